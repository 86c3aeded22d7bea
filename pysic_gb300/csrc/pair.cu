// pair.cu -- pair potentials, real-space Ewald and single-atom charge terms.
//
// Replaces, for non-bond-order terms, the doublet part of
// core_loop_over_local_interactions (Core.f90:3249-3946 with
// core_evaluate_local_doublet_energy_B / _forces_B, 4257-4385 and 5371-5606),
// the inline real-space Ewald sum (Core.f90:3416-3460) and the singlet loop
// (core_evaluate_local_singlet, 4095-4239).
//
// The reference visits each pair once (pick, Geometry.f90:648-676) and
// scatters the force to both atoms.  Here a group of G lanes owns atom i and
// walks i's full list, so each pair is evaluated from both ends: atom i takes
// half the pair energy, its own force and half the pair virial.  Every force
// and electronegativity is a gather; no atomics, bit-reproducible.
#include <algorithm>

#include "args.cuh"
#include "common.cuh"
#include "kernels.cuh"
#include "pairvec.cuh"
#include "atomfactor.cuh"
#include "pair_body.cuh"

namespace pg {


template <typename R, int G, bool AF>
__global__ void __launch_bounds__(256) pair_kernel(const __grid_constant__ PairArgs A) {
    pair_body<R, G, AF>(A, blockIdx.x);
}

// many systems in one launch (tiles[t] = system, block of that system)
template <typename R, int G>
__global__ void __launch_bounds__(256)
    pair_kernel_batch(const PairArgs* __restrict__ sys, const int2* __restrict__ tiles, int ntiles) {
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 tl = tiles[t];
        pair_body<R, G>(sys[tl.x], tl.y);
        __syncthreads();
    }
}

// Relaxation loops keep the positions fixed, so the real-space Ewald part of
// the electronegativities, chi_i -= q_j erfc(r_ij / (sqrt2 sigma)) / (4 pi eps
// r_ij) (Core.f90:3453-3456), is a fixed sparse matrix over the full list.
// chi_cache_build stores its entries once (the same arithmetic as the pair
// kernel: 0 beyond the cutoff or at r = 0); chi_cache_apply forms
// chi = -sum_e k_e q_j plus the charge_self terms per step (energy, forces and
// the charge-independent pair terms are not wanted there).
template <typename R, int G>
__global__ void __launch_bounds__(256) chi_cache_build(const __grid_constant__ PairArgs A, R* __restrict__ kc) {
    const int lane = threadIdx.x % G;
    const int i = blockIdx.x * (blockDim.x / G) + threadIdx.x / G;
    if (i >= A.n) return;
    double xi = 0, yi = 0, zi = 0;
    if constexpr (sizeof(R) == 8) {
        xi = A.pos[3 * i];
        yi = A.pos[3 * i + 1];
        zi = A.pos[3 * i + 2];
    }
    const R ew_rc = (R)A.ew_rc, ew_is2 = (R)A.ew_is2, ew_k = (R)A.ew_k;
    for (int e = A.start[i] + lane; e < A.start[i + 1]; e += G) {
        R x, y, z;
        pair_vector<R>(A, i, e, xi, yi, zi, x, y, z);
        const R r = sqrt_(x * x + y * y + z * z);
        R k = R(0);
        if (A.ewald && r != R(0) && r < ew_rc) k = ew_k * erfc_(r * ew_is2) * (R(1) / r);
        kc[e] = k;
    }
}

template <typename R, int G>
__global__ void __launch_bounds__(256) chi_cache_apply(const __grid_constant__ PairArgs A, const R* __restrict__ kc) {
    if (A.skip && *A.skip) return;
    const int lane = threadIdx.x % G;
    const int i = blockIdx.x * (blockDim.x / G) + threadIdx.x / G;
    const bool act = i < A.n;
    R chi = 0;
    if (act)
        for (int e = A.start[i] + lane; e < A.start[i + 1]; e += G) chi -= kc[e] * charge_of<R>(A, A.idx[e]);
    double cs = 0.0;
    if (act && lane == 0) {
        const int2 sx = A.sindex[A.type[i]];
        for (int t = sx.x; t < sx.x + sx.y; ++t) {
            const SingleTerm S = A.sterms[t];
            if (S.kind == 0) cs += -(S.p[0] * S.n * powi_(A.charge[i], S.n - 1));
        }
    }
    auto schi = group_sum_f<G>(chi);
    if (act && lane == 0) {
        if constexpr (sizeof(R) == 4) schi.f += fix_from_double(cs);
        else schi.s += cs;
        store_sum(A.out_chi + i, schi, true);
    }
}

// atoms per block: enough blocks to cover every SM twice, at most 256 threads
int pair_atoms_per_block(int n, int G) {
    const int maxa = 256 / G;
    const int sms = sm_count();
    int a = (n + 2 * sms - 1) / (2 * sms);
    if (a < 1) a = 1;
    if (a > maxa) a = maxa;
    const int warp_atoms = 32 / G > 0 ? 32 / G : 1;  // whole warps
    a = ((a + warp_atoms - 1) / warp_atoms) * warp_atoms;
    return a > maxa ? maxa : a;
}

int pair_kernel_blocks(int n, int G) {
    const int a = pair_atoms_per_block(n, G);
    return (n + a - 1) / a;
}

PairArgs make_pair_args(pg_context* ctx, int precision, int flags, bool first_f, bool first_chi, FxAcc* acc,
                        const int* skip) {
    PairArgs A{};
    A.skip = skip;
    A.n = ctx->n;
    A.T = std::max(ctx->n_types, 1);
    A.pos = ctx->pos.p;
    A.charge = ctx->charge.p;
    A.type = ctx->type.p;
    A.C = cell_kernel_view(ctx->cell);
    A.start = ctx->nb_start.p;
    A.idx = ctx->nb_idx.p;
    A.off = ctx->nb_off.p;
    A.terms = precision == PG_PREC_FP64 ? (const void*)ctx->d_pair_terms.p : (const void*)ctx->d_pair_terms32.p;
    A.tab = precision == PG_PREC_FP64 ? (const void*)ctx->d_tab64.p : (const void*)ctx->d_tab32.p;
    A.index = ctx->d_pair_index.p;
    A.sterms = ctx->d_single_terms.p;
    A.sindex = ctx->d_single_index.p;
    A.ewald = ctx->ewald ? 1 : 0;
    A.qpair = ctx->have_charge_pairs ? 1 : 0;
    if (ctx->ewald) {
        const double pi = 3.14159265358979323846;
        A.ew_rc = ctx->ew_rc;
        A.ew_is2 = 1.0 / (std::sqrt(2.0) * ctx->ew_sigma);
        A.ew_k = 1.0 / (4.0 * pi * ctx->ew_eps);
        A.ew_c2 = 2.0 / (std::sqrt(2.0 * pi) * ctx->ew_sigma);
        A.ew_isq2 = A.ew_is2 * A.ew_is2;
    }
    A.flags = flags;
    A.first_f = first_f;
    A.first_chi = first_chi;
    A.out_f = ctx->out_f.p;
    A.out_chi = ctx->out_chi.p;
    A.acc = acc;
    A.sep0 = ctx->nb_sep0.p;
    A.disp = ctx->disp32.p;
    set_atom_factor_args(ctx, precision, A);
    return A;
}

void launch_pair_kernel_skip(pg_context* ctx, int precision, int flags, bool first_f, bool first_chi, int G,
                             FxAcc* acc, const int* skip) {
    const PairArgs A = make_pair_args(ctx, precision, flags, first_f, first_chi, acc, skip);
    const int nbk = pair_kernel_blocks(ctx->n, G);
    const int threads = pair_atoms_per_block(ctx->n, G) * G;
    cudaStream_t st = ctx->stream;
#define PG_PAIR_LAUNCH(R_, G_)                                                   \
    do {                                                                         \
        if (A.af_fused && (flags & PG_WANT_FORCES))                              \
            pair_kernel<R_, G_, true><<<nbk, threads, 0, st>>>(A);               \
        else                                                                     \
            pair_kernel<R_, G_, false><<<nbk, threads, 0, st>>>(A);              \
    } while (0)
    if (precision == PG_PREC_FP64) {
        if (G == 8) PG_PAIR_LAUNCH(double, 8);
        else if (G == 16) PG_PAIR_LAUNCH(double, 16);
        else PG_PAIR_LAUNCH(double, 32);
    } else {
        if (G == 8) PG_PAIR_LAUNCH(float, 8);
        else if (G == 16) PG_PAIR_LAUNCH(float, 16);
        else PG_PAIR_LAUNCH(float, 32);
    }
#undef PG_PAIR_LAUNCH
    PG_CHECK_LAUNCH();
    ctx->launches++;
}

void launch_pair_batch(const PairArgs* sys, const int2* tiles, int ntiles, int grid, int threads, int precision, int G,
                       cudaStream_t st) {
#define PG_PAIR_BATCH(R_, G_) pair_kernel_batch<R_, G_><<<grid, threads, 0, st>>>(sys, tiles, ntiles)
    if (precision == PG_PREC_FP64) {
        if (G == 8) PG_PAIR_BATCH(double, 8);
        else if (G == 16) PG_PAIR_BATCH(double, 16);
        else PG_PAIR_BATCH(double, 32);
    } else {
        if (G == 8) PG_PAIR_BATCH(float, 8);
        else if (G == 16) PG_PAIR_BATCH(float, 16);
        else PG_PAIR_BATCH(float, 32);
    }
#undef PG_PAIR_BATCH
    PG_CHECK_LAUNCH();
}

// the cache of the current list generation and positions (called at the
// start of a relaxation loop); false when the electronegativities have other
// pair contributions (charge_pair), which then need the full pair kernel
bool chi_cache_prepare(pg_context* ctx, int precision) {
    if (ctx->have_charge_pairs || ctx->n == 0) return false;
    const int G = pair_lanes_for(ctx);
    const PairArgs A = make_pair_args(ctx, precision, PG_WANT_ENEGS, true, true, nullptr, nullptr);
    ctx->chi_k.resize((size_t)std::max<long long>(ctx->nb_total, 1));
    const int nbk = pair_kernel_blocks(ctx->n, G), threads = pair_atoms_per_block(ctx->n, G) * G;
    cudaStream_t st = ctx->stream;
#define PG_CACHE_BUILD(R_, G_) chi_cache_build<R_, G_><<<nbk, threads, 0, st>>>(A, (R_*)ctx->chi_k.p)
    if (precision == PG_PREC_FP64) {
        if (G == 8) PG_CACHE_BUILD(double, 8);
        else if (G == 16) PG_CACHE_BUILD(double, 16);
        else PG_CACHE_BUILD(double, 32);
    } else {
        if (G == 8) PG_CACHE_BUILD(float, 8);
        else if (G == 16) PG_CACHE_BUILD(float, 16);
        else PG_CACHE_BUILD(float, 32);
    }
#undef PG_CACHE_BUILD
    PG_CHECK_LAUNCH();
    return true;
}

void launch_chi_cache_apply(pg_context* ctx, int precision, const int* skip) {
    const int G = pair_lanes_for(ctx);
    const PairArgs A = make_pair_args(ctx, precision, PG_WANT_ENEGS, true, true, nullptr, skip);
    const int nbk = pair_kernel_blocks(ctx->n, G), threads = pair_atoms_per_block(ctx->n, G) * G;
    cudaStream_t st = ctx->stream;
#define PG_CACHE_APPLY(R_, G_) chi_cache_apply<R_, G_><<<nbk, threads, 0, st>>>(A, (const R_*)ctx->chi_k.p)
    if (precision == PG_PREC_FP64) {
        if (G == 8) PG_CACHE_APPLY(double, 8);
        else if (G == 16) PG_CACHE_APPLY(double, 16);
        else PG_CACHE_APPLY(double, 32);
    } else {
        if (G == 8) PG_CACHE_APPLY(float, 8);
        else if (G == 16) PG_CACHE_APPLY(float, 16);
        else PG_CACHE_APPLY(float, 32);
    }
#undef PG_CACHE_APPLY
    PG_CHECK_LAUNCH();
    ctx->launches++;
}

void launch_pair_kernel_impl(pg_context* ctx, int precision, int flags, bool first_f, bool first_chi, int G,
                             FxAcc* acc) {
    launch_pair_kernel_skip(ctx, precision, flags, first_f, first_chi, G, acc, nullptr);
}

}  // namespace pg
