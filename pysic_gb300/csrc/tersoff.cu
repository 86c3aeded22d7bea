// tersoff.cu -- pair-bond-order (Tersoff) energy and forces.
//
// Replaces, for bond-order scaled pair potentials, core_evaluate_local_doublet_
// energy_B / _forces_B (Core.f90:4257-4385, 5371-5606) together with
// core_calculate_pair_bond_order_factor (2439-2637),
// core_post_process_pair_bond_order_factor (2763-2807) and
// core_add_pair_bond_order_forces (4952-5353).
//
// Energy of an unordered pair i-j in the reference:
//     V(r) f(r) (B_ij + B_ji)/2 + (plain pair terms) V f
// = sum over the two ordered bonds of  1/2 V f B_ij  (+ 1/2 of the plain terms),
// with B_ij = B(zeta_ij), zeta_ij = sum_k xi_ijk g_ijk over i's neighbours.
//
// Two kernels, one group of G lanes per atom, one lane per ordered bond:
//  bond_pass   per bond i->j: zeta_ij, B, dB/dzeta, the bond energy, the radial
//              pair force and the three-body gradient of zeta_ij.  The part that
//              acts on i is summed in registers; the parts that act on j and on
//              each k are written to per-bond / per-triplet slots (FP32 in the
//              mixed path) so that no other atom's force is touched.
//  gather_pass per atom m: own centre part + the j-parts of the bonds i->m
//              (through the reverse-bond index) + the k-parts of every bond
//              i->x with k = m.  No atomics: each force is produced by exactly
//              one lane group, bit-reproducibly.
// The virial uses the reference's convention sum(r_rel (x) F): pair part
// r_ij (x) F_j, three-body part r_ij (x) F_j + r_ik (x) F_k (Core.f90:5146-5172).
//
// Precision.  The FP64 path computes every bond vector from the FP64 positions
// like separation_vector (Geometry.f90:449-466).  The mixed path keeps FP64 out
// of the per-term work: bond vectors are taken once per short-list build in
// FP64 (rounded to FP32), and every evaluation adds the FP32 displacement of
// both atoms since that build (prepared per atom in FP64 by disp_pass).  Lane
// partial sums are FP32; the lanes of an atom are combined exactly in integer
// fixed point and the energy / virial totals are exact 128-bit integers
// (fixed.cuh), so the mixed path issues no FP64 instruction at all.
// Per bond, the staging step keeps the unit vector, 1/r and (when every j
// type shares it) the bond-order cutoff factor f(r_ik), which every triplet
// through the bond reuses.
#include <functional>
#include <type_traits>

#include "args.cuh"
#include "bond.cuh"
#include "common.cuh"
#include "kernels.cuh"
#include "bond_body.cuh"

namespace pg {


// Electronegativities of the Tersoff-scaled charge-dependent and product
// terms (core_evaluate_local_doublet_electronegativities_B with bond-order
// factors, Core.f90:5622-5775): per atom i and short-list entry i -> j,
// chi_i += -dV/dq_i f (B_ij + B_ji) / 2, the B of both directions kept by the
// bond pass (B[e], B[rev e]).  One thread per atom; the sum is a gather.
template <typename R>
__global__ void bond_chi(const __grid_constant__ BondArgs A, const R* __restrict__ B, int first,
                         double* __restrict__ out_chi) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    if (A.skip && *A.skip) return;
    const PairT<R>* terms = (const PairT<R>*)A.terms;
    const int ti = A.type[i];
    const int s = A.start[i], s1 = A.start[i + 1];
    double xi = 0, yi = 0, zi = 0;
    if constexpr (sizeof(R) == 8) {
        xi = A.pos[3 * i];
        yi = A.pos[3 * i + 1];
        zi = A.pos[3 * i + 2];
    }
    R chi = 0;
    for (int e = s; e < s1; ++e) {
        const auto g = bond_vector<R>(A, i, e, xi, yi, zi);
        const R r = g.w;
        if (r == R(0)) continue;
        const int tj = A.etype[e];
        const int2 ix = A.index[ti * A.T + tj];
        const R bsum = R(0.5) * (B[e] + B[A.rev[e]]);
        for (int t = ix.x; t < ix.x + ix.y; ++t) {
            const PairT<R>& PT = terms[t];
            if (!PT.in_bond_kernel || PT.group < 0 || !(PT.kind >= 7 || PT.nmul > 0) || !(r < PT.rc)) continue;
            R V, dV, en;
            bond_charge_term<R>(A, PT, terms, i, e, ti, tj, r, V, dV, en);
            chi += en * bsum;
        }
    }
    out_chi[i] = first ? (double)chi : out_chi[i] + (double)chi;
}

__global__ void disp_pass(const __grid_constant__ DispArgs A) {
    pdl_trigger();
    disp_body(A, blockIdx.x * blockDim.x + threadIdx.x);
}
__global__ void disp_pass_batch(const DispArgs* __restrict__ sys, const int2* __restrict__ tiles, int ntiles) {
    pdl_trigger();
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 tl = tiles[t];
        disp_body(sys[tl.x], tl.y * blockDim.x + threadIdx.x);
    }
}

// One system: the kernel argument is read in place (no copy to local memory).
template <typename R, int G, bool SPEC>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 7 : 4) bond_pass(const __grid_constant__ BondArgs A) {
    bond_body<R, G, SPEC>(A, blockIdx.x, gridDim.x);
}
template <typename R, int G>
__global__ void __launch_bounds__(128) gather_pass(const __grid_constant__ BondArgs A) {
    gather_body<R, G>(A, blockIdx.x, gridDim.x);
}

// Many systems in one launch: tiles[t] = (system, block of that system); the
// resident blocks walk the tile list.
template <typename R, int G, bool SPEC>
__global__ void __launch_bounds__(128, sizeof(R) == 4 ? 7 : 4)
    bond_pass_batch(const BondArgs* __restrict__ sys, const int2* __restrict__ tiles, int ntiles) {
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 tl = tiles[t];
        bond_body<R, G, SPEC>(sys[tl.x], tl.y, sys[tl.x].nblocks);
        __syncthreads();
    }
}
template <typename R, int G>
__global__ void __launch_bounds__(128)
    gather_pass_batch(const BondArgs* __restrict__ sys, const int2* __restrict__ tiles, int ntiles) {
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int2 tl = tiles[t];
        gather_body<R, G>(sys[tl.x], tl.y, sys[tl.x].nblocks);
    }
}

// blocks of 128 threads over n atoms at G lanes per atom (the triplet tile: 16
// lanes, 8 atoms per block)
int bond_blocks(int n, int G) {
    const int ap = G == PG_LANES_TRIPLET ? 8 : 128 / G;
    return (n + ap - 1) / ap;
}

// Entries per section of the bond-pass scratch: the short list's length with
// headroom, kept while the list fits, so that the sections (and the captured
// kernels' arguments) stay put across list rebuilds of similar length.
static size_t bond_stride(pg_context* ctx) {
    const long long need = std::max<long long>(ctx->sh_total, 1);
    if (ctx->bo_stride < need) ctx->bo_stride = need + need / 4 + 64;
    return (size_t)ctx->bo_stride;
}

void prepare_bond_scratch(pg_context* ctx, int precision) {
    const size_t ne = bond_stride(ctx);
    if (ctx->have_bond_charge_terms) ctx->bo_b.resize(ne);
    // per short-list entry: bond geometry | force from the partner's bonds | k-part
    // sums | unstaged j parts
    if (precision == PG_PREC_FP64) ctx->bo_fj64.resize(4 * ne);
    else ctx->bo_fj.resize(4 * ne);
    ctx->bo_fc.resize(3 * (size_t)std::max(ctx->n, 1));
}

DispArgs make_disp_args(pg_context* ctx, F4* d, const int* skip, FxAcc* zero8) {
    DispArgs A{};
    A.n = ctx->n;
    A.pos = ctx->pos.p;
    A.pos0 = ctx->pos0.p;
    A.q = ctx->charge.p;
    A.d = d;
    A.skip = skip;
    A.zero8 = zero8;
    return A;
}

BondArgs make_bond_args(pg_context* ctx, int precision, int flags, bool first_f, FxAcc* acc) {
    BondArgs A{};
    A.n = ctx->n;
    A.T = std::max(ctx->n_types, 1);
    A.pos = ctx->pos.p;
    A.type = ctx->type.p;
    A.C = cell_kernel_view(ctx->cell);
    A.start = ctx->sh_start.p;
    A.idx = ctx->sh_idx.p;
    A.off = ctx->sh_off.p;
    A.rev = ctx->sh_rev.p;
    A.etype = ctx->sh_type.p;
    A.order = ctx->sh_order.p;
    A.slot = ctx->sh_slot.p;
    A.n_terms = ctx->n_pair_terms;
    A.index = ctx->d_pair_index.p;
    A.bcut_uniform = ctx->bcut_uniform ? 1 : 0;
    A.spec = ctx->spec_ok ? 1 : 0;
    A.spec_nterm = ctx->spec_nterm;
    A.spec_bomask = ctx->spec_bomask;
    for (int q = 0; q < SP_COUNT; ++q) {
        A.spd[q] = ctx->spec[q];
        A.spf[q] = (float)ctx->spec[q];
    }
    A.flags = flags;
    A.first_f = first_f;
    const size_t ne = bond_stride(ctx);
    if (precision == PG_PREC_FP64) {
        A.terms = ctx->d_pair_terms.p;
        A.tab = ctx->d_tab64.p;
        A.trip = ctx->d_trip.p;
        A.post = ctx->d_post.p;
        A.maxbr = ctx->d_maxbr.p;
        A.bcut = ctx->d_bcut.p;
        A.geo = ctx->bo_fj64.p;
        A.fj = ctx->bo_fj64.p + ne;
        A.kacc = ctx->bo_fj64.p + 2 * ne;
        A.bscr = ctx->bo_fj64.p + 3 * ne;
    } else {
        A.terms = ctx->d_pair_terms32.p;
        A.tab = ctx->d_tab32.p;
        A.trip = ctx->d_trip32.p;
        A.post = ctx->d_post32.p;
        A.maxbr = ctx->d_maxbr32.p;
        A.bcut = ctx->d_bcut32.p;
        A.geo = ctx->bo_fj.p;
        A.fj = ctx->bo_fj.p + ne;
        A.kacc = ctx->bo_fj.p + 2 * ne;
        A.bscr = ctx->bo_fj.p + 3 * ne;
        A.sep0 = ctx->sh_sep0.p;
        A.disp = ctx->disp32.p;
    }
    A.fc = ctx->bo_fc.p;
    A.out_f = ctx->out_f.p;
    A.acc = acc;
    A.zeta_out = nullptr;
    A.q = ctx->charge.p;
    A.b_out = nullptr;
    return A;
}

template <typename R, int G>
static void launch_pair(const BondArgs& A, int n, cudaStream_t st, bool forces, const std::function<void()>& between) {
    // each pass may start while its predecessor drains (programmatic dependent launch)
    const dim3 grid(bond_blocks(n, G)), block(128);
    if (A.spec) launch_pdl(bond_pass<R, G, true>, grid, block, st, A);
    else launch_pdl(bond_pass<R, G, false>, grid, block, st, A);
    between();
    if (forces) launch_pdl(gather_pass<R, G>, grid, block, st, A);
}

void launch_tri_pass(const BondArgs& A, int n, int precision, cudaStream_t st);  // tersoff_tri.cu
void launch_tri_batch(const BondArgs* sys, const int2* tiles, int ntiles, int grid, int precision, bool spec,
                      cudaStream_t st);

template <typename R>
static void launch_by_lanes(const BondArgs& A, int n, cudaStream_t st, int G, bool forces,
                            const std::function<void()>& between) {
    if (G == PG_LANES_TRIPLET) {  // triplet tile, then the 4-lane gather
        launch_tri_pass(A, n, sizeof(R) == 8 ? PG_PREC_FP64 : PG_PREC_MIXED, st);
        between();
        if (forces) launch_pdl(gather_pass<R, 4>, dim3(bond_blocks(n, 4)), dim3(128), st, A);
        return;
    }
    switch (G) {
        case 4: launch_pair<R, 4>(A, n, st, forces, between); break;
        case 8: launch_pair<R, 8>(A, n, st, forces, between); break;
        case 16: launch_pair<R, 16>(A, n, st, forces, between); break;
        default: launch_pair<R, 32>(A, n, st, forces, between); break;
    }
}

// `between` runs between the two passes
void launch_bond_order_impl(pg_context* ctx, int precision, int flags, bool first_f, int G, FxAcc* acc,
                            const std::function<void()>& between, const int* skip, HostTotals* pub,
                            const int* pub_bad) {
    prepare_bond_scratch(ctx, precision);
    BondArgs A = make_bond_args(ctx, precision, flags, first_f, acc);
    A.skip = skip;
    A.pub = pub;
    A.pub_bad = pub_bad;
    if (ctx->have_bond_charge_terms) A.b_out = ctx->bo_b.p;  // kept for bond_chi
    const bool forces = (flags & PG_WANT_FORCES) != 0;
    if (precision == PG_PREC_FP64) launch_by_lanes<double>(A, ctx->n, ctx->stream, G, forces, between);
    else launch_by_lanes<float>(A, ctx->n, ctx->stream, G, forces, between);
    PG_CHECK_LAUNCH();
    ctx->launches += forces ? 2 : 1;
}

// The two passes on scratch the caller provides instead of the context's
// buffers (the no-allocation entry point): bonds holds 4 records per short-list
// entry, fc 3 values per atom, disp (mixed path) one record per atom.  Energy
// and virial go to acc, forces to out_f (written).
void launch_bond_order_scratch(pg_context* ctx, int precision, int G, void* bonds, void* fc, F4* disp, FxAcc* acc,
                               double* out_f) {
    BondArgs A = make_bond_args(ctx, precision, PG_WANT_ENERGY | PG_WANT_FORCES, true, acc);
    const size_t ne = (size_t)std::max<long long>(ctx->sh_total, 1);
    const size_t rec = precision == PG_PREC_FP64 ? sizeof(D4) : sizeof(F4);
    A.geo = bonds;
    A.fj = (char*)bonds + ne * rec;
    A.kacc = (char*)bonds + 2 * ne * rec;
    A.bscr = (char*)bonds + 3 * ne * rec;
    A.fc = fc;
    A.out_f = out_f;
    auto none = [] {};
    if (precision == PG_PREC_FP64) {
        launch_by_lanes<double>(A, ctx->n, ctx->stream, G, true, none);
    } else {
        disp_pass<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(make_disp_args(ctx, disp, nullptr, nullptr));
        A.disp = disp;
        launch_by_lanes<float>(A, ctx->n, ctx->stream, G, true, none);
    }
    PG_CHECK_LAUNCH();
}

// The bond pass for its B values only (no totals, no forces): the
// electronegativity pass of a relaxation, whose positions stay fixed, needs
// them once per loop.
void launch_bond_b(pg_context* ctx, int precision, int G, const int* skip) {
    prepare_bond_scratch(ctx, precision);
    BondArgs A = make_bond_args(ctx, precision, PG_WANT_ENERGY, true, nullptr);
    A.skip = skip;
    A.b_out = ctx->bo_b.p;
    auto none = [] {};
    if (precision == PG_PREC_FP64) launch_by_lanes<double>(A, ctx->n, ctx->stream, G, false, none);
    else launch_by_lanes<float>(A, ctx->n, ctx->stream, G, false, none);
    PG_CHECK_LAUNCH();
    ctx->launches++;
}

// bond_chi into out_chi (written when first, added otherwise)
void launch_bond_chi(pg_context* ctx, int precision, bool first, const int* skip) {
    BondArgs A = make_bond_args(ctx, precision, PG_WANT_ENEGS, true, nullptr);
    A.skip = skip;
    const int blocks = (ctx->n + 127) / 128;
    if (precision == PG_PREC_FP64)
        bond_chi<double><<<blocks, 128, 0, ctx->stream>>>(A, (const double*)ctx->bo_b.p, first ? 1 : 0, ctx->out_chi.p);
    else
        bond_chi<float><<<blocks, 128, 0, ctx->stream>>>(A, (const float*)ctx->bo_b.p, first ? 1 : 0, ctx->out_chi.p);
    PG_CHECK_LAUNCH();
    ctx->launches++;
}

void launch_disp(pg_context* ctx, const int* skip, FxAcc* zero8, bool commit) {
    ctx->disp32.resize((size_t)std::max(ctx->n, 1));
    DispArgs A = make_disp_args(ctx, ctx->disp32.p, skip, zero8);
    if (commit) {  // the staged coordinates (pos_in) committed by the same pass
        A.pos_in = ctx->pos_in.p;
        A.pos_out = ctx->pos.p;
        A.pos_prev = ctx->pos_prev.p;
        A.bad = ctx->pos_bad.p;
    }
    disp_pass<<<(ctx->n + 255) / 256, 256, 0, ctx->stream>>>(A);
    PG_CHECK_LAUNCH();
    ctx->launches++;
}

void bond_zeta_diag(pg_context* ctx) {
    prepare_bond_scratch(ctx, PG_PREC_FP64);
    ctx->bo_zeta.resize((size_t)std::max<long long>(ctx->sh_total, 1));
    ctx->bo_zeta.zero(ctx->stream);
    BondArgs A = make_bond_args(ctx, PG_PREC_FP64, PG_WANT_ENERGY, true, nullptr);
    A.zeta_out = ctx->bo_zeta.p;
    bond_pass<double, 8, false><<<bond_blocks(ctx->n, 8), 128, 0, ctx->stream>>>(A);
    PG_CHECK_LAUNCH();
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
}

void launch_bond_batch(const BondArgs* sys, const int2* tiles, int ntiles, int grid, int precision, int G, bool spec,
                       bool forces, cudaStream_t st) {
    const dim3 g(grid), b(128);
    if (G == PG_LANES_TRIPLET) {  // triplet tile (8 atoms per tile), then the gather
        launch_tri_batch(sys, tiles, ntiles, grid, precision, spec, st);
        if (forces) {  // 16 lanes per atom: the gather's tiles are the bond tiles (8 atoms each)
            if (precision == PG_PREC_FP64) launch_pdl(gather_pass_batch<double, 16>, g, b, st, sys, tiles, ntiles);
            else launch_pdl(gather_pass_batch<float, 16>, g, b, st, sys, tiles, ntiles);
        }
        PG_CHECK_LAUNCH();
        return;
    }
    auto go = [&](auto rtag, auto gtag) {
        using R = decltype(rtag);
        constexpr int GG = decltype(gtag)::value;
        if (spec) launch_pdl(bond_pass_batch<R, GG, true>, g, b, st, sys, tiles, ntiles);
        else launch_pdl(bond_pass_batch<R, GG, false>, g, b, st, sys, tiles, ntiles);
        if (forces) launch_pdl(gather_pass_batch<R, GG>, g, b, st, sys, tiles, ntiles);
    };
    auto by_lanes = [&](auto rtag) {
        switch (G) {
            case 4: go(rtag, std::integral_constant<int, 4>{}); break;
            case 8: go(rtag, std::integral_constant<int, 8>{}); break;
            case 16: go(rtag, std::integral_constant<int, 16>{}); break;
            default: go(rtag, std::integral_constant<int, 32>{}); break;
        }
    };
    if (precision == PG_PREC_FP64) by_lanes(double{});
    else by_lanes(float{});
    PG_CHECK_LAUNCH();
}

void launch_disp_batch(const DispArgs* sys, const int2* tiles, int ntiles, int grid, cudaStream_t st) {
    disp_pass_batch<<<grid, 256, 0, st>>>(sys, tiles, ntiles);
    PG_CHECK_LAUNCH();
}

}  // namespace pg
