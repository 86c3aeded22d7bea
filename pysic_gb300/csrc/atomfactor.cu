// atomfactor.cu -- per-atom (level-1) bond-order factors: neighbors,
// power_bond, table_bond, c_scale, sqrt_scale, table_scale.
//
// Replaces, for Coordinators of per-atom factors, core_calculate_bond_order_
// factors (Core.f90:2015-2404, the two-target level-1 part),
// core_post_process_bond_order_factors (2671-2735) and
// core_add_bond_order_forces (4745-4933), as the singlet and doublet loops use
// them (core_evaluate_local_singlet, 4095-4239; core_evaluate_local_doublet_
// energy_B / _forces_B, 4257-4385, 5371-5606).
//
// In the reference an atom's raw sum b_i collects, over the pairs the loop
// picks (pick, Geometry.f90:648-676), the factor c(r) of every record whose
// position 1 holds atom1's element and position 2 atom2's, added to both
// atoms; B_i = post(b_i) with the first scaler of the atom's element in the
// group.  A term scaled by the group multiplies its energy by B_i (single-atom)
// or (B_i + B_j)/2 (pair), and its prefactor P_i (the singlet's V, or half of
// each pair's V f) multiplies -grad B_i, taken over all of atom i's neighbours
// (no pick) with the records of atom i's element at position 1.
//
// Three launches, one group of G lanes per atom, every result a gather:
//   af_sum     b_i over i's full list (the pick decides which atom is atom1,
//              so which records apply), B_i and S_i = dB/db at b_i
//   pair       (pair.cu) the scaled energies and forces, and W_i = S_i P_i
//   af_force   F_k = sum_j c'(r_kj) u_kj [W_k (records k, j) + W_j (records
//              j, k)], u_kj the unit vector from k to j, a record of both
//              lists evaluated once; virial of atom k's own terms,
//              sep (x) (-W_k c' u) as the reference sums it
// No atomics; with a fixed tile the results are bit-reproducible.
#include <algorithm>
#include <map>
#include <vector>

#include "args.cuh"
#include "common.cuh"
#include "kernels.cuh"
#include "pairvec.cuh"
#include "atomfactor.cuh"

namespace pg {

namespace {

template <typename R>
__device__ __forceinline__ void add_at(R (&a)[PG_MAX_AGROUPS], int g, R v) {
#pragma unroll
    for (int q = 0; q < PG_MAX_AGROUPS; ++q)
        if (q == g) a[q] += v;
}

template <typename R, int G>
__global__ void __launch_bounds__(256) af_sum(const __grid_constant__ PairArgs A) {
    if (A.skip && *A.skip) return;
    const int lane = threadIdx.x % G;
    const int i = blockIdx.x * (blockDim.x / G) + threadIdx.x / G;
    const bool act = i < A.n;
    R b[PG_MAX_AGROUPS] = {};
    int ti = 0;
    if (act) {
        ti = A.type[i];
        double xi = 0, yi = 0, zi = 0;
        if constexpr (sizeof(R) == 8) {
            xi = A.pos[3 * i];
            yi = A.pos[3 * i + 1];
            zi = A.pos[3 * i + 2];
        }
        const AfT<R>* recs = (const AfT<R>*)A.af;
        for (int e = A.start[i] + lane; e < A.start[i + 1]; e += G) {
            const int j = A.idx[e];
            R x, y, z;
            pair_vector<R>(A, i, e, xi, yi, zi, x, y, z);
            const R r = sqrt_(x * x + y * y + z * z);
            if (r == R(0)) continue;
            const int tj = A.type[j];
            // the reference visits the pair once, from the atom pick makes atom1
            const bool first = pick(i, j, A.off[3 * e], A.off[3 * e + 1], A.off[3 * e + 2]);
            const int2 ix = A.af_index[first ? ti * A.T + tj : tj * A.T + ti];
            const R ir = rcp_(r);
            for (int t = ix.x; t < ix.x + ix.y; ++t) {
                const AfT<R> F = recs[t];
                if (!(r < F.rc)) continue;
                R c, dc;
                af_term<R>(F, r, ir, (const R*)A.tab, c, dc);
                add_at<R>(b, F.group, c);
            }
        }
    }
    R* Bv = (R*)A.afB;
    R* Sv = (R*)A.afS;
    const AfPostT<R>* post = (const AfPostT<R>*)A.af_post;
#pragma unroll
    for (int g = 0; g < PG_MAX_AGROUPS; ++g) {
        if (g >= A.ng) break;
        const auto s = group_sum_f<G>(b[g]);
        if (!(act && lane == 0)) continue;
        const R raw = (R)s.d();
        const AfPostT<R> P = post[g * A.T + ti];
        R B, S;
        if (P.kind == 3) {  // sqrt_scale: epsilon sqrt(b), 0 for b <= 0
            if (raw <= R(0)) {
                B = R(0);
                S = R(0);
            } else {
                const R sq = sqrt_(raw);
                B = P.p[0] * sq;
                S = P.p[0] / (R(2) * sq);
            }
        } else if (P.kind == 5) {  // table_scale: 0 for b <= 0, the last value (unscaled) beyond the range
            const R* T = (const R*)A.tab + 2 * (long long)P.t0;
            if (raw <= R(0)) {
                B = R(0);
                S = R(0);
            } else if (raw >= P.p[2]) {
                B = T[2 * (P.tn - 1)];
                S = R(0);
            } else {
                af_hermite<R>(T, P.tn, P.p[2], P.p[3], raw, B, S);
            }
        } else if (P.kind == 2) {  // c_scale: epsilon dN / (1 + exp(gamma dN)), dN = C (b - N) > min
            const R dN = (raw - P.p[1]) * P.p[2];
            if (dN > P.p[4]) {
                const R ex = exp_(P.p[3] * dN), ie = R(1) / (R(1) + ex);
                B = P.p[0] * dN * ie;
                S = P.p[0] * P.p[2] * (ie - dN * ie * ie * P.p[3] * ex);
            } else {
                B = R(0);
                S = R(0);
            }
        } else {
            B = raw;
            S = R(1);
        }
        Bv[(size_t)g * A.n + i] = B;
        Sv[(size_t)g * A.n + i] = S;
        if (A.af_fused) {
            // no scaled pair term: the prefactor is the scaled singlets' V, known
            // here, and the pair kernel adds the factor forces in its own pass
            double V = 0.0;
            const int2 sx = A.sindex[ti];
            for (int t = sx.x; t < sx.x + sx.y; ++t) {
                const SingleTerm T1 = A.sterms[t];
                if (T1.agroup != g) continue;
                V += T1.kind == 1 ? T1.p[0]
                                  : -(T1.p[0] * A.pos[3 * i] + T1.p[1] * A.pos[3 * i + 1] + T1.p[2] * A.pos[3 * i + 2]);
            }
            ((R*)A.afW)[(size_t)g * A.n + i] = (R)((double)S * V);
        }
    }
}

template <typename R, int G>
__global__ void __launch_bounds__(256) af_force(const __grid_constant__ PairArgs A) {
    __shared__ Fx128 wsum[256 / 32][7];
    __shared__ unsigned done;
    if (threadIdx.x == 0) done = 0u;
    __syncthreads();
    if (A.skip && *A.skip) return;
    const int lane = threadIdx.x % G;
    const int k = blockIdx.x * (blockDim.x / G) + threadIdx.x / G;
    const bool act = k < A.n;
    const R* W = (const R*)A.afW;
    R fx = 0, fy = 0, fz = 0;
    R w0 = 0, w1 = 0, w2 = 0, w3 = 0, w4 = 0, w5 = 0;
    if (act) {
        const int tk = A.type[k];
        R wk[PG_MAX_AGROUPS] = {};
#pragma unroll
        for (int g = 0; g < PG_MAX_AGROUPS; ++g)
            if (g < A.ng) wk[g] = W[(size_t)g * A.n + k];
        double xk = 0, yk = 0, zk = 0;
        if constexpr (sizeof(R) == 8) {
            xk = A.pos[3 * k];
            yk = A.pos[3 * k + 1];
            zk = A.pos[3 * k + 2];
        }
        for (int e = A.start[k] + lane; e < A.start[k + 1]; e += G) {
            const int j = A.idx[e];
            R x, y, z;
            pair_vector<R>(A, k, e, xk, yk, zk, x, y, z);
            const R r = sqrt_(x * x + y * y + z * z);
            if (r == R(0)) continue;
            R cf, h;
            af_entry<R>(A, wk, tk, j, A.type[j], r, rcp_(r), cf, h);
            fx += cf * x;
            fy += cf * y;
            fz += cf * z;
            w0 += h * x * x;
            w1 += h * y * y;
            w2 += h * z * z;
            w3 += h * y * z;
            w4 += h * x * z;
            w5 += h * x * y;
        }
    }
    auto sfx = group_sum_f<G>(fx), sfy = group_sum_f<G>(fy), sfz = group_sum_f<G>(fz);
    if (act && lane == 0) {
        store_sum(A.out_f + 3 * k, sfx, A.first_f);
        store_sum(A.out_f + 3 * k + 1, sfy, A.first_f);
        store_sum(A.out_f + 3 * k + 2, sfz, A.first_f);
    }
    if (A.acc) {
        const Fx128 v[7] = {fx_zero(), warp_total(w0), warp_total(w1), warp_total(w2),
                            warp_total(w3), warp_total(w4), warp_total(w5)};
        block_totals_publish(v, wsum, &done, A.acc);
    }
}

// Gradients of group g's factors (core_calculate_bond_order_gradients and
// _of_factor, Core.f90:1157-1989, with the post-processing of 2842-3080): one
// thread walks atom a's list in order, so the sums are deterministic; out is
// n x 3, zeroed by the caller.  of_factor 0: every factor with respect to
// moving a; 1: a's factor with respect to moving every atom.
template <typename R>
__global__ void af_grad(const __grid_constant__ PairArgs A, int g, int a, int of_factor, double* __restrict__ out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    const int ta = A.type[a];
    double xa = 0, ya = 0, za = 0;
    if constexpr (sizeof(R) == 8) {
        xa = A.pos[3 * a];
        ya = A.pos[3 * a + 1];
        za = A.pos[3 * a + 2];
    }
    const AfT<R>* recs = (const AfT<R>*)A.af;
    for (int e = A.start[a]; e < A.start[a + 1]; ++e) {
        const int j = A.idx[e];
        R x, y, z;
        pair_vector<R>(A, a, e, xa, ya, za, x, y, z);
        const R r = sqrt_(x * x + y * y + z * z);
        if (r == R(0)) continue;
        const R ir = rcp_(r);
        const int2 ix = A.af_index[ta * A.T + A.type[j]];
        for (int t = ix.x; t < ix.x + ix.y; ++t) {
            const AfT<R> F = recs[t];
            if (F.group != g || !(r < F.rc)) continue;
            R c, dc;
            af_term<R>(F, r, ir, (const R*)A.tab, c, dc);
            // gradient of the pair's factor with respect to a: -c'(r) u
            const double s = -(double)(dc * ir);
            const double gx = s * (double)x, gy = s * (double)y, gz = s * (double)z;
            out[3 * a] += gx;
            out[3 * a + 1] += gy;
            out[3 * a + 2] += gz;
            const double sj = of_factor ? -1.0 : 1.0;
            out[3 * j] += sj * gx;
            out[3 * j + 1] += sj * gy;
            out[3 * j + 2] += sj * gz;
        }
    }
    const R* S = (const R*)A.afS + (size_t)g * A.n;
    for (int i = 0; i < A.n; ++i) {
        const double f = (double)S[of_factor ? a : i];
        out[3 * i] *= f;
        out[3 * i + 1] *= f;
        out[3 * i + 2] *= f;
    }
}

}  // namespace

void atom_factor_gradients(pg_context* ctx, int precision, int group, int atom, int of_factor, double* out) {
    const size_t n = (size_t)std::max(ctx->n, 1);
    ctx->af_grad.resize(3 * n);
    PG_CUDA(cudaMemsetAsync(ctx->af_grad.p, 0, sizeof(double) * 3 * n, ctx->stream));
    auto it = ctx->agroup_of.find(group);
    if (it != ctx->agroup_of.end()) {
        const PairArgs A = make_pair_args(ctx, precision, PG_WANT_FORCES, true, true, nullptr, nullptr);
        if (precision == PG_PREC_FP64) af_grad<double><<<1, 32, 0, ctx->stream>>>(A, it->second, atom, of_factor, ctx->af_grad.p);
        else af_grad<float><<<1, 32, 0, ctx->stream>>>(A, it->second, atom, of_factor, ctx->af_grad.p);
        PG_CHECK_LAUNCH();
    }
    ctx->af_grad.download(out, 3 * (size_t)ctx->n, ctx->stream);
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
}

// Fold the per-atom factor records into per-(atom1 type, atom2 type) lists and
// per-(group, type) scalers.  gmap: coordinator group id -> level-1 index.
void fold_atom_factors(pg_context* ctx, const std::map<int, int>& gmap) {
    const int T = std::max(ctx->n_types, 1);
    const int nr = (int)ctx->af_kind.size();
    auto has = [](uint64_t m, int t) { return ((m >> t) & 1ull) != 0; };
    auto two_target = [](int kind) { return kind == 0 || kind == 1 || kind == 4; };
    // tabulated factors: params first row, rows, range, scale; the kernels read
    // rows t0 .. t0 + tn - 1 only, checked here
    const size_t rows = ctx->pr_table.size() / 2;
    for (int r = 0; r < nr; ++r)
        if (ctx->af_kind[r] == 4 || ctx->af_kind[r] == 5) {
            const double* p = &ctx->af_params[5 * (size_t)r];
            require(p[0] >= 0.0 && p[1] >= 2.0 && p[0] + p[1] <= (double)rows && p[2] > 0.0, PG_ERR_INVALID,
                    "tabulated bond-order factor: table rows or range out of bounds");
        }
    auto set_table = [&](auto& F, const double* p) {
        F.t0 = (int)p[0];
        F.tn = (int)p[1];
    };
    std::vector<AfT<double>> recs;
    std::vector<int2> index((size_t)T * T, make_int2(0, 0));
    for (int ta = 0; ta < T; ++ta)
        for (int tb = 0; tb < T; ++tb) {
            int2& ix = index[(size_t)ta * T + tb];
            ix.x = (int)recs.size();
            for (int r = 0; r < nr; ++r) {
                if (!two_target(ctx->af_kind[r]) || !has(ctx->af_m1[r], ta) || !has(ctx->af_m2[r], tb)) continue;
                const double* p = &ctx->af_params[5 * (size_t)r];
                AfT<double> F{};
                F.kind = ctx->af_kind[r];
                F.group = gmap.at(ctx->af_group[r]);
                F.rc = ctx->af_cut[r];
                // smoothening_factor with soft = cutoff - margin; evaluated below the cutoff only
                F.rs = std::min(ctx->af_soft[r], ctx->af_cut[r]);
                F.a = F.kind == 4 ? p[2] : p[0];
                F.n = F.kind == 4 ? p[3] : p[1];
                F.ni = F.kind == 1 ? integral_exponent(p[1]) : PG_NOT_INT;
                F.flags = 0;
                if (F.kind == 4) set_table(F, p);
                recs.push_back(F);
            }
            ix.y = (int)recs.size() - ix.x;
        }
    // force records: per (k type, j type) every two-target record with k at
    // position 1 and j at 2 (k's factor) or j at 1 and k at 2 (j's factor)
    std::vector<AfT<double>> frecs;
    std::vector<int2> findex((size_t)T * T, make_int2(0, 0));
    for (int tk = 0; tk < T; ++tk)
        for (int tj = 0; tj < T; ++tj) {
            int2& ix = findex[(size_t)tk * T + tj];
            ix.x = (int)frecs.size();
            for (int r = 0; r < nr; ++r) {
                if (!two_target(ctx->af_kind[r])) continue;
                const bool own = has(ctx->af_m1[r], tk) && has(ctx->af_m2[r], tj);
                const bool other = has(ctx->af_m1[r], tj) && has(ctx->af_m2[r], tk);
                if (!own && !other) continue;
                const double* p = &ctx->af_params[5 * (size_t)r];
                AfT<double> F{};
                F.kind = ctx->af_kind[r];
                F.group = gmap.at(ctx->af_group[r]);
                F.rc = ctx->af_cut[r];
                F.rs = std::min(ctx->af_soft[r], ctx->af_cut[r]);
                F.a = F.kind == 4 ? p[2] : p[0];
                F.n = F.kind == 4 ? p[3] : p[1];
                F.ni = F.kind == 1 ? integral_exponent(p[1]) : PG_NOT_INT;
                F.flags = (own ? 1 : 0) | (other ? 2 : 0);
                if (F.kind == 4) set_table(F, p);
                frecs.push_back(F);
            }
            ix.y = (int)frecs.size() - ix.x;
        }
    const int ng = std::max(ctx->n_agroups, 1);
    std::vector<AfPostT<double>> post((size_t)ng * T);
    for (auto& q : post) q = AfPostT<double>{-1, {0, 0, 0, 0, 0}, 0, 0};
    for (int t = 0; t < T; ++t)
        for (int r = 0; r < nr; ++r) {
            if (two_target(ctx->af_kind[r]) || !has(ctx->af_m1[r], t)) continue;
            AfPostT<double>& q = post[(size_t)gmap.at(ctx->af_group[r]) * T + t];
            if (q.kind >= 0) continue;  // the first scaler of the element in the group
            q.kind = ctx->af_kind[r];
            for (int c = 0; c < 5; ++c) q.p[c] = ctx->af_params[5 * (size_t)r + c];
            if (q.kind == 5) set_table(q, &ctx->af_params[5 * (size_t)r]);
        }
    if (recs.empty()) recs.push_back(AfT<double>{});
    if (frecs.empty()) frecs.push_back(AfT<double>{});
    auto to32 = [](const AfT<double>& q) {
        return AfT<float>{q.kind, q.group, (float)q.rc, (float)q.rs, (float)q.a, (float)q.n, q.ni, q.flags, q.t0, q.tn};
    };
    std::vector<AfT<float>> recs32(recs.size()), frecs32(frecs.size());
    for (size_t q = 0; q < recs.size(); ++q) recs32[q] = to32(recs[q]);
    for (size_t q = 0; q < frecs.size(); ++q) frecs32[q] = to32(frecs[q]);
    std::vector<AfPostT<float>> post32(post.size());
    for (size_t q = 0; q < post.size(); ++q) {
        post32[q].kind = post[q].kind;
        for (int c = 0; c < 5; ++c) post32[q].p[c] = (float)post[q].p[c];
        post32[q].t0 = post[q].t0;
        post32[q].tn = post[q].tn;
    }
    cudaStream_t st = ctx->stream;
    ctx->d_af.upload(recs.data(), recs.size(), st);
    ctx->d_af32.upload(recs32.data(), recs32.size(), st);
    ctx->d_af_index.upload(index.data(), index.size(), st);
    ctx->d_aff.upload(frecs.data(), frecs.size(), st);
    ctx->d_aff32.upload(frecs32.data(), frecs32.size(), st);
    ctx->d_aff_index.upload(findex.data(), findex.size(), st);
    ctx->d_af_post.upload(post.data(), post.size(), st);
    ctx->d_af_post32.upload(post32.data(), post32.size(), st);
}

void set_atom_factor_args(pg_context* ctx, int precision, PairArgs& A) {
    A.ng = ctx->n_agroups;
    if (A.ng == 0) return;
    const size_t m = (size_t)ctx->n_agroups * (size_t)std::max(ctx->n, 1);
    ctx->af_B.resize(m);
    ctx->af_S.resize(m);
    ctx->af_W.resize(m);
    A.af = precision == PG_PREC_FP64 ? (const void*)ctx->d_af.p : (const void*)ctx->d_af32.p;
    A.af_index = ctx->d_af_index.p;
    A.aff = precision == PG_PREC_FP64 ? (const void*)ctx->d_aff.p : (const void*)ctx->d_aff32.p;
    A.aff_index = ctx->d_aff_index.p;
    A.af_post = precision == PG_PREC_FP64 ? (const void*)ctx->d_af_post.p : (const void*)ctx->d_af_post32.p;
    A.afB = ctx->af_B.p;
    A.afS = ctx->af_S.p;
    A.afW = ctx->af_W.p;
    A.af_fused = ctx->af_fused ? 1 : 0;
}

// stage 0: the sums and factors (before the pair kernel); stage 1: the forces
// (after it, adding to out_f)
void launch_atom_factors(pg_context* ctx, int precision, int stage, bool first_f, FxAcc* acc, const int* skip) {
    const int G = pair_lanes_for(ctx);
    PairArgs A = make_pair_args(ctx, precision, PG_WANT_FORCES, first_f, true, acc, skip);
    const int nbk = pair_kernel_blocks(ctx->n, G), threads = pair_atoms_per_block(ctx->n, G) * G;
    cudaStream_t st = ctx->stream;
#define PG_AF_LAUNCH(K_, R_, G_) K_<R_, G_><<<nbk, threads, 0, st>>>(A)
#define PG_AF_G(K_, R_)                   \
    do {                                  \
        if (G == 8) PG_AF_LAUNCH(K_, R_, 8);  \
        else if (G == 16) PG_AF_LAUNCH(K_, R_, 16); \
        else PG_AF_LAUNCH(K_, R_, 32);    \
    } while (0)
    if (stage == 0) {
        if (precision == PG_PREC_FP64) PG_AF_G(af_sum, double);
        else PG_AF_G(af_sum, float);
    } else {
        if (precision == PG_PREC_FP64) PG_AF_G(af_force, double);
        else PG_AF_G(af_force, float);
    }
#undef PG_AF_G
#undef PG_AF_LAUNCH
    PG_CHECK_LAUNCH();
    ctx->launches++;
}

}  // namespace pg
