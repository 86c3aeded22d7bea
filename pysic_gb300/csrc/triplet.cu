// triplet.cu -- three-body potentials (bond_bend) in the reference's triplet
// enumeration.
//
// core_loop_over_local_interactions (Core.f90:3249-3943) finds triplets from
// the pairs it already visits: for every picked pair (atom1, atom2) within a
// many-body potential's cutoff that affects atom2 at target position 2, it
//   A  walks atom1's neighbours atom3 with pick(atom2, atom3): triplet
//      atom2 - atom1 - atom3, centre atom1;
//   B  walks atom2's neighbours atom3 with pick(atom1, atom3): triplet
//      atom1 - atom2 - atom3, centre atom2;
// and core_evaluate_local_triplet_B (6656-7028) applies each many-body record
// whose position-2 target is the triplet's second listed atom and whose
// position-3 target is atom3, within the cutoff for both bonds; the bond_bend
// evaluator (Potentials.f90:3206-3314) further requires the unpermuted tuple's
// middle element at the centre.  This kernel walks the same loops: one warp
// per atom1, lanes over atom1's list entries (atom2), each lane the two atom3
// loops of its pair.  Forces on the three atoms go to per-atom 2^-40 fixed-point
// accumulators by 64-bit integer atomics (order-independent, so results do
// not depend on scheduling).  A signed 64-bit word in these units holds
// magnitudes below 2^23 (8.4e6 eV/A) exactly; beside the three components
// every atom has a magnitude word, the sum of |Fx| + |Fy| + |Fz| of its terms
// in units of 2^-8 (rounded up), with its top bit set by any non-finite term
// or term of 2^30 eV/A or more.  While that sum stays below 2^23 eV/A no
// component can have wrapped; otherwise the atom's force reads back as NaN
// instead of a wrong value.  Energy and the reference's virial
// (sep1 (x) F_centre + (sep1 + sep2) (x) F_3, Core.f90:6980-6991) to the exact
// block totals.  The centre's smooth-cutoff gradient terms are those of
// 6860-6888.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "fixed.cuh"
#include "kernels.cuh"

namespace pg {

namespace {

constexpr int TT = 128;
constexpr double FIX40 = 1099511627776.0;  // 2^40

struct TriArgs {
    int n;
    const double* pos;
    const int* type;
    CellK C;
    const int* start;
    const int* idx;
    const int* off;
    const F4* sep0;   // mixed path: full-list bond vectors at the list build
    const F4* disp;   // mixed path: displacements since the build
    const void* rec;  // TriT<R>
    int nrec;
    long long* facc;  // n x 3 fixed-point forces
    FxAcc* acc;       // energy, virial totals (null: none)
    const int* skip;
};

// bond vector of list entry e of atom a (the separation a -> partner)
template <typename R>
__device__ __forceinline__ V3<R> entry_vector(const TriArgs& A, int a, int e);
template <>
__device__ __forceinline__ V3<double> entry_vector<double>(const TriArgs& A, int a, int e) {
    const int j = A.idx[e];
    const double o0 = A.off[3 * e], o1 = A.off[3 * e + 1], o2 = A.off[3 * e + 2];
    V3<double> s;
    s.x = A.pos[3 * j] - A.pos[3 * a] + (o0 * A.C.vc[0][0] + o1 * A.C.vc[0][1] + o2 * A.C.vc[0][2]);
    s.y = A.pos[3 * j + 1] - A.pos[3 * a + 1] + (o0 * A.C.vc[1][0] + o1 * A.C.vc[1][1] + o2 * A.C.vc[1][2]);
    s.z = A.pos[3 * j + 2] - A.pos[3 * a + 2] + (o0 * A.C.vc[2][0] + o1 * A.C.vc[2][1] + o2 * A.C.vc[2][2]);
    return s;
}
template <>
__device__ __forceinline__ V3<float> entry_vector<float>(const TriArgs& A, int a, int e) {
    const int j = A.idx[e];
    const F4 s0 = A.sep0[e], dj = A.disp[j], da = A.disp[a];
    return V3<float>{s0.x + (dj.x - da.x), s0.y + (dj.y - da.y), s0.z + (dj.z - da.z)};
}

// magnitude words (one per atom after the 3 n components): the top bit marks
// a term that cannot be accumulated; sums from 2^23 eV/A (2^31 units of 2^-8)
// on may have wrapped a component
constexpr unsigned long long MAG_BAD = 1ull << 63;
constexpr unsigned long long MAG_LIMIT = 1ull << 31;

__device__ __forceinline__ long long fix40(float v) { return __float2ll_rn(v * 1099511627776.0f); }
__device__ __forceinline__ long long fix40(double v) { return __double2ll_rn(v * FIX40); }

// facc: 3 n components, then n magnitude words
template <typename R>
__device__ __forceinline__ void add_force(long long* facc, int n, int a, const V3<R>& f) {
    const R m = fabs(f.x) + fabs(f.y) + fabs(f.z);
    unsigned long long* mag = (unsigned long long*)(facc + 3 * (size_t)n + a);
    if (!(m < R(1073741824))) {  // 2^30 eV/A, infinities and NaN: nothing is added
        atomicOr(mag, MAG_BAD);
        return;
    }
    atomicAdd(mag, (unsigned long long)ceil(m * R(256)));
    atomicAdd((unsigned long long*)(facc + 3 * a), (unsigned long long)fix40(f.x));
    atomicAdd((unsigned long long*)(facc + 3 * a + 1), (unsigned long long)fix40(f.y));
    atomicAdd((unsigned long long*)(facc + 3 * a + 2), (unsigned long long)fix40(f.z));
}

// One bond_bend term of the triplet x - c - y: s1 = x -> c, s2 = c -> y.
// Forces on x, c, y and the energy, smooth cutoffs included
// (evaluate_energy/force_bond_bending, Potentials.f90:3206-3314, and the
// cut-factor products of Core.f90:6860-6888).
template <typename R>
__device__ __forceinline__ void bend_term(const TriT<R>& T, const V3<R>& s1, R d1, const V3<R>& s2, R d2, V3<R>& fx,
                                          V3<R>& fc, V3<R>& fy, R& e) {
    const V3<R> t1{-s1.x, -s1.y, -s1.z};
    const R r3 = t1.x * s2.x + t1.y * s2.y + t1.z * s2.z;
    const R ratio = R(1) / (d1 * d2);
    const R cosplain = r3 * ratio;
    const R cospower = ipow(cosplain, T.n - 1);
    const R v = T.eps * ipow(ipow(r3 / (d1 * d2), T.n) - T.c0, T.m);
    const R r6 = T.eps * (R)(T.m * T.n) * ipow(cospower * cosplain - T.c0, T.m - 1) * cospower;
    const R a = r3 / (d1 * d1), b = r3 / (d2 * d2);
    const V3<R> t3{s2.x - a * t1.x, s2.y - a * t1.y, s2.z - a * t1.z};
    const V3<R> t4{t1.x - b * s2.x, t1.y - b * s2.y, t1.z - b * s2.z};
    const R k = ratio * r6;
    V3<R> px{-t3.x * k, -t3.y * k, -t3.z * k};
    V3<R> pc{(t3.x + t4.x) * k, (t3.y + t4.y) * k, (t3.z + t4.z) * k};
    V3<R> py{-t4.x * k, -t4.y * k, -t4.z * k};
    if (T.smooth) {
        R f1, g1, f2, g2;
        smooth<R>(d1, T.rc, T.rs, f1, g1);
        smooth<R>(d2, T.rc, T.rs, f2, g2);
        // cut_gradients = f'(d) * direction of the separation
        const V3<R> c1{g1 * s1.x / d1, g1 * s1.y / d1, g1 * s1.z / d1};
        const V3<R> c2{g2 * s2.x / d2, g2 * s2.y / d2, g2 * s2.z / d2};
        const R ff = f1 * f2;
        fx = V3<R>{px.x * ff + c1.x * f2 * v, px.y * ff + c1.y * f2 * v, px.z * ff + c1.z * f2 * v};
        fc = V3<R>{pc.x * ff + (-c1.x * f2 + c2.x * f1) * v, pc.y * ff + (-c1.y * f2 + c2.y * f1) * v,
                   pc.z * ff + (-c1.z * f2 + c2.z * f1) * v};
        fy = V3<R>{py.x * ff - c2.x * f1 * v, py.y * ff - c2.y * f1 * v, py.z * ff - c2.z * f1 * v};
        e = v * ff;
    } else {
        fx = px;
        fc = pc;
        fy = py;
        e = v;
    }
}

__device__ __forceinline__ bool bit(unsigned long long m, int t) { return (m >> t) & 1ull; }

template <typename R>
__global__ void __launch_bounds__(TT) tri_kernel(const __grid_constant__ TriArgs A) {
    __shared__ Fx128 wsum[TT / 32][7];
    __shared__ unsigned done;
    if (threadIdx.x == 0) done = 0u;
    __syncthreads();
    if (A.skip && *A.skip) return;  // uniform over the grid
    const TriT<R>* recs = (const TriT<R>*)A.rec;
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // atom1
    R En = 0, W0 = 0, W1 = 0, W2 = 0, W3 = 0, W4 = 0, W5 = 0;
    auto account = [&](const TriT<R>& T, int x, int c, int y, const V3<R>& s1, R d1, const V3<R>& s2, R d2) {
        V3<R> fx, fc, fy;
        R e;
        bend_term<R>(T, s1, d1, s2, d2, fx, fc, fy, e);
        En += e;
        add_force(A.facc, A.n, x, fx);
        add_force(A.facc, A.n, c, fc);
        add_force(A.facc, A.n, y, fy);
        const V3<R> s12{s1.x + s2.x, s1.y + s2.y, s1.z + s2.z};
        W0 += s1.x * fc.x + s12.x * fy.x;
        W1 += s1.y * fc.y + s12.y * fy.y;
        W2 += s1.z * fc.z + s12.z * fy.z;
        W3 += s1.y * fc.z + s12.y * fy.z;
        W4 += s1.x * fc.z + s12.x * fy.z;
        W5 += s1.x * fc.y + s12.x * fy.y;
    };
    if (i < A.n) {
        const int ti = A.type[i];
        const int b1 = A.start[i], e1 = A.start[i + 1];
        for (int e = b1 + lane; e < e1; e += 32) {
            const int j = A.idx[e];
            const int o0 = A.off[3 * e], o1 = A.off[3 * e + 1], o2 = A.off[3 * e + 2];
            if (!pick(i, j, o0, o1, o2)) continue;
            const V3<R> s12 = entry_vector<R>(A, i, e);
            const R d12 = sqrt_(s12.x * s12.x + s12.y * s12.y + s12.z * s12.z);
            if (d12 == R(0)) continue;
            const int tj = A.type[j];
            // the many-body records of this pair (core_evaluate_local_doublet_*_B)
            unsigned long long rm = 0;
            for (int r = 0; r < A.nrec; ++r)
                if (recs[r].rc > d12 && bit(recs[r].many, ti) && bit(recs[r].m2, tj)) rm |= 1ull << r;
            if (!rm) continue;
            const V3<R> s21{-s12.x, -s12.y, -s12.z};
            // A: atom2 - atom1 - atom3 over atom1's neighbours
            for (int l = b1; l < e1; ++l) {
                const int k = A.idx[l];
                const int p0 = A.off[3 * l] - o0, p1 = A.off[3 * l + 1] - o1, p2 = A.off[3 * l + 2] - o2;
                if (!pick(j, k, p0, p1, p2)) continue;
                const V3<R> s13 = entry_vector<R>(A, i, l);
                const R d13 = sqrt_(s13.x * s13.x + s13.y * s13.y + s13.z * s13.z);
                if (d13 == R(0)) continue;
                const int tk = A.type[k];
                for (unsigned long long q = rm; q; q &= q - 1) {
                    const TriT<R>& T = recs[__ffsll((long long)q) - 1];
                    if (bit(T.m3, tk) && bit(T.center, ti) && T.rc > d13) account(T, j, i, k, s21, d12, s13, d13);
                }
            }
            // B: atom1 - atom2 - atom3 over atom2's neighbours
            const int b2 = A.start[j], e2 = A.start[j + 1];
            for (int l = b2; l < e2; ++l) {
                const int k = A.idx[l];
                const int p0 = A.off[3 * l] + o0, p1 = A.off[3 * l + 1] + o1, p2 = A.off[3 * l + 2] + o2;
                if (!pick(i, k, p0, p1, p2)) continue;
                const V3<R> s23 = entry_vector<R>(A, j, l);
                const R d23 = sqrt_(s23.x * s23.x + s23.y * s23.y + s23.z * s23.z);
                if (d23 == R(0)) continue;
                const int tk = A.type[k];
                for (unsigned long long q = rm; q; q &= q - 1) {
                    const TriT<R>& T = recs[__ffsll((long long)q) - 1];
                    if (bit(T.m3, tk) && bit(T.center, tj) && T.rc > d23) account(T, i, j, k, s12, d12, s23, d23);
                }
            }
        }
    }
    if (A.acc) {
        const Fx128 v[7] = {warp_total(En), warp_total(W0), warp_total(W1), warp_total(W2),
                            warp_total(W3), warp_total(W4), warp_total(W5)};
        block_totals_publish(v, wsum, &done, A.acc);
    }
}

// the accumulated forces into out_f (written or added), accumulators back to zero
__global__ void tri_forces(int n, long long* __restrict__ facc, double* __restrict__ out_f, int first,
                           const int* skip) {
    if (skip && *skip) return;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= 3 * n) return;
    const unsigned long long mag = (unsigned long long)facc[3 * (size_t)n + q / 3];
    const double v = mag >= MAG_LIMIT ? fx_nan() : (double)facc[q] * (1.0 / FIX40);
    facc[q] = 0;
    out_f[q] = first ? v : out_f[q] + v;
}

// the magnitude words back to zero (after tri_forces has read them)
__global__ void tri_clear_mag(int n, long long* __restrict__ facc, const int* skip) {
    if (skip && *skip) return;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < n) facc[3 * (size_t)n + a] = 0;
}

}  // namespace

void launch_triplets(pg_context* ctx, int precision, int flags, bool first_f, FxAcc* acc, const int* skip) {
    const int n = ctx->n;
    if (n == 0 || ctx->n_tri == 0) return;
    cudaStream_t st = ctx->stream;
    if (ctx->tri_facc.n != 4 * (size_t)n) {  // 3 n components, n magnitude words; zero between calls
        ctx->tri_facc.resize(4 * (size_t)n);
        PG_CUDA(cudaMemsetAsync(ctx->tri_facc.p, 0, sizeof(long long) * 4 * (size_t)n, st));
    }
    TriArgs A{};
    A.n = n;
    A.pos = ctx->pos.p;
    A.type = ctx->type.p;
    A.C = cell_kernel_view(ctx->cell);
    A.start = ctx->nb_start.p;
    A.idx = ctx->nb_idx.p;
    A.off = ctx->nb_off.p;
    A.sep0 = ctx->nb_sep0.p;
    A.disp = ctx->disp32.p;
    A.nrec = ctx->n_tri;
    A.facc = ctx->tri_facc.p;
    A.acc = (flags & (PG_WANT_ENERGY | PG_WANT_FORCES)) ? acc : nullptr;
    A.skip = skip;
    const int blocks = (int)(((long long)n * 32 + TT - 1) / TT);
    if (precision == PG_PREC_FP64) {
        A.rec = ctx->d_tri.p;
        tri_kernel<double><<<blocks, TT, 0, st>>>(A);
    } else {
        A.rec = ctx->d_tri32.p;
        tri_kernel<float><<<blocks, TT, 0, st>>>(A);
    }
    if (flags & PG_WANT_FORCES) {
        tri_forces<<<(3 * n + 255) / 256, 256, 0, st>>>(n, ctx->tri_facc.p, ctx->out_f.p, first_f ? 1 : 0, skip);
        tri_clear_mag<<<(n + 255) / 256, 256, 0, st>>>(n, ctx->tri_facc.p, skip);
    } else {  // energy only: the accumulated forces are dropped
        PG_CUDA(cudaMemsetAsync(ctx->tri_facc.p, 0, sizeof(long long) * 4 * (size_t)n, st));
    }
    PG_CHECK_LAUNCH();
    ctx->launches += (flags & PG_WANT_FORCES) ? 3 : 1;
}

}  // namespace pg
