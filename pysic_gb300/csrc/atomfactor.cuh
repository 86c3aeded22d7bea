// atomfactor.cuh -- device functions of the per-atom (level-1) bond-order
// factors, shared by the factor kernels (atomfactor.cu) and the pair kernel,
// which adds the factor forces in its own pass when no pair term is scaled.
#pragma once
#include "args.cuh"
#include "common.cuh"
#include "kernels.cuh"

namespace pg {

// Cubic Hermite value and derivative at x < range on rows (V, d)
// (Potentials.f90:6496-6576, 6663-6765)
template <typename R>
__device__ __forceinline__ void af_hermite(const R* T, int nv, R range, R scale, R x, R& v, R& dv) {
    const R dr = range / (R)(nv - 1);
    const R u = x / dr;
    const int l = min(max((int)u, 0), nv - 2);
    const R t = u - (R)l, t2 = t * t, t3 = t2 * t;
    const R* a = T + 2 * l;
    v = scale * (a[0] * (R(2) * t3 - R(3) * t2 + R(1)) + a[1] * dr / range * (t3 - R(2) * t2 + t) +
                 a[2] * (R(3) * t2 - R(2) * t3) + a[3] * dr / range * (t3 - t2));
    dv = scale * (a[0] / dr * R(6) * (t2 - t) + a[1] / range * (R(3) * t2 - R(4) * t + R(1)) +
                  a[2] / dr * R(6) * (t - t2) + a[3] / range * (R(3) * t2 - R(2) * t));
}

// c(r) and dc/dr of a two-target record (evaluate_bond_order_factor_ /
// _gradient_coordination, Potentials.f90:5631-5673; _power, 6293-6347;
// _table, 6663-6765: beyond the range the last value, neither scaled nor
// smoothed, with zero gradient)
template <typename R>
__device__ __forceinline__ void af_term(const AfT<R>& F, R r, R ir, const R* tab, R& c, R& dc) {
    R f, fp;
    smooth<R>(r, F.rc, F.rs, f, fp);
    if (F.kind == 0) {
        c = f;
        dc = fp;
        return;
    }
    if (F.kind == 4) {
        const R* T = tab + 2 * (long long)F.t0;
        if (r >= F.a) {
            c = T[2 * (F.tn - 1)];
            dc = R(0);
            return;
        }
        R v, dv;
        af_hermite<R>(T, F.tn, F.a, F.n, r, v, dv);
        c = v * f;
        dc = v * fp + f * dv;
        return;
    }
    const R rn = powk(F.a * ir, F.n, F.ni);
    c = f * rn;
    dc = rn * (fp - F.n * f * ir);
}

// The factor force terms of one list entry k -> j at distance r (ir = 1/r):
// over the records of k's factor (k at position 1, flag 1, weight W_k) and of
// j's factor (j at position 1, flag 2, weight W_j) in one merged list per
// (k type, j type), a record of both lists evaluated once.  cf: force on k per
// unit bond vector; hv: virial weight of k's own terms, sep (x) (-W_k c' u).
template <typename R>
__device__ __forceinline__ void af_entry(const PairArgs& A, const R (&wk)[PG_MAX_AGROUPS], int tk, int j, int tj, R r,
                                         R ir, R& cf, R& hv) {
    const AfT<R>* recs = (const AfT<R>*)A.aff;
    const R* W = (const R*)A.afW;
    R own = 0, other = 0;
    const int2 io = A.aff_index[tk * A.T + tj];
    for (int t = io.x; t < io.x + io.y; ++t) {
        const AfT<R> F = recs[t];
        if (!(r < F.rc)) continue;
        R c, dc;
        af_term<R>(F, r, ir, (const R*)A.tab, c, dc);
        if (F.flags & 1) {
            R wg = 0;
#pragma unroll
            for (int q = 0; q < PG_MAX_AGROUPS; ++q)
                if (q == F.group) wg = wk[q];
            own += dc * wg;
        }
        if (F.flags & 2) other += dc * W[(size_t)F.group * A.n + j];
    }
    cf = (own + other) * ir;
    hv = -own * ir;
}

}  // namespace pg
