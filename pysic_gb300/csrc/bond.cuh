// bond.cuh -- bond geometry of the bond-order kernels (tersoff.cu), shared by
// the bond-per-lane and triplet-per-lane tiles.
#pragma once
#include "args.cuh"
#include "kernels.cuh"

namespace pg {

template <typename R>
__device__ __forceinline__ typename Vec4T<R>::T bond_vector(const BondArgs& A, int i, int e, double xi, double yi,
                                                            double zi);

template <>
__device__ __forceinline__ D4 bond_vector<double>(const BondArgs& A, int i, int e, double xi, double yi, double zi) {
    const int j = A.idx[e];
    const double o0 = A.off[3 * e], o1 = A.off[3 * e + 1], o2 = A.off[3 * e + 2];
    double sx = A.pos[3 * j] - xi, sy = A.pos[3 * j + 1] - yi, sz = A.pos[3 * j + 2] - zi;
    sx += o0 * A.C.vc[0][0] + o1 * A.C.vc[0][1] + o2 * A.C.vc[0][2];
    sy += o0 * A.C.vc[1][0] + o1 * A.C.vc[1][1] + o2 * A.C.vc[1][2];
    sz += o0 * A.C.vc[2][0] + o1 * A.C.vc[2][1] + o2 * A.C.vc[2][2];
    return D4{sx, sy, sz, sqrt(sx * sx + sy * sy + sz * sz)};
}

template <>
__device__ __forceinline__ F4 bond_vector<float>(const BondArgs& A, int i, int e, double, double, double) {
    const int j = A.idx[e];
    const F4 s0 = A.sep0[e];
    const F4 dj = A.disp[j], di = A.disp[i];
    const float x = s0.x + (dj.x - di.x), y = s0.y + (dj.y - di.y), z = s0.z + (dj.z - di.z);
    return F4{x, y, z, sqrtf(x * x + y * y + z * z)};
}

template <typename R>
struct Vec2T;
template <>
struct Vec2T<float> {
    using T = float2;
};
template <>
struct Vec2T<double> {
    using T = double2;
};

// A bond-order scaled charge-dependent or product term of short-list entry
// `ent` (atom i -> its partner): V f, d(V f)/dr and f times the
// electronegativity of atom i (-dV/dq_i), with the pair's atom1 as the
// reference's loop picks it (pick on the entry's image offset) and the charges
// of both atoms (FP64 charges, or the FP32 copy of the mixed path).
template <typename R>
__device__ __forceinline__ void bond_charge_term(const BondArgs& A, const PairT<R>& PT, const PairT<R>* terms, int i,
                                                 int ent, int ti, int tj, R r, R& V, R& dV, R& en) {
    const int j = A.idx[ent];
    const bool first = pick(i, j, A.off[3 * ent], A.off[3 * ent + 1], A.off[3 * ent + 2]);
    R qi, qj;
    if constexpr (sizeof(R) == 4) {
        qi = A.disp[i].w;
        qj = A.disp[j].w;
    } else {
        qi = A.q[i];
        qj = A.q[j];
    }
    product_value<R>(PT, terms, (const R*)A.tab, r, qi, qj, first, ti, tj, V, dV, en);
    if (PT.smooth) {
        R f, fp;
        smooth<R>(r, PT.rc, PT.rs, f, fp);
        dV = dV * f + V * fp;
        V *= f;
        en *= f;
    }
}

}  // namespace pg
