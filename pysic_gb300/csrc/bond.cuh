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

}  // namespace pg
