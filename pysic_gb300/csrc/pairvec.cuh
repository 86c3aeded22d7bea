// pairvec.cuh -- per-entry geometry of the full neighbour list, shared by the
// pair kernel (pair.cu) and the per-atom bond-order factor kernels
// (atomfactor.cu).
#pragma once
#include "args.cuh"
#include "common.cuh"

namespace pg {

// bond vector of entry e of atom i: FP64 from the positions, or (mixed path)
// build-time vector plus the FP32 displacements of both atoms
template <typename R>
__device__ __forceinline__ void pair_vector(const PairArgs& A, int i, int e, double xi, double yi, double zi, R& x,
                                            R& y, R& z);
template <>
__device__ __forceinline__ void pair_vector<double>(const PairArgs& A, int i, int e, double xi, double yi, double zi,
                                                    double& x, double& y, double& z) {
    const int j = A.idx[e];
    const double o0 = A.off[3 * e], o1 = A.off[3 * e + 1], o2 = A.off[3 * e + 2];
    // separation_vector (Geometry.f90:449-466)
    x = A.pos[3 * j] - xi + (o0 * A.C.vc[0][0] + o1 * A.C.vc[0][1] + o2 * A.C.vc[0][2]);
    y = A.pos[3 * j + 1] - yi + (o0 * A.C.vc[1][0] + o1 * A.C.vc[1][1] + o2 * A.C.vc[1][2]);
    z = A.pos[3 * j + 2] - zi + (o0 * A.C.vc[2][0] + o1 * A.C.vc[2][1] + o2 * A.C.vc[2][2]);
}
template <>
__device__ __forceinline__ void pair_vector<float>(const PairArgs& A, int i, int e, double, double, double, float& x,
                                                   float& y, float& z) {
    const int j = A.idx[e];
    const F4 s0 = A.sep0[e], dj = A.disp[j], di = A.disp[i];
    x = s0.x + (dj.x - di.x);
    y = s0.y + (dj.y - di.y);
    z = s0.z + (dj.z - di.z);
}

// charge of atom j in the working precision (mixed path: the FP32 copy kept
// beside the displacement)
template <typename R>
__device__ __forceinline__ R charge_of(const PairArgs& A, int j);
template <>
__device__ __forceinline__ double charge_of<double>(const PairArgs& A, int j) {
    return A.charge[j];
}
template <>
__device__ __forceinline__ float charge_of<float>(const PairArgs& A, int j) {
    return A.disp[j].w;
}

}  // namespace pg
