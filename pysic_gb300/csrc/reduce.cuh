// reduce.cuh -- block reductions and the "last block" ticket shared by the
// charge-relaxation and charge-optimisation kernels.  Every reduction runs in
// a fixed order (shuffle trees, then blocks in index order), so results do not
// depend on scheduling.
#pragma once
#include <cuda_runtime.h>

namespace pg {

// block-wide sum or max of v; the result is valid in thread 0.  sh holds one
// double per warp.
__device__ __forceinline__ double block_reduce(double v, bool is_max, double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, v, o);
        v = is_max ? fmax(v, u) : v + u;
    }
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < nw ? sh[lane] : (is_max ? -1e300 : 0.0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double u = __shfl_xor_sync(0xffffffffu, v, o);
            v = is_max ? fmax(v, u) : v + u;
        }
    }
    return v;
}

// true in thread 0 of the block that takes the last ticket: by then every other
// block has published its partial (fence before the ticket).  The last block
// puts the counter back to zero for the next launch.  No block waits.
__device__ __forceinline__ bool last_block(int* ticket) {
    __shared__ int is_last;
    if (threadIdx.x == 0) {
        __threadfence();
        const int last = atomicAdd(ticket, 1) == (int)gridDim.x - 1;
        if (last) *ticket = 0;
        is_last = last;
    }
    __syncthreads();
    return is_last && threadIdx.x == 0;
}

}  // namespace pg
