// reduce.cu -- deterministic final reduction of the per-block energy / virial
// partials that the evaluation kernels write.
//
// The reference sums energy and stress with plain FP64 additions in atom order
// (Core.f90:3249-4082).  Here every kernel leaves one FP64 partial per thread
// block, and this kernel adds them exactly in 128-bit fixed point (fixed.cuh):
// one block per component, integer additions only, no FP64 dependency chain,
// and a result that does not depend on the order of the terms.
#include "common.cuh"
#include "fixed.cuh"

namespace pg {

constexpr int RED_THREADS = 256;

__global__ void __launch_bounds__(RED_THREADS) final_reduce(const double* __restrict__ partial, int nslots,
                                                            double* __restrict__ out) {
    __shared__ Fx128 ws[RED_THREADS / 32];
    const int c = blockIdx.x;
    const int t = threadIdx.x;
    Fx128 acc = fx_zero();
    for (int k = t; k < nslots; k += RED_THREADS) acc = fx_add(acc, fx_from_double(partial[8 * k + c]));
    acc = fx_warp_sum(acc);
    if ((t & 31) == 0) ws[t >> 5] = acc;
    __syncthreads();
    if (t < 32) {
        acc = t < RED_THREADS / 32 ? ws[t] : fx_zero();
        acc = fx_warp_sum(acc);
        if (t == 0) out[c] = fx_to_double(acc);
    }
}

void launch_final_reduce(pg_context* ctx, int nslots) {
    final_reduce<<<7, RED_THREADS, 0, ctx->stream>>>(ctx->red_part.p, nslots, ctx->out_tot.p);
    PG_CHECK_LAUNCH();
    ctx->launches++;
}

}  // namespace pg
