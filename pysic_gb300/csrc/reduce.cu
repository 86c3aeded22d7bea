// reduce.cu -- deterministic, compensated FP64 reduction of the per-block
// energy / virial partials that the evaluation kernels write.
//
// The reference sums energy and stress with plain FP64 additions in atom order
// (Core.f90:3249-4082); here every kernel leaves one partial per thread block
// and this single-block kernel adds them with Kahan compensation in a fixed
// order, so repeated evaluations are bit-identical.
#include "common.cuh"

namespace pg {

__global__ void final_reduce(const double* __restrict__ partial, int nslots, double* __restrict__ out) {
    __shared__ double hi[256], lo[256];
    const int t = threadIdx.x;
    for (int c = 0; c < 7; ++c) {
        double s = 0.0, comp = 0.0;
        for (int k = t; k < nslots; k += blockDim.x) {
            const double y = partial[8 * k + c] - comp;
            const double u = s + y;
            comp = (u - s) - y;
            s = u;
        }
        hi[t] = s;
        lo[t] = -comp;
        __syncthreads();
        if (t == 0) {
            double S = 0.0, C = 0.0;
            for (int k = 0; k < (int)blockDim.x; ++k) {
                for (int h = 0; h < 2; ++h) {
                    const double y = (h ? lo[k] : hi[k]) - C;
                    const double u = S + y;
                    C = (u - S) - y;
                    S = u;
                }
            }
            out[c] = S;
        }
        __syncthreads();
    }
}

void launch_final_reduce(pg_context* ctx, int nslots) {
    final_reduce<<<1, 256, 0, ctx->stream>>>(ctx->red_part.p, nslots, ctx->out_tot.p);
    PG_CHECK_LAUNCH();
    ctx->launches++;
}

}  // namespace pg
