// peak.cu -- the FP32 issue rate this GPU sustains, measured with a kernel of
// independent fused multiply-add chains (no counterpart in the reference).
//
// The Tersoff bond-order kernels are bound by FP32 instruction issue and
// dependency latency, not by HBM bandwidth; their roofline is reported against
// the FP32 rate measured here, in the same process and at the clocks of the
// same run, instead of a nominal figure.  Every thread runs CHAINS independent
// chains x = x * a + b (2 FLOP each), enough to hide the FMA latency; the grid
// fills every SM with 2048 threads.
#include <algorithm>

#include "common.cuh"

namespace pg {
namespace {

constexpr int CHAINS = 8;
constexpr int THREADS = 256;

__global__ void __launch_bounds__(THREADS) fma_chains(int iters, float a, float b, float* __restrict__ sink) {
    float x[CHAINS];
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) x[c] = (float)(threadIdx.x + c) * 1e-3f;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int c = 0; c < CHAINS; ++c) x[c] = fmaf(x[c], a, b);
    }
    float s = 0.f;
#pragma unroll
    for (int c = 0; c < CHAINS; ++c) s += x[c];
    if (s == -1.0f) sink[threadIdx.x] = s;  // never true for these inputs; keeps the chains live
}

}  // namespace

void measure_fp32_peak(int device, double* tflops, double* ms) {
    require(tflops != nullptr, PG_ERR_INVALID, "null output pointer");
    if (device >= 0) PG_CUDA(cudaSetDevice(device));
    const int sms = sm_count();
    const int blocks = sms * (2048 / THREADS);
    const int iters = 4096;
    float* sink = nullptr;
    PG_CUDA(cudaMalloc(&sink, sizeof(float) * THREADS));
    cudaStream_t st = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    float best = 1e30f;
    cudaError_t err = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking);
    if (err == cudaSuccess) err = cudaEventCreate(&e0);
    if (err == cudaSuccess) err = cudaEventCreate(&e1);
    for (int rep = 0; rep < 8 && err == cudaSuccess; ++rep) {
        fma_chains<<<blocks, THREADS, 0, st>>>(iters, 0.9999999f, 1e-7f, sink);
        err = cudaGetLastError();
        if (rep < 2 || err != cudaSuccess) continue;  // warm-up: clocks ramp
        cudaEventRecord(e0, st);
        fma_chains<<<blocks, THREADS, 0, st>>>(iters, 0.9999999f, 1e-7f, sink);
        cudaEventRecord(e1, st);
        err = cudaEventSynchronize(e1);
        float t = 0.f;
        if (err == cudaSuccess) err = cudaEventElapsedTime(&t, e0, e1);
        best = std::min(best, t);
    }
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
    if (st) cudaStreamDestroy(st);
    cudaFree(sink);
    PG_CUDA(err);
    const double flop = 2.0 * CHAINS * (double)iters * (double)blocks * THREADS;
    *tflops = flop / (best * 1e-3) / 1e12;
    if (ms) *ms = best;
}

}  // namespace pg
