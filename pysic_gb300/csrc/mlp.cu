// mlp.cu -- learned warm start for charge relaxation: per-atom radial
// descriptors and a small multilayer perceptron (descriptors -> H1 -> H2 -> 1)
// with BF16 weights and FP32 arithmetic, trained on the GPU by the kernels of
// this file (forward, backward, Adam).
//
// No counterpart in the reference: its ChargeRelaxation always starts from the
// current charges (pysic/charges/relaxation.py:394-450).  The network only
// supplies the starting charges; the plain relaxation then runs to the same
// tolerance, so the result is the reference's own fixed point.
//
// Descriptors of atom i: for every element type t and Gaussian k,
//   G[t][k] = sum over neighbours j of type t with r_ij < rc of
//             exp(-(r_ij - mu_k)^2 / (2 w^2)) * 1/2 (1 + cos(pi r_ij / rc)),
// mu_k evenly spaced on [r0, r1].  One warp per atom, lanes over features.
//
// Network: z1 = W1 x + b1, h1 = tanh(z1), z2 = W2 h1 + b2, h2 = tanh(z2),
// y = w3 . h2 + b3.  Parameters are kept in FP32 (Adam's master copy) and as a
// BF16 copy that every forward pass reads; all sums are FP32.  Loss: mean
// squared error.  Every reduction over samples runs in a fixed order (one
// thread per parameter), so training is deterministic.
#include <algorithm>
#include <cmath>
#include <random>
#include <vector>

#include "common.cuh"


namespace pg {

namespace {

constexpr int MLP_THREADS = 128;
constexpr int MAX_IN = 64, MAX_H = 128;

struct Layout {
    int n_in, n_h1, n_h2;
    __host__ __device__ int w1() const { return 0; }
    __host__ __device__ int b1() const { return n_h1 * n_in; }
    __host__ __device__ int w2() const { return b1() + n_h1; }
    __host__ __device__ int b2() const { return w2() + n_h2 * n_h1; }
    __host__ __device__ int w3() const { return b2() + n_h2; }
    __host__ __device__ int b3() const { return w3() + n_h2; }
    __host__ __device__ int total() const { return b3() + 1; }
};

// ---- descriptors -----------------------------------------------------------

struct DescArgs {
    int n, T, n_gauss;
    const double* pos;
    const int* type;
    CellK C;
    const int* start;
    const int* idx;
    const int* off;
    float r0, dmu, inv2w2, rc;
    float* out;  // n x (T * n_gauss)
};

__global__ void desc_kernel(DescArgs A) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= A.n) return;
    const int i = warp;
    const int nf = A.T * A.n_gauss;
    const double xi = A.pos[3 * i], yi = A.pos[3 * i + 1], zi = A.pos[3 * i + 2];
    for (int f0 = 0; f0 < nf; f0 += 32) {
        const int f = f0 + lane;
        const int tf = f < nf ? f / A.n_gauss : -1;
        const float mu = A.r0 + A.dmu * (float)(f < nf ? f % A.n_gauss : 0);
        float acc = 0.0f;
        for (int e = A.start[i]; e < A.start[i + 1]; ++e) {
            const int j = A.idx[e];
            if (A.type[j] != tf) continue;
            const double o0 = A.off[3 * e], o1 = A.off[3 * e + 1], o2 = A.off[3 * e + 2];
            const double x = A.pos[3 * j] - xi + (o0 * A.C.vc[0][0] + o1 * A.C.vc[0][1] + o2 * A.C.vc[0][2]);
            const double y = A.pos[3 * j + 1] - yi + (o0 * A.C.vc[1][0] + o1 * A.C.vc[1][1] + o2 * A.C.vc[1][2]);
            const double z = A.pos[3 * j + 2] - zi + (o0 * A.C.vc[2][0] + o1 * A.C.vc[2][1] + o2 * A.C.vc[2][2]);
            const float r = (float)sqrt(x * x + y * y + z * z);
            if (!(r < A.rc)) continue;
            const float d = r - mu;
            acc += expf(-d * d * A.inv2w2) * 0.5f * (1.0f + cospif(r / A.rc));
        }
        if (f < nf) A.out[(long long)i * nf + f] = acc;
    }
}

// Fast form for NG Gaussians and at most TMAX types: lanes over the atom's
// entries (one separation per entry instead of one per feature), features in
// registers, then a fixed-order shuffle tree per feature.
template <int NG, int TMAX>
__global__ void desc_kernel_lanes(DescArgs A) {
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (warp >= A.n) return;  // whole warps leave together
    const int i = warp;
    const double xi = A.pos[3 * i], yi = A.pos[3 * i + 1], zi = A.pos[3 * i + 2];
    float acc[TMAX][NG];
#pragma unroll
    for (int t = 0; t < TMAX; ++t)
#pragma unroll
        for (int k = 0; k < NG; ++k) acc[t][k] = 0.0f;
    for (int e = A.start[i] + lane; e < A.start[i + 1]; e += 32) {
        const int j = A.idx[e];
        const double o0 = A.off[3 * e], o1 = A.off[3 * e + 1], o2 = A.off[3 * e + 2];
        const double x = A.pos[3 * j] - xi + (o0 * A.C.vc[0][0] + o1 * A.C.vc[0][1] + o2 * A.C.vc[0][2]);
        const double y = A.pos[3 * j + 1] - yi + (o0 * A.C.vc[1][0] + o1 * A.C.vc[1][1] + o2 * A.C.vc[1][2]);
        const double z = A.pos[3 * j + 2] - zi + (o0 * A.C.vc[2][0] + o1 * A.C.vc[2][1] + o2 * A.C.vc[2][2]);
        const float r = (float)sqrt(x * x + y * y + z * z);
        if (!(r < A.rc)) continue;
        const int tj = A.type[j];
        const float fc = 0.5f * (1.0f + cospif(r / A.rc));
#pragma unroll
        for (int t = 0; t < TMAX; ++t) {
            if (t != tj) continue;
#pragma unroll
            for (int k = 0; k < NG; ++k) {
                const float d = r - (A.r0 + A.dmu * (float)k);
                acc[t][k] += expf(-d * d * A.inv2w2) * fc;
            }
        }
    }
    const int nf = A.T * NG;
#pragma unroll
    for (int t = 0; t < TMAX; ++t)
#pragma unroll
        for (int k = 0; k < NG; ++k) {
            float v = acc[t][k];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0 && t < A.T) A.out[(long long)i * nf + t * NG + k] = v;
        }
}

// ---- network -----------------------------------------------------------------

// parameters (BF16) into shared memory as FP32
__device__ __forceinline__ void load_params(float* sw, const __nv_bfloat16* wb, int total) {
    for (int q = threadIdx.x; q < total; q += blockDim.x) sw[q] = __bfloat162float(wb[q]);
    __syncthreads();
}

// forward pass of sample rows[s] (or s); keeps h1, h2 when training
template <bool TRAIN>
__global__ void __launch_bounds__(MLP_THREADS) mlp_forward(Layout Lp, const __nv_bfloat16* __restrict__ wb,
                                                           const float* __restrict__ x, const int* __restrict__ rows,
                                                           int nb, float* __restrict__ out, float* __restrict__ h1o,
                                                           float* __restrict__ h2o) {
    extern __shared__ float sw[];
    load_params(sw, wb, Lp.total());
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= nb) return;
    const long long row = rows ? rows[s] : s;
    float xin[MAX_IN], h1[MAX_H];
    for (int a = 0; a < Lp.n_in; ++a) xin[a] = x[row * Lp.n_in + a];
    for (int j = 0; j < Lp.n_h1; ++j) {
        const float* wr = sw + Lp.w1() + j * Lp.n_in;
        float z = sw[Lp.b1() + j];
        for (int a = 0; a < Lp.n_in; ++a) z = fmaf(wr[a], xin[a], z);
        h1[j] = tanhf(z);
        if (TRAIN) h1o[(long long)s * Lp.n_h1 + j] = h1[j];
    }
    float y = sw[Lp.b3()];
    for (int k = 0; k < Lp.n_h2; ++k) {
        const float* wr = sw + Lp.w2() + k * Lp.n_h1;
        float z = sw[Lp.b2() + k];
        for (int j = 0; j < Lp.n_h1; ++j) z = fmaf(wr[j], h1[j], z);
        const float h2 = tanhf(z);
        if (TRAIN) h2o[(long long)s * Lp.n_h2 + k] = h2;
        y = fmaf(sw[Lp.w3() + k], h2, y);
    }
    out[s] = y;
}

// output and hidden-layer errors of one batch; per-block partial loss
__global__ void __launch_bounds__(MLP_THREADS) mlp_backward(Layout Lp, const __nv_bfloat16* __restrict__ wb,
                                                            const float* __restrict__ target,
                                                            const int* __restrict__ rows, int nb,
                                                            const float* __restrict__ out,
                                                            const float* __restrict__ h1, const float* __restrict__ h2,
                                                            float* __restrict__ dy, float* __restrict__ dz1,
                                                            float* __restrict__ dz2, float* __restrict__ lpart) {
    extern __shared__ float sw[];
    __shared__ float sl[MLP_THREADS];
    load_params(sw, wb, Lp.total());
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    float l = 0.0f;
    if (s < nb) {
        const long long row = rows ? rows[s] : s;
        const float err = out[s] - target[row];
        l = err * err;
        const float g = 2.0f * err / (float)nb;
        dy[s] = g;
        float d2[MAX_H];
        for (int k = 0; k < Lp.n_h2; ++k) {
            const float h = h2[(long long)s * Lp.n_h2 + k];
            d2[k] = g * sw[Lp.w3() + k] * (1.0f - h * h);
            dz2[(long long)s * Lp.n_h2 + k] = d2[k];
        }
        for (int j = 0; j < Lp.n_h1; ++j) {
            float a = 0.0f;
            for (int k = 0; k < Lp.n_h2; ++k) a = fmaf(d2[k], sw[Lp.w2() + k * Lp.n_h1 + j], a);
            const float h = h1[(long long)s * Lp.n_h1 + j];
            dz1[(long long)s * Lp.n_h1 + j] = a * (1.0f - h * h);
        }
    }
    sl[threadIdx.x] = l;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sl[threadIdx.x] += sl[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) lpart[blockIdx.x] = sl[0];
}

// gradient of every parameter: one thread per parameter, sum over the batch
// in sample order
__global__ void mlp_grad(Layout Lp, const float* __restrict__ x, const int* __restrict__ rows, int nb,
                         const float* __restrict__ h1, const float* __restrict__ h2, const float* __restrict__ dy,
                         const float* __restrict__ dz1, const float* __restrict__ dz2, float* __restrict__ grad) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= Lp.total()) return;
    float g = 0.0f;
    if (p < Lp.b1()) {
        const int j = p / Lp.n_in, a = p % Lp.n_in;
        for (int s = 0; s < nb; ++s) {
            const long long row = rows ? rows[s] : s;
            g = fmaf(dz1[(long long)s * Lp.n_h1 + j], x[row * Lp.n_in + a], g);
        }
    } else if (p < Lp.w2()) {
        const int j = p - Lp.b1();
        for (int s = 0; s < nb; ++s) g += dz1[(long long)s * Lp.n_h1 + j];
    } else if (p < Lp.b2()) {
        const int q = p - Lp.w2(), k = q / Lp.n_h1, j = q % Lp.n_h1;
        for (int s = 0; s < nb; ++s) g = fmaf(dz2[(long long)s * Lp.n_h2 + k], h1[(long long)s * Lp.n_h1 + j], g);
    } else if (p < Lp.w3()) {
        const int k = p - Lp.b2();
        for (int s = 0; s < nb; ++s) g += dz2[(long long)s * Lp.n_h2 + k];
    } else if (p < Lp.b3()) {
        const int k = p - Lp.w3();
        for (int s = 0; s < nb; ++s) g = fmaf(dy[s], h2[(long long)s * Lp.n_h2 + k], g);
    } else {
        for (int s = 0; s < nb; ++s) g += dy[s];
    }
    grad[p] = g;
}

// Adam (Kingma & Ba 2015) on the FP32 master copy, then the BF16 copy
__global__ void mlp_adam(int np, float* __restrict__ w, float* __restrict__ m, float* __restrict__ v,
                         const float* __restrict__ g, __nv_bfloat16* __restrict__ wb, float lr, float b1, float b2,
                         float eps, float c1, float c2) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= np) return;
    const float gp = g[p];
    const float mp = b1 * m[p] + (1.0f - b1) * gp;
    const float vp = b2 * v[p] + (1.0f - b2) * gp * gp;
    m[p] = mp;
    v[p] = vp;
    const float wp = w[p] - lr * (mp / c1) / (sqrtf(vp / c2) + eps);
    w[p] = wp;
    wb[p] = __float2bfloat16_rn(wp);
}

__global__ void to_bf16(int np, const float* __restrict__ w, __nv_bfloat16* __restrict__ wb) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < np) wb[p] = __float2bfloat16_rn(w[p]);
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace

Layout mlp_layout(const pg_mlp* M) { return Layout{M->n_in, M->n_h1, M->n_h2}; }

size_t mlp_smem(const pg_mlp* M) { return sizeof(float) * (size_t)M->n_params; }

// ---- host side ---------------------------------------------------------------

void descriptors(pg_context* ctx, int n_gauss, double r0, double r1, double width, double cutoff, float* out) {
    require(ctx->have_list && ctx->have_atoms && ctx->have_cell, PG_ERR_NOT_READY,
            "descriptors need atoms, a cell and neighbour lists");
    require(n_gauss >= 1 && width > 0 && cutoff > 0 && r1 >= r0, PG_ERR_INVALID, "invalid descriptor parameters");
    require(cutoff <= ctx->list_min_cutoff + 1e-12, PG_ERR_INVALID,
            "the neighbour lists are shorter than the descriptor cutoff");
    const int T = std::max(ctx->n_types, 1);
    const int nf = T * n_gauss;
    ctx->mlp_desc.resize((size_t)std::max(ctx->n, 1) * nf);
    DescArgs A{};
    A.n = ctx->n;
    A.T = T;
    A.n_gauss = n_gauss;
    A.pos = ctx->pos.p;
    A.type = ctx->type.p;
    A.C = cell_kernel_view(ctx->cell);
    A.start = ctx->nb_start.p;
    A.idx = ctx->nb_idx.p;
    A.off = ctx->nb_off.p;
    A.r0 = (float)r0;
    A.dmu = n_gauss > 1 ? (float)((r1 - r0) / (n_gauss - 1)) : 0.0f;
    A.inv2w2 = (float)(1.0 / (2.0 * width * width));
    A.rc = (float)cutoff;
    A.out = ctx->mlp_desc.p;
    if (ctx->n > 0) {
        if (n_gauss == 16 && T <= 2)
            desc_kernel_lanes<16, 2><<<cdiv((long long)ctx->n * 32, 128), 128, 0, ctx->stream>>>(A);
        else
            desc_kernel<<<cdiv((long long)ctx->n * 32, 128), 128, 0, ctx->stream>>>(A);
        PG_CHECK_LAUNCH();
    }
    ctx->mlp_desc.download(out, (size_t)ctx->n * nf, ctx->stream);
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
}

void mlp_create(pg_mlp** out, int n_in, int n_h1, int n_h2, int device) {
    require(n_in >= 1 && n_in <= MAX_IN && n_h1 >= 1 && n_h1 <= MAX_H && n_h2 >= 1 && n_h2 <= MAX_H, PG_ERR_INVALID,
            "network sizes: inputs 1..64, hidden layers 1..128");
    if (device >= 0) PG_CUDA(cudaSetDevice(device));
    int dev = 0;
    PG_CUDA(cudaGetDevice(&dev));
    pg_mlp* M = new pg_mlp();
    M->device = dev;
    M->n_in = n_in;
    M->n_h1 = n_h1;
    M->n_h2 = n_h2;
    M->n_params = Layout{n_in, n_h1, n_h2}.total();
    cudaError_t e = cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete M;
        PG_CUDA(e);
    }
    const size_t smem = mlp_smem(M);
    if (smem > 48 * 1024) {
        PG_CUDA(cudaFuncSetAttribute(mlp_forward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        PG_CUDA(cudaFuncSetAttribute(mlp_forward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        PG_CUDA(cudaFuncSetAttribute(mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    // Glorot-uniform weights and zero biases from a fixed seed
    std::vector<float> w((size_t)M->n_params, 0.0f);
    std::mt19937_64 rng(0x5eedull);
    const Layout Lp = mlp_layout(M);
    auto fill = [&](int at, int rows, int cols) {
        std::uniform_real_distribution<float> u(-std::sqrt(6.0f / (rows + cols)), std::sqrt(6.0f / (rows + cols)));
        for (int q = 0; q < rows * cols; ++q) w[(size_t)at + q] = u(rng);
    };
    fill(Lp.w1(), n_h1, n_in);
    fill(Lp.w2(), n_h2, n_h1);
    fill(Lp.w3(), 1, n_h2);
    M->w.upload(w.data(), w.size(), M->stream);
    std::vector<float> z(w.size(), 0.0f);
    M->m.upload(z.data(), z.size(), M->stream);
    M->v.upload(z.data(), z.size(), M->stream);
    M->grad.resize(w.size());
    M->wb.resize(w.size());
    to_bf16<<<cdiv(M->n_params, 256), 256, 0, M->stream>>>((int)M->n_params, M->w.p, M->wb.p);
    PG_CHECK_LAUNCH();
    PG_CUDA(cudaStreamSynchronize(M->stream));
    *out = M;
}

void mlp_set_params(pg_mlp* M, const float* params, long long n) {
    require(n == M->n_params, PG_ERR_INVALID, "parameter count does not match the network");
    M->w.upload(params, (size_t)n, M->stream);
    std::vector<float> z((size_t)n, 0.0f);
    M->m.upload(z.data(), z.size(), M->stream);
    M->v.upload(z.data(), z.size(), M->stream);
    M->step = 0;
    to_bf16<<<cdiv(n, 256), 256, 0, M->stream>>>((int)n, M->w.p, M->wb.p);
    PG_CHECK_LAUNCH();
    PG_CUDA(cudaStreamSynchronize(M->stream));
}

void mlp_get_params(pg_mlp* M, float* params, long long n) {
    require(n == M->n_params, PG_ERR_INVALID, "parameter count does not match the network");
    M->w.download(params, (size_t)n, M->stream);
    PG_CUDA(cudaStreamSynchronize(M->stream));
}

void mlp_add_samples(pg_mlp* M, const float* x, const float* y, long long n) {
    require(n >= 0, PG_ERR_INVALID, "negative sample count");
    const long long total = M->n_samples + n;
    // grow keeping the samples already on the device
    if ((size_t)total * M->n_in > M->x.cap || (size_t)total > M->y.cap) {
        DevBuf<float> nx, ny;
        nx.resize((size_t)std::max(total, 1ll) * M->n_in * 2);
        ny.resize((size_t)std::max(total, 1ll) * 2);
        if (M->n_samples) {
            PG_CUDA(cudaMemcpyAsync(nx.p, M->x.p, sizeof(float) * M->n_samples * M->n_in, cudaMemcpyDeviceToDevice,
                                    M->stream));
            PG_CUDA(cudaMemcpyAsync(ny.p, M->y.p, sizeof(float) * M->n_samples, cudaMemcpyDeviceToDevice, M->stream));
        }
        PG_CUDA(cudaStreamSynchronize(M->stream));
        std::swap(M->x.p, nx.p);
        std::swap(M->x.cap, nx.cap);
        std::swap(M->y.p, ny.p);
        std::swap(M->y.cap, ny.cap);
    }
    if (n) {
        PG_CUDA(cudaMemcpyAsync(M->x.p + M->n_samples * M->n_in, x, sizeof(float) * n * M->n_in,
                                cudaMemcpyHostToDevice, M->stream));
        PG_CUDA(cudaMemcpyAsync(M->y.p + M->n_samples, y, sizeof(float) * n, cudaMemcpyHostToDevice, M->stream));
        PG_CUDA(cudaStreamSynchronize(M->stream));
    }
    M->n_samples = total;
}

void mlp_clear_samples(pg_mlp* M) { M->n_samples = 0; }

// forward + backward of one batch (rows into the sample arrays, or the first
// nb samples); leaves the gradient in M->grad and returns the summed squared error
static double batch_grad(pg_mlp* M, const float* x, const float* y, const int* rows, int nb) {
    const Layout Lp = mlp_layout(M);
    const size_t smem = mlp_smem(M);
    M->h1.resize((size_t)nb * M->n_h1);
    M->h2.resize((size_t)nb * M->n_h2);
    M->dz1.resize((size_t)nb * M->n_h1);
    M->dz2.resize((size_t)nb * M->n_h2);
    M->out.resize((size_t)nb);
    M->dy.resize((size_t)nb);
    const int blocks = cdiv(nb, MLP_THREADS);
    M->lpart.resize((size_t)blocks);
    mlp_forward<true><<<blocks, MLP_THREADS, smem, M->stream>>>(Lp, M->wb.p, x, rows, nb, M->out.p, M->h1.p, M->h2.p);
    mlp_backward<<<blocks, MLP_THREADS, smem, M->stream>>>(Lp, M->wb.p, y, rows, nb, M->out.p, M->h1.p, M->h2.p,
                                                           M->dy.p, M->dz1.p, M->dz2.p, M->lpart.p);
    mlp_grad<<<cdiv(M->n_params, 128), 128, 0, M->stream>>>(Lp, x, rows, nb, M->h1.p, M->h2.p, M->dy.p, M->dz1.p,
                                                            M->dz2.p, M->grad.p);
    PG_CHECK_LAUNCH();
    std::vector<float> lp((size_t)blocks);
    M->lpart.download(lp.data(), lp.size(), M->stream);
    PG_CUDA(cudaStreamSynchronize(M->stream));
    double l = 0.0;
    for (float v : lp) l += v;
    return l;
}

void mlp_train(pg_mlp* M, int epochs, int batch, float lr, unsigned long long seed, float* epoch_loss) {
    require(M->n_samples > 0, PG_ERR_NOT_READY, "no training samples");
    require(epochs >= 0 && batch >= 1 && lr > 0.0f, PG_ERR_INVALID, "invalid training settings");
    const long long n = M->n_samples;
    require(n < (1ll << 31), PG_ERR_INVALID, "too many samples");
    std::vector<int> order((size_t)n);
    for (long long q = 0; q < n; ++q) order[(size_t)q] = (int)q;
    std::mt19937_64 rng(seed);
    M->order.resize((size_t)n);
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(order.begin(), order.end(), rng);
        M->order.upload(order.data(), order.size(), M->stream);
        double loss = 0.0;
        for (long long b0 = 0; b0 < n; b0 += batch) {
            const int nb = (int)std::min<long long>(batch, n - b0);
            loss += batch_grad(M, M->x.p, M->y.p, M->order.p + b0, nb);
            M->step++;
            const float c1 = 1.0f - std::pow(b1, (float)M->step), c2 = 1.0f - std::pow(b2, (float)M->step);
            mlp_adam<<<cdiv(M->n_params, 256), 256, 0, M->stream>>>((int)M->n_params, M->w.p, M->m.p, M->v.p,
                                                                    M->grad.p, M->wb.p, lr, b1, b2, eps, c1, c2);
            PG_CHECK_LAUNCH();
        }
        if (epoch_loss) epoch_loss[ep] = (float)(loss / (double)n);
    }
    PG_CUDA(cudaStreamSynchronize(M->stream));
}

void mlp_gradients(pg_mlp* M, const float* x, const float* y, long long n, float* grad, double* loss) {
    require(n >= 1 && n < (1ll << 31), PG_ERR_INVALID, "sample count out of range");
    M->px.resize((size_t)n * M->n_in);
    M->py.resize((size_t)n);
    M->px.upload(x, (size_t)n * M->n_in, M->stream);
    M->py.upload(y, (size_t)n, M->stream);
    const double l = batch_grad(M, M->px.p, M->py.p, nullptr, (int)n);
    M->grad.download(grad, (size_t)M->n_params, M->stream);
    PG_CUDA(cudaStreamSynchronize(M->stream));
    if (loss) *loss = l / (double)n;
}

void mlp_predict(pg_mlp* M, const float* x, long long n, float* y) {
    require(n >= 0 && n < (1ll << 31), PG_ERR_INVALID, "sample count out of range");
    if (n == 0) return;
    M->px.resize((size_t)n * M->n_in);
    M->py.resize((size_t)n);
    M->px.upload(x, (size_t)n * M->n_in, M->stream);
    mlp_forward<false><<<cdiv(n, MLP_THREADS), MLP_THREADS, mlp_smem(M), M->stream>>>(
        mlp_layout(M), M->wb.p, M->px.p, nullptr, (int)n, M->py.p, nullptr, nullptr);
    PG_CHECK_LAUNCH();
    M->py.download(y, (size_t)n, M->stream);
    PG_CUDA(cudaStreamSynchronize(M->stream));
}

}  // namespace pg
