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
// Network: z1 = W1 x~ + b1, h1 = tanh(z1), z2 = W2 h1~ + b2, h2 = tanh(z2),
// y = w3 . h2 + b3, where x~ and h1~ are the inputs and the first-layer
// activations rounded to BF16 (the operands of the tensor-core path,
// mlp_tc.cu, which trains networks of two 64-unit layers; every path here
// computes the same function).  Parameters are kept in FP32 (Adam's master
// copy) and as a BF16 copy that every forward pass reads; all sums are FP32.
// Loss: mean squared error.  Every reduction over samples runs in a fixed
// order, so training is deterministic.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <memory>
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

// v rounded to the nearest BF16 (ties to even), as an FP32 value
__device__ __forceinline__ float rbf(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

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
    for (int a = 0; a < Lp.n_in; ++a) xin[a] = rbf(x[row * Lp.n_in + a]);
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
        for (int j = 0; j < Lp.n_h1; ++j) z = fmaf(wr[j], rbf(h1[j]), z);
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
            g = fmaf(dz1[(long long)s * Lp.n_h1 + j], rbf(x[row * Lp.n_in + a]), g);
        }
    } else if (p < Lp.w2()) {
        const int j = p - Lp.b1();
        for (int s = 0; s < nb; ++s) g += dz1[(long long)s * Lp.n_h1 + j];
    } else if (p < Lp.b2()) {
        const int q = p - Lp.w2(), k = q / Lp.n_h1, j = q % Lp.n_h1;
        for (int s = 0; s < nb; ++s) g = fmaf(dz2[(long long)s * Lp.n_h2 + k], rbf(h1[(long long)s * Lp.n_h1 + j]), g);
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

// ---- inference -----------------------------------------------------------------

// Parameters in shared memory with odd row strides, so that the lanes of a
// warp (one hidden unit each) read different banks.
struct PadLayout {
    int n_in, n_h1, n_h2, p1, p2;
    __host__ __device__ explicit PadLayout(const Layout& L)
        : n_in(L.n_in), n_h1(L.n_h1), n_h2(L.n_h2), p1(L.n_in | 1), p2(L.n_h1 | 1) {}
    __host__ __device__ int w1() const { return 0; }
    __host__ __device__ int b1() const { return n_h1 * p1; }
    __host__ __device__ int w2() const { return b1() + n_h1; }
    __host__ __device__ int b2() const { return w2() + n_h2 * p2; }
    __host__ __device__ int w3() const { return b2() + n_h2; }
    __host__ __device__ int b3() const { return w3() + n_h2; }
    __host__ __device__ int total() const { return b3() + 1; }
};

// What the charge prediction needs besides the network: the raw descriptors
// (per atom type and Gaussian), the element of each type, the input
// normalisation and the output scale.
struct FoldArgs {
    const float* raw;       // n x (T * G)
    const int* type;        // per atom
    const int* elem;        // per type: element index
    const float* x_mean;    // n_in
    const float* x_scale;   // n_in
    int T, G, E;
    double y_mean, y_scale;
    double* q;              // per atom: predicted charge before the total-charge shift
    double* part;           // per block: sum of q (block order)
};

constexpr int INF_THREADS = 256;
constexpr int INF_WARPS = INF_THREADS / 32;

// One warp per sample (grid-stride), lanes over the hidden units.  Every unit
// is the same sequential FMA chain as in mlp_forward, and the output the same
// chain over the second layer, so both kernels give identical results.
// FOLD: the inputs are formed from the raw descriptors as the host-side
// fold does (per-type columns added in type order into per-element columns,
// one-hot element code, (x - mean) / scale), and the charge
// y * y_scale + y_mean is written in FP64 with per-block sums in a fixed order.
template <bool FOLD>
__global__ void __launch_bounds__(INF_THREADS) mlp_infer(Layout L0, const __nv_bfloat16* __restrict__ wb,
                                                         const float* __restrict__ x, int n, float* __restrict__ out,
                                                         FoldArgs F) {
    extern __shared__ float sw[];
    __shared__ float sx[INF_WARPS][MAX_IN], sh1[INF_WARPS][MAX_H], sh2[INF_WARPS][MAX_H];
    __shared__ double sq[INF_WARPS];
    const PadLayout P(L0);
    for (int q = threadIdx.x; q < L0.total(); q += blockDim.x) {
        int d;
        if (q < L0.b1()) d = P.w1() + (q / L0.n_in) * P.p1 + q % L0.n_in;
        else if (q < L0.w2()) d = P.b1() + (q - L0.b1());
        else if (q < L0.b2()) d = P.w2() + ((q - L0.w2()) / L0.n_h1) * P.p2 + (q - L0.w2()) % L0.n_h1;
        else d = P.b2() + (q - L0.b2());  // b2, w3, b3 keep their order
        sw[d] = __bfloat162float(wb[q]);
    }
    __syncthreads();
    const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
    double qsum = 0.0;
    for (int s = blockIdx.x * INF_WARPS + w; s < n; s += gridDim.x * INF_WARPS) {
        for (int a = lane; a < L0.n_in; a += 32) {
            float v;
            if constexpr (FOLD) {
                const int EG = F.E * F.G;
                if (a < EG) {
                    const int e = a / F.G, k = a % F.G;
                    v = 0.0f;
                    for (int t = 0; t < F.T; ++t)
                        if (F.elem[t] == e) v += F.raw[(long long)s * F.T * F.G + t * F.G + k];
                } else {
                    v = F.elem[F.type[s]] == a - EG ? 1.0f : 0.0f;
                }
                v = __fdiv_rn(__fsub_rn(v, F.x_mean[a]), F.x_scale[a]);
            } else {
                v = x[(long long)s * L0.n_in + a];
            }
            sx[w][a] = rbf(v);
        }
        __syncwarp();
        for (int j = lane; j < L0.n_h1; j += 32) {
            const float* wr = sw + P.w1() + j * P.p1;
            float z = sw[P.b1() + j];
            for (int a = 0; a < L0.n_in; ++a) z = fmaf(wr[a], sx[w][a], z);
            sh1[w][j] = rbf(tanhf(z));
        }
        __syncwarp();
        for (int k = lane; k < L0.n_h2; k += 32) {
            const float* wr = sw + P.w2() + k * P.p2;
            float z = sw[P.b2() + k];
            for (int j = 0; j < L0.n_h1; ++j) z = fmaf(wr[j], sh1[w][j], z);
            sh2[w][k] = tanhf(z);
        }
        __syncwarp();
        if (lane == 0) {
            float y = sw[P.b3()];
            for (int k = 0; k < L0.n_h2; ++k) y = fmaf(sw[P.w3() + k], sh2[w][k], y);
            if constexpr (FOLD) {
                const double qv = __dadd_rn(__dmul_rn((double)y, F.y_scale), F.y_mean);
                F.q[s] = qv;
                qsum += qv;
            } else {
                out[s] = y;
            }
        }
        __syncwarp();
    }
    if constexpr (FOLD) {
        if (lane == 0) sq[w] = qsum;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = 0.0;
            for (int k = 0; k < INF_WARPS; ++k) t += sq[k];
            F.part[blockIdx.x] = t;
        }
    }
}

// q_i - (sum q - total) / n into the charges; every block forms the sum from
// the block partials in the same order
__global__ void mlp_charge_shift(const double* __restrict__ q, const double* __restrict__ part, int nparts, int n,
                                 double total, double* __restrict__ charge) {
    __shared__ double shift;
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int b = 0; b < nparts; ++b) t += part[b];
        shift = (t - total) / n;
    }
    __syncthreads();
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) charge[i] = q[i] - shift;
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

// blocks of the inference kernel: at most two per SM, each reading the
// parameters into shared memory once
inline int infer_blocks(long long n) { return std::max(1, std::min(cdiv(n, INF_WARPS), 2 * sm_count())); }

}  // namespace

Layout mlp_layout(const pg_mlp* M) { return Layout{M->n_in, M->n_h1, M->n_h2}; }

size_t mlp_smem(const pg_mlp* M) { return sizeof(float) * (size_t)M->n_params; }
size_t infer_smem(const pg_mlp* M) { return sizeof(float) * (size_t)PadLayout(mlp_layout(M)).total(); }

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
    if (out) {
        ctx->mlp_desc.download(out, (size_t)ctx->n * nf, ctx->stream);
        PG_CUDA(cudaStreamSynchronize(ctx->stream));
    }
}

void mlp_create(pg_mlp** out, int n_in, int n_h1, int n_h2, int device) {
    require(n_in >= 1 && n_in <= MAX_IN && n_h1 >= 1 && n_h1 <= MAX_H && n_h2 >= 1 && n_h2 <= MAX_H, PG_ERR_INVALID,
            "network sizes: inputs 1..64, hidden layers 1..128");
    if (device >= 0) PG_CUDA(cudaSetDevice(device));
    int dev = 0;
    PG_CUDA(cudaGetDevice(&dev));
    std::unique_ptr<pg_mlp> hold(new pg_mlp());
    pg_mlp* M = hold.get();
    M->device = dev;
    M->n_in = n_in;
    M->n_h1 = n_h1;
    M->n_h2 = n_h2;
    M->n_params = Layout{n_in, n_h1, n_h2}.total();
    PG_CUDA(cudaStreamCreateWithFlags(&M->stream, cudaStreamNonBlocking));
    // shared-memory limits of the network kernels, set once to what the
    // largest network allowed here needs (a per-network value would shrink
    // the limit under a larger network created before)
    const Layout big{MAX_IN, MAX_H, MAX_H};
    const int fwd_max = (int)(sizeof(float) * (size_t)big.total());
    const int inf_max = (int)(sizeof(float) * (size_t)PadLayout(big).total());
    PG_CUDA(cudaFuncSetAttribute(mlp_infer<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, inf_max));
    PG_CUDA(cudaFuncSetAttribute(mlp_infer<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, inf_max));
    PG_CUDA(cudaFuncSetAttribute(mlp_forward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, fwd_max));
    PG_CUDA(cudaFuncSetAttribute(mlp_forward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, fwd_max));
    PG_CUDA(cudaFuncSetAttribute(mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize, fwd_max));
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
    *out = hold.release();
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
    if (mlp_tc_eligible(M)) {
        M->dloss.resize(1);
        PG_CUDA(cudaMemsetAsync(M->dloss.p, 0, sizeof(double), M->stream));
        mlp_tc_batch_grad(M, x, y, rows, nb, M->dloss.p);
        double l = 0.0;
        M->dloss.download(&l, 1, M->stream);
        PG_CUDA(cudaStreamSynchronize(M->stream));
        return l;
    }
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
    const bool tc = mlp_tc_eligible(M);
    M->dloss.resize(1);
    for (int ep = 0; ep < epochs; ++ep) {
        std::shuffle(order.begin(), order.end(), rng);
        M->order.upload(order.data(), order.size(), M->stream);
        double loss = 0.0;
        // tensor-core path: the epoch's loss stays on the device until its end
        if (tc) PG_CUDA(cudaMemsetAsync(M->dloss.p, 0, sizeof(double), M->stream));
        for (long long b0 = 0; b0 < n; b0 += batch) {
            const int nb = (int)std::min<long long>(batch, n - b0);
            if (tc) mlp_tc_batch_grad(M, M->x.p, M->y.p, M->order.p + b0, nb, M->dloss.p);
            else loss += batch_grad(M, M->x.p, M->y.p, M->order.p + b0, nb);
            M->step++;
            const float c1 = 1.0f - std::pow(b1, (float)M->step), c2 = 1.0f - std::pow(b2, (float)M->step);
            mlp_adam<<<cdiv(M->n_params, 256), 256, 0, M->stream>>>((int)M->n_params, M->w.p, M->m.p, M->v.p,
                                                                    M->grad.p, M->wb.p, lr, b1, b2, eps, c1, c2);
            PG_CHECK_LAUNCH();
        }
        if (tc) {
            M->dloss.download(&loss, 1, M->stream);
            PG_CUDA(cudaStreamSynchronize(M->stream));
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
    mlp_infer<false><<<infer_blocks(n), INF_THREADS, infer_smem(M), M->stream>>>(mlp_layout(M), M->wb.p, M->px.p,
                                                                                  (int)n, M->py.p, FoldArgs{});
    PG_CHECK_LAUNCH();
    M->py.download(y, (size_t)n, M->stream);
    PG_CUDA(cudaStreamSynchronize(M->stream));
}

void mlp_predict_charges(pg_mlp* M, pg_context* ctx, int n_gauss, double r0, double r1, double width, double cutoff,
                         int n_elements, const int* type_element, const float* x_mean, const float* x_scale,
                         double y_mean, double y_scale, double total_charge, double* charges) {
    require(M->device == ctx->device, PG_ERR_INVALID, "network and context on different devices");
    const int T = std::max(ctx->n_types, 1);
    require(n_elements >= 1 && M->n_in == n_elements * (n_gauss + 1), PG_ERR_INVALID,
            "network inputs must be n_elements x (n_gauss + 1)");
    for (int t = 0; t < T; ++t)
        require(type_element[t] >= 0 && type_element[t] < n_elements, PG_ERR_INVALID, "type without an element");
    const int n = ctx->n;
    // descriptors into ctx->mlp_desc, on the context's stream
    descriptors(ctx, n_gauss, r0, r1, width, cutoff, nullptr);
    if (n == 0) return;
    // small per-call inputs in one upload: type -> element, mean, scale
    std::vector<float> h((size_t)T + 2 * (size_t)M->n_in);
    static_assert(sizeof(float) == sizeof(int), "packed upload");
    std::memcpy(h.data(), type_element, sizeof(int) * T);
    std::memcpy(h.data() + T, x_mean, sizeof(float) * M->n_in);
    std::memcpy(h.data() + T + M->n_in, x_scale, sizeof(float) * M->n_in);
    ctx->mlp_fold.upload(h.data(), h.size(), ctx->stream);
    const int nb = infer_blocks(n);
    ctx->mlp_q.resize((size_t)n + (size_t)nb);
    FoldArgs F{};
    F.raw = ctx->mlp_desc.p;
    F.type = ctx->type.p;
    F.elem = (const int*)ctx->mlp_fold.p;
    F.x_mean = ctx->mlp_fold.p + T;
    F.x_scale = ctx->mlp_fold.p + T + M->n_in;
    F.T = T;
    F.G = n_gauss;
    F.E = n_elements;
    F.y_mean = y_mean;
    F.y_scale = y_scale;
    F.q = ctx->mlp_q.p;
    F.part = ctx->mlp_q.p + n;
    // the weights may have been written on the network's own stream
    PG_CUDA(cudaStreamSynchronize(M->stream));
    mlp_infer<true><<<nb, INF_THREADS, infer_smem(M), ctx->stream>>>(mlp_layout(M), M->wb.p, nullptr, n, nullptr, F);
    mlp_charge_shift<<<cdiv(n, 256), 256, 0, ctx->stream>>>(F.q, F.part, nb, n, total_charge, ctx->charge.p);
    PG_CHECK_LAUNCH();
    if (charges) ctx->charge.download(charges, (size_t)n, ctx->stream);
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
}

}  // namespace pg
