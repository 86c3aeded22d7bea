// mlp_tc.cu -- training step of the warm-start network (mlp.cu) on the tensor
// cores: forward pass, backward pass and the parameter gradient of one
// mini-batch as BF16 matrix products with FP32 accumulation (mma.sync
// m16n8k16), for networks with two hidden layers of 64 units and at most 64
// inputs -- the shape of the SiO2 warm start.  Other shapes train with the
// scalar kernels of mlp.cu.
//
// The network computed is the one every path of mlp.cu computes: inputs and
// first-layer activations rounded to BF16, BF16 weights, FP32 sums:
//   x~ = bf16(x), a1 = tanh(W1 x~ + b1), a1~ = bf16(a1),
//   a2 = tanh(W2 a1~ + b2), y = w3 . a2 + b3.
// The backward pass rounds the layer errors dz2, dz1 to BF16 where they enter
// a matrix product (dz2 W2, dz2^T a1~, dz1^T x~) and keeps everything else in
// FP32.
//
// One block of 4 warps takes 64 samples (16 per warp):
//   Z1 = X~ W1^T, Z2 = A1~ W2^T, dA1 = dZ2 W2            (16 rows per warp)
//   dW2 = dZ2^T A1~, dW1 = dZ1^T X~                      (16 output rows per warp)
// Operands are staged in shared memory with rows padded to a stride of 4 mod 8
// words, so that fragment loads hit distinct banks.  Each block writes its
// gradient to its own row of a partial buffer; a second kernel sums the rows
// in block order, so the gradient is deterministic.
#include <algorithm>

#include "common.cuh"

namespace pg {

namespace {

using bf16 = __nv_bfloat16;

constexpr int TCH = 64;       // hidden units per layer
constexpr int TCS = 64;       // samples per block
constexpr int TCT = 128;      // threads: 4 warps of 16 samples
constexpr int LDH = TCH + 8;  // row stride (bf16) of the 64-wide operands

// parameter offsets for n_in inputs and two hidden layers of TCH units
struct TcLayout {
    int n_in;
    __host__ __device__ int w1() const { return 0; }
    __host__ __device__ int b1() const { return TCH * n_in; }
    __host__ __device__ int w2() const { return b1() + TCH; }
    __host__ __device__ int b2() const { return w2() + TCH * TCH; }
    __host__ __device__ int w3() const { return b2() + TCH; }
    __host__ __device__ int b3() const { return w3() + TCH; }
    __host__ __device__ int total() const { return b3() + 1; }
};

__device__ __forceinline__ uint32_t pack2(float lo, float hi) {
    __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<uint32_t*>(&v);
}

__device__ __forceinline__ float rbf(float v) { return __bfloat162float(__float2bfloat16_rn(v)); }

// D += A B for one 16 x 8 tile, K = 16, BF16 inputs, FP32 accumulator
__device__ __forceinline__ void mma16816(float (&d)[4], const uint32_t (&a)[4], const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0, %1, %2, %3}, {%4, %5, %6, %7}, {%8, %9}, "
        "{%0, %1, %2, %3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

// A fragment: rows r0 .. r0 + 15, columns k0 .. k0 + 15 of a row-major [row][k]
// array with row stride ld
__device__ __forceinline__ void load_a(uint32_t (&a)[4], const bf16* s, int ld, int r0, int k0, int g, int q) {
    a[0] = *reinterpret_cast<const uint32_t*>(s + (r0 + g) * ld + k0 + 2 * q);
    a[1] = *reinterpret_cast<const uint32_t*>(s + (r0 + g + 8) * ld + k0 + 2 * q);
    a[2] = *reinterpret_cast<const uint32_t*>(s + (r0 + g) * ld + k0 + 8 + 2 * q);
    a[3] = *reinterpret_cast<const uint32_t*>(s + (r0 + g + 8) * ld + k0 + 8 + 2 * q);
}

// B fragment (K x 8, K = 16) from an array stored [n][k] (row n holds column n of B)
__device__ __forceinline__ void load_b(uint32_t (&b)[2], const bf16* s, int ld, int n0, int k0, int g, int q) {
    b[0] = *reinterpret_cast<const uint32_t*>(s + (n0 + g) * ld + k0 + 2 * q);
    b[1] = *reinterpret_cast<const uint32_t*>(s + (n0 + g) * ld + k0 + 8 + 2 * q);
}

template <int NT>
__device__ __forceinline__ void zero(float (&acc)[NT][4]) {
#pragma unroll
    for (int t = 0; t < NT; ++t)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[t][c] = 0.0f;
}

// 16 rows (r0 ..) x (8 NT) columns of A B, A [row][k] (stride lda), B stored [n][k]
// (stride ldb), K = KD
template <int NT, int KD>
__device__ __forceinline__ void tile_product(float (&acc)[NT][4], const bf16* A, int lda, const bf16* B, int ldb,
                                             int r0, int g, int q) {
    zero(acc);
#pragma unroll
    for (int k0 = 0; k0 < KD; k0 += 16) {
        uint32_t a[4];
        load_a(a, A, lda, r0, k0, g, q);
#pragma unroll
        for (int t = 0; t < NT; ++t) {
            uint32_t b[2];
            load_b(b, B, ldb, 8 * t, k0, g, q);
            mma16816(acc[t], a, b);
        }
    }
}

template <int KI>
constexpr size_t tc_smem_bytes() {
    return sizeof(bf16) * ((size_t)TCH * (KI + 8) + 2 * (size_t)TCH * LDH + (size_t)TCS * (KI + 8) + (size_t)KI * LDH +
                           5 * (size_t)TCH * LDH) +
           sizeof(float) * (3 * (size_t)TCH + (size_t)TCS + (size_t)TCS * (TCH + 1) + 8);
}

// Loss and parameter gradient of the samples blockIdx.x * 64 .. + 63 of the
// batch (rows: sample indices, or the first nb samples); KI: inputs padded to
// a multiple of 16.  gpart row blockIdx.x receives the block's gradient,
// lpart[blockIdx.x] its summed squared error.
template <int KI>
__global__ void __launch_bounds__(TCT) mlp_tc_grad(TcLayout Lp, const bf16* __restrict__ wb,
                                                   const float* __restrict__ x, const float* __restrict__ yt,
                                                   const int* __restrict__ rows, int nb, float* __restrict__ gpart,
                                                   float* __restrict__ lpart) {
    constexpr int KIP = KI + 8;
    extern __shared__ __align__(16) unsigned char smem[];
    bf16* sW1 = reinterpret_cast<bf16*>(smem);  // [j][a]
    bf16* sW2 = sW1 + TCH * KIP;                // [k][j]
    bf16* sW2t = sW2 + TCH * LDH;               // [j][k]
    bf16* sX = sW2t + TCH * LDH;                // [s][a]
    bf16* sXt = sX + TCS * KIP;                 // [a][s]
    bf16* sH1 = sXt + KI * LDH;                 // [s][j]
    bf16* sH1t = sH1 + TCS * LDH;               // [j][s]
    bf16* sD2 = sH1t + TCH * LDH;               // [s][k]
    bf16* sD2t = sD2 + TCS * LDH;               // [k][s]
    bf16* sD1t = sD2t + TCH * LDH;              // [j][s]
    float* sb1 = reinterpret_cast<float*>(sD1t + TCH * LDH);
    float* sb2 = sb1 + TCH;
    float* sw3 = sb2 + TCH;
    float* sdy = sw3 + TCH;
    float* sA2 = sdy + TCS;  // [s][k], stride TCH + 1
    float* sl = sA2 + TCS * (TCH + 1);
    const int n_in = Lp.n_in;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31, g = lane >> 2, q = lane & 3;
    const int s0 = blockIdx.x * TCS;
    const bf16 zero_bf = __float2bfloat16_rn(0.0f);
    for (int e = tid; e < TCH * KI; e += TCT) {
        const int j = e / KI, a = e % KI;
        sW1[j * KIP + a] = a < n_in ? wb[Lp.w1() + j * n_in + a] : zero_bf;
    }
    for (int e = tid; e < TCH * TCH; e += TCT) {
        const int k = e / TCH, j = e % TCH;
        const bf16 v = wb[Lp.w2() + e];
        sW2[k * LDH + j] = v;
        sW2t[j * LDH + k] = v;
    }
    for (int e = tid; e < TCH; e += TCT) {
        sb1[e] = __bfloat162float(wb[Lp.b1() + e]);
        sb2[e] = __bfloat162float(wb[Lp.b2() + e]);
        sw3[e] = __bfloat162float(wb[Lp.w3() + e]);
    }
    const float b3 = __bfloat162float(wb[Lp.b3()]);
    for (int e = tid; e < TCS * KI; e += TCT) {
        const int s = e / KI, a = e % KI, gs = s0 + s;
        float v = 0.0f;
        if (gs < nb && a < n_in) {
            const long long row = rows ? rows[gs] : gs;
            v = x[row * n_in + a];
        }
        const bf16 b = __float2bfloat16_rn(v);
        sX[s * KIP + a] = b;
        sXt[a * LDH + s] = b;
    }
    __syncthreads();
    const int r0 = 16 * warp;

    // layer 1: a1 = tanh(x~ W1^T + b1), kept in FP32 for its derivative
    float h1[8][4];
    tile_product<8, KI>(h1, sX, KIP, sW1, KIP, r0, g, q);
#pragma unroll
    for (int t = 0; t < 8; ++t)
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {
            const int row = r0 + g + 8 * hf, col = 8 * t + 2 * q;
            const float u0 = tanhf(h1[t][2 * hf] + sb1[col]), u1 = tanhf(h1[t][2 * hf + 1] + sb1[col + 1]);
            h1[t][2 * hf] = u0;
            h1[t][2 * hf + 1] = u1;
            *reinterpret_cast<uint32_t*>(sH1 + row * LDH + col) = pack2(u0, u1);
            sH1t[col * LDH + row] = __float2bfloat16_rn(u0);
            sH1t[(col + 1) * LDH + row] = __float2bfloat16_rn(u1);
        }
    __syncwarp();

    // layer 2 and the output: a2 = tanh(a1~ W2^T + b2), y = w3 . a2 + b3
    float a2[8][4];
    tile_product<8, TCH>(a2, sH1, LDH, sW2, LDH, r0, g, q);
    float y0 = 0.0f, y1 = 0.0f;
#pragma unroll
    for (int t = 0; t < 8; ++t) {
        const int col = 8 * t + 2 * q;
#pragma unroll
        for (int c = 0; c < 4; ++c) a2[t][c] = tanhf(a2[t][c] + sb2[col + (c & 1)]);
        y0 = fmaf(sw3[col + 1], a2[t][1], fmaf(sw3[col], a2[t][0], y0));
        y1 = fmaf(sw3[col + 1], a2[t][3], fmaf(sw3[col], a2[t][2], y1));
    }
    y0 += __shfl_xor_sync(0xffffffffu, y0, 1);
    y0 += __shfl_xor_sync(0xffffffffu, y0, 2);
    y1 += __shfl_xor_sync(0xffffffffu, y1, 1);
    y1 += __shfl_xor_sync(0xffffffffu, y1, 2);
    const int gr0 = s0 + r0 + g, gr1 = gr0 + 8;
    const float e0 = gr0 < nb ? y0 + b3 - yt[rows ? rows[gr0] : gr0] : 0.0f;
    const float e1 = gr1 < nb ? y1 + b3 - yt[rows ? rows[gr1] : gr1] : 0.0f;
    const float dy0 = 2.0f * e0 / (float)nb, dy1 = 2.0f * e1 / (float)nb;
    float l = q == 0 ? e0 * e0 + e1 * e1 : 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if (lane == 0) sl[warp] = l;
    if (q == 0) {
        sdy[r0 + g] = dy0;
        sdy[r0 + g + 8] = dy1;
    }
    // dz2 = dy w3 (1 - a2^2)
#pragma unroll
    for (int t = 0; t < 8; ++t)
#pragma unroll
        for (int hf = 0; hf < 2; ++hf) {
            const int row = r0 + g + 8 * hf, col = 8 * t + 2 * q;
            const float dy = hf ? dy1 : dy0;
            const float v0 = a2[t][2 * hf], v1 = a2[t][2 * hf + 1];
            const float d0 = dy * sw3[col] * (1.0f - v0 * v0), d1 = dy * sw3[col + 1] * (1.0f - v1 * v1);
            *reinterpret_cast<uint32_t*>(sD2 + row * LDH + col) = pack2(d0, d1);
            sD2t[col * LDH + row] = __float2bfloat16_rn(d0);
            sD2t[(col + 1) * LDH + row] = __float2bfloat16_rn(d1);
            sA2[row * (TCH + 1) + col] = v0;
            sA2[row * (TCH + 1) + col + 1] = v1;
        }
    __syncwarp();

    // dz1 = (dz2~ W2) (1 - a1^2); B = W2 as (k x j), stored [j][k]
    float d1[8][4];
    tile_product<8, TCH>(d1, sD2, LDH, sW2t, LDH, r0, g, q);
#pragma unroll
    for (int t = 0; t < 8; ++t)
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const int row = r0 + g + 8 * (c >> 1), col = 8 * t + 2 * q + (c & 1);
            sD1t[col * LDH + row] = __float2bfloat16_rn(d1[t][c] * (1.0f - h1[t][c] * h1[t][c]));
        }
    __syncthreads();

    // the block's gradient: dW2 = dz2~^T a1~ (rows k of this warp), dW1 = dz1~^T x~ (rows j)
    float* gp = gpart + (size_t)blockIdx.x * Lp.total();
    {
        float acc[8][4];
        tile_product<8, TCS>(acc, sD2t, LDH, sH1t, LDH, r0, g, q);
#pragma unroll
        for (int t = 0; t < 8; ++t)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int row = r0 + g + 8 * (c >> 1), col = 8 * t + 2 * q + (c & 1);
                gp[Lp.w2() + row * TCH + col] = acc[t][c];
            }
    }
    {
        float acc[KI / 8][4];
        tile_product<KI / 8, TCS>(acc, sD1t, LDH, sXt, LDH, r0, g, q);
#pragma unroll
        for (int t = 0; t < KI / 8; ++t)
#pragma unroll
            for (int c = 0; c < 4; ++c) {
                const int row = r0 + g + 8 * (c >> 1), col = 8 * t + 2 * q + (c & 1);
                if (col < n_in) gp[Lp.w1() + row * n_in + col] = acc[t][c];
            }
    }
    // biases and output weights, one thread per parameter, samples in order
    for (int e = tid; e < TCH; e += TCT) {
        float db1 = 0.0f, db2 = 0.0f, dw3 = 0.0f;
        for (int s = 0; s < TCS; ++s) {
            db1 += __bfloat162float(sD1t[e * LDH + s]);
            db2 += __bfloat162float(sD2t[e * LDH + s]);
            dw3 = fmaf(sdy[s], sA2[s * (TCH + 1) + e], dw3);
        }
        gp[Lp.b1() + e] = db1;
        gp[Lp.b2() + e] = db2;
        gp[Lp.w3() + e] = dw3;
    }
    if (tid == 0) {
        float db3 = 0.0f;
        for (int s = 0; s < TCS; ++s) db3 += sdy[s];
        gp[Lp.b3()] = db3;
        lpart[blockIdx.x] = sl[0] + sl[1] + sl[2] + sl[3];
    }
}

// grad[p] = sum of the blocks' partial gradients in block order; loss += the
// blocks' squared errors in block order (thread 0)
__global__ void mlp_tc_reduce(int np, int nblk, const float* __restrict__ gpart, const float* __restrict__ lpart,
                              float* __restrict__ grad, double* __restrict__ loss) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p < np) {
        float s = 0.0f;
        for (int b = 0; b < nblk; ++b) s += gpart[(size_t)b * np + p];
        grad[p] = s;
    }
    if (p == 0 && loss) {
        double l = 0.0;
        for (int b = 0; b < nblk; ++b) l += lpart[b];
        *loss += l;
    }
}

template <int KI>
void launch_tc(const pg_mlp* M, const float* x, const float* y, const int* rows, int nb, float* gpart, float* lpart,
               int blocks) {
    constexpr size_t smem = tc_smem_bytes<KI>();
    static bool attr = false;
    if (!attr) {
        PG_CUDA(cudaFuncSetAttribute(mlp_tc_grad<KI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        attr = true;
    }
    mlp_tc_grad<KI><<<blocks, TCT, smem, M->stream>>>(TcLayout{M->n_in}, M->wb.p, x, y, rows, nb, gpart, lpart);
}

}  // namespace

bool mlp_tc_eligible(const pg_mlp* M) { return M->n_h1 == TCH && M->n_h2 == TCH && M->n_in >= 1 && M->n_in <= 64; }

// Gradient of one batch into M->grad on the tensor cores; the batch's summed
// squared error is added to *loss_dev (device memory, may be null).
void mlp_tc_batch_grad(pg_mlp* M, const float* x, const float* y, const int* rows, int nb, double* loss_dev) {
    const int blocks = (nb + TCS - 1) / TCS;
    const int np = (int)M->n_params;
    M->gpart.resize((size_t)blocks * np);
    M->lpart.resize((size_t)blocks);
    const int ki = ((M->n_in + 15) / 16) * 16;
    switch (ki) {
        case 16: launch_tc<16>(M, x, y, rows, nb, M->gpart.p, M->lpart.p, blocks); break;
        case 32: launch_tc<32>(M, x, y, rows, nb, M->gpart.p, M->lpart.p, blocks); break;
        case 48: launch_tc<48>(M, x, y, rows, nb, M->gpart.p, M->lpart.p, blocks); break;
        default: launch_tc<64>(M, x, y, rows, nb, M->gpart.p, M->lpart.p, blocks); break;
    }
    mlp_tc_reduce<<<(np + 255) / 256, 256, 0, M->stream>>>(np, blocks, M->gpart.p, M->lpart.p, M->grad.p, loss_dev);
    PG_CHECK_LAUNCH();
}

}  // namespace pg
