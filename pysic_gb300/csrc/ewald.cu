// ewald.cu -- reciprocal-space Ewald sum: energy, forces (+ the reference's
// k-space stress term) and electronegativities.
//
// Replaces the k-space parts of calculate_ewald_energy (Potentials.f90:1428-1653),
// calculate_ewald_forces (1675-1971) and calculate_ewald_electronegativities
// (1992-2249).  The listed k vectors are exactly the reference's: k = k1 b1 +
// k2 b2 + k3 b3 with k3 >= 0, (k1,k2,k3) != 0 and |k|^2 < k_radius^2, weight 1
// for k3 = 0 and 2 otherwise.
//
// Phases.  The reference evaluates sin/cos(k . r) in FP64 with arguments of
// ~100 rad.  Here k . r = 2 pi (n1 f1 + n2 f2 + n3 f3) with f the fractional
// coordinates; f is held as 32-bit fixed point, so the phase modulo one turn is
// an exact integer sum and sincospi gets an argument in [-1, 1).  Along n3 the
// phase factor is advanced by multiplying with exp(2 pi i f3) within segments
// of at most 8 consecutive k vectors.
//
// Passes (per-atom and per-k values are gathers; only the energy / virial
// totals are exact fixed-point integer atomics, fixed.cuh):
//  ew_prep     per atom: fixed-point fractions, scaled charge; block sums of q, q^2
//  ew_sfac     per (segment, atom chunk): partial structure factors
//  ew_sreduce  per k: sum the chunk partials (compensated FP32 or FP64),
//              c_k |S_k|^2 into the energy total; block 0 also forms sum q,
//              sum q^2 and the self + background energy
//  ew_field    per (atom, k split): force / electronegativity partials
//  ew_finish   per atom: sum of the splits, constants, self/background
//              electronegativity, output, the reference's stress term r (x) F.
#include <algorithm>
#include <cmath>
#include <type_traits>
#include <vector>

#include "common.cuh"
#include "fixed.cuh"
#include "kernels.cuh"

namespace pg {

namespace {

constexpr int SEG = 8;
constexpr int EW_THREADS = 128;
constexpr double PI = 3.14159265358979323846;

template <typename R>
struct C2 {
    R re, im;
};

// Fixed-point fractional coordinates: 32 bits for the FP32 path, 64 bits for
// the FP64 path (no precision lost beyond the FP64 fraction itself).
struct alignas(32) U64x4 {
    unsigned long long x, y, z, w;
};
template <typename R>
struct Frac;
template <>
struct Frac<float> {
    using U = uint32_t;
    using U4 = uint4;
};
template <>
struct Frac<double> {
    using U = unsigned long long;
    using U4 = U64x4;
};

// sincospi argument 2 u / 2^bits in [-1, 1): (cos, sin)(2 pi u / 2^bits)
__device__ __forceinline__ float turn_(uint32_t u) { return (float)(int32_t)u * 4.656612873077393e-10f; }
__device__ __forceinline__ double turn_(unsigned long long u) { return (double)(long long)u * 1.0842021724855044e-19; }

template <typename R>
__device__ __forceinline__ void phase(typename Frac<R>::U u, R& c, R& s) {
    sincospi_(turn_(u), &s, &c);
}

__device__ __forceinline__ uint32_t to_fixed(double fr, uint32_t) {
    return (uint32_t)(unsigned long long)llrint(fr * 4294967296.0);
}
__device__ __forceinline__ unsigned long long to_fixed(double fr, unsigned long long) {
    // fr in [0, 1): exact scaling by 2^64; 2^64 itself wraps to 0 (one full turn)
    const double v = fr * 18446744073709551616.0;
    return v >= 18446744073709551615.0 ? 0ull : (unsigned long long)v;
}

struct EwArgs {
    int n, nk, nseg, chunks, chunk, splits, seg_per_split;
    const double* pos;
    const double* charge;
    const double* scaler;
    CellK C;
    const int4* seg;      // n1, n2, n3 start, count
    const int* seg_k0;    // first listed k of the segment
    const D4* kvec64;     // kx, ky, kz, c_k (FP64)
    void* frac;           // per atom: fixed-point fractions (Frac<R>::U4)
    double* qs;           // per atom: charge * scaler
    double* qpart;        // per prep block: sum q, sum q^2
    int prep_blocks;
    void* Spart;          // chunks x nk complex (working precision)
    double2* S;           // nk
    void* wS;             // nk: c_k S_k in working precision
    const void* kvecR;    // nk x 4: kx, ky, kz, c_k in working precision
    double* Ssum;         // sum q, sum q^2 (device scalars)
    void* Fpart;          // splits x n x 4 (working precision)
    double inv_eps_2v, inv_eps_4pi, inv_sigma_sqrt_2pi, sigma2, volume_eps;
    int flags, first_f, first_chi;
    double* out_f;
    double* out_chi;
    FxAcc* acc;           // global energy / virial totals (null: not wanted)
    const int* skip;      // optional device flag: nonzero = do nothing
};

template <typename R>
__global__ void ew_prep(EwArgs A) {
    using U = typename Frac<R>::U;
    using U4 = typename Frac<R>::U4;
    __shared__ double sq[EW_THREADS], sq2[EW_THREADS];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (A.skip && *A.skip) return;
    double q = 0.0;
    if (i < A.n) {
        const double p[3] = {A.pos[3 * i], A.pos[3 * i + 1], A.pos[3 * i + 2]};
        U u[3];
        for (int r = 0; r < 3; ++r) {
            const double f = A.C.ic[r][0] * p[0] + A.C.ic[r][1] * p[1] + A.C.ic[r][2] * p[2];
            const double fr = f - floor(f);
            u[r] = to_fixed(fr, U(0));
        }
        U4 v;
        v.x = u[0];
        v.y = u[1];
        v.z = u[2];
        v.w = 0;
        ((U4*)A.frac)[i] = v;
        q = A.charge[i] * A.scaler[i];
        A.qs[i] = q;
    }
    // block sums of q and q^2: shuffle trees (no sequential FP64 chain)
    double a = group_sum<32>(q), b = group_sum<32>(q * q);
    if ((threadIdx.x & 31) == 0) {
        sq[threadIdx.x >> 5] = a;
        sq2[threadIdx.x >> 5] = b;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x >> 5;
        a = group_sum<32>(threadIdx.x < nw ? sq[threadIdx.x] : 0.0);
        b = group_sum<32>(threadIdx.x < nw ? sq2[threadIdx.x] : 0.0);
        if (threadIdx.x == 0) {
            A.qpart[2 * blockIdx.x] = a;
            A.qpart[2 * blockIdx.x + 1] = b;
        }
    }
}

template <typename R>
__global__ void __launch_bounds__(EW_THREADS) ew_sfac(EwArgs A) {
    using U = typename Frac<R>::U;
    using U4 = typename Frac<R>::U4;
    __shared__ U4 sf[EW_THREADS];
    __shared__ R sq[EW_THREADS];
    __shared__ R sc3[EW_THREADS], ss3[EW_THREADS];
    if (A.skip && *A.skip) return;
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    const int chunk = blockIdx.y;
    const int a0 = chunk * A.chunk, a1 = min(A.n, a0 + A.chunk);
    int4 sg = make_int4(0, 0, 0, 0);
    if (g < A.nseg) sg = A.seg[g];
    C2<R> acc[SEG];
#pragma unroll
    for (int t = 0; t < SEG; ++t) acc[t] = C2<R>{0, 0};
    for (int b = a0; b < a1; b += EW_THREADS) {
        const int i = b + threadIdx.x;
        __syncthreads();
        if (i < a1) {
            const U4 f = ((const U4*)A.frac)[i];
            sf[threadIdx.x] = f;
            sq[threadIdx.x] = (R)A.qs[i];
            R c, s;
            phase<R>(f.z, c, s);
            sc3[threadIdx.x] = c;
            ss3[threadIdx.x] = s;
        }
        __syncthreads();
        const int m = min(EW_THREADS, a1 - b);
        if (g < A.nseg) {
            for (int a = 0; a < m; ++a) {
                const U4 f = sf[a];
                const U ph = (U)(long long)sg.x * f.x + (U)(long long)sg.y * f.y + (U)(long long)sg.z * f.z;
                R c, s;
                phase<R>(ph, c, s);
                const R q = sq[a];
                R zr = q * c, zi = q * s;
                const R c3 = sc3[a], s3 = ss3[a];
#pragma unroll
                for (int t = 0; t < SEG; ++t) {
                    if (t < sg.w) {
                        acc[t].re += zr;
                        acc[t].im += zi;
                        const R nr = zr * c3 - zi * s3;
                        zi = zr * s3 + zi * c3;
                        zr = nr;
                    }
                }
            }
        }
    }
    if (g < A.nseg) {
        C2<R>* out = (C2<R>*)A.Spart + (long long)chunk * A.nk + A.seg_k0[g];
#pragma unroll
        for (int t = 0; t < SEG; ++t)
            if (t < sg.w) out[t] = acc[t];
    }
}

// sum of the chunk partials of one k: compensated FP32 (two-sum) in the mixed
// path, plain FP64 in the FP64 path
__device__ __forceinline__ void add_c(float v, float& s, float& c) {
    const float t = s + v;
    const float bp = t - s;
    c += (s - (t - bp)) + (v - bp);
    s = t;
}
// Sum of the chunk partials of one k by KL lanes: lane l takes chunks l,
// l + KL, ...; the lanes are then combined by a fixed shuffle tree.  Mixed
// path: compensated FP32 (two-sum) throughout, widened once; FP64 path: FP64.
constexpr int KL = 8;

template <typename R>
__device__ __forceinline__ double2 chunk_sum(const C2<R>* sp, int chunks, int nk, int k, int l);
template <>
__device__ __forceinline__ double2 chunk_sum<float>(const C2<float>* sp, int chunks, int nk, int k, int l) {
    float rs = 0.f, rc = 0.f, is = 0.f, ic = 0.f;
    if (k < nk)
        for (int c = l; c < chunks; c += KL) {
            const C2<float> v = sp[(long long)c * nk + k];
            add_c(v.re, rs, rc);
            add_c(v.im, is, ic);
        }
#pragma unroll
    for (int o = KL / 2; o > 0; o >>= 1) {
        const float ors = __shfl_xor_sync(0xffffffffu, rs, o, KL), orc = __shfl_xor_sync(0xffffffffu, rc, o, KL);
        const float ois = __shfl_xor_sync(0xffffffffu, is, o, KL), oic = __shfl_xor_sync(0xffffffffu, ic, o, KL);
        add_c(ors, rs, rc);
        rc += orc;
        add_c(ois, is, ic);
        ic += oic;
    }
    return make_double2((double)rs + (double)rc, (double)is + (double)ic);
}
template <>
__device__ __forceinline__ double2 chunk_sum<double>(const C2<double>* sp, int chunks, int nk, int k, int l) {
    double re = 0.0, im = 0.0;
    if (k < nk)
        for (int c = l; c < chunks; c += KL) {
            const C2<double> v = sp[(long long)c * nk + k];
            re += v.re;
            im += v.im;
        }
#pragma unroll
    for (int o = KL / 2; o > 0; o >>= 1) {
        re += __shfl_xor_sync(0xffffffffu, re, o, KL);
        im += __shfl_xor_sync(0xffffffffu, im, o, KL);
    }
    return make_double2(re, im);
}

template <typename R>
__global__ void ew_sreduce(EwArgs A) {
    __shared__ Fx128 se[8], sq1[8], sq2[8];
    if (A.skip && *A.skip) return;
    const int k = (blockIdx.x * blockDim.x + threadIdx.x) / KL;
    const int l = threadIdx.x % KL;
    double e = 0.0;
    const double2 S = chunk_sum<R>((const C2<R>*)A.Spart, A.chunks, A.nk, k, l);
    if (k < A.nk && l == 0) {
        A.S[k] = S;
        const double ck = A.kvec64[k].w;
        ((C2<R>*)A.wS)[k] = C2<R>{(R)(ck * S.x), (R)(ck * S.y)};
        e = ck * (S.x * S.x + S.y * S.y) * A.inv_eps_2v;
    }
    // block sum of c_k |S_k|^2, exact in fixed point
    Fx128 acc = fx_warp_sum(fx_from_double(e));
    if ((threadIdx.x & 31) == 0) se[threadIdx.x >> 5] = acc;
    // block 0: sum q and sum q^2 over the prep blocks
    Fx128 a1 = fx_zero(), a2 = fx_zero();
    if (blockIdx.x == 0) {
        for (int b = threadIdx.x; b < A.prep_blocks; b += blockDim.x) {
            a1 = fx_add(a1, fx_from_double(A.qpart[2 * b]));
            a2 = fx_add(a2, fx_from_double(A.qpart[2 * b + 1]));
        }
        a1 = fx_warp_sum(a1);
        a2 = fx_warp_sum(a2);
        if ((threadIdx.x & 31) == 0) {
            sq1[threadIdx.x >> 5] = a1;
            sq2[threadIdx.x >> 5] = a2;
        }
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x >> 5;
        acc = fx_warp_sum(threadIdx.x < nw ? se[threadIdx.x] : fx_zero());
        if (blockIdx.x == 0) {
            a1 = fx_warp_sum(threadIdx.x < nw ? sq1[threadIdx.x] : fx_zero());
            a2 = fx_warp_sum(threadIdx.x < nw ? sq2[threadIdx.x] : fx_zero());
        }
        if (threadIdx.x == 0) {
            if (A.acc) fx_red(&A.acc[0], acc);
            if (blockIdx.x == 0) {
                // self and background energies (Potentials.f90:1643-1646)
                const double q1 = fx_to_double(a1), q2 = fx_to_double(a2);
                A.Ssum[0] = q1;
                A.Ssum[1] = q2;
                const double eb = -(q2 * A.inv_eps_4pi * A.inv_sigma_sqrt_2pi) - q1 * q1 * 0.5 * A.inv_eps_2v * A.sigma2;
                if (A.acc) fx_red(&A.acc[0], fx_from_double(eb));
            }
        }
    }
}

constexpr int SEG_TILE = 64;

// two atoms per thread: every staged k record is read once for both
constexpr int FIELD_ATOMS = 2;

template <typename R>
__global__ void __launch_bounds__(EW_THREADS) ew_field(EwArgs A) {
    using V4 = typename std::conditional<sizeof(R) == 4, F4, D4>::type;
    __shared__ int4 sseg[SEG_TILE];
    __shared__ int sk0[SEG_TILE];
    __shared__ V4 sk[SEG_TILE * SEG];  // kx, ky, kz, c_k Re S(k)
    __shared__ R sSs[SEG_TILE * SEG];  // c_k Im S(k)
    if (A.skip && *A.skip) return;
    const int split = blockIdx.y;
    const int s0 = split * A.seg_per_split, s1 = min(A.nseg, s0 + A.seg_per_split);
    using U = typename Frac<R>::U;
    using U4 = typename Frac<R>::U4;
    int ia[FIELD_ATOMS];
    U4 f[FIELD_ATOMS];
    R c3[FIELD_ATOMS], s3[FIELD_ATOMS];
    R fx[FIELD_ATOMS], fy[FIELD_ATOMS], fz[FIELD_ATOMS], ch[FIELD_ATOMS];
#pragma unroll
    for (int a = 0; a < FIELD_ATOMS; ++a) {
        ia[a] = (blockIdx.x * FIELD_ATOMS + a) * blockDim.x + threadIdx.x;
        f[a].x = f[a].y = f[a].z = f[a].w = 0;
        if (ia[a] < A.n) f[a] = ((const U4*)A.frac)[ia[a]];
        phase<R>(f[a].z, c3[a], s3[a]);
        fx[a] = fy[a] = fz[a] = ch[a] = 0;
    }
    const C2<R>* wS = (const C2<R>*)A.wS;
    const R* kv = (const R*)A.kvecR;
    for (int b = s0; b < s1; b += SEG_TILE) {
        const int m = min(SEG_TILE, s1 - b);
        const int kb = A.seg_k0[b];
        const int ke = A.seg_k0[b + m - 1] + A.seg[b + m - 1].w;
        __syncthreads();
        for (int t = threadIdx.x; t < m; t += blockDim.x) {
            sseg[t] = A.seg[b + t];
            sk0[t] = A.seg_k0[b + t] - kb;
        }
        for (int t = threadIdx.x; t < ke - kb; t += blockDim.x) {
            const C2<R> v = wS[kb + t];
            sk[t] = V4{kv[4 * (kb + t)], kv[4 * (kb + t) + 1], kv[4 * (kb + t) + 2], v.re};
            sSs[t] = v.im;
        }
        __syncthreads();
        for (int q = 0; q < m; ++q) {
            const int4 sg = sseg[q];
            const int k0 = sk0[q];
            R c[FIELD_ATOMS], sn[FIELD_ATOMS];
#pragma unroll
            for (int a = 0; a < FIELD_ATOMS; ++a) {
                const U ph = (U)(long long)sg.x * f[a].x + (U)(long long)sg.y * f[a].y + (U)(long long)sg.z * f[a].z;
                phase<R>(ph, c[a], sn[a]);
            }
            for (int t = 0; t < sg.w; ++t) {
                const V4 kk = sk[k0 + t];
                const R Ss = sSs[k0 + t];
#pragma unroll
                for (int a = 0; a < FIELD_ATOMS; ++a) {
                    const R ff = kk.w * sn[a] - Ss * c[a];
                    fx[a] += ff * kk.x;
                    fy[a] += ff * kk.y;
                    fz[a] += ff * kk.z;
                    ch[a] += kk.w * c[a] + Ss * sn[a];
                    const R nr = c[a] * c3[a] - sn[a] * s3[a];
                    sn[a] = c[a] * s3[a] + sn[a] * c3[a];
                    c[a] = nr;
                }
            }
        }
    }
#pragma unroll
    for (int a = 0; a < FIELD_ATOMS; ++a) {
        if (ia[a] < A.n) {
            R* out = (R*)A.Fpart + 4 * ((long long)split * A.n + ia[a]);
            out[0] = fx[a];
            out[1] = fy[a];
            out[2] = fz[a];
            out[3] = ch[a];
        }
    }
}

// Sum of the k-split partials of one atom by FL lanes (lane l takes splits l,
// l + FL, ...), combined by a fixed shuffle tree: compensated FP32 (two-sum)
// widened once in the mixed path, FP64 in the FP64 path.  Every lane of the
// group ends with the sums.
constexpr int FL = 8;

template <typename R>
__device__ __forceinline__ void split_sum(const R* fp, int splits, int n, int i, int l, double f[4]);
template <>
__device__ __forceinline__ void split_sum<float>(const float* fp, int splits, int n, int i, int l, double f[4]) {
    float s[4] = {0, 0, 0, 0}, c[4] = {0, 0, 0, 0};
    if (i < n)
        for (int q = l; q < splits; q += FL) {
            const F4 v = *(const F4*)(fp + 4 * ((long long)q * n + i));
            add_c(v.x, s[0], c[0]);
            add_c(v.y, s[1], c[1]);
            add_c(v.z, s[2], c[2]);
            add_c(v.w, s[3], c[3]);
        }
#pragma unroll
    for (int o = FL / 2; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const float os = __shfl_xor_sync(0xffffffffu, s[k], o, FL), oc = __shfl_xor_sync(0xffffffffu, c[k], o, FL);
            add_c(os, s[k], c[k]);
            c[k] += oc;
        }
    for (int k = 0; k < 4; ++k) f[k] = (double)s[k] + (double)c[k];
}
template <>
__device__ __forceinline__ void split_sum<double>(const double* fp, int splits, int n, int i, int l, double f[4]) {
    for (int k = 0; k < 4; ++k) f[k] = 0.0;
    if (i < n)
        for (int q = l; q < splits; q += FL)
            for (int k = 0; k < 4; ++k) f[k] += fp[4 * ((long long)q * n + i) + k];
#pragma unroll
    for (int o = FL / 2; o > 0; o >>= 1)
#pragma unroll
        for (int k = 0; k < 4; ++k) f[k] += __shfl_xor_sync(0xffffffffu, f[k], o, FL);
}

template <typename R>
__global__ void ew_finish(EwArgs A) {
    __shared__ Fx128 sw[EW_THREADS / 32][6];
    if (A.skip && *A.skip) return;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) / FL;
    const int l = threadIdx.x % FL;
    double w[6] = {0, 0, 0, 0, 0, 0};
    double f[4];
    split_sum<R>((const R*)A.Fpart, A.splits, A.n, i, l, f);
    if (i < A.n && l == 0) {
        const double q = A.qs[i];
        const double pre = q / A.volume_eps;
        const double F0 = pre * f[0], F1 = pre * f[1], F2 = pre * f[2];
        if (A.flags & PG_WANT_FORCES) {
            if (A.first_f) {
                A.out_f[3 * i] = F0;
                A.out_f[3 * i + 1] = F1;
                A.out_f[3 * i + 2] = F2;
            } else {
                A.out_f[3 * i] += F0;
                A.out_f[3 * i + 1] += F1;
                A.out_f[3 * i + 2] += F2;
            }
            // the reference's k-space stress term: absolute position (x) k-space force
            // (Potentials.f90:1949-1954)
            const double r0 = A.pos[3 * i], r1 = A.pos[3 * i + 1], r2 = A.pos[3 * i + 2];
            w[0] = r0 * F0;
            w[1] = r1 * F1;
            w[2] = r2 * F2;
            w[3] = r1 * F2;
            w[4] = r0 * F2;
            w[5] = r0 * F1;
        }
        if (A.flags & PG_WANT_ENEGS) {
            // k sum, self term 2 q/(4 pi eps sqrt(2 pi) sigma), background
            // scaler sigma^2 Q/(2 V eps) (Potentials.f90:2121-2196)
            const double x = -f[3] / A.volume_eps + 2.0 * q * A.inv_eps_4pi * A.inv_sigma_sqrt_2pi +
                             A.scaler[i] * A.inv_eps_2v * A.sigma2 * A.Ssum[0];
            if (A.first_chi) A.out_chi[i] = x;
            else A.out_chi[i] += x;
        }
    }
    // block sums of the six stress components, exact in fixed point
    if (A.acc == nullptr || !(A.flags & PG_WANT_FORCES)) return;
    const int wl = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int c = 0; c < 6; ++c) {
        const Fx128 v = fx_warp_sum(fx_from_double(w[c]));
        if (wl == 0) sw[wid][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < 32) {
        const int nw = blockDim.x >> 5;
        for (int c = 0; c < 6; ++c) {
            const Fx128 v = fx_warp_sum(threadIdx.x < nw ? sw[threadIdx.x][c] : fx_zero());
            if (threadIdx.x == 0) fx_red(&A.acc[1 + c], v);
        }
    }
}

inline int cdiv(long long a, long long b) { return (int)((a + b - 1) / b); }

}  // namespace

void ewald_prepare(pg_context* ctx) {
    if (!ctx->ew_tables_dirty) return;
    const Cell& C = ctx->cell;
    const int K1 = ctx->ew_kmax[0], K2 = ctx->ew_kmax[1], K3 = ctx->ew_kmax[2];
    const double kcsq = ctx->ew_kc * ctx->ew_kc;
    const double sig = ctx->ew_sigma;
    std::vector<int4> seg;
    std::vector<int> seg_k0;
    std::vector<D4> kv;
    for (int k1 = -K1; k1 <= K1; ++k1)
        for (int k2 = -K2; k2 <= K2; ++k2) {
            int last_n3 = -2;
            for (int k3 = 0; k3 <= K3; ++k3) {
                if (!(k1 != 0 || k2 != 0 || k3 != 0)) continue;
                double v[3];
                for (int c = 0; c < 3; ++c)
                    v[c] = (double)k1 * C.rc[c][0] + (double)k2 * C.rc[c][1] + (double)k3 * C.rc[c][2];
                const double d = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
                if (!(d < kcsq)) continue;
                const double w = k3 == 0 ? 1.0 : 2.0;
                const double ck = w * std::exp(-(sig * sig * d * 0.5)) / d;
                if (seg.empty() || last_n3 != k3 - 1 || seg.back().x != k1 || seg.back().y != k2 ||
                    seg.back().w >= SEG) {
                    seg.push_back(make_int4(k1, k2, k3, 0));
                    seg_k0.push_back((int)kv.size());
                }
                seg.back().w += 1;
                last_n3 = k3;
                kv.push_back(D4{v[0], v[1], v[2], ck});
            }
        }
    ctx->ew_nk = (int)kv.size();
    ctx->ew_nseg = (int)seg.size();
    if (seg.empty()) {
        seg.push_back(make_int4(0, 0, 0, 0));
        seg_k0.push_back(0);
        kv.push_back(D4{0, 0, 0, 0});
    }
    ctx->ew_seg.upload(seg.data(), seg.size(), ctx->stream);
    ctx->ew_seg_k0.upload(seg_k0.data(), seg_k0.size(), ctx->stream);
    ctx->ew_kvec64.upload(kv.data(), kv.size(), ctx->stream);
    std::vector<F4> kv32(kv.size());
    for (size_t q = 0; q < kv.size(); ++q) kv32[q] = F4{(float)kv[q].x, (float)kv[q].y, (float)kv[q].z, (float)kv[q].w};
    ctx->ew_kvec.upload(kv32.data(), kv32.size(), ctx->stream);
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->ew_tables_dirty = false;
    ctx->state_epoch++;
}

static void ew_shape(const pg_context* ctx, int& chunks, int& chunk, int& splits, int& sps, int& prep_blocks,
                     int& kred_blocks, int& fin_blocks) {
    const int n = std::max(ctx->n, 1);
    const int nseg = std::max(ctx->ew_nseg, 1);
    const int seg_blocks = cdiv(nseg, EW_THREADS);
    chunks = std::max(1, std::min(64, cdiv(4 * sm_count(), seg_blocks)));
    chunks = std::min(chunks, std::max(1, n / 32));
    chunk = cdiv(n, chunks);
    chunks = cdiv(n, chunk);
    const int atom_blocks = cdiv(n, EW_THREADS * FIELD_ATOMS);
    splits = std::max(1, std::min(32, cdiv(4 * sm_count(), atom_blocks)));
    splits = std::min(splits, nseg);
    sps = cdiv(nseg, splits);
    splits = cdiv(nseg, sps);
    prep_blocks = cdiv(n, EW_THREADS);
    kred_blocks = cdiv((long long)std::max(ctx->ew_nk, 1) * KL, 256);
    fin_blocks = cdiv((long long)n * FL, EW_THREADS);
}

template <typename R>
static void ew_launch(pg_context* ctx, EwArgs& A, int prep_blocks, int kred_blocks, int fin_blocks) {
    cudaStream_t st = ctx->stream;
    ew_prep<R><<<prep_blocks, EW_THREADS, 0, st>>>(A);
    ew_sfac<R><<<dim3(cdiv(std::max(A.nseg, 1), EW_THREADS), A.chunks), EW_THREADS, 0, st>>>(A);
    ew_sreduce<R><<<kred_blocks, 256, 0, st>>>(A);
    ctx->launches += 3;
    if (A.flags & (PG_WANT_FORCES | PG_WANT_ENEGS)) {
        ew_field<R><<<dim3(cdiv(A.n, EW_THREADS * FIELD_ATOMS), A.splits), EW_THREADS, 0, st>>>(A);
        ew_finish<R><<<fin_blocks, EW_THREADS, 0, st>>>(A);
        ctx->launches += 2;
    }
    PG_CHECK_LAUNCH();
}

void launch_ewald_kspace_skip(pg_context* ctx, int precision, int flags, bool first_f, bool first_chi, FxAcc* acc,
                              const int* skip) {
    const int n = ctx->n;
    int chunks, chunk, splits, sps, prep_blocks, kred_blocks, fin_blocks;
    ew_shape(ctx, chunks, chunk, splits, sps, prep_blocks, kred_blocks, fin_blocks);
    const size_t cs = precision == PG_PREC_FP64 ? sizeof(double) : sizeof(float);
    ctx->ew_frac.resize(8 * (size_t)std::max(n, 1));
    ctx->ew_qs.resize((size_t)std::max(n, 1));
    ctx->ew_qpart.resize(2 * (size_t)prep_blocks);
    ctx->ew_S.resize((size_t)std::max(ctx->ew_nk, 1));
    ctx->ew_Ssum.resize(2);
    ctx->ew_spart_bytes.resize((2 * cs * (size_t)chunks * std::max(ctx->ew_nk, 1) + 7) / 8);
    ctx->ew_fpart_bytes.resize((4 * cs * (size_t)splits * std::max(n, 1) + 7) / 8);
    EwArgs A{};
    A.n = n;
    A.nk = ctx->ew_nk;
    A.nseg = ctx->ew_nseg;
    A.chunks = chunks;
    A.chunk = chunk;
    A.splits = splits;
    A.seg_per_split = sps;
    A.pos = ctx->pos.p;
    A.charge = ctx->charge.p;
    A.scaler = ctx->ew_scaler.p;
    A.C = cell_kernel_view(ctx->cell);
    A.seg = ctx->ew_seg.p;
    A.seg_k0 = ctx->ew_seg_k0.p;
    A.kvec64 = ctx->ew_kvec64.p;
    A.frac = ctx->ew_frac.p;
    A.qs = ctx->ew_qs.p;
    A.qpart = ctx->ew_qpart.p;
    A.prep_blocks = prep_blocks;
    A.Spart = ctx->ew_spart_bytes.p;
    A.S = ctx->ew_S.p;
    ctx->ew_wS_bytes.resize((2 * cs * (size_t)std::max(ctx->ew_nk, 1) + 7) / 8);
    A.wS = ctx->ew_wS_bytes.p;
    A.kvecR = precision == PG_PREC_FP64 ? (const void*)ctx->ew_kvec64.p : (const void*)ctx->ew_kvec.p;
    A.Ssum = ctx->ew_Ssum.p;
    A.Fpart = ctx->ew_fpart_bytes.p;
    const double eps = ctx->ew_eps, sig = ctx->ew_sigma;
    A.inv_eps_2v = 1.0 / (2.0 * ctx->cell.volume * eps);
    A.inv_eps_4pi = 1.0 / (4.0 * PI * eps);
    A.inv_sigma_sqrt_2pi = 1.0 / (std::sqrt(2.0 * PI) * sig);
    A.sigma2 = sig * sig;
    A.volume_eps = ctx->cell.volume * eps;
    A.flags = flags;
    A.first_f = first_f;
    A.first_chi = first_chi;
    A.out_f = ctx->out_f.p;
    A.out_chi = ctx->out_chi.p;
    A.acc = (flags & (PG_WANT_ENERGY | PG_WANT_FORCES)) ? acc : nullptr;
    A.skip = skip;
    if (precision == PG_PREC_FP64) ew_launch<double>(ctx, A, prep_blocks, kred_blocks, fin_blocks);
    else ew_launch<float>(ctx, A, prep_blocks, kred_blocks, fin_blocks);
}

void launch_ewald_kspace(pg_context* ctx, int precision, int flags, bool first_f, bool first_chi, FxAcc* acc) {
    launch_ewald_kspace_skip(ctx, precision, flags, first_f, first_chi, acc, nullptr);
}

}  // namespace pg
