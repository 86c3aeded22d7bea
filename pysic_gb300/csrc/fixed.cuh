// fixed.cuh -- exact accumulation of FP64 values in 128-bit fixed point.
//
// Energies and virials are summed over all atoms.  A compensated FP64 sum is a
// long chain of dependent FP64 additions, and FP64 latency on this GPU is high,
// so a few-thousand-term tree of two-sums costs microseconds.  Instead every
// FP64 term is converted exactly (integer operations on its bit pattern) to a
// signed 128-bit integer in units of 2^-64 and added with integer carries.  The
// sum is exact for |terms| < 2^62 and independent of the order of addition, so
// the result is deterministic by construction; it is rounded to FP64 once.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pg {

struct Fx128 {
    unsigned long long lo;
    long long hi;
};

__device__ __forceinline__ Fx128 fx_zero() { return Fx128{0ull, 0ll}; }

__device__ __forceinline__ Fx128 fx_add(Fx128 a, Fx128 b) {
    Fx128 r;
    r.lo = a.lo + b.lo;
    r.hi = a.hi + b.hi + (r.lo < a.lo ? 1 : 0);
    return r;
}

__device__ __forceinline__ Fx128 fx_neg(Fx128 a) {
    Fx128 r;
    r.lo = ~a.lo + 1ull;
    r.hi = ~a.hi + (r.lo == 0ull ? 1 : 0);
    return r;
}

// exact for |x| < 2^62; bits below 2^-64 are truncated
__device__ __forceinline__ Fx128 fx_from_double(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0) return fx_zero();  // zero and subnormals (below 2^-1022)
    const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
    // value = m * 2^(ex - 1075); in units of 2^-64: m * 2^(ex - 1011)
    const int sh = ex - 1011;
    Fx128 r;
    if (sh >= 0) {
        if (sh >= 64) {
            r.lo = 0ull;
            r.hi = (long long)(m << (sh - 64));
        } else {
            r.lo = m << sh;
            r.hi = sh == 0 ? 0ll : (long long)(m >> (64 - sh));
        }
    } else {
        r.lo = -sh >= 64 ? 0ull : (m >> -sh);
        r.hi = 0ll;
    }
    return (b >> 63) ? fx_neg(r) : r;
}

__device__ __forceinline__ double fx_to_double(Fx128 a) {
    const bool neg = a.hi < 0;
    if (neg) a = fx_neg(a);
    // a = hi * 2^64 + lo in units of 2^-64
    return (neg ? -1.0 : 1.0) * ((double)(unsigned long long)a.hi + (double)a.lo * 5.421010862427522e-20);
}

__device__ __forceinline__ Fx128 fx_shfl_xor(Fx128 a, int o) {
    Fx128 r;
    r.lo = __shfl_xor_sync(0xffffffffu, a.lo, o);
    r.hi = __shfl_xor_sync(0xffffffffu, a.hi, o);
    return r;
}

__device__ __forceinline__ Fx128 fx_warp_sum(Fx128 a) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) a = fx_add(a, fx_shfl_xor(a, o));
    return a;
}

}  // namespace pg
