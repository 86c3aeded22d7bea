// fixed.cuh -- exact accumulation in fixed point, with integer operations only.
//
// Energies and virials are summed over all atoms.  A compensated FP64 sum is a
// long chain of dependent FP64 additions, and this GPU issues one FP64 warp
// instruction per 64 cycles per scheduler, so even the conversions of a few
// per-atom values to FP64 cost more than the FP32 physics around them.  Here
//
//   * totals (energy, virial) are signed 128-bit integers in units of 2^-64
//     (Fx128).  Every FP32 or FP64 term is converted exactly from its bit
//     pattern, block sums are integer shuffles, and each block adds its sums to
//     one global accumulator with three 64-bit integer reductions (FxAcc).
//     Integer addition is associative, so the total is exact and independent
//     of the order in which blocks finish: deterministic by construction.  It
//     is rounded to FP64 once, on the host.
//   * per-atom values of the mixed path (forces, electronegativities) are
//     signed 64-bit integers in units of 2^-32 (about 2.3e-10).  FP32 lane
//     partials are converted with rounding to nearest, summed exactly as
//     integers, and turned into FP64 by an integer routine that rounds to
//     nearest even -- no FP64 instruction anywhere.  Magnitudes up to 2^26
//     (6.7e7 eV/A) are exact; larger values, infinities and NaN saturate, and a
//     saturated total reads back as NaN.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace pg {

struct Fx128 {
    unsigned long long lo;
    long long hi;
};

__host__ __device__ __forceinline__ double fx_nan() {
    union {
        unsigned long long u;
        double d;
    } c;
    c.u = 0x7ff8000000000000ull;
    return c.d;
}

__host__ __device__ __forceinline__ Fx128 fx_zero() { return Fx128{0ull, 0ll}; }

// non-finite terms make the total huge; it reads back as NaN
__host__ __device__ __forceinline__ Fx128 fx_poison() { return Fx128{0ull, 1ll << 61}; }

__device__ __forceinline__ Fx128 fx_add(Fx128 a, Fx128 b) {
    Fx128 r;
    r.lo = a.lo + b.lo;
    r.hi = a.hi + b.hi + (r.lo < a.lo ? 1 : 0);
    return r;
}

__host__ __device__ __forceinline__ Fx128 fx_neg(Fx128 a) {
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
    if (ex >= 1011 + 62 + 64 - 52) return fx_poison();  // |x| >= 2^62, infinities, NaN
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

__host__ __device__ __forceinline__ double fx_to_double(Fx128 a) {
    if (a.hi >= (1ll << 60) || a.hi <= -(1ll << 60)) return fx_nan();
    const bool neg = a.hi < 0;
    if (neg) a = fx_neg(a);
    // a = hi * 2^64 + lo in units of 2^-64
    return (neg ? -1.0 : 1.0) * ((double)(unsigned long long)a.hi + (double)a.lo * 5.421010862427522e-20);
}

// exact for any finite float (units 2^-64: bits below 2^-64 are truncated)
__device__ __forceinline__ Fx128 fx_from_float(float x) {
    const unsigned b = __float_as_uint(x);
    const int ex = (int)((b >> 23) & 0xffu);
    if (ex == 0) return fx_zero();  // zero and subnormals
    if (ex == 255) return fx_poison();
    const unsigned long long m = (unsigned long long)((b & 0x7fffffu) | 0x800000u);
    // value = m 2^(ex - 150); in units of 2^-64: m 2^(ex - 86)
    const int sh = ex - 86;
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
    return (b >> 31) ? fx_neg(r) : r;
}

// 2^-32 fixed point (per-atom values) widened to a 128-bit total: exact
__device__ __forceinline__ Fx128 fx_from_fix(long long v) {
    Fx128 r;
    r.lo = (unsigned long long)v << 32;
    r.hi = v >> 32;
    return r;
}

// A global 128-bit total kept as three 64-bit limb sums (bits 0-41, 42-83 and
// 84-127 of the two's complement value).  A block adds its value with three
// independent reductions that return nothing, so no thread waits for a round
// trip and no carry has to be passed between words; every limb sum stays exact
// for up to 2^22 additions.  fx_from_limbs puts the limbs back together
// (modulo 2^128, which is exact for any total that fits in 128 bits).
struct FxAcc {
    unsigned long long l[3];
};

__device__ __forceinline__ void fx_red(FxAcc* dst, Fx128 v) {
    const unsigned long long lo = v.lo, hi = (unsigned long long)v.hi;
    const unsigned long long m42 = (1ull << 42) - 1ull;
    const unsigned long long l0 = lo & m42;
    const unsigned long long l1 = ((lo >> 42) | (hi << 22)) & m42;
    const unsigned long long l2 = hi >> 20;
    if (l0) atomicAdd(&dst->l[0], l0);
    if (l1) atomicAdd(&dst->l[1], l1);
    if (l2) atomicAdd(&dst->l[2], l2);
}

__host__ __device__ __forceinline__ Fx128 fx_from_limbs(const FxAcc& a) {
    // t = l0 + l1 2^42 + l2 2^84 (mod 2^128), with explicit carries
    const unsigned long long l0 = a.l[0], l1 = a.l[1], l2 = a.l[2];
    unsigned long long lo = l0, hi = 0ull;
    const unsigned long long s1lo = l1 << 42, s1hi = l1 >> 22;
    const unsigned long long t = lo + s1lo;
    hi += s1hi + (t < lo ? 1ull : 0ull);
    lo = t;
    hi += l2 << 20;  // l2 2^84 has no bits below 2^64
    return Fx128{lo, (long long)hi};
}

// ---- per-atom 2^-32 fixed point ----
constexpr long long FIX_SAT = 1ll << 61;

// float to 2^-32 units, rounded to nearest (ties away from zero)
__device__ __forceinline__ long long fix_from_float(float x) {
    const unsigned b = __float_as_uint(x);
    const int ex = (int)((b >> 23) & 0xffu);
    if (ex == 0) return 0;
    const unsigned long long m = (unsigned long long)((b & 0x7fffffu) | 0x800000u);
    // value = m 2^(ex - 150); in units of 2^-32: m 2^(ex - 118)
    const int sh = ex - 118;
    unsigned long long u;
    if (sh >= 0) {
        u = sh > 34 ? (unsigned long long)FIX_SAT : (m << sh);
    } else {
        const int rs = -sh;
        u = rs > 25 ? 0ull : ((m + (1ull << (rs - 1))) >> rs);
    }
    return (b >> 31) ? -(long long)u : (long long)u;
}

// double to 2^-32 units, rounded to nearest (ties away from zero)
__device__ __forceinline__ long long fix_from_double(double x) {
    const unsigned long long b = (unsigned long long)__double_as_longlong(x);
    const int ex = (int)((b >> 52) & 0x7ff);
    if (ex == 0) return 0;
    const unsigned long long m = (b & 0xfffffffffffffull) | (1ull << 52);
    // value = m 2^(ex - 1075); in units of 2^-32: m 2^(ex - 1043)
    const int sh = ex - 1043;
    unsigned long long u;
    if (sh >= 0) {
        u = sh > 5 ? (unsigned long long)FIX_SAT : (m << sh);
    } else {
        const int rs = -sh;
        u = rs > 54 ? 0ull : ((m + (1ull << (rs - 1))) >> rs);
    }
    return (b >> 63) ? -(long long)u : (long long)u;
}

// 2^-32 units to the nearest double (ties to even); saturated values give NaN
__device__ __forceinline__ double fix_to_double(long long v) {
    if (v == 0) return 0.0;
    const unsigned long long sgn = v < 0 ? 1ull : 0ull;
    const unsigned long long u = sgn ? (unsigned long long)(-v) : (unsigned long long)v;
    if (u >= (1ull << 60)) return __longlong_as_double(0x7ff8000000000000ll);
    const int p = 63 - __clzll((long long)u);  // position of the leading one, < 60
    int e = p - 32;
    unsigned long long mant;
    if (p <= 52) {
        mant = u << (52 - p);
    } else {
        const int rs = p - 52;
        const unsigned long long rem = u & ((1ull << rs) - 1ull), half = 1ull << (rs - 1);
        mant = u >> rs;
        if (rem > half || (rem == half && (mant & 1ull))) {
            ++mant;
            if (mant == (1ull << 53)) {
                mant >>= 1;
                ++e;
            }
        }
    }
    const unsigned long long bits = (sgn << 63) | ((unsigned long long)(e + 1023) << 52) | (mant & 0xfffffffffffffull);
    return __longlong_as_double((long long)bits);
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
