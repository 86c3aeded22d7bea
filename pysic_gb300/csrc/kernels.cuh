// kernels.cuh -- device-side physics shared by the pair, bond-order and batched
// kernels, templated on the per-term arithmetic type R (double for the FP64
// path, float for the mixed path).
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"
#include "fixed.cuh"

namespace pg {

template <typename R>
struct V3 {
    R x, y, z;
};

__device__ __forceinline__ void sincospi_(float x, float* s, float* c) { sincospif(x, s, c); }
__device__ __forceinline__ void sincospi_(double x, double* s, double* c) { sincospi(x, s, c); }
__device__ __forceinline__ float sinpi_(float x) { return sinpif(x); }
__device__ __forceinline__ double sinpi_(double x) { return sinpi(x); }
__device__ __forceinline__ float cospi_(float x) { return cospif(x); }
__device__ __forceinline__ double cospi_(double x) { return cospi(x); }
__device__ __forceinline__ float exp_(float x) { return expf(x); }
__device__ __forceinline__ double exp_(double x) { return exp(x); }
__device__ __forceinline__ float pow_(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double pow_(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }

// x^k by repeated squaring for an integer k, or pow(x, y) otherwise (k =
// PG_NOT_INT): power-law terms whose exponent is integral skip the general pow
template <typename R>
__device__ __forceinline__ R powk(R x, R y, int k) {
    if (k == PG_NOT_INT) return pow_(x, y);
    unsigned a = k < 0 ? (unsigned)(-k) : (unsigned)k;
    R r = R(1);
    while (a) {
        if (a & 1u) r *= x;
        x *= x;
        a >>= 1;
    }
    return k < 0 ? R(1) / r : r;
}

__device__ __forceinline__ float erfc_(float x) { return erfcf(x); }
__device__ __forceinline__ double erfc_(double x) { return erfc(x); }
// reciprocal: the FP32 path uses the fast approximate division (a few ulp),
// the FP64 path the correctly rounded one
__device__ __forceinline__ float rcp_(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ double rcp_(double x) { return 1.0 / x; }

// Smooth cutoff f(r) = 1/2 (1 + cos(pi (r - rs)/(rc - rs))) on [rs, rc] and its
// derivative (smoothening_factor / smoothening_derivative, Potentials.f90:442-498).
template <typename R>
__device__ __forceinline__ void smooth(R r, R rc, R rs, R& f, R& fp) {
    if (r > rc) {
        f = R(0);
        fp = R(0);
    } else if (r < rs) {
        f = R(1);
        fp = R(0);
    } else {
        const R w = rc - rs;
        R s, c;
        sincospi_((r - rs) / w, &s, &c);
        f = R(0.5) * (R(1) + c);
        fp = R(-0.5) * R(3.14159265358979323846) / w * s;
    }
}
// FP32: one approximate reciprocal of the band width (a few ulp) in place of
// two IEEE divisions, which cost more than the sine and cosine themselves in
// the bond pass's per-bond set-up
template <>
__device__ __forceinline__ void smooth<float>(float r, float rc, float rs, float& f, float& fp) {
    if (r > rc) {
        f = 0.0f;
        fp = 0.0f;
    } else if (r < rs) {
        f = 1.0f;
        fp = 0.0f;
    } else {
        const float iw = __fdividef(1.0f, rc - rs);
        float s, c;
        sincospif((r - rs) * iw, &s, &c);
        f = 0.5f * (1.0f + c);
        fp = -0.5f * 3.14159265358979323846f * iw * s;
    }
}

// V(r) and the radial derivative dV/dr of LJ (Potentials.f90:2971-3005),
// exponential (3643-3680) and Buckingham (4009-4045); no factor 4 in LJ.
// tab: the rows (V, d) of every tabulated potential, 2 values per row
template <typename R>
__device__ __forceinline__ void pair_eval(const PairT<R>& P, R r, R& V, R& dV, const R* tab) {
    const R p0 = P.p0, p1 = P.p1, p2 = P.p2;
    switch (P.kind) {
        case 0: {  // LJ: eps ((s/r)^12 - (s/r)^6), no factor 4 (evaluate_energy_LJ, Potentials.f90:2993-3005)
            const R ratio = p1 / r;
            const R r2 = ratio * ratio;
            const R r6 = r2 * r2 * r2;
            V = p0 * (r6 * r6 - r6);
            dV = p0 * (R(6) * r6 - R(12) * r6 * r6) / r;
            break;
        }
        case 1: {  // exponential: eps exp(-zeta r) (3666-3677)
            const R e = p0 * exp_(-p1 * r);
            V = e;
            dV = -p1 * e;
            break;
        }
        case 2: {  // Buckingham: A exp(-r/s) - C (s/r)^6 (4033-4045)
            const R ratio = r / p2;
            const R q2 = R(1) / (ratio * ratio);
            const R r6 = q2 * q2 * q2;
            const R e = p0 * exp_(-ratio);
            V = e - p1 * r6;
            dV = (-e * ratio + R(6) * p1 * r6) / r;
            break;
        }
        case 3: {  // spring: k/2 ((r - R0)^2 - (rc - R0)^2) while |r - R0| < |rc - R0|, else 0 (3042-3085)
            const R d = r - p1, dc = P.rc - p1;
            if (d * d < dc * dc) {
                V = p0 * R(0.5) * (d * d - dc * dc);
                dV = p0 * d;
            } else {
                V = R(0);
                dV = R(0);
            }
            break;
        }
        case 4: {  // power: eps (a/r)^n (4119-4152)
            const R t = p0 * powk(p1 / r, p2, P.ni);
            V = t;
            dV = -p2 * t / r;
            break;
        }
        case 5: {  // shift_power: eps ((r1 - r)/(r1 - r2))^n (4803-4842)
            const R w = p1 - p2;
            const R x = (p1 - r) / w;
            V = p0 * powk(x, P.p3, P.ni);
            dV = -p0 * P.p3 / w * powk(x, P.p3 - R(1), P.ni == PG_NOT_INT ? PG_NOT_INT : P.ni - 1);
            break;
        }
        case 6: {  // tabulated: cubic Hermite on rows (V, d), range p0, scale p1 (4227-4298);
                   // beyond the range the last V, unscaled, as the reference returns it
            const R* T = tab + 2 * (long long)P.t0;
            const int nv = P.tn;
            if (r >= p0) {
                V = T[2 * (nv - 1)];
                dV = R(0);
            } else {
                const R dr = p0 / (R)(nv - 1);
                const R x = r / dr;
                const int l = min(max((int)x, 0), nv - 2);
                const R t = x - (R)l, t2 = t * t, t3 = t2 * t;
                const R* a = T + 2 * l;
                V = p1 * (a[0] * (R(2) * t3 - R(3) * t2 + R(1)) + a[1] * dr / p0 * (t3 - R(2) * t2 + t) +
                          a[2] * (R(3) * t2 - R(2) * t3) + a[3] * dr / p0 * (t3 - t2));
                dV = p1 * (a[0] / dr * R(6) * (t2 - t) + a[1] / p0 * (R(3) * t2 - R(4) * t + R(1)) +
                           a[2] / dr * R(6) * (t - t2) + a[3] / p0 * (R(3) * t2 - R(2) * t));
            }
            break;
        }
        case 10: {  // step: e1 below r1, e2 above r2, (e1 + e2)/2 (1 + cos(pi t)/2) between
                    // (evaluate_energy_step, 4946-4967); its force is not radial: the pair
                    // kernel adds it (step_force), dV is 0
            V = r < P.p2 ? p0 : r > P.p3 ? p1 : (p0 + p1) * R(0.5) * (R(1) + R(0.5) * cospi_((r - P.p2) / (P.p3 - P.p2)));
            dV = R(0);
            break;
        }
        default:  // charge-dependent terms are evaluated by the pair kernel itself
            V = R(0);
            dV = R(0);
            break;
    }
}

// The step potential's force as the reference evaluates it (evaluate_force_step,
// Potentials.f90:4917-4937): the same value c on all three components of the
// force on the pair's atom 1, -c on atom 2, c = (e1 + e2) pi/(4 (r2 - r1))
// sin(pi (r - r1)/(r2 - r1)) on [r1, r2], else 0 (not the gradient of the
// energy, and not along the bond).
template <typename R>
__device__ __forceinline__ R step_force(const PairT<R>& P, R r) {
    if (r < P.p2 || r > P.p3) return R(0);
    const R w = P.p3 - P.p2;
    return (P.p0 + P.p1) * R(0.25) * R(3.14159265358979323846) / w * sinpi_((r - P.p2) / w);
}

// pick (Core.f90): each pair once -- the higher index, or for one atom and
// its own image the lexicographically positive offset
__device__ __forceinline__ bool pick(int i1, int i2, int o0, int o1, int o2) {
    if (i2 > i1) return true;
    if (i2 == i1 && o0 >= 0) {
        if (o0 > 0) return true;
        if (o1 > 0) return true;
        if (o1 == 0 && o2 > 0) return true;
    }
    return false;
}

// x^k for an integer k (the reference's integer powers), negative k as 1 / x^-k
template <typename R>
__device__ __forceinline__ R ipow(R x, int k) {
    R r = R(1);
    const int a = k < 0 ? -k : k;
    for (int q = 0; q < a; ++q) r *= x;
    return k < 0 ? R(1) / r : r;
}

// V f and d(V f)/dr of one pair term, smoothing included
template <typename R>
__device__ __forceinline__ void pair_term(const PairT<R>& P, R r, R& V, R& dV, const R* tab) {
    pair_eval<R>(P, r, V, dV, tab);
    if (P.smooth) {
        R f, fp;
        smooth<R>(r, P.rc, P.rs, f, fp);
        dV = dV * f + V * fp;
        V = V * f;
    }
}

// One factor of a product of potentials for the pair (i, j): its value V, dV/dr
// and its electronegativity of atom i (-dV/dq_i), without any cut factor
// (evaluate_energy_component / _force_component /
// _electronegativity_component, Potentials.f90:2512-2890).  first: i is the
// pair's atom1 as the reference's loop picks it; charge-dependent factors take
// the parameters of the product's first target on atom1 when its type is that
// target's, as their plain records do below.
template <typename R>
__device__ __forceinline__ void factor_raw(const PairT<R>& P, const R* tab, R r, R qi, R qj, bool first, int ti, int tj,
                                           R& V, R& dV, R& en) {
    en = R(0);
    if (P.kind < 7) {
        pair_eval<R>(P, r, V, dV, tab);
        return;
    }
    dV = R(0);
    const R q1 = first ? qi : qj, q2 = first ? qj : qi;
    const bool direct = (P.first >> (first ? ti : tj)) & 1ull;
    if (P.kind == 7) {  // charge_pair
        const int n1 = direct ? (int)P.p1 : (int)P.p2, n2 = direct ? (int)P.p2 : (int)P.p1;
        V = P.p0 * (ipow(q1, n1) * ipow(q2, n2));
        const int nm = first ? n1 : n2;
        if (nm > 0)
            en = -(first ? P.p0 * (R(n1) * ipow(q1, n1 - 1) * ipow(q2, n2))
                         : P.p0 * (R(n2) * ipow(q1, n1) * ipow(q2, n2 - 1)));
    } else if (P.kind == 8) {  // charge_exp
        const R* c = tab + 2 * (long long)P.t0;
        const int a1 = direct ? 0 : 4, a2 = direct ? 4 : 0;
        const R eta1 = c[direct ? 11 : 12], eta2 = c[direct ? 12 : 11];
        const R beta1 = c[direct ? 13 : 14], beta2 = c[direct ? 14 : 13];
        const R xi1 = c[direct ? 9 : 10], xi2 = c[direct ? 10 : 9];
        const R d5 = beta1 * (c[3 + a1] - q1), d6 = beta2 * (c[3 + a2] - q2);
        const R D1 = c[1 + a1] + pow_(fabs(d5), eta1), D2 = c[1 + a2] + pow_(fabs(d6), eta2);
        V = c[0] * exp_(R(0.5) * (xi1 * D1 + xi2 * D2));
        en = first ? V * xi1 * R(0.5) * eta1 * pow_(fabs(d5), eta1 - R(1)) * copysign(R(1), d5) * beta1
                   : V * xi2 * R(0.5) * eta2 * pow_(fabs(d6), eta2 - R(1)) * copysign(R(1), d6) * beta2;
    } else {  // charge_abs
        const R* c = tab + 2 * (long long)P.t0;
        const R* s1 = c + (direct ? 0 : 4);
        const R* s2 = c + (direct ? 4 : 0);
        const R ab1 = fabs(q1 - s1[2]), ab2 = fabs(q2 - s2[2]);
        const R pw1 = pow_(ab1, s1[3] - R(1)), pw2 = pow_(ab2, s2[3] - R(1));
        R f1 = s1[0] + s1[1] * ab1 * pw1, f2 = s2[0] + s2[1] * ab2 * pw2;
        R is = R(0.5) / sqrt_(f1 * f2);
        if (f1 < R(0)) {
            f1 = R(0);
            is = R(0);
        }
        if (f2 < R(0)) {
            f2 = R(0);
            is = R(0);
        }
        const R e1 = fmax(s1[0] + s1[1] * pow_(ab1, s1[3]), R(0));
        const R e2 = fmax(s2[0] + s2[1] * pow_(ab2, s2[3]), R(0));
        V = sqrt_(e1 * e2);
        en = first ? is * (-s1[3] * pw1 * copysign(R(1), q1 - s1[2]) * s1[1]) * f2
                   : is * (-s2[3] * pw2 * copysign(R(1), q2 - s2[2]) * s2[1]) * f1;
    }
}

// A record and its factors (P.nmul of them from terms[P.mul0]; a record with
// none is one factor): V = prod V_k, dV/dr and the electronegativity of atom
// i by the running product rule (V <- V e_k, V' <- V' e_k + V d_k), without
// the record's smooth cut.
template <typename R>
__device__ __forceinline__ void product_value(const PairT<R>& P, const PairT<R>* terms, const R* tab, R r, R qi, R qj,
                                              bool first, int ti, int tj, R& V, R& dV, R& en) {
    V = R(1);
    dV = R(0);
    en = R(0);
    for (int k = 0; k <= P.nmul; ++k) {
        R ek, dk, nk;
        factor_raw<R>(k == 0 ? P : terms[P.mul0 + k - 1], tab, r, qi, qj, first, ti, tj, ek, dk, nk);
        dV = dV * ek + V * dk;
        en = en * ek + V * nk;
        V *= ek;
    }
}

// Angular function g = 1 + c^2/d^2 - c^2/(d^2 + (h - cos)^2) of
// evaluate_pair_bond_order_factor_tersoff (Potentials.f90:5790), written in the
// algebraically equal form 1 + (c^2/d^2) x / (d^2 + x), x = (h - cos)^2, which
// does not cancel catastrophically in FP32 (c^2/d^2 is ~4e7 for silicon);
// dg/dcos = -2 c^2 (h - cos) / (d^2 + x)^2.
template <typename R>
__device__ __forceinline__ void angular(const TripT<R>& t, R cs, R& g, R& dg) {
    const R hc = t.h - cs;
    const R x = hc * hc;
    const R den = t.d2 + x;
    const R inv = rcp_(den);
    g = R(1) + t.c2d2 * x * inv;
    dg = R(-2) * t.c2 * hc * inv * inv;
}

// exp((a (r1 - r2))^mu) and its derivative with respect to r1 - r2
template <typename R>
__device__ __forceinline__ void radial_exp(const TripT<R>& t, R dr, R& X, R& Xp) {
    if (t.a == R(0)) {
        X = R(1);
        Xp = R(0);
    } else {
        const R u = t.a * dr;
        const R um1 = pow_(u, t.mu - R(1));
        X = exp_(u * um1);
        Xp = X * t.mu * t.a * um1;
    }
}

// zeta term xi_ijk g_ijk for bond ij (vector a, length r1) and neighbour k
// (vector b, length r2), Potentials.f90:5744-5795
template <typename R>
__device__ __forceinline__ R tersoff_term(const TripT<R>& t, const V3<R>& a, R r1, const V3<R>& b, R r2) {
    R f, fp;
    smooth(r2, t.rc, t.rs, f, fp);
    if (f == R(0)) return R(0);
    const R cs = (a.x * b.x + a.y * b.y + a.z * b.z) / (r1 * r2);
    R g, dg;
    angular(t, cs, g, dg);
    R X, Xp;
    radial_exp(t, r1 - r2, X, Xp);
    return f * X * g;
}

// gradient of the zeta term with respect to the positions of j and k
// (the gradient with respect to the centre i is minus their sum);
// Potentials.f90:5806-5902 computes the same derivatives.
template <typename R>
__device__ __forceinline__ bool tersoff_grad(const TripT<R>& t, const V3<R>& a, R r1, const V3<R>& b, R r2, V3<R>& gj,
                                             V3<R>& gk) {
    R f, fp;
    smooth(r2, t.rc, t.rs, f, fp);
    if (f == R(0) && fp == R(0)) return false;
    const R i1 = R(1) / r1, i2 = R(1) / r2;
    const V3<R> ua{a.x * i1, a.y * i1, a.z * i1};
    const V3<R> ub{b.x * i2, b.y * i2, b.z * i2};
    const R cs = ua.x * ub.x + ua.y * ub.y + ua.z * ub.z;
    R g, dg;
    angular(t, cs, g, dg);
    R X, Xp;
    radial_exp(t, r1 - r2, X, Xp);
    const R xi = f * X;
    // d/dr_j : g f Xp ua + xi dg (ub - cs ua)/r1
    const R cj = g * f * Xp - xi * dg * cs * i1;
    const R cjb = xi * dg * i1;
    gj.x = cj * ua.x + cjb * ub.x;
    gj.y = cj * ua.y + cjb * ub.y;
    gj.z = cj * ua.z + cjb * ub.z;
    // d/dr_k : g (fp X - f Xp) ub + xi dg (ua - cs ub)/r2
    const R ck = g * (fp * X - f * Xp) - xi * dg * cs * i2;
    const R cka = xi * dg * i2;
    gk.x = ck * ub.x + cka * ua.x;
    gk.y = ck * ub.y + cka * ua.y;
    gk.z = ck * ub.z + cka * ua.z;
    return true;
}

// The same zeta term and gradient from per-bond quantities computed once per
// bond instead of once per triplet: unit vectors ua, ub, inverse lengths and
// the cutoff factor f(r_ik), f'(r_ik) of bond ik.
template <typename R>
__device__ __forceinline__ R tersoff_term_c(const TripT<R>& t, const V3<R>& ua, R r1, const V3<R>& ub, R r2, R f) {
    const R cs = ua.x * ub.x + ua.y * ub.y + ua.z * ub.z;
    R g, dg;
    angular(t, cs, g, dg);
    R X, Xp;
    radial_exp(t, r1 - r2, X, Xp);
    return f * X * g;
}

template <typename R>
__device__ __forceinline__ void tersoff_grad_c(const TripT<R>& t, const V3<R>& ua, R r1, R i1, const V3<R>& ub, R r2,
                                               R i2, R f, R fp, V3<R>& gj, V3<R>& gk) {
    const R cs = ua.x * ub.x + ua.y * ub.y + ua.z * ub.z;
    R g, dg;
    angular(t, cs, g, dg);
    R X, Xp;
    radial_exp(t, r1 - r2, X, Xp);
    const R xi = f * X;
    const R xdg = xi * dg;
    const R cj = g * f * Xp - xdg * cs * i1;
    const R cjb = xdg * i1;
    gj.x = cj * ua.x + cjb * ub.x;
    gj.y = cj * ua.y + cjb * ub.y;
    gj.z = cj * ua.z + cjb * ub.z;
    const R ck = g * (fp * X - f * Xp) - xdg * cs * i2;
    const R cka = xdg * i2;
    gk.x = ck * ub.x + cka * ua.x;
    gk.y = ck * ub.y + cka * ua.y;
    gk.z = ck * ub.z + cka * ua.z;
}

// B(zeta) = (1 + (beta zeta)^eta)^(-1/(2 eta)) and dB/dzeta
// (post_process_bond_order_factor_tersoff / _gradient_tersoff, Potentials.f90:5910-5961)
template <typename R>
__device__ __forceinline__ void post_process(R beta, R eta, R zeta, R& B, R& dB) {
    const R tt = pow_(beta * zeta, eta);
    B = pow_(R(1) + tt, R(-0.5) / eta);
    dB = zeta > R(0) ? R(-0.5) * B * tt / ((R(1) + tt) * zeta) : R(0);
}
// FP32: x^y written as 2^(y log2 x), and (1 + t)^p as exp(p log1p(t)) so that
// the small t = (beta zeta)^eta keeps its relative accuracy
template <>
__device__ __forceinline__ void post_process<float>(float beta, float eta, float zeta, float& B, float& dB) {
    if (zeta > 0.0f) {
        const float tt = exp2f(eta * log2f(beta * zeta));
        B = expf(__fdividef(-0.5f, eta) * log1pf(tt));
        dB = __fdividef(-0.5f * B * tt, (1.0f + tt) * zeta);
    } else {
        B = 1.0f;
        dB = 0.0f;
    }
}

// Slot of the atom a lane group handles.  The atoms, sorted by list length,
// are cut into warp-sized runs that are dealt round-robin over the blocks, so
// that the lanes of a warp loop equally long and every block gets a similar
// mix of light and heavy warps.  blk is the block's index among the nblk
// blocks of one system; a bijection onto [0, nblk * blockDim.x / G).
template <int G>
__device__ __forceinline__ int dealt_slot(int blk, int nblk) {
    constexpr int APW = 32 / G;
    const int wi = threadIdx.x >> 5, si = (threadIdx.x & 31) / G;
    return (wi * nblk + blk) * APW + si;
}

// warp-segment reductions over groups of G lanes
template <int G, typename T>
__device__ __forceinline__ T group_sum(T v) {
#pragma unroll
    for (int o = G / 2; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o, G);
    return v;
}

// Per-atom group sums: XSum (mixed path) holds 2^-32 fixed point, DSum (FP64
// path) an FP64 value; fixed.cuh explains the fixed-point formats.
struct XSum {
    long long f;
    __device__ __forceinline__ double d() const { return fix_to_double(f); }
    __device__ __forceinline__ Fx128 fx() const { return fx_from_fix(f); }
};
struct DSum {
    double s;
    __device__ __forceinline__ double d() const { return s; }
    __device__ __forceinline__ Fx128 fx() const { return fx_from_double(s); }
};

// Group sum in the working precision and, in the mixed path, one conversion to
// 2^-32 fixed point afterwards: an FP32 shuffle tree over the G lanes of an atom
// (a fixed order, so deterministic), exact from there on.
template <int G>
__device__ __forceinline__ XSum group_sum_f(float v) {
    return XSum{fix_from_float(group_sum<G>(v))};
}
template <int G>
__device__ __forceinline__ DSum group_sum_f(double v) {
    return DSum{group_sum<G>(v)};
}

// sum over the 32 lanes of a warp in the working precision, widened exactly to
// a 128-bit total (the same in every lane)
__device__ __forceinline__ Fx128 warp_total(float v) { return fx_from_float(group_sum<32>(v)); }
__device__ __forceinline__ Fx128 warp_total(double v) { return fx_from_double(group_sum<32>(v)); }

__device__ __forceinline__ Fx128 fx_from(float v) { return fx_from_float(v); }
__device__ __forceinline__ Fx128 fx_from(double v) { return fx_from_double(v); }

// Sums 8 values over the 32 lanes of a warp with 9 shuffles instead of 8 x 5:
// at each of the first three levels (lane distance 16, 8, 4) a lane keeps half
// of its values and trades the other half with its partner, then the last two
// levels sum the one value left.  Lane l ends with the warp total of value
// `which` = 4 b4 + 2 b3 + b2 (b: the bits of l); a fixed order, so the result
// is reproducible.
template <typename R>
__device__ __forceinline__ R warp_sum8(const R (&v)[8], int& which) {
    const int l = threadIdx.x & 31;
    const bool h4 = (l & 16) != 0, h3 = (l & 8) != 0, h2 = (l & 4) != 0;
    R a[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
        const R keep = h4 ? v[j + 4] : v[j], send = h4 ? v[j] : v[j + 4];
        a[j] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
    R b[2];
#pragma unroll
    for (int j = 0; j < 2; ++j) {
        const R keep = h3 ? a[j + 2] : a[j], send = h3 ? a[j] : a[j + 2];
        b[j] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
    R c = (h2 ? b[1] : b[0]) + __shfl_xor_sync(0xffffffffu, h2 ? b[0] : b[1], 4);
    c += __shfl_xor_sync(0xffffffffu, c, 2);
    c += __shfl_xor_sync(0xffffffffu, c, 1);
    which = (h4 ? 4 : 0) + (h3 ? 2 : 0) + (h2 ? 1 : 0);
    return c;
}

// Adds a block's energy and virial to the global totals acc[0..6] (null: none)
// from every lane's 7 terms t, with the result of block_totals_publish: each
// warp sums its lanes in the working precision (warp_sum8) and leaves the 7
// sums in shared memory (wpart); the last warp of the block to arrive widens
// them exactly, lane c taking value c over the block's warps in warp order,
// and sends value c's limbs to acc from lane c.  Only one warp per block
// converts, and the 7 values go out in parallel.  `done` is a shared counter
// set to zero before the block's first barrier.  x0, wx (both null, or both
// set): an exact 128-bit warp total (the same in every lane) added to value 0,
// through the per-warp shared slots wx.
template <typename R>
__device__ __forceinline__ void block_totals_add(const R (&t)[7], R (*wpart)[7], unsigned* done, FxAcc* acc,
                                                 const Fx128* x0 = nullptr, Fx128* wx = nullptr) {
    if (acc == nullptr) return;
    const int wl = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const R t8[8] = {t[0], t[1], t[2], t[3], t[4], t[5], t[6], R(0)};
    int which;
    const R tot = warp_sum8(t8, which);
    if ((wl & 3) == 0 && which < 7) wpart[w][which] = tot;
    if (x0 && wl == 0) wx[w] = *x0;
    __syncwarp();
    unsigned last = 0;
    if (wl == 0) {
        __threadfence_block();
        last = atomicAdd(done, 1u) == (unsigned)(nw - 1) ? 1u : 0u;
    }
    if (__shfl_sync(0xffffffffu, last, 0) == 0u) return;
    __threadfence_block();
    if (wl < 7) {
        Fx128 x = fx_zero();
        for (int k = 0; k < nw; ++k) {
            const volatile R* q = &wpart[k][wl];
            x = fx_add(x, fx_from((R)*q));
            if (x0 && wl == 0) {
                const volatile Fx128* e = &wx[k];
                x = fx_add(x, Fx128{e->lo, e->hi});
            }
        }
        fx_red(&acc[wl], x);
    }
}

// write (first) or add a group sum into a per-atom FP64 output; the mixed
// path adds in fixed point
__device__ __forceinline__ void store_sum(double* p, const XSum& v, bool first) {
    *p = first ? v.d() : fix_to_double(v.f + fix_from_double(*p));
}
__device__ __forceinline__ void store_sum(double* p, const DSum& v, bool first) { *p = first ? v.s : *p + v.s; }

// Adds a block's energy and virial to the global totals acc[0..6] (null: none)
// without a block-wide barrier.  v holds the 7 totals of the calling warp
// (read in lane 0).  Each warp publishes its sums in shared memory; the last
// warp of the block to arrive adds all of them to acc.  `done` is a shared
// counter set to zero before the block's first barrier.
__device__ __forceinline__ void block_totals_publish(const Fx128 (&v)[7], Fx128 (*wsum)[7], unsigned* done,
                                                     FxAcc* acc) {
    if (acc == nullptr) return;
    const int wl = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
    if (wl == 0) {
#pragma unroll
        for (int c = 0; c < 7; ++c) wsum[w][c] = v[c];
        __threadfence_block();
        if (atomicAdd(done, 1u) == (unsigned)(nw - 1)) {
            __threadfence_block();
            for (int c = 0; c < 7; ++c) {
                Fx128 t = fx_zero();
                for (int k = 0; k < nw; ++k) {
                    const volatile Fx128* q = &wsum[k][c];
                    t = fx_add(t, Fx128{q->lo, q->hi});
                }
                fx_red(&acc[c], t);
            }
        }
    }
}

}  // namespace pg
