// pair_body.cuh -- the per-block body of the pair kernel (pair terms,
// products of pair potentials, real-space Ewald, single-atom terms), shared by
// the one-system kernel, the many-system kernel and the persistent batch
// kernel.  The arithmetic and its citations are those of pair.cu.
#pragma once

#include "args.cuh"
#include "atomfactor.cuh"
#include "common.cuh"
#include "kernels.cuh"
#include "pairvec.cuh"

namespace pg {

__device__ __forceinline__ double powi_(double x, int n) {
    double r = 1.0;
    for (int k = 0; k < n; ++k) r *= x;
    return r;
}

// AF: also add the per-atom factor forces (no scaled pair term; W from af_sum)
template <typename R, int G, bool AF = false>
__device__ __forceinline__ void pair_body(const PairArgs& A, int blk) {
    __shared__ R wpart[256 / 32][7];
    __shared__ Fx128 wx[256 / 32];
    __shared__ unsigned done;
    if (threadIdx.x == 0) done = 0u;
    __syncthreads();
    const int lane = threadIdx.x % G;
    const int slot = threadIdx.x / G;
    const int i = blk * (blockDim.x / G) + slot;
    if (A.skip && *A.skip) return;
    const bool act = i < A.n;
    R fx = 0, fy = 0, fz = 0, en = 0, chi = 0;
    R w0 = 0, w1 = 0, w2 = 0, w3 = 0, w4 = 0, w5 = 0;
    R pre[PG_MAX_AGROUPS] = {};  // per-atom factor groups: this atom's prefactors (half of each pair's V f)
    const bool wantE = A.flags & PG_WANT_ENERGY, wantF = A.flags & PG_WANT_FORCES, wantC = A.flags & PG_WANT_ENEGS;
    int ti = 0;
    R wk[PG_MAX_AGROUPS] = {};
    if (act) {
        ti = A.type[i];
        if constexpr (AF) {
#pragma unroll
            for (int g = 0; g < PG_MAX_AGROUPS; ++g)
                if (g < A.ng) wk[g] = ((const R*)A.afW)[(size_t)g * A.n + i];
        }
        const R qi = charge_of<R>(A, i);
        const R ew_rc = (R)A.ew_rc, ew_is2 = (R)A.ew_is2, ew_k = (R)A.ew_k, ew_c2 = (R)A.ew_c2,
                ew_isq2 = (R)A.ew_isq2;
        double xi = 0, yi = 0, zi = 0;
        if constexpr (sizeof(R) == 8) {
            xi = A.pos[3 * i];
            yi = A.pos[3 * i + 1];
            zi = A.pos[3 * i + 2];
        }
        const int e1 = A.start[i + 1];
        for (int e = A.start[i] + lane; e < e1; e += G) {
            const int j = A.idx[e];
            R x, y, z;
            pair_vector<R>(A, i, e, xi, yi, zi, x, y, z);
            const R r = sqrt_(x * x + y * y + z * z);
            if (r == R(0)) continue;
            const R ir = R(1) / r;
            R U = 0, dU = 0;
            R gs = 0;  // step terms: the same force on every component (not radial)
            if (A.ewald && r < ew_rc) {
                const R qj = charge_of<R>(A, j);
                const R qq = qi * qj;
                const R ec = erfc_(r * ew_is2);
                U += ew_k * qq * ec * ir;
                if (wantF) dU -= ew_k * qq * (ec * ir * ir + ew_c2 * exp_(-r * r * ew_isq2) * ir);
                if (wantC) chi -= qj * ew_k * ec * ir;
            }
            const int tj = A.type[j];
            // charge-independent pair terms have zero electronegativity
            const int2 ix = (wantE || wantF || (wantC && A.qpair)) ? A.index[ti * A.T + tj] : make_int2(0, 0);
            for (int t = ix.x; t < ix.x + ix.y; ++t) {
                const PairT<R> P = ((const PairT<R>*)A.terms)[t];
                if (P.in_bond_kernel || !(r < P.rc)) continue;
                if (P.nmul > 0) {
                    // a product of potentials (Potentials.f90:2512-2700), then the
                    // record's smooth cut
                    const bool first = pick(i, j, A.off[3 * e], A.off[3 * e + 1], A.off[3 * e + 2]);
                    R V, dV, en;
                    product_value<R>(P, (const PairT<R>*)A.terms, (const R*)A.tab, r, qi, charge_of<R>(A, j), first,
                                     ti, tj, V, dV, en);
                    R f = R(1), fp = R(0);
                    if (P.smooth) smooth<R>(r, P.rc, P.rs, f, fp);
                    U += V * f;
                    dU += dV * f + V * fp;
                    if (wantC) chi += en * f;
                    continue;
                }
                if (P.kind == 7) {
                    // charge_pair: eps q1^n1 q2^n2 of the pair's (atom1, atom2) as the
                    // reference's loop picks them; the exponents follow the unpermuted
                    // first target (evaluate_energy/electronegativity_charge_pair,
                    // Potentials.f90:4415-4513).  No r dependence but the smooth cutoff.
                    const bool first = pick(i, j, A.off[3 * e], A.off[3 * e + 1], A.off[3 * e + 2]);
                    const R qj = charge_of<R>(A, j);
                    const R q1 = first ? qi : qj, q2 = first ? qj : qi;
                    const bool direct = (P.first >> (first ? ti : tj)) & 1ull;
                    const int n1 = direct ? (int)P.p1 : (int)P.p2, n2 = direct ? (int)P.p2 : (int)P.p1;
                    R f = R(1), fp = R(0);
                    if (P.smooth) smooth<R>(r, P.rc, P.rs, f, fp);
                    const R v = P.p0 * (ipow(q1, n1) * ipow(q2, n2));
                    U += v * f;
                    dU += v * fp;
                    if (wantC) {
                        const int nm = first ? n1 : n2;  // the exponent of this atom's charge
                        if (nm > 0)
                            chi -= (first ? P.p0 * (R(n1) * ipow(q1, n1 - 1) * ipow(q2, n2))
                                          : P.p0 * (R(n2) * ipow(q1, n1) * ipow(q2, n2 - 1))) * f;
                    }
                    continue;
                }
                if (P.kind == 8) {
                    // charge_exp, V = eps exp((xi_1 D_1(q_1) + xi_2 D_2(q_2))/2),
                    // D(q) = Rmax + |beta (Qmax - q)|^eta, with the parameters of the
                    // unpermuted first target on the pair's atom1 when its type is that
                    // target's (Potentials.f90:3691-3903; no r dependence but the cut)
                    const R* c = (const R*)A.tab + 2 * (long long)P.t0;
                    const bool first = pick(i, j, A.off[3 * e], A.off[3 * e + 1], A.off[3 * e + 2]);
                    const R qj = charge_of<R>(A, j);
                    const R q1 = first ? qi : qj, q2 = first ? qj : qi;
                    const bool direct = (P.first >> (first ? ti : tj)) & 1ull;
                    const int a1 = direct ? 0 : 4, a2 = direct ? 4 : 0;  // Rmax at 1 + a, Qmax at 3 + a
                    const R eta1 = c[direct ? 11 : 12], eta2 = c[direct ? 12 : 11];
                    const R beta1 = c[direct ? 13 : 14], beta2 = c[direct ? 14 : 13];
                    const R xi1 = c[direct ? 9 : 10], xi2 = c[direct ? 10 : 9];
                    const R d5 = beta1 * (c[3 + a1] - q1), d6 = beta2 * (c[3 + a2] - q2);
                    const R D1 = c[1 + a1] + pow_(fabs(d5), eta1), D2 = c[1 + a2] + pow_(fabs(d6), eta2);
                    R f = R(1), fp = R(0);
                    if (P.smooth) smooth<R>(r, P.rc, P.rs, f, fp);
                    const R v = c[0] * exp_(R(0.5) * (xi1 * D1 + xi2 * D2));
                    U += v * f;
                    dU += v * fp;
                    if (wantC) {
                        chi += first ? v * xi1 * R(0.5) * eta1 * pow_(fabs(d5), eta1 - R(1)) * copysign(R(1), d5) * beta1 * f
                                     : v * xi2 * R(0.5) * eta2 * pow_(fabs(d6), eta2 - R(1)) * copysign(R(1), d6) * beta2 * f;
                    }
                    continue;
                }
                if (P.kind == 9) {
                    // charge_abs, V = sqrt(f_1(q_1) f_2(q_2)), f(q) = a + b |q - Q|^n, f < 0
                    // taken as 0, parameters (a, b, Q, n) of the unpermuted first target on
                    // atom1 when its type is that target's (Potentials.f90:4525-4728); no
                    // r dependence but the cut
                    const R* c = (const R*)A.tab + 2 * (long long)P.t0;
                    const bool first = pick(i, j, A.off[3 * e], A.off[3 * e + 1], A.off[3 * e + 2]);
                    const R qj = charge_of<R>(A, j);
                    const R q1 = first ? qi : qj, q2 = first ? qj : qi;
                    const bool direct = (P.first >> (first ? ti : tj)) & 1ull;
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
                    R f = R(1), fp = R(0);
                    if (P.smooth) smooth<R>(r, P.rc, P.rs, f, fp);
                    // the energy routine takes |q - Q|^n directly
                    const R e1 = fmax(s1[0] + s1[1] * pow_(ab1, s1[3]), R(0));
                    const R e2 = fmax(s2[0] + s2[1] * pow_(ab2, s2[3]), R(0));
                    const R v = sqrt_(e1 * e2);
                    U += v * f;
                    dU += v * fp;
                    if (wantC) {
                        chi += first ? is * (-s1[3] * pw1 * copysign(R(1), q1 - s1[2]) * s1[1]) * f2 * f
                                     : is * (-s2[3] * pw2 * copysign(R(1), q2 - s2[2]) * s2[1]) * f1 * f;
                    }
                    continue;
                }
                if (!(wantE || wantF)) continue;
                R V, dV;
                pair_term<R>(P, r, V, dV, (const R*)A.tab);
                if (P.kind == 10 && wantF) {
                    // force (c, c, c) on the pair's atom 1, -(c, c, c) on atom 2, times the cut
                    const bool first = pick(i, j, A.off[3 * e], A.off[3 * e + 1], A.off[3 * e + 2]);
                    R f = R(1), fp = R(0);
                    if (P.smooth) smooth<R>(r, P.rc, P.rs, f, fp);
                    const R c = step_force<R>(P, r) * f;
                    gs += first ? c : -c;
                }
                if (P.agroup >= 0) {
                    // scaled by the pair's mean per-atom factor (B_i + B_j)/2
                    // (Core.f90:4345-4350, 5553-5560); half of V f is each atom's
                    // prefactor of the gradient of its factor (5486-5491)
                    const R* B = (const R*)A.afB + (size_t)P.agroup * A.n;
                    const R bm = R(0.5) * (B[i] + B[j]);
#pragma unroll
                    for (int q = 0; q < PG_MAX_AGROUPS; ++q)
                        if (q == P.agroup) pre[q] += R(0.5) * V;
                    V *= bm;
                    dV *= bm;
                }
                U += V;
                dU += dV;
            }
            en += R(0.5) * U;
            // force on i: U'(r) r_hat; half of the pair virial sep (x) F_j, F_j = -U' r_hat
            R c = dU * ir;
            R h = R(-0.5) * c;
            if constexpr (AF) {
                if (wantF) {
                    R cf, hv;
                    af_entry<R>(A, wk, ti, j, tj, r, ir, cf, hv);
                    c += cf;
                    h += hv;
                }
            }
            fx += c * x;
            fy += c * y;
            fz += c * z;
            w0 += h * x * x;
            w1 += h * y * y;
            w2 += h * z * z;
            w3 += h * y * z;
            w4 += h * x * z;
            w5 += h * x * y;
            if (gs != R(0)) {
                // half of the reference's stress term sep12 (x) F2 taken component by
                // component (xx, yy, zz, yz, xz, xy; Core.f90:5593-5598) for F2 = -(gs, gs, gs)
                // seen from atom 1, the same from either side
                const R hg = R(-0.5) * gs;
                fx += gs;
                fy += gs;
                fz += gs;
                w0 += hg * x;
                w1 += hg * y;
                w2 += hg * z;
                w3 += hg * y;
                w4 += hg * x;
                w5 += hg * x;
            }
        }
    }
    // single-atom terms in FP64, added by the group's lane 0
    // (core_evaluate_local_singlet, Core.f90:4095-4239): charge_self eps q^n with
    // chi = -eps n q^(n-1) (Potentials.f90:4341-4375), constant V (3959-3966),
    // constant force F with energy -F . r at the absolute position (3122-3147);
    // singlets add nothing to the virial
    // With a per-atom factor (constant and force only) the energy is V B_i and the
    // term's own force gives way to -V grad B_i (V joins the prefactor).
    double cs = 0.0, es = 0.0, sf0 = 0.0, sf1 = 0.0, sf2 = 0.0;
    double spre[PG_MAX_AGROUPS] = {};
    if (act && lane == 0) {
        const int2 sx = A.sindex[ti];
        for (int t = sx.x; t < sx.x + sx.y; ++t) {
            const SingleTerm S = A.sterms[t];
            if (S.kind == 0) {
                const double qd = A.charge[i];
                es += S.p[0] * powi_(qd, S.n);
                cs += -(S.p[0] * S.n * powi_(qd, S.n - 1));
            } else {
                const double V =
                    S.kind == 1 ? S.p[0] : -(S.p[0] * A.pos[3 * i] + S.p[1] * A.pos[3 * i + 1] + S.p[2] * A.pos[3 * i + 2]);
                if (S.agroup >= 0) {
                    if (wantE || wantF) es += V * (double)((const R*)A.afB)[(size_t)S.agroup * A.n + i];
#pragma unroll
                    for (int q = 0; q < PG_MAX_AGROUPS; ++q)
                        if (q == S.agroup) spre[q] += V;
                } else {
                    es += V;
                    if (S.kind == 2) {
                        sf0 += S.p[0];
                        sf1 += S.p[1];
                        sf2 += S.p[2];
                    }
                }
            }
        }
    }
    // W_i = dB/dsum times the prefactor, for the per-atom factor forces
    if (wantF && A.ng > 0 && !AF) {
#pragma unroll
        for (int q = 0; q < PG_MAX_AGROUPS; ++q) {
            if (q >= A.ng) break;
            const auto sp = group_sum_f<G>(pre[q]);
            if (act && lane == 0) {
                const size_t o = (size_t)q * A.n + i;
                ((R*)A.afW)[o] = (R)(((const R*)A.afS)[o] * (sp.d() + spre[q]));
            }
        }
    }
    if (wantF) {
        auto sfx = group_sum_f<G>(fx), sfy = group_sum_f<G>(fy), sfz = group_sum_f<G>(fz);
        if (act && lane == 0) {
            if constexpr (sizeof(R) == 4) {
                sfx.f += fix_from_double(sf0);
                sfy.f += fix_from_double(sf1);
                sfz.f += fix_from_double(sf2);
            } else {
                sfx.s += sf0;
                sfy.s += sf1;
                sfz.s += sf2;
            }
            store_sum(A.out_f + 3 * i, sfx, A.first_f);
            store_sum(A.out_f + 3 * i + 1, sfy, A.first_f);
            store_sum(A.out_f + 3 * i + 2, sfz, A.first_f);
        }
    }
    if (wantC) {
        auto schi = group_sum_f<G>(chi);
        if (act && lane == 0) {
            if constexpr (sizeof(R) == 4) schi.f += fix_from_double(cs);
            else schi.s += cs;
            store_sum(A.out_chi + i, schi, A.first_chi);
        }
    }
    // energy and virial: warp sums, exact from there on
    if (A.acc && (wantE || wantF)) {
        // the single-atom energies join the total exactly, outside the working precision
        // (skipped, as zero, when no lane of the warp has one)
        Fx128 xs = fx_zero();
        if (__any_sync(0xffffffffu, es != 0.0)) xs = fx_warp_sum(fx_from_double(es));
        const R t[7] = {en, w0, w1, w2, w3, w4, w5};
        block_totals_add(t, wpart, &done, A.acc, &xs, wx);
    }
}

}  // namespace pg
