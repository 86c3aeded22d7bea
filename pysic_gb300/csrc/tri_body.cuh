// tri_body.cuh -- the triplet tile of the bond pass (16 lanes per atom as a
// 4 x 4 tile of triplets), shared by the one-system and many-system kernels of
// tersoff_tri.cu and the persistent batch kernel.  The method is described at
// the top of tersoff_tri.cu.
#pragma once

#include "args.cuh"
#include "bond.cuh"
#include "common.cuh"
#include "kernels.cuh"

namespace pg {

constexpr int TRI_THREADS = 128;             // 4 warps, 8 atoms per round
constexpr int TRI_ATOMS = TRI_THREADS / 16;  // atoms per block and round
constexpr int TRI_CAP = 16;                  // bonds per atom staged in shared memory

// per atom (half warp): staged bond geometry, per-bond prefactor and the j / k
// force parts being summed
template <typename R>
struct TriStage {
    typename Vec4T<R>::T geo[TRI_CAP];   // bond vector, length
    typename Vec4T<R>::T unit[TRI_CAP];  // unit vector, 1/r
    typename Vec2T<R>::T cut[TRI_CAP];   // f(r), f'(r) of the bond-order cutoff (uniform cutoffs)
    typename Vec4T<R>::T jp[TRI_CAP];    // j part of bond e (xyz)
    typename Vec4T<R>::T kp[TRI_CAP];    // k parts landing on entry k (xyz)
    R pref[TRI_CAP];                     // 1/2 V f dB/dzeta of bond e (0: no three-body force)
    int typ[TRI_CAP];
};

// running energy and virial of a lane
template <typename R>
struct TriAcc {
    R En = 0, W0 = 0, W1 = 0, W2 = 0, W3 = 0, W4 = 0, W5 = 0;
};

// sum over the column of a 4 x 4 tile: lanes t, t ^ 4, t ^ 8, t ^ 12 of a half warp
template <typename R>
__device__ __forceinline__ R column_sum(R v) {
    v += __shfl_xor_sync(0xffffffffu, v, 4, 16);
    v += __shfl_xor_sync(0xffffffffu, v, 8, 16);
    return v;
}

// One atom per half warp: gslot is the atom's slot in the order of list length
// (>= A.n: an idle half warp that still takes part in every shuffle).
template <typename R, bool SPEC>
__device__ __forceinline__ void tri_atom(const BondArgs& A, int gslot, TriStage<R>& S, TriAcc<R>& acc) {
    using V4 = typename Vec4T<R>::T;
    using V2 = typename Vec2T<R>::T;
    const int t = threadIdx.x & 15, a = t >> 2, b = t & 3;
    const bool act = gslot < A.n;
    int i = 0, s = 0, ni = 0;
    if (act) {
        if (A.slot) {
            const int4 rec = A.slot[gslot];
            i = rec.x;
            s = rec.y;
            ni = rec.z;
        } else {
            i = A.order ? A.order[gslot] : gslot;
            s = A.start[i];
            ni = A.start[i + 1] - s;
        }
    }
    auto SPV = [&](int q) -> R {
        if constexpr (sizeof(R) == 4) return A.spf[q];
        else return A.spd[q];
    };
    // bonds beyond the shared capacity live in the context's per-entry scratch
    const bool staged = ni <= TRI_CAP;
    V4* geo = staged ? S.geo : (V4*)A.geo + s;
    V4* jp = staged ? S.jp : (V4*)A.bscr + s;
    V4* kp = staged ? S.kp : (V4*)A.kacc + s;
    const bool cached_cut = staged && (SPEC || A.bcut_uniform);
    const int ti = (act && !SPEC) ? A.type[i] : 0;
    const int T = A.T;
    const PairT<R>* terms = (const PairT<R>*)A.terms;
    const TripT<R>* trip = (const TripT<R>*)A.trip;
    TripT<R> TS{};
    if constexpr (SPEC)
        TS = TripT<R>{SPV(SP_A), SPV(SP_C2), SPV(SP_D2), SPV(SP_H), SPV(SP_MU), SPV(SP_RC), SPV(SP_RS), SPV(SP_C2D2), 1};
    auto type_of = [&](int k) -> int {
        if constexpr (SPEC) return 0;
        else return staged ? S.typ[k] : A.etype[s + k];
    };
    auto trip_of = [&](int tj, int tk) -> TripT<R> {
        if constexpr (SPEC) return TS;
        else return trip[(ti * T + tj) * T + tk];
    };
    auto unit_of = [&](int k, const V4& g, V3<R>& u, R& ir) {
        if (staged) {
            const V4 v = S.unit[k];
            u = V3<R>{v.x, v.y, v.z};
            ir = v.w;
        } else {
            ir = g.w > R(0) ? rcp_(g.w) : R(0);
            u = V3<R>{g.x * ir, g.y * ir, g.z * ir};
        }
    };
    R maxbr = R(0);
    if constexpr (SPEC) maxbr = SPV(SP_RC);
    else if (act) maxbr = ((const R*)A.maxbr)[ti];

    // 1. geometry, one bond per lane; the force parts start at zero
    if (act) {
        double xi = 0, yi = 0, zi = 0;
        if constexpr (sizeof(R) == 8) {
            xi = A.pos[3 * i];
            yi = A.pos[3 * i + 1];
            zi = A.pos[3 * i + 2];
        }
        for (int e = t; e < ni; e += 16) {
            const V4 g = bond_vector<R>(A, i, s + e, xi, yi, zi);
            geo[e] = g;
            jp[e] = V4{0, 0, 0, 0};
            kp[e] = V4{0, 0, 0, 0};
            if (staged) {
                S.pref[e] = R(0);
                const R ir = g.w > R(0) ? rcp_(g.w) : R(0);
                S.unit[e] = V4{g.x * ir, g.y * ir, g.z * ir, ir};
                if constexpr (SPEC) {
                    R f, fp;
                    smooth<R>(g.w, SPV(SP_RC), SPV(SP_RS), f, fp);
                    S.cut[e] = V2{f, fp};
                } else {
                    const int te = A.etype[s + e];
                    S.typ[e] = te;
                    if (A.bcut_uniform) {
                        const V2 c = ((const V2*)A.bcut)[ti * T + te];
                        R f, fp;
                        smooth<R>(g.w, c.x, c.y, f, fp);
                        S.cut[e] = V2{f, fp};
                    }
                }
            }
        }
    }
    __syncwarp();
    // the prefactor of bond e: shared memory, or (unstaged atoms) the .w of its
    // j part, which the j-part sums below never write
    auto pref_of = [&](int e) -> R { return staged ? S.pref[e] : jp[e].w; };
    const int nb = (int)__reduce_max_sync(0xffffffffu, (unsigned)((ni + 3) >> 2));  // 4-bond blocks, warp-wide
    R Fx = 0, Fy = 0, Fz = 0;  // this lane's part of the force on the centre

    // 2. zeta of each bond (row sums), then B, the pair terms and the radial force
    for (int eb = 0; eb < nb; ++eb) {
        const int e = 4 * eb + a;
        const bool ve = act && e < ni;
        V4 gij = ve ? geo[e] : V4{0, 0, 0, 0};
        const R r = gij.w;
        const int tj = ve ? type_of(e) : 0;
        int2 ix = make_int2(0, 0);
        bool any = false, bo = false;
        if (ve) {
            if constexpr (SPEC) {
                any = bo = r < SPV(SP_RC);
            } else {
                ix = A.index[ti * T + tj];
                for (int q = ix.x; q < ix.x + ix.y; ++q) {
                    const PairT<R>& P = terms[q];
                    if (P.in_bond_kernel && r < P.rc) {
                        any = true;
                        bo |= P.group >= 0;
                    }
                }
            }
        }
        V3<R> ua{0, 0, 0};
        R i1 = 0;
        if (ve) unit_of(e, gij, ua, i1);
        R zp = 0;
        if (ve && (bo || A.zeta_out) && r != R(0)) {
            for (int kb = 0; kb < nb; ++kb) {
                const int k = 4 * kb + b;
                if (k >= ni || k == e) continue;
                const V4 gik = geo[k];
                if (!(gik.w < maxbr)) continue;
                const TripT<R> TT = trip_of(tj, type_of(k));
                if (!TT.valid) continue;
                R f, fp;
                if (cached_cut) f = S.cut[k].x;
                else smooth<R>(gik.w, TT.rc, TT.rs, f, fp);
                if (f == R(0)) continue;
                V3<R> ub;
                R i2;
                unit_of(k, gik, ub, i2);
                zp += tersoff_term_c<R>(TT, ua, r, ub, gik.w, f);
            }
        }
        const R zeta = group_sum<4>(zp);
        if (A.zeta_out && ve && b == 0) A.zeta_out[s + e] = (double)zeta;
        if (A.b_out && ve && b == 0 && (!any || r == R(0))) ((R*)A.b_out)[s + e] = R(1);
        if (!ve || !any || r == R(0)) continue;
        R B = 1, dB = 0;
        if (bo) {
            PostT<R> pp{};
            if constexpr (SPEC) pp = PostT<R>{SPV(SP_BETA), SPV(SP_ETA), 1};
            else pp = ((const PostT<R>*)A.post)[ti * T + tj];  // the pair type's group
            if (pp.valid) {
                post_process<R>(pp.beta, pp.eta, zeta, B, dB);
            } else {
                B = zeta;
                dB = 1;
            }
        }
        if (A.b_out && b == 0) ((R*)A.b_out)[s + e] = B;
        R U = 0, dU = 0, P = 0;
        if constexpr (SPEC) {
            R f, fp;
            if (cached_cut) {
                const V2 fc = S.cut[e];
                f = fc.x;
                fp = fc.y;
            } else {
                smooth<R>(r, SPV(SP_RC), SPV(SP_RS), f, fp);
            }
#pragma unroll
            for (int q = 0; q < PG_SPEC_MAX_TERMS; ++q) {
                if (q >= A.spec_nterm) break;
                const R p1 = SPV(SP_TERMS + 2 * q + 1);
                const R ex = SPV(SP_TERMS + 2 * q) * exp_(-p1 * r);
                const R V = ex * f, dV = ex * (fp - p1 * f);
                if ((A.spec_bomask >> q) & 1) {
                    U += V * B;
                    dU += dV * B;
                    P += V;
                } else {
                    U += V;
                    dU += dV;
                }
            }
        } else {
            V2 bc{R(-1), R(-1)};
            if (cached_cut) bc = ((const V2*)A.bcut)[ti * T + tj];
            for (int q = ix.x; q < ix.x + ix.y; ++q) {
                const PairT<R>& PT = terms[q];
                if (!PT.in_bond_kernel || !(r < PT.rc)) continue;
                R V, dV;
                if (PT.kind >= 7 || PT.nmul > 0) {  // charge-dependent or product (bond-order scaled)
                    R en;
                    bond_charge_term<R>(A, PT, terms, i, s + e, ti, tj, r, V, dV, en);
                } else if (PT.smooth && PT.rc == bc.x && PT.rs == bc.y) {
                    pair_eval<R>(PT, r, V, dV, (const R*)A.tab);
                    const V2 fc = S.cut[e];
                    dV = dV * fc.x + V * fc.y;
                    V = V * fc.x;
                } else {
                    pair_term<R>(PT, r, V, dV, (const R*)A.tab);
                }
                if (PT.group < 0) {
                    U += V;
                    dU += dV;
                } else {
                    U += V * B;
                    dU += dV * B;
                    P += V;
                }
            }
        }
        if (b == 0) {  // one lane of the row keeps the bond's own terms
            const R c = R(0.5) * dU * i1;
            acc.En += R(0.5) * U;
            Fx += c * gij.x;
            Fy += c * gij.y;
            Fz += c * gij.z;
            acc.W0 -= gij.x * c * gij.x;
            acc.W1 -= gij.y * c * gij.y;
            acc.W2 -= gij.z * c * gij.z;
            acc.W3 -= gij.y * c * gij.z;
            acc.W4 -= gij.x * c * gij.z;
            acc.W5 -= gij.x * c * gij.y;
            const R pr = bo ? R(0.5) * P * dB : R(0);
            jp[e] = V4{-c * gij.x, -c * gij.y, -c * gij.z, staged ? R(0) : pr};
            if (staged) S.pref[e] = pr;
        }
    }
    __syncwarp();

    // 3. three-body forces: triplet (e, k) per lane; j parts summed over the row,
    // k parts over the column; written component by component by one lane each
    for (int eb = 0; eb < nb; ++eb) {
        const int e = 4 * eb + a;
        const bool ve = act && e < ni;
        const R pe = ve ? pref_of(e) : R(0);
        V4 gij = V4{0, 0, 0, 0};
        V3<R> ua{0, 0, 0};
        R i1 = 0;
        int tj = 0;
        if (ve && pe != R(0)) {
            gij = geo[e];
            unit_of(e, gij, ua, i1);
            tj = type_of(e);
        }
        R jx = 0, jy = 0, jz = 0;
        for (int kb = 0; kb < nb; ++kb) {
            const int k = 4 * kb + b;
            R kx = 0, ky = 0, kz = 0;
            if (pe != R(0) && k < ni && k != e) {
                const V4 gik = geo[k];
                if (gik.w < maxbr) {
                    const TripT<R> TT = trip_of(tj, type_of(k));
                    if (TT.valid) {
                        R f, fp;
                        if (cached_cut) {
                            const V2 cc = S.cut[k];
                            f = cc.x;
                            fp = cc.y;
                        } else {
                            smooth<R>(gik.w, TT.rc, TT.rs, f, fp);
                        }
                        if (!(f == R(0) && fp == R(0))) {
                            V3<R> ub, gj, gk;
                            R i2;
                            unit_of(k, gik, ub, i2);
                            tersoff_grad_c<R>(TT, ua, gij.w, i1, ub, gik.w, i2, f, fp, gj, gk);
                            const R qjx = -pe * gj.x, qjy = -pe * gj.y, qjz = -pe * gj.z;
                            kx = -pe * gk.x;
                            ky = -pe * gk.y;
                            kz = -pe * gk.z;
                            jx += qjx;
                            jy += qjy;
                            jz += qjz;
                            Fx -= qjx + kx;
                            Fy -= qjy + ky;
                            Fz -= qjz + kz;
                            acc.W0 += gij.x * qjx + gik.x * kx;
                            acc.W1 += gij.y * qjy + gik.y * ky;
                            acc.W2 += gij.z * qjz + gik.z * kz;
                            acc.W3 += gij.y * qjz + gik.y * kz;
                            acc.W4 += gij.x * qjz + gik.x * kz;
                            acc.W5 += gij.x * qjy + gik.x * ky;
                        }
                    }
                }
            }
            // the k parts of this block of bonds on neighbour k, summed over the column
            kx = column_sum(kx);
            ky = column_sum(ky);
            kz = column_sum(kz);
            if (act && a == 0 && k < ni) {
                kp[k].x += kx;
                kp[k].y += ky;
                kp[k].z += kz;
            }
        }
        jx = group_sum<4>(jx);
        jy = group_sum<4>(jy);
        jz = group_sum<4>(jz);
        if (ve && b == 0) {
            jp[e].x += jx;
            jp[e].y += jy;
            jp[e].z += jz;
        }
    }
    __syncwarp();
    // 4. per entry i->x: the force of this atom's bonds on x, stored in x's own
    // entry x->i; the centre part summed over the 16 lanes
    V4* fj = (V4*)A.fj;
    if (act) {
        for (int e = t; e < ni; e += 16) {
            const V4 jv = jp[e], kv = kp[e];
            fj[A.rev[s + e]] = V4{jv.x + kv.x, jv.y + kv.y, jv.z + kv.z, 0};
        }
    }
    const auto d0 = group_sum_f<16>(Fx), d1 = group_sum_f<16>(Fy), d2 = group_sum_f<16>(Fz);
    if (act && t == 0) {
        if constexpr (sizeof(R) == 4) {
            long long* fc = (long long*)A.fc + 3 * i;
            fc[0] = d0.f;
            fc[1] = d1.f;
            fc[2] = d2.f;
        } else {
            double* fc = (double*)A.fc + 3 * i;
            fc[0] = d0.s;
            fc[1] = d1.s;
            fc[2] = d2.s;
        }
    }
    __syncwarp();  // the stage is reused by the next atom
}

// energy and virial of the block's warps to the totals
template <typename R>
__device__ __forceinline__ void tri_publish(const TriAcc<R>& acc, Fx128 (*wsum)[7], unsigned* done, FxAcc* dst) {
    if (dst == nullptr) return;
    const Fx128 v[7] = {warp_total(acc.En), warp_total(acc.W0), warp_total(acc.W1), warp_total(acc.W2),
                        warp_total(acc.W3), warp_total(acc.W4), warp_total(acc.W5)};
    block_totals_publish(v, wsum, done, dst);
}

}  // namespace pg
