// bond_body.cuh -- per-block bodies of the pair-bond-order (Tersoff) passes
// (displacement, bond pass, gather pass), shared by the one-system kernels,
// the many-system kernels and the persistent batch kernel.  The arithmetic and
// its citations are those described at the top of tersoff.cu.
#pragma once

#include <type_traits>

#include "args.cuh"
#include "bond.cuh"
#include "common.cuh"
#include "kernels.cuh"

namespace pg {

// per-atom displacement since the list build (FP64 difference rounded to FP32)
// and the FP32 charge, one 16-byte record per atom for the mixed-path kernels;
// block 0 also clears the energy / virial totals (zero8, 8 records; may be null)
// that the kernels after it add to.  With a staged coordinate update (pos_in)
// each thread commits its atom's new coordinates first: no separate check and
// commit kernels in front of the evaluation.  A non-finite value sets the
// verdict flag; the host puts pos_prev back when it reads that verdict, so a
// rejected update still leaves the old coordinates.
__device__ __forceinline__ void disp_body(const DispArgs& A, int i) {
    if (A.zero8 && i < 8) A.zero8[i] = FxAcc{{0ull, 0ull, 0ull}};
    if (A.skip && *A.skip) return;
    if (i >= A.n || A.d == nullptr) return;
    const double* pos0 = A.pos0;
    double x, y, z;
    if (A.pos_in) {
        x = A.pos_in[3 * i];
        y = A.pos_in[3 * i + 1];
        z = A.pos_in[3 * i + 2];
        if (!(isfinite(x) && isfinite(y) && isfinite(z))) *A.bad = 1;
        A.pos_prev[3 * i] = A.pos[3 * i];
        A.pos_prev[3 * i + 1] = A.pos[3 * i + 1];
        A.pos_prev[3 * i + 2] = A.pos[3 * i + 2];
        A.pos_out[3 * i] = x;
        A.pos_out[3 * i + 1] = y;
        A.pos_out[3 * i + 2] = z;
    } else {
        x = A.pos[3 * i];
        y = A.pos[3 * i + 1];
        z = A.pos[3 * i + 2];
    }
    A.d[i] = F4{(float)(x - pos0[3 * i]), (float)(y - pos0[3 * i + 1]), (float)(z - pos0[3 * i + 2]), (float)A.q[i]};
}

// SPEC: single-species Tersoff, every parameter a kernel argument (no table
// lookups per bond or triplet); the same arithmetic as the table path.
template <typename R, int G, bool SPEC>
__device__ __forceinline__ void bond_body(const BondArgs& A, int blk, int nblk) {
    using V4 = typename Vec4T<R>::T;
    using V2 = typename Vec2T<R>::T;
    constexpr int AP = 128 / G;  // atoms per block
    // bonds per atom staged in shared memory with their unit vectors and cutoff
    // factors; an atom with more bonds reads its geometry from global memory
    // and recomputes the rest per triplet
    constexpr int CAP = (sizeof(R) == 4 && G > 4) ? 16 : 8;
    constexpr int CAPP = CAP + 1;  // padded stride: the groups of a warp hit different banks
    __shared__ V4 sgeo[AP * CAPP];
    __shared__ V4 sunit[AP * CAPP];
    __shared__ V2 scut[AP * CAPP];
    __shared__ V4 sbacc[AP * CAPP];
    __shared__ int styp[AP * CAPP];
    __shared__ TripT<R> strip[64];
    __shared__ PairT<R> sterm[32];
    __shared__ int2 sindex[64];
    __shared__ R wpart[128 / 32][7];
    __shared__ unsigned done;
    // small interaction tables in shared memory
    const PairT<R>* terms = (const PairT<R>*)A.terms;
    const int2* index = A.index;
    const int T2 = A.T * A.T, T3 = T2 * A.T;
    const TripT<R>* trip = (const TripT<R>*)A.trip;
    if (T3 <= 64) {
        for (int q = threadIdx.x; q < T3; q += blockDim.x) strip[q] = trip[q];
        trip = strip;
    }
    if (A.n_terms <= 32 && T2 <= 64) {
        for (int q = threadIdx.x; q < A.n_terms; q += blockDim.x) sterm[q] = terms[q];
        for (int q = threadIdx.x; q < T2; q += blockDim.x) sindex[q] = index[q];
        terms = sterm;
        index = sindex;
    }
    if (threadIdx.x == 0) done = 0u;
    pdl_trigger();
    __syncthreads();
    const int lane = threadIdx.x % G;
    const int slot = threadIdx.x / G;
    const int gslot = A.order ? dealt_slot<G>(blk, nblk) : blk * AP + slot;
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
    const bool staged = ni <= CAP;
    auto SPV = [&](int k) -> R {
        if constexpr (sizeof(R) == 4) return A.spf[k];
        else return A.spd[k];
    };
    V4* geo = staged ? sgeo + slot * CAPP : (V4*)A.geo + s;
    const int* typ = staged ? styp + slot * CAPP : A.etype + s;
    V4* unit = sunit + slot * CAPP;  // staged atoms: unit vector, 1/r
    V2* cut = scut + slot * CAPP;    // staged atoms with uniform cutoffs: f(r), f'(r)
    const bool cached_cut = staged && (SPEC || A.bcut_uniform);
    const int ti = (act && !SPEC) ? A.type[i] : 0;
    TripT<R> TS{};
    if constexpr (SPEC)
        TS = TripT<R>{SPV(SP_A), SPV(SP_C2), SPV(SP_D2), SPV(SP_H), SPV(SP_MU), SPV(SP_RC), SPV(SP_RS), SPV(SP_C2D2), 1};
    // triplet parameters of (i, j, k) and the partner type of entry k
    auto trip_of = [&](int tj, int tk) -> const TripT<R>& {
        if constexpr (SPEC) return TS;
        else return trip[(ti * A.T + tj) * A.T + tk];
    };
    auto type_of = [&](int k) -> int {
        if constexpr (SPEC) return 0;
        else return typ[k];
    };
    V4* fj = (V4*)A.fj;
    // the lane's first bond: partner index and build-time bond vector are not
    // written by the kernel before, so they are fetched ahead of the wait
    int j_pre = 0;
    F4 s0_pre{};
    if constexpr (sizeof(R) == 4) {
        if (act && lane < ni) {
            j_pre = A.idx[s + lane];
            s0_pre = A.sep0[s + lane];
        }
    }
    // the displacements (mixed path) and the totals come from the kernel before
    pdl_wait();
    if (A.skip && *A.skip) return;  // uniform over the block
    // geometry of i's bonds in the working precision, and per bond what every
    // triplet through it reuses
    if (act) {
        double xi = 0, yi = 0, zi = 0;
        if constexpr (sizeof(R) == 8) {
            xi = A.pos[3 * i];
            yi = A.pos[3 * i + 1];
            zi = A.pos[3 * i + 2];
        }
        for (int e = lane; e < ni; e += G) {
            V4 g;
            if constexpr (sizeof(R) == 4) {
                if (e == lane) {
                    const F4 dj = A.disp[j_pre], di = A.disp[i];
                    const float x = s0_pre.x + (dj.x - di.x), y = s0_pre.y + (dj.y - di.y),
                                z = s0_pre.z + (dj.z - di.z);
                    g = F4{x, y, z, sqrtf(x * x + y * y + z * z)};
                } else {
                    g = bond_vector<R>(A, i, s + e, xi, yi, zi);
                }
            } else {
                g = bond_vector<R>(A, i, s + e, xi, yi, zi);
            }
            geo[e] = g;
            if (staged) {
                const R ir = g.w > R(0) ? rcp_(g.w) : R(0);
                unit[e] = V4{g.x * ir, g.y * ir, g.z * ir, ir};
                if constexpr (SPEC) {
                    R f, fp;
                    smooth<R>(g.w, SPV(SP_RC), SPV(SP_RS), f, fp);
                    cut[e] = V2{f, fp};
                } else {
                    const int te = A.etype[s + e];
                    styp[slot * CAPP + e] = te;
                    if (A.bcut_uniform) {
                        const V2 c = ((const V2*)A.bcut)[ti * A.T + te];
                        R f, fp;
                        smooth<R>(g.w, c.x, c.y, f, fp);
                        cut[e] = V2{f, fp};
                    }
                }
            }
        }
    }
    __syncwarp();
    // unit vector and inverse length of bond k
    auto unit_of = [&](int k, const V4& g, V3<R>& u, R& ir) {
        if (staged) {
            const V4 v = unit[k];
            u = V3<R>{v.x, v.y, v.z};
            ir = v.w;
        } else {
            ir = g.w > R(0) ? rcp_(g.w) : R(0);
            u = V3<R>{g.x * ir, g.y * ir, g.z * ir};
        }
    };
    R Fx = 0, Fy = 0, Fz = 0, En = 0;
    R W0 = 0, W1 = 0, W2 = 0, W3 = 0, W4 = 0, W5 = 0;
    // per bond e (owned by lane e % G): the force on its partner j so far, and
    // in .w the three-body prefactor 1/2 V f dB/dzeta
    V4* bacc = staged ? sbacc + slot * CAPP : (V4*)A.bscr + s;
    V4* kacc = (V4*)A.kacc + s;  // per bond k: the group's k parts, written once
    R maxbr = R(0);
    if constexpr (SPEC) maxbr = SPV(SP_RC);
    else if (act) maxbr = ((const R*)A.maxbr)[ti];
    if (act) {
        PostT<R> pp{};
        if constexpr (SPEC) pp = PostT<R>{SPV(SP_BETA), SPV(SP_ETA), 1};
        for (int e = lane; e < ni; e += G) {
            const V4 gij = geo[e];
            const V3<R> a{gij.x, gij.y, gij.z};
            const R r = gij.w;
            const int tj = type_of(e);
            V3<R> ua;
            R i1;
            unit_of(e, gij, ua, i1);
            int2 ix = make_int2(0, 0);
            bool any = false, bo = false;
            if constexpr (SPEC) {
                any = bo = r < SPV(SP_RC);
            } else {
                ix = index[ti * A.T + tj];
                for (int t = ix.x; t < ix.x + ix.y; ++t) {
                    const PairT<R>& P = terms[t];
                    if (P.in_bond_kernel && r < P.rc) {
                        any = true;
                        bo |= P.group >= 0;
                    }
                }
            }
            // zeta_ij (core_calculate_pair_bond_order_factor, first neighbour loop)
            R zeta = 0, B = 1, dB = 0;
            if ((bo || A.zeta_out) && r != R(0)) {
                for (int k = 0; k < ni; ++k) {
                    if (k == e) continue;
                    const V4 gik = geo[k];
                    if (!(gik.w < maxbr)) continue;
                    const TripT<R>& TT = trip_of(tj, type_of(k));
                    if (!TT.valid) continue;
                    R f, fp;
                    if (cached_cut) f = cut[k].x;
                    else smooth<R>(gik.w, TT.rc, TT.rs, f, fp);
                    if (f == R(0)) continue;
                    V3<R> ub;
                    R i2;
                    unit_of(k, gik, ub, i2);
                    zeta += tersoff_term_c<R>(TT, ua, r, ub, gik.w, f);
                }
            }
            if (A.zeta_out) A.zeta_out[s + e] = (double)zeta;
            if (!any || r == R(0)) {
                bacc[e] = V4{0, 0, 0, 0};
                if (A.b_out) ((R*)A.b_out)[s + e] = R(1);
                continue;
            }
            if (bo) {
                // post-processing of the centre type in the pair type's group
                if constexpr (!SPEC) pp = ((const PostT<R>*)A.post)[ti * A.T + tj];
                if (pp.valid) post_process<R>(pp.beta, pp.eta, zeta, B, dB);
                else {
                    B = zeta;
                    dB = 1;
                }
            }
            if (A.b_out) ((R*)A.b_out)[s + e] = B;
            R U = 0, dU = 0, P = 0;
            if constexpr (SPEC) {
                // exponential terms p0 exp(-p1 r) with the bond-order cutoff
                R f, fp;
                if (cached_cut) {
                    const V2 fc = cut[e];
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
            }
            // the cutoff factor of bond e, reused by pair terms with the same cutoff
            V2 bc{R(-1), R(-1)};
            if (!SPEC && cached_cut) bc = ((const V2*)A.bcut)[ti * A.T + tj];
            for (int t = ix.x; t < ix.x + ix.y; ++t) {
                const PairT<R>& PT = terms[t];
                if (!PT.in_bond_kernel || !(r < PT.rc)) continue;
                R V, dV;
                if (PT.kind >= 7 || PT.nmul > 0) {  // charge-dependent or product (bond-order scaled)
                    R en;
                    bond_charge_term<R>(A, PT, terms, i, s + e, ti, tj, r, V, dV, en);
                } else if (PT.smooth && PT.rc == bc.x && PT.rs == bc.y) {
                    pair_eval<R>(PT, r, V, dV, (const R*)A.tab);
                    const V2 fc = cut[e];
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
            En += R(0.5) * U;
            // radial part: force on j = -1/2 U' r_hat (on i the opposite, added
            // with everything else from the entry records below)
            const R c = R(0.5) * dU * i1;
            bacc[e] = V4{-c * a.x, -c * a.y, -c * a.z, bo ? R(0.5) * P * dB : R(0)};
        }
    }
    // Three-body part, F = -(1/2 V f dB/dzeta) grad zeta_ij, with the loop over
    // k outside: for each k the k parts of all bonds e of i are summed over the
    // group with shuffles, so the force on k from atom i leaves as one record.
    // The lanes of a warp run to the warp's longest list (empty turns for the
    // shorter ones) because the shuffles need every lane.
    const int nloop = (int)__reduce_max_sync(0xffffffffu, (unsigned)ni);
    // the lane's first bond stays in registers through the k loop (its
    // geometry, unit vector, type and the force on its partner so far)
    const bool own = act && lane < ni;
    V4 b0{}, g0{};
    V3<R> u0{};
    R i0 = 0;
    int t0 = 0;
    if (own) {
        b0 = bacc[lane];
        g0 = geo[lane];
        unit_of(lane, g0, u0, i0);
        t0 = type_of(lane);
    }
    for (int k = 0; k < nloop; ++k) {
        R kx = 0, ky = 0, kz = 0;
        if (k < ni) {
            const V4 gik = geo[k];
            if (gik.w < maxbr) {
                const int tk = type_of(k);
                V3<R> ub;
                R i2;
                unit_of(k, gik, ub, i2);
                V2 ck{R(0), R(0)};
                if (cached_cut) ck = cut[k];
                // one triplet term (bond e = gij, k): its j part onto be, its k part onto k
                auto term = [&](const V4& gij, const V3<R>& ua, R i1, int te, V4& be) {
                    const R pref = be.w;
                    if (pref == R(0)) return;
                    const TripT<R>& TT = trip_of(te, tk);
                    if (!TT.valid) return;
                    R f, fp;
                    if (cached_cut) {
                        f = ck.x;
                        fp = ck.y;
                    } else {
                        smooth<R>(gik.w, TT.rc, TT.rs, f, fp);
                    }
                    if (f == R(0) && fp == R(0)) return;
                    V3<R> gj, gk;
                    tersoff_grad_c<R>(TT, ua, gij.w, i1, ub, gik.w, i2, f, fp, gj, gk);
                    be.x -= pref * gj.x;
                    be.y -= pref * gj.y;
                    be.z -= pref * gj.z;
                    kx -= pref * gk.x;
                    ky -= pref * gk.y;
                    kz -= pref * gk.z;
                };
                if (own && lane != k) term(g0, u0, i0, t0, b0);
                for (int e = lane + G; e < ni; e += G) {
                    if (e == k) continue;
                    V4 be = bacc[e];
                    const V4 gij = geo[e];
                    V3<R> ua;
                    R i1;
                    unit_of(e, gij, ua, i1);
                    term(gij, ua, i1, type_of(e), be);
                    bacc[e] = be;
                }
            }
        }
        kx = group_sum<G>(kx);
        ky = group_sum<G>(ky);
        kz = group_sum<G>(kz);
        if (k < ni && lane == k % G) kacc[k] = V4{kx, ky, kz, 0};
    }
    if (own) bacc[lane] = b0;
    // per entry i->x: the force F_x of this atom's bonds on x (j part + k
    // parts), stored in x's own entry x->i (the reverse), so that the gather
    // pass reads each atom's records contiguously.  The force on i is minus
    // their sum and the virial the sum of r_ix (x) F_x (components xx, yy, zz,
    // yz, xz, xy), once per entry instead of once per triplet term.
    for (int e = lane; e < ni; e += G) {
        const V4 be = bacc[e], ke = kacc[e], g = geo[e];
        const R x = be.x + ke.x, y = be.y + ke.y, z = be.z + ke.z;
        fj[A.rev[s + e]] = V4{x, y, z, 0};
        Fx -= x;
        Fy -= y;
        Fz -= z;
        W0 += g.x * x;
        W1 += g.y * y;
        W2 += g.z * z;
        W3 += g.y * z;
        W4 += g.x * z;
        W5 += g.x * y;
    }
    const auto d0 = group_sum_f<G>(Fx), d1 = group_sum_f<G>(Fy), d2 = group_sum_f<G>(Fz);
    if (lane == 0) {
        if (act) {
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
    }
    // energy and virial: warp sums (empty slots hold zeros), exact from there on
    if (A.acc) {
        const R t[7] = {En, W0, W1, W2, W3, W4, W5};
        block_totals_add(t, wpart, &done, A.acc);
    }
}

template <typename R, int G>
__device__ __forceinline__ void gather_body(const BondArgs& A, int blk, int nblk) {
    using V4 = typename Vec4T<R>::T;
    const V4* fj = (const V4*)A.fj;
    const int lane = threadIdx.x % G;
    const int slot = threadIdx.x / G;
    // atoms in index order: every atom's records are short and contiguous, so
    // no load balancing by list length is needed here
    const int m = blk * (blockDim.x / G) + slot;
    const bool act = m < A.n;
    R Fx = 0, Fy = 0, Fz = 0;
    // the list bounds are not written by the bond pass: read before the wait
    const int s = act ? A.start[m] : 0, nm = act ? A.start[m + 1] - s : 0;
    pdl_wait();  // the bond pass's records
    if (A.skip && *A.skip) return;
    if (A.pub && blk == 0 && threadIdx.x < 8) {
        // every kernel that adds to the totals has completed (the bond pass
        // waited for the ones before it)
        if (threadIdx.x < 7) A.pub->totals[threadIdx.x] = fx_to_double(fx_from_limbs(A.acc[threadIdx.x]));
        else A.pub->bad = A.pub_bad ? *A.pub_bad : 0;
        __threadfence_system();
    }
    // the part on m as a centre, left by the bond pass (2^-32 fixed point in the
    // mixed path), fetched together with the records rather than after the sums
    using C = typename std::conditional<sizeof(R) == 4, long long, double>::type;
    C c0 = 0, c1 = 0, c2 = 0;
    if (act && lane == 0) {
        const C* fc = (const C*)A.fc + 3 * m;
        c0 = fc[0];
        c1 = fc[1];
        c2 = fc[2];
    }
    if (act) {
        // every neighbour x left the force of its bonds on m in m's entry m->x
        for (int e = lane; e < nm; e += G) {
            const V4 a = fj[s + e];
            Fx += a.x;
            Fy += a.y;
            Fz += a.z;
        }
    }
    auto sx = group_sum_f<G>(Fx), sy = group_sum_f<G>(Fy), sz = group_sum_f<G>(Fz);
    if (act && lane == 0) {
        if constexpr (sizeof(R) == 4) {
            sx.f += c0;
            sy.f += c1;
            sz.f += c2;
        } else {
            sx.s += c0;
            sy.s += c1;
            sz.s += c2;
        }
        store_sum(A.out_f + 3 * m, sx, A.first_f);
        store_sum(A.out_f + 3 * m + 1, sy, A.first_f);
        store_sum(A.out_f + 3 * m + 2, sz, A.first_f);
    }
}

}  // namespace pg
