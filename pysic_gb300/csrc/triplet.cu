// triplet.cu -- three-body potentials (bond_bend) in the reference's triplet
// enumeration.
//
// core_loop_over_local_interactions (Core.f90:3249-3943) finds triplets from
// the pairs it already visits: for every picked pair (atom1, atom2) within a
// many-body potential's cutoff that affects atom2 at target position 2, it
//   A  walks atom1's neighbours atom3 with pick(atom2, atom3): triplet
//      atom2 - atom1 - atom3, centre atom1;
//   B  walks atom2's neighbours atom3 with pick(atom1, atom3): triplet
//      atom1 - atom2 - atom3, centre atom2;
// and core_evaluate_local_triplet_B (6656-7028) applies each many-body record
// whose position-2 target is the triplet's second listed atom and whose
// position-3 target is atom3, within the cutoff for both bonds; the bond_bend
// evaluator (Potentials.f90:3206-3314) further requires the unpermuted tuple's
// middle element at the centre.  This kernel walks the same loops: one warp
// per atom1, lanes over atom1's list entries (atom2), each lane the two atom3
// loops of its pair.  Forces on the three atoms go to per-atom 2^-40 fixed-point
// accumulators by 64-bit integer atomics (order-independent, so results do
// not depend on scheduling).  A signed 64-bit word in these units holds
// magnitudes below 2^23 (8.4e6 eV/A) exactly; beside the three components
// every atom has a magnitude word, the sum of |Fx| + |Fy| + |Fz| of its terms
// in units of 2^-8 (rounded up), with its top bit set by any non-finite term
// or term of 2^30 eV/A or more.  While that sum stays below 2^23 eV/A no
// component can have wrapped; otherwise the atom's force reads back as NaN
// instead of a wrong value.  Energy and the reference's virial
// (sep1 (x) F_centre + (sep1 + sep2) (x) F_3, Core.f90:6980-6991) to the exact
// block totals.  The centre's smooth-cutoff gradient terms are those of
// 6860-6888.
//
// Four-body (dihedral) chains come from the same loops (Core.f90:3614-3940):
// every triplet x - c - y above is extended by a fourth atom among the
// neighbours of either end, giving the chains
//   A1 w - atom2 - atom1 - atom3   (w among atom2's neighbours),
//   A2 atom2 - atom1 - atom3 - w   (w among atom3's neighbours),
//   B1 w - atom1 - atom2 - atom3   (w among atom1's neighbours),
//   B2 atom1 - atom2 - atom3 - w   (w among atom3's neighbours),
// each pair of a chain picked once by its image offset, w never the triplet's
// far end.  core_evaluate_local_quadruplet_B (7450-7883) tests three of the
// chain's types as the record's target positions 2, 3, 4 (which three depends
// on the loop: the list positions as the reference passes them), every bond
// within the cutoff; the dihedral evaluator (Potentials.f90:3380-3611) then
// requires the unpermuted target tuple along the chain, forwards or
// backwards.  The quadruplet variant of the kernel is a separate
// instantiation, so bond_bend-only models keep the smaller kernel.
#include <algorithm>
#include <cmath>

#include "common.cuh"
#include "fixed.cuh"
#include "kernels.cuh"

namespace pg {

namespace {

constexpr int TT = 128;
constexpr double FIX40 = 1099511627776.0;  // 2^40

struct TriArgs {
    int n;
    const double* pos;
    const int* type;
    CellK C;
    const int* start;
    const int* idx;
    const int* off;
    const F4* sep0;   // mixed path: full-list bond vectors at the list build
    const F4* disp;   // mixed path: displacements since the build
    const void* rec;  // TriT<R>
    int nrec;
    const void* qrec;  // QuadT<R>
    int nqrec;
    long long* facc;  // n x 3 fixed-point forces
    FxAcc* acc;       // energy, virial totals (null: none)
    const int* skip;
};

// bond vector of list entry e of atom a (the separation a -> partner)
template <typename R>
__device__ __forceinline__ V3<R> entry_vector(const TriArgs& A, int a, int e);
template <>
__device__ __forceinline__ V3<double> entry_vector<double>(const TriArgs& A, int a, int e) {
    const int j = A.idx[e];
    const double o0 = A.off[3 * e], o1 = A.off[3 * e + 1], o2 = A.off[3 * e + 2];
    V3<double> s;
    s.x = A.pos[3 * j] - A.pos[3 * a] + (o0 * A.C.vc[0][0] + o1 * A.C.vc[0][1] + o2 * A.C.vc[0][2]);
    s.y = A.pos[3 * j + 1] - A.pos[3 * a + 1] + (o0 * A.C.vc[1][0] + o1 * A.C.vc[1][1] + o2 * A.C.vc[1][2]);
    s.z = A.pos[3 * j + 2] - A.pos[3 * a + 2] + (o0 * A.C.vc[2][0] + o1 * A.C.vc[2][1] + o2 * A.C.vc[2][2]);
    return s;
}
template <>
__device__ __forceinline__ V3<float> entry_vector<float>(const TriArgs& A, int a, int e) {
    const int j = A.idx[e];
    const F4 s0 = A.sep0[e], dj = A.disp[j], da = A.disp[a];
    return V3<float>{s0.x + (dj.x - da.x), s0.y + (dj.y - da.y), s0.z + (dj.z - da.z)};
}

// magnitude words (one per atom after the 3 n components): the top bit marks
// a term that cannot be accumulated; sums from 2^23 eV/A (2^31 units of 2^-8)
// on may have wrapped a component
constexpr unsigned long long MAG_BAD = 1ull << 63;
constexpr unsigned long long MAG_LIMIT = 1ull << 31;

__device__ __forceinline__ long long fix40(float v) { return __float2ll_rn(v * 1099511627776.0f); }
__device__ __forceinline__ long long fix40(double v) { return __double2ll_rn(v * FIX40); }

// facc: 3 n components, then n magnitude words
template <typename R>
__device__ __forceinline__ void add_force(long long* facc, int n, int a, const V3<R>& f) {
    const R m = fabs(f.x) + fabs(f.y) + fabs(f.z);
    unsigned long long* mag = (unsigned long long*)(facc + 3 * (size_t)n + a);
    if (!(m < R(1073741824))) {  // 2^30 eV/A, infinities and NaN: nothing is added
        atomicOr(mag, MAG_BAD);
        return;
    }
    atomicAdd(mag, (unsigned long long)ceil(m * R(256)));
    atomicAdd((unsigned long long*)(facc + 3 * a), (unsigned long long)fix40(f.x));
    atomicAdd((unsigned long long*)(facc + 3 * a + 1), (unsigned long long)fix40(f.y));
    atomicAdd((unsigned long long*)(facc + 3 * a + 2), (unsigned long long)fix40(f.z));
}

// One bond_bend term of the triplet x - c - y: s1 = x -> c, s2 = c -> y.
// Forces on x, c, y and the energy, smooth cutoffs included
// (evaluate_energy/force_bond_bending, Potentials.f90:3206-3314, and the
// cut-factor products of Core.f90:6860-6888).
template <typename R>
__device__ __forceinline__ void bend_term(const TriT<R>& T, const V3<R>& s1, R d1, const V3<R>& s2, R d2, V3<R>& fx,
                                          V3<R>& fc, V3<R>& fy, R& e) {
    const V3<R> t1{-s1.x, -s1.y, -s1.z};
    const R r3 = t1.x * s2.x + t1.y * s2.y + t1.z * s2.z;
    const R ratio = R(1) / (d1 * d2);
    const R cosplain = r3 * ratio;
    const R cospower = ipow(cosplain, T.n - 1);
    const R v = T.eps * ipow(ipow(r3 / (d1 * d2), T.n) - T.c0, T.m);
    const R r6 = T.eps * (R)(T.m * T.n) * ipow(cospower * cosplain - T.c0, T.m - 1) * cospower;
    const R a = r3 / (d1 * d1), b = r3 / (d2 * d2);
    const V3<R> t3{s2.x - a * t1.x, s2.y - a * t1.y, s2.z - a * t1.z};
    const V3<R> t4{t1.x - b * s2.x, t1.y - b * s2.y, t1.z - b * s2.z};
    const R k = ratio * r6;
    V3<R> px{-t3.x * k, -t3.y * k, -t3.z * k};
    V3<R> pc{(t3.x + t4.x) * k, (t3.y + t4.y) * k, (t3.z + t4.z) * k};
    V3<R> py{-t4.x * k, -t4.y * k, -t4.z * k};
    if (T.smooth) {
        R f1, g1, f2, g2;
        smooth<R>(d1, T.rc, T.rs, f1, g1);
        smooth<R>(d2, T.rc, T.rs, f2, g2);
        // cut_gradients = f'(d) * direction of the separation
        const V3<R> c1{g1 * s1.x / d1, g1 * s1.y / d1, g1 * s1.z / d1};
        const V3<R> c2{g2 * s2.x / d2, g2 * s2.y / d2, g2 * s2.z / d2};
        const R ff = f1 * f2;
        fx = V3<R>{px.x * ff + c1.x * f2 * v, px.y * ff + c1.y * f2 * v, px.z * ff + c1.z * f2 * v};
        fc = V3<R>{pc.x * ff + (-c1.x * f2 + c2.x * f1) * v, pc.y * ff + (-c1.y * f2 + c2.y * f1) * v,
                   pc.z * ff + (-c1.z * f2 + c2.z * f1) * v};
        fy = V3<R>{py.x * ff - c2.x * f1 * v, py.y * ff - c2.y * f1 * v, py.z * ff - c2.z * f1 * v};
        e = v * ff;
    } else {
        fx = px;
        fc = pc;
        fy = py;
        e = v;
    }
}

__device__ __forceinline__ bool bit(unsigned long long m, int t) { return (m >> t) & 1ull; }

template <typename R>
__device__ __forceinline__ R dot(const V3<R>& a, const V3<R>& b) {
    return a.x * b.x + a.y * b.y + a.z * b.z;
}

// One dihedral term of the chain 1-2-3-4 with separations v12, v23, v34
// (evaluate_energy_dihedral / evaluate_force_dihedral, Potentials.f90:
// 3380-3611): V = k/2 (cos phi - cos phi_0)^2, cos phi the cosine between the
// parts of v12 (reversed) and v34 perpendicular to v23; f[a] the force on
// chain atom a, without the cut factors.  With p1, p2 those parts and
// c = p1.p2 / (|p1| |p2|), F_a = k (c - cos phi_0) / (|p1| |p2|)
// (D_a + c |p2| / |p1| Q1_a + c |p1| / |p2| Q2_a), where D_a, Q1_a, Q2_a are
// minus the gradients of p1.p2, |p1|^2 / 2, |p2|^2 / 2 with respect to atom a.
template <typename R>
__device__ __forceinline__ void dihedral_term(const QuadT<R>& Q, const V3<R>& v12, const V3<R>& v23,
                                              const V3<R>& v34, R& e, V3<R> f[4]) {
    const R ir = R(1) / dot(v23, v23);
    const R a12 = dot(v12, v23), a34 = dot(v34, v23);
    const R u = a12 * ir, w = a34 * ir;
    const V3<R> p1{-(v12.x - u * v23.x), -(v12.y - u * v23.y), -(v12.z - u * v23.z)};
    const V3<R> p2{v34.x - w * v23.x, v34.y - w * v23.y, v34.z - w * v23.z};
    const R pp = dot(p1, p2);
    const R i1 = R(1) / sqrt_(dot(p1, p1)), i2 = R(1) / sqrt_(dot(p2, p2));
    const R ratio = i1 * i2;
    const R off = pp * ratio - Q.cos0;
    e = R(0.5) * Q.k * off * off;
    const R pre = Q.k * off * ratio;
    const R g1 = pp * i1 * i1, g2 = pp * i2 * i2;  // weights of Q1_a, Q2_a
    const R uw2 = R(2) * u * w, uu = u * u, ww = w * w;
    // atom 1: D = -p2, Q1 = p1, Q2 = 0; atom 4: D = -p1, Q1 = 0, Q2 = p2
    f[0] = V3<R>{pre * (-p2.x + g1 * p1.x), pre * (-p2.y + g1 * p1.y), pre * (-p2.z + g1 * p1.z)};
    f[3] = V3<R>{pre * (-p1.x + g2 * p2.x), pre * (-p1.y + g2 * p2.y), pre * (-p1.z + g2 * p2.z)};
    // atoms 2 and 3 (the centre bond)
    auto mid = [&](R a, R b, R c, R& r2, R& r3) {  // components of v12, v23, v34
        const R d2 = c - w * (b - a) + u * c - uw2 * b;
        const R q22 = w * c - ww * b;
        const R q12 = a - u * (b - a) - uu * b;
        r2 = pre * (d2 + q12 * g1 + q22 * g2);
        const R d3 = -(a + w * a + u * (c - b) - uw2 * b);
        const R q23 = -c + w * (b - c) + ww * b;
        const R q13 = -u * a + uu * b;
        r3 = pre * (d3 + q13 * g1 + q23 * g2);
    };
    mid(v12.x, v23.x, v34.x, f[1].x, f[2].x);
    mid(v12.y, v23.y, v34.y, f[1].y, f[2].y);
    mid(v12.z, v23.z, v34.z, f[1].z, f[2].z);
}

template <typename R, bool QUAD>
__global__ void __launch_bounds__(TT) tri_kernel(const __grid_constant__ TriArgs A) {
    __shared__ Fx128 wsum[TT / 32][7];
    __shared__ unsigned done;
    if (threadIdx.x == 0) done = 0u;
    __syncthreads();
    if (A.skip && *A.skip) return;  // uniform over the grid
    const TriT<R>* recs = (const TriT<R>*)A.rec;
    const int lane = threadIdx.x & 31;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // atom1
    R En = 0, W0 = 0, W1 = 0, W2 = 0, W3 = 0, W4 = 0, W5 = 0;
    auto account = [&](const TriT<R>& T, int x, int c, int y, const V3<R>& s1, R d1, const V3<R>& s2, R d2) {
        V3<R> fx, fc, fy;
        R e;
        bend_term<R>(T, s1, d1, s2, d2, fx, fc, fy, e);
        En += e;
        add_force(A.facc, A.n, x, fx);
        add_force(A.facc, A.n, c, fc);
        add_force(A.facc, A.n, y, fy);
        const V3<R> s12{s1.x + s2.x, s1.y + s2.y, s1.z + s2.z};
        W0 += s1.x * fc.x + s12.x * fy.x;
        W1 += s1.y * fc.y + s12.y * fy.y;
        W2 += s1.z * fc.z + s12.z * fy.z;
        W3 += s1.y * fc.z + s12.y * fy.z;
        W4 += s1.x * fc.z + s12.x * fy.z;
        W5 += s1.x * fc.y + s12.x * fy.y;
    };
    const QuadT<R>* qrecs = (const QuadT<R>*)A.qrec;
    // the chain x[0..3] with separations s1, s2, s3: the records of qm whose
    // target positions 2, 3, 4 hold the types of chain positions tp0, tp1, tp2
    auto chain = [&](unsigned long long qm, const int x[4], int tp0, int tp1, int tp2, const V3<R>& s1, R d1,
                     const V3<R>& s2, R d2, const V3<R>& s3, R d3) {
        if (d1 == R(0) || d2 == R(0) || d3 == R(0)) return;
        const int t[4] = {A.type[x[0]], A.type[x[1]], A.type[x[2]], A.type[x[3]]};
        for (unsigned long long q = qm; q; q &= q - 1) {
            const QuadT<R>& Q = qrecs[__ffsll((long long)q) - 1];
            if (!(bit(Q.m2, t[tp0]) && bit(Q.m3, t[tp1]) && bit(Q.m4, t[tp2]) && Q.rc > d1 && Q.rc > d2 &&
                  Q.rc > d3))
                continue;
            const bool fwd = bit(Q.orig[0], t[0]) && bit(Q.orig[1], t[1]) && bit(Q.orig[2], t[2]) &&
                             bit(Q.orig[3], t[3]);
            const bool bwd = bit(Q.orig[0], t[3]) && bit(Q.orig[1], t[2]) && bit(Q.orig[2], t[1]) &&
                             bit(Q.orig[3], t[0]);
            if (!fwd && !bwd) continue;
            R e;
            V3<R> f[4];
            dihedral_term<R>(Q, s1, s2, s3, e, f);
            if (Q.smooth) {  // cut factors of the three bonds and their gradients (Core.f90:7587-7725)
                R c1, g1, c2, g2, c3, g3;
                smooth<R>(d1, Q.rc, Q.rs, c1, g1);
                smooth<R>(d2, Q.rc, Q.rs, c2, g2);
                smooth<R>(d3, Q.rc, Q.rs, c3, g3);
                const R c123 = c1 * c2 * c3;
                const R h1 = g1 / d1 * c2 * c3 * e, h2 = g2 / d2 * c1 * c3 * e, h3 = g3 / d3 * c1 * c2 * e;
                f[0] = V3<R>{f[0].x * c123 + h1 * s1.x, f[0].y * c123 + h1 * s1.y, f[0].z * c123 + h1 * s1.z};
                f[1] = V3<R>{f[1].x * c123 - h1 * s1.x + h2 * s2.x, f[1].y * c123 - h1 * s1.y + h2 * s2.y,
                             f[1].z * c123 - h1 * s1.z + h2 * s2.z};
                f[2] = V3<R>{f[2].x * c123 - h2 * s2.x + h3 * s3.x, f[2].y * c123 - h2 * s2.y + h3 * s3.y,
                             f[2].z * c123 - h2 * s2.z + h3 * s3.z};
                f[3] = V3<R>{f[3].x * c123 - h3 * s3.x, f[3].y * c123 - h3 * s3.y, f[3].z * c123 - h3 * s3.z};
                e *= c123;
            }
            En += e;
            for (int a = 0; a < 4; ++a) add_force(A.facc, A.n, x[a], f[a]);
            // virial s1 (x) F2 + (s1 + s2) (x) F3 + (s1 + s2 + s3) (x) F4
            const V3<R> u2{s1.x + s2.x, s1.y + s2.y, s1.z + s2.z};
            const V3<R> u3{u2.x + s3.x, u2.y + s3.y, u2.z + s3.z};
            W0 += s1.x * f[1].x + u2.x * f[2].x + u3.x * f[3].x;
            W1 += s1.y * f[1].y + u2.y * f[2].y + u3.y * f[3].y;
            W2 += s1.z * f[1].z + u2.z * f[2].z + u3.z * f[3].z;
            W3 += s1.y * f[1].z + u2.y * f[2].z + u3.y * f[3].z;
            W4 += s1.x * f[1].z + u2.x * f[2].z + u3.x * f[3].z;
            W5 += s1.x * f[1].y + u2.x * f[2].y + u3.x * f[3].y;
        }
    };
    auto norm = [](const V3<R>& v) { return sqrt_(v.x * v.x + v.y * v.y + v.z * v.z); };
    if (i < A.n) {
        const int ti = A.type[i];
        const int b1 = A.start[i], e1 = A.start[i + 1];
        for (int e = b1 + lane; e < e1; e += 32) {
            const int j = A.idx[e];
            const int o0 = A.off[3 * e], o1 = A.off[3 * e + 1], o2 = A.off[3 * e + 2];
            if (!pick(i, j, o0, o1, o2)) continue;
            const V3<R> s12 = entry_vector<R>(A, i, e);
            const R d12 = sqrt_(s12.x * s12.x + s12.y * s12.y + s12.z * s12.z);
            if (d12 == R(0)) continue;
            const int tj = A.type[j];
            // the many-body records of this pair (core_evaluate_local_doublet_*_B)
            unsigned long long rm = 0;
            for (int r = 0; r < A.nrec; ++r)
                if (recs[r].rc > d12 && bit(recs[r].many, ti) && bit(recs[r].m2, tj)) rm |= 1ull << r;
            unsigned long long qm = 0;
            if (QUAD)
                for (int r = 0; r < A.nqrec; ++r)
                    if (qrecs[r].rc > d12 && bit(qrecs[r].many, ti) && bit(qrecs[r].m2, tj)) qm |= 1ull << r;
            if (!rm && !qm) continue;
            const V3<R> s21{-s12.x, -s12.y, -s12.z};
            // A: atom2 - atom1 - atom3 over atom1's neighbours
            for (int l = b1; l < e1; ++l) {
                const int k = A.idx[l];
                const int p0 = A.off[3 * l] - o0, p1 = A.off[3 * l + 1] - o1, p2 = A.off[3 * l + 2] - o2;
                if (!pick(j, k, p0, p1, p2)) continue;
                const V3<R> s13 = entry_vector<R>(A, i, l);
                const R d13 = sqrt_(s13.x * s13.x + s13.y * s13.y + s13.z * s13.z);
                if (d13 == R(0)) continue;
                const int tk = A.type[k];
                for (unsigned long long q = rm; q; q &= q - 1) {
                    const TriT<R>& T = recs[__ffsll((long long)q) - 1];
                    if (bit(T.m3, tk) && bit(T.center, ti) && T.rc > d13) account(T, j, i, k, s21, d12, s13, d13);
                }
                if (!QUAD || !qm) continue;
                // A1: w - atom2 - atom1 - atom3, w among atom2's neighbours
                for (int q = A.start[j]; q < A.start[j + 1]; ++q) {
                    const int w = A.idx[q];
                    if (w == i || !pick(k, w, A.off[3 * q] - p0, A.off[3 * q + 1] - p1, A.off[3 * q + 2] - p2)) continue;
                    const V3<R> v = entry_vector<R>(A, j, q);
                    const V3<R> s42{-v.x, -v.y, -v.z};
                    const int x[4] = {w, j, i, k};
                    chain(qm, x, 0, 1, 3, s42, norm(s42), s21, d12, s13, d13);
                }
                // A2: atom2 - atom1 - atom3 - w, w among atom3's neighbours
                for (int q = A.start[k]; q < A.start[k + 1]; ++q) {
                    const int w = A.idx[q];
                    if (w == i || !pick(j, w, A.off[3 * q] + p0, A.off[3 * q + 1] + p1, A.off[3 * q + 2] + p2)) continue;
                    const V3<R> s34 = entry_vector<R>(A, k, q);
                    const int x[4] = {j, i, k, w};
                    chain(qm, x, 0, 2, 3, s21, d12, s13, d13, s34, norm(s34));
                }
            }
            // B: atom1 - atom2 - atom3 over atom2's neighbours
            const int b2 = A.start[j], e2 = A.start[j + 1];
            for (int l = b2; l < e2; ++l) {
                const int k = A.idx[l];
                const int p0 = A.off[3 * l] + o0, p1 = A.off[3 * l + 1] + o1, p2 = A.off[3 * l + 2] + o2;
                if (!pick(i, k, p0, p1, p2)) continue;
                const V3<R> s23 = entry_vector<R>(A, j, l);
                const R d23 = sqrt_(s23.x * s23.x + s23.y * s23.y + s23.z * s23.z);
                if (d23 == R(0)) continue;
                const int tk = A.type[k];
                for (unsigned long long q = rm; q; q &= q - 1) {
                    const TriT<R>& T = recs[__ffsll((long long)q) - 1];
                    if (bit(T.m3, tk) && bit(T.center, tj) && T.rc > d23) account(T, i, j, k, s12, d12, s23, d23);
                }
                if (!QUAD || !qm) continue;
                // B1: w - atom1 - atom2 - atom3, w among atom1's neighbours
                for (int q = b1; q < e1; ++q) {
                    const int w = A.idx[q];
                    if (w == j || !pick(k, w, A.off[3 * q] - p0, A.off[3 * q + 1] - p1, A.off[3 * q + 2] - p2)) continue;
                    const V3<R> v = entry_vector<R>(A, i, q);
                    const V3<R> s41{-v.x, -v.y, -v.z};
                    const int x[4] = {w, i, j, k};
                    chain(qm, x, 0, 2, 3, s41, norm(s41), s12, d12, s23, d23);
                }
                // B2: atom1 - atom2 - atom3 - w, w among atom3's neighbours
                for (int q = A.start[k]; q < A.start[k + 1]; ++q) {
                    const int w = A.idx[q];
                    if (w == j || !pick(i, w, A.off[3 * q] + p0, A.off[3 * q + 1] + p1, A.off[3 * q + 2] + p2)) continue;
                    const V3<R> s34 = entry_vector<R>(A, k, q);
                    const int x[4] = {i, j, k, w};
                    chain(qm, x, 1, 2, 3, s12, d12, s23, d23, s34, norm(s34));
                }
            }
        }
    }
    if (A.acc) {
        const Fx128 v[7] = {warp_total(En), warp_total(W0), warp_total(W1), warp_total(W2),
                            warp_total(W3), warp_total(W4), warp_total(W5)};
        block_totals_publish(v, wsum, &done, A.acc);
    }
}

// the accumulated forces into out_f (written or added), accumulators back to zero
__global__ void tri_forces(int n, long long* __restrict__ facc, double* __restrict__ out_f, int first,
                           const int* skip) {
    if (skip && *skip) return;
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= 3 * n) return;
    const unsigned long long mag = (unsigned long long)facc[3 * (size_t)n + q / 3];
    const double v = mag >= MAG_LIMIT ? fx_nan() : (double)facc[q] * (1.0 / FIX40);
    facc[q] = 0;
    out_f[q] = first ? v : out_f[q] + v;
}

// the magnitude words back to zero (after tri_forces has read them)
__global__ void tri_clear_mag(int n, long long* __restrict__ facc, const int* skip) {
    if (skip && *skip) return;
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a < n) facc[3 * (size_t)n + a] = 0;
}

}  // namespace

void launch_triplets(pg_context* ctx, int precision, int flags, bool first_f, FxAcc* acc, const int* skip) {
    const int n = ctx->n;
    if (n == 0 || ctx->n_tri + ctx->n_quad == 0) return;
    cudaStream_t st = ctx->stream;
    if (ctx->tri_facc.n != 4 * (size_t)n) {  // 3 n components, n magnitude words; zero between calls
        ctx->tri_facc.resize(4 * (size_t)n);
        PG_CUDA(cudaMemsetAsync(ctx->tri_facc.p, 0, sizeof(long long) * 4 * (size_t)n, st));
    }
    TriArgs A{};
    A.n = n;
    A.pos = ctx->pos.p;
    A.type = ctx->type.p;
    A.C = cell_kernel_view(ctx->cell);
    A.start = ctx->nb_start.p;
    A.idx = ctx->nb_idx.p;
    A.off = ctx->nb_off.p;
    A.sep0 = ctx->nb_sep0.p;
    A.disp = ctx->disp32.p;
    A.nrec = ctx->n_tri;
    A.nqrec = ctx->n_quad;
    A.facc = ctx->tri_facc.p;
    A.acc = (flags & (PG_WANT_ENERGY | PG_WANT_FORCES)) ? acc : nullptr;
    A.skip = skip;
    const int blocks = (int)(((long long)n * 32 + TT - 1) / TT);
    const bool quad = ctx->n_quad > 0;
    if (precision == PG_PREC_FP64) {
        A.rec = ctx->d_tri.p;
        A.qrec = ctx->d_quad.p;
        if (quad) tri_kernel<double, true><<<blocks, TT, 0, st>>>(A);
        else tri_kernel<double, false><<<blocks, TT, 0, st>>>(A);
    } else {
        A.rec = ctx->d_tri32.p;
        A.qrec = ctx->d_quad32.p;
        if (quad) tri_kernel<float, true><<<blocks, TT, 0, st>>>(A);
        else tri_kernel<float, false><<<blocks, TT, 0, st>>>(A);
    }
    if (flags & PG_WANT_FORCES) {
        tri_forces<<<(3 * n + 255) / 256, 256, 0, st>>>(n, ctx->tri_facc.p, ctx->out_f.p, first_f ? 1 : 0, skip);
        tri_clear_mag<<<(n + 255) / 256, 256, 0, st>>>(n, ctx->tri_facc.p, skip);
    } else {  // energy only: the accumulated forces are dropped
        PG_CUDA(cudaMemsetAsync(ctx->tri_facc.p, 0, sizeof(long long) * 4 * (size_t)n, st));
    }
    PG_CHECK_LAUNCH();
    ctx->launches += (flags & PG_WANT_FORCES) ? 3 : 1;
}

}  // namespace pg
