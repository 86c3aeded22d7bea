// common.cuh -- shared types of the GB300 engine: device buffers, the engine
// context, interaction tables and error handling.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include <functional>
#include <utility>
#include <stdexcept>
#include <string>
#include <map>
#include <vector>

#include "../../include/pysic_gb300.h"
#include "fixed.cuh"

namespace pg {

struct Error : std::runtime_error {
    int status;
    Error(int s, const std::string& m) : std::runtime_error(m), status(s) {}
};

#define PG_CUDA(call)                                                                                  \
    do {                                                                                               \
        cudaError_t e_ = (call);                                                                       \
        if (e_ != cudaSuccess)                                                                         \
            throw ::pg::Error(PG_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_));         \
    } while (0)

#define PG_CHECK_LAUNCH() PG_CUDA(cudaGetLastError())

// the literal overload builds no std::string unless the check fails (some
// checks run once per atom)
inline void require(bool ok, int status, const char* msg) {
    if (!ok) throw Error(status, msg);
}
inline void require(bool ok, int status, const std::string& msg) {
    if (!ok) throw Error(status, msg);
}

// Bumped on every device (re)allocation: captured CUDA graphs hold raw
// pointers and are replayed only while this has not changed.
inline unsigned long long& alloc_epoch() {
    static unsigned long long e = 0;
    return e;
}

// FNV-1a over the values a captured launch sequence was built from.
struct SigHash {
    unsigned long long h = 1469598103934665603ull;
    template <typename T>
    SigHash& add(const T& v) {
        const unsigned char* p = (const unsigned char*)&v;
        for (size_t i = 0; i < sizeof(T); ++i) {
            h ^= p[i];
            h *= 1099511628211ull;
        }
        return *this;
    }
};

// A launch sequence kept as an instantiated CUDA graph (the list-build
// stages): replayed while the values it was built from (sig: buffer
// addresses through alloc_epoch, sizes, kernel arguments) are unchanged,
// otherwise captured anew and the executable graph updated in place.
struct SegGraph {
    cudaGraphExec_t exec = nullptr;
    unsigned long long sig = 0;
    SegGraph() = default;
    SegGraph(const SegGraph&) = delete;
    SegGraph& operator=(const SegGraph&) = delete;
    ~SegGraph() {
        if (exec) cudaGraphExecDestroy(exec);
    }
};

// Streaming multiprocessors of the current device (cudaDevAttrMultiProcessorCount),
// queried once per device; grids are sized in multiples of it.
inline int sm_count() {
    constexpr int MAXDEV = 64;
    static int cache[MAXDEV] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) dev = 0;
    if (dev >= MAXDEV) dev = MAXDEV - 1;
    int v = __atomic_load_n(&cache[dev], __ATOMIC_RELAXED);
    if (v == 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
        __atomic_store_n(&cache[dev], v, __ATOMIC_RELAXED);
    }
    return v;
}

// Grow-only device buffer.
template <typename T>
struct DevBuf {
    T* p = nullptr;
    size_t cap = 0;
    size_t n = 0;
    DevBuf() = default;
    DevBuf(const DevBuf&) = delete;
    DevBuf& operator=(const DevBuf&) = delete;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    void resize(size_t count) {
        if (count > cap) {
            if (p) cudaFree(p);
            p = nullptr;
            size_t c = count + count / 8 + 16;
            PG_CUDA(cudaMalloc(&p, c * sizeof(T)));
            cap = c;
            ++alloc_epoch();
        }
        n = count;
    }
    void upload(const T* h, size_t count, cudaStream_t s) {
        resize(count);
        if (count) PG_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void download(T* h, size_t count, cudaStream_t s) const {
        if (count) PG_CUDA(cudaMemcpyAsync(h, p, count * sizeof(T), cudaMemcpyDeviceToHost, s));
    }
    void zero(cudaStream_t s) {
        if (n) PG_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

// Page-locked host memory for small per-call results (totals, flags), so that
// their device-to-host copies are asynchronous and share one synchronisation.
template <typename T>
struct PinnedBuf {
    T* p = nullptr;
    size_t cap = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() {
        if (p) cudaFreeHost(p);
    }
    T* get(size_t count) {
        if (count > cap) {
            if (p) cudaFreeHost(p);
            p = nullptr;
            cap = 0;
            PG_CUDA(cudaMallocHost(&p, count * sizeof(T)));
            cap = count;
        }
        return p;
    }
};

// Host-side copy of the cell in the reference's layout (Geometry.f90:50-145).
struct Cell {
    double vc[3][3];  // cell%vectors(r,c): component r of cell vector c
    double ic[3][3];  // cell%inverse_cell(r,c)
    double rc[3][3];  // reciprocal_cell(r,c) = 2 pi inverse(c,r)
    double volume;
    int pbc[3];
};

// Kernel-side view of the cell (passed by value).
struct CellK {
    double vc[3][3];
    double ic[3][3];
    int pbc[3];
};

// One pair term folded per type pair (an interaction record whose two target
// masks contain the pair of types).  Every table exists in FP64 and in FP32 so
// that the mixed-precision kernels never convert parameters per term.
template <typename R>
struct PairT {
    int kind;            // 0 LJ, 1 exponential, 2 Buckingham, 3 spring, 4 power, 5 shift_power, 6 tabulated,
                         // 7 charge_pair
    int group;           // -1: plain, else bond-order group
    int smooth;          // smoothing active (create_potential, Potentials.f90:2382-2388)
    int in_bond_kernel;  // evaluated by the bond-order kernels (short list) rather than the pair kernel
    R p0, p1, p2, p3, rc, rs;
    int t0, tn;          // tabulated: first row and row count in the context's table rows
    unsigned long long first;  // charge_pair: types of the unpermuted first target (original_elements(1))
    int agroup;          // -1, or the per-atom bond-order group whose factors scale the term
    int ni;              // power / shift_power: the exponent when it is an integer, else PG_NOT_INT
    int mul0, nmul;      // a product of potentials: its nmul other factors are the records mul0 .. (never
                         // evaluated on their own; kept after every type pair's records)
};

// marks a non-integer exponent (general pow instead of repeated squaring)
constexpr int PG_NOT_INT = -1000000;

// the exponent as an int when it is integral and small, else PG_NOT_INT
inline int integral_exponent(double x) {
    return (x == (double)(long long)x && x >= -64.0 && x <= 64.0) ? (int)x : PG_NOT_INT;
}

// Per-atom (level-1) bond-order factors: at most this many groups (Coordinators
// of per-atom factors) per calculator.
constexpr int PG_MAX_AGROUPS = 4;

// Two-target per-atom factor record of an oriented type pair (atom1 type,
// atom2 type): kind 0 neighbors f(r), 1 power_bond f(r) (a/r)^n
// (Potentials.f90:5631-5645, 6293-6306).
template <typename R>
struct AfT {
    int kind, group;  // kind 0 neighbors, 1 power_bond, 4 table_bond; group: level-1 group index
    R rc, rs, a, n;   // power_bond: a, n; table_bond: range, scale
    int ni;     // n when it is an integer, else PG_NOT_INT
    int flags;  // force records: 1 the first atom's factor, 2 the second atom's, 3 both
    int t0, tn; // table_bond: first row and rows in the context's table rows
};

// Post-processing of a level-1 group's sum for one atom type: kind -1 none,
// 2 c_scale (epsilon, N, C, gamma, min), 3 sqrt_scale (epsilon)
// (Potentials.f90:6021-6063, 6402-6436).
template <typename R>
struct AfPostT {
    int kind;   // 5: table_scale, p[2] range, p[3] scale, rows t0 .. t0 + tn - 1
    R p[5];
    int t0, tn;
};

// Tersoff triplet parameters for (centre type, j type, k type) of group 0.
template <typename R>
struct TripT {
    R a, c2, d2, h, mu, rc, rs, c2d2;  // c2d2 = c^2 / d^2
    int valid;
};

// Post-processing (B(zeta)) parameters per centre type for group 0.
template <typename R>
struct PostT {
    R beta, eta;
    int valid;
};

// Three-body record (bond_bend: V = eps (cos^n theta - cos^n theta_0)^m,
// Potentials.f90:3206-3314) with the target masks of the reference's
// permuted record: position 2 and 3 types, the types at any position, and the
// types that may sit in the middle (the unpermuted tuple's second element).
template <typename R>
struct TriT {
    R eps, c0, rc, rs;  // c0 = cos(theta_0)^n, the reference's derived parameter
    int n, m, smooth, kind;
    unsigned long long m2, m3, many, center;
};

// Four-body record (dihedral: V = k/2 (cos phi - cos phi_0)^2,
// Potentials.f90:3329-3611): the masks of the permuted record's target
// positions 2, 3, 4, the types at any position, and the unpermuted tuple's
// types (the evaluator's forward / backward match).
template <typename R>
struct QuadT {
    R k, cos0, rc, rs;
    int smooth, kind;
    unsigned long long m2, m3, m4, many;
    unsigned long long orig[4];
};

template <typename R, typename S>
inline PairT<R> cast_pair(const PairT<S>& a) {
    return PairT<R>{a.kind, a.group, a.smooth, a.in_bond_kernel, (R)a.p0, (R)a.p1, (R)a.p2, (R)a.p3, (R)a.rc, (R)a.rs,
                    a.t0, a.tn, a.first, a.agroup, a.ni, a.mul0, a.nmul};
}
template <typename R, typename S>
inline TripT<R> cast_trip(const TripT<S>& a) {
    return TripT<R>{(R)a.a, (R)a.c2, (R)a.d2, (R)a.h, (R)a.mu, (R)a.rc, (R)a.rs, (R)a.c2d2, a.valid};
}
template <typename R, typename S>
inline PostT<R> cast_post(const PostT<S>& a) {
    return PostT<R>{(R)a.beta, (R)a.eta, a.valid};
}

// Programmatic dependent launch: a kernel launched with launch_pdl may start
// while its predecessor in the stream finishes; it runs its prologue (reads of
// data that the predecessor does not write) and then calls pdl_wait(), which
// returns once the predecessor has completed and its writes are visible.  A
// kernel calls pdl_trigger() to let its own dependent start early.  Both are
// no-ops for kernels launched the ordinary way.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline void launch_pdl(void (*kernel)(KArgs...), dim3 grid, dim3 block, cudaStream_t st, Args&&... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    PG_CUDA(cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...));
}

// State of a coordinate update (pg_update_atom_coordinates): none
// outstanding; staged on the device, not yet checked; checked and committed by
// an evaluation whose verdict the host has not read yet.
constexpr int PG_UPD_NONE = 0, PG_UPD_STAGED = 1, PG_UPD_CHECKED = 2;

// Page-locked, device-mapped record that the last kernel of a pg_calculate
// sequence fills: the totals as doubles and the verdict of the coordinate
// update it committed, so that only the per-atom arrays travel by the copy
// engine.
struct HostTotals {
    double totals[8];  // energy, virial (xx, yy, zz, yz, xz, xy), spare
    int bad;           // the committed update held a non-finite value
    int pad;
};

// Parameters of the single-species Tersoff fast path, by index.
constexpr int PG_SPEC_MAX_TERMS = 3;
enum SpecIndex {
    SP_RC = 0,
    SP_RS,
    SP_BETA,
    SP_ETA,
    SP_A,
    SP_C2,
    SP_D2,
    SP_C2D2,
    SP_H,
    SP_MU,
    SP_TERMS,  // then p0, p1 of each exponential pair term
    SP_COUNT = SP_TERMS + 2 * PG_SPEC_MAX_TERMS
};

// single-atom terms: 0 charge_self (eps q^n: p[0] = eps, n = (int)p[1]),
// 1 constant (V = p[0]), 2 constant force (F = p[0..2], V = -F . r)
struct SingleTerm {
    int kind;
    int n;
    int agroup;  // -1, or the per-atom bond-order group whose factor scales the term
    double p[3];
};

// 16- and 32-byte aligned 4-vectors (bond geometry, per-bond forces)
struct alignas(16) F4 {
    float x, y, z, w;
};
struct alignas(32) D4 {
    double x, y, z, w;
};

}  // namespace pg

// ---- the engine context --------------------------------------------------
struct pg_context {
    int device = 0;
    cudaStream_t stream = nullptr;

    // system
    int n = 0;
    bool have_cell = false, have_atoms = false;
    pg::Cell cell{};
    double cell_rows[9]{}, inv_rows[9]{};
    pg::DevBuf<double> pos;     // n x 3
    pg::DevBuf<double> pos_in;  // coordinate updates land here first and are checked on the device
    pg::DevBuf<int> pos_bad;    // 1 element: nonzero when an update held a non-finite value
    pg::DevBuf<double> pos_prev;  // the coordinates before an update the displacement pass committed
    bool commit_in_disp = false;  // the outstanding update was committed by the displacement pass
    int upd_state = 0;          // pg::PG_UPD_*: an outstanding coordinate update
    pg::PinnedBuf<pg::FxAcc> h_acc; // energy / virial totals on their way to the host
    pg::PinnedBuf<int> h_flag;
    pg::PinnedBuf<pg::HostTotals> h_tot;  // filled by the results kernel of pg_calculate sequences
    pg::DevBuf<double> charge;  // n
    pg::DevBuf<int> type;       // n
    std::vector<int> h_type;

    // interaction records (host copies) and folded tables
    int n_types = 0;
    std::vector<int> pr_kind, pr_group;
    std::vector<double> pr_params, pr_cut, pr_soft;
    std::vector<uint64_t> pr_m1, pr_m2;
    std::vector<int> sr_kind;
    std::vector<double> sr_params;
    std::vector<uint64_t> sr_m;
    std::vector<double> br_params, br_cut, br_soft;
    std::vector<uint64_t> br_m1, br_m2, br_m3;
    std::vector<int> br_group;
    bool tables_dirty = true;
    bool have_bond_terms = false, have_pair_kernel_terms = false, have_singles = false;
    bool have_triplets = false;
    double bo_radius = 0.0;          // largest cutoff handled by the bond-order kernels
    pg::DevBuf<pg::PairT<double>> d_pair_terms;
    pg::DevBuf<pg::PairT<float>> d_pair_terms32;
    pg::DevBuf<int2> d_pair_index;     // per (ti, tj): offset, count into d_pair_terms
    std::vector<double> pr_table;      // tabulated potentials: rows (V, d) of every table, concatenated
    std::vector<uint64_t> pr_first;    // per pair record: types of its unpermuted first target
    std::vector<int> pr_nmul, pr_mul0; // per pair record: factors of a product (0: a plain record), first factor
    std::vector<int> pm_kind;          // product factors: kind, 4 parameters, types of the product's first target
    std::vector<double> pm_params;
    std::vector<uint64_t> pm_first;
    bool have_charge_pairs = false;    // a charge-dependent pair term (charge_pair)
    bool have_bond_charge_terms = false;  // a Tersoff-scaled charge-dependent or product term
    pg::DevBuf<double> bo_b;           // per short entry: B of the bond (R), for bond_chi
    pg::DevBuf<double> d_tab64;        // the rows on the device, FP64 and FP32
    pg::DevBuf<float> d_tab32;
    pg::DevBuf<pg::TripT<double>> d_trip;  // n_types^3
    pg::DevBuf<pg::TripT<float>> d_trip32;
    pg::DevBuf<pg::PostT<double>> d_post;  // n_types x n_types (centre, partner)
    pg::DevBuf<pg::PostT<float>> d_post32;
    std::vector<int> tr_kind;            // three-body records as set through the C ABI
    std::vector<double> tr_params, tr_cut, tr_soft;
    std::vector<uint64_t> tr_m1, tr_m2, tr_m3, tr_center;
    pg::DevBuf<pg::TriT<double>> d_tri;  // folded records, FP64 and FP32
    pg::DevBuf<pg::TriT<float>> d_tri32;
    int n_tri = 0;
    std::vector<int> qd_kind;            // four-body records as set through the C ABI
    std::vector<double> qd_params, qd_cut, qd_soft;
    std::vector<uint64_t> qd_mask, qd_orig;  // 4 per record
    pg::DevBuf<pg::QuadT<double>> d_quad;    // folded records, FP64 and FP32
    pg::DevBuf<pg::QuadT<float>> d_quad32;
    int n_quad = 0;
    pg::DevBuf<long long> tri_facc;      // per atom x 3: three-body forces in 2^-40 fixed point
    pg::DevBuf<double> d_maxbr;          // per type: max bond-order cutoff (max_bond_radius)
    pg::DevBuf<float> d_maxbr32;
    // per (centre type, k type): bond-order cutoff rc, rs of the triplets, valid
    // for every j type when bcut_uniform (then f(r_ik) is computed once per bond)
    pg::DevBuf<double2> d_bcut;
    pg::DevBuf<float2> d_bcut32;
    bool bcut_uniform = false;
    int n_pair_terms = 0;  // records in d_pair_terms
    // single-species Tersoff fast path (tables.cu): parameters by value
    bool spec_ok = false;
    double spec[pg::SP_COUNT] = {};
    int spec_nterm = 0, spec_bomask = 0;
    pg::DevBuf<pg::SingleTerm> d_single_terms;
    pg::DevBuf<int2> d_single_index;     // per type
    // per-atom (level-1) bond-order factors (atomfactor.cu)
    std::vector<int> af_kind, af_group;  // records as set through the C ABI
    std::vector<double> af_params, af_cut, af_soft;
    std::vector<uint64_t> af_m1, af_m2;
    std::vector<int> sr_group;           // per single record: coordinator group or -1
    int pair_lanes = 0;                  // lanes per atom of the full-list kernels (0: by list length)
    int n_agroups = 0;                   // level-1 groups in use
    bool af_fused = false;               // no scaled pair term: factor forces inside the pair kernel
    std::map<int, int> agroup_of;        // coordinator group -> level-1 group
    pg::DevBuf<pg::AfT<double>> d_af;    // folded per oriented type pair, FP64 and FP32
    pg::DevBuf<pg::AfT<float>> d_af32;
    pg::DevBuf<int2> d_af_index;         // per (atom1 type, atom2 type): offset, count into d_af
    pg::DevBuf<pg::AfT<double>> d_aff;   // force records per (type k, type j), own / partner flags
    pg::DevBuf<pg::AfT<float>> d_aff32;
    pg::DevBuf<int2> d_aff_index;
    pg::DevBuf<pg::AfPostT<double>> d_af_post;  // per (group, type)
    pg::DevBuf<pg::AfPostT<float>> d_af_post32;
    // per (group, atom), in the working precision: the factor B, dB/dsum and
    // W = (the atom's prefactor) dB/dsum
    pg::DevBuf<double> af_B, af_S, af_W;
    pg::DevBuf<double> af_grad;          // n x 3: factor gradients handed to the caller

    // Ewald
    bool ewald = false;
    double ew_rc = 0, ew_kc = 0, ew_sigma = 0, ew_eps = 0;
    int ew_kmax[3] = {0, 0, 0};
    pg::DevBuf<double> ew_scaler;
    bool ew_tables_dirty = true;
    int ew_nk = 0, ew_ncol = 0, ew_nseg = 0;
    pg::DevBuf<int4> ew_seg;       // per segment: n1, n2, n3 start, count (+ k index base in .w via separate array)
    pg::DevBuf<int> ew_seg_k0;     // first listed-k index of each segment
    pg::DevBuf<pg::F4> ew_kvec;    // per listed k: kx, ky, kz, weight * exp(-s^2 k^2/2)/k^2 (FP32)
    pg::DevBuf<pg::D4> ew_kvec64; // same in FP64
    pg::DevBuf<double2> ew_S;      // structure factor per listed k (FP64 accumulated)
    pg::DevBuf<float2> ew_Spart;   // per (atom chunk, k) partial sums
    pg::DevBuf<double2> ew_Spart64;
    pg::DevBuf<uint32_t> ew_frac;  // per atom: fixed-point fractional coordinates (4 words)
    pg::DevBuf<double> ew_qs, ew_qpart, ew_Ssum;
    pg::DevBuf<double> ew_spart_bytes, ew_fpart_bytes, ew_wS_bytes;  // raw storage, precision-dependent layout

    // neighbour lists: full list (CSR) and the short list of bond-order terms
    bool have_list = false;
    double list_min_cutoff = 0.0;   // smallest per-atom list radius (0: unknown)
    pg::DevBuf<float> mlp_desc;     // descriptors of the warm-start network
    pg::DevBuf<float> mlp_fold;     // per prediction: type -> element, input mean and scale
    pg::DevBuf<double> mlp_q;       // per prediction: charges before the total-charge shift, block sums
    double skin = 0.5;
    pg::DevBuf<int> nb_start, nb_idx, nb_off;  // nb_off: 3 per entry
    pg::DevBuf<int> nb_g0;                     // per atom: entries coming from lower-index atoms
    long long nb_total = 0;
    bool short_dirty = true;
    bool short_is_full = false;
    pg::DevBuf<int> sh_start, sh_idx, sh_off, sh_rev, sh_count;
    pg::DevBuf<int4> sh_slot;  // per lane-group slot: atom, first entry, count (sh_order applied)
    pg::DevBuf<int> sh_order;      // atoms in order of their short-list length (lane groups of equal work)
    pg::DevBuf<int> sh_type;       // per short entry: type of the partner atom
    // mixed path: bond vectors of both lists taken once per list generation in
    // FP64 (rounded to FP32) at the positions pos0; an evaluation adds the FP32
    // displacements pos - pos0 of the two atoms
    pg::DevBuf<pg::F4> sh_sep0, nb_sep0;
    pg::DevBuf<double> pos0;
    pg::DevBuf<pg::F4> disp32;
    unsigned long long list_epoch = 0, sep0_epoch = ~0ull;
    long long sh_total = 0;
    long long bo_stride = 0;  // entries per section of the bond-pass scratch (>= sh_total)

    // neighbour-build scratch
    pg::DevBuf<float4> nb_posf;     // positions rounded to FP32 for the stencil scan's screen
    // the multi-block prefix scans' tile records and ticket / done counters
    // (zero between scans: the last block of each scan clears them)
    pg::DevBuf<unsigned long long> scan_rec;
    pg::DevBuf<unsigned> scan_ctr;
    pg::DevBuf<int> cell_of, cell_start, sorted_atoms, wrap, keys_a, keys_b, vals_a, vals_b, radix_hist, count_tmp,
        invisible;
    pg::DevBuf<long long> g0_keys;
    pg::DevBuf<int4> g0_vals;
    pg::DevBuf<int> g0_start;
    pg::DevBuf<double> cutoffs;
    pg::DevBuf<int> scan_tmp;
    pg::DevBuf<int> nb_totals;     // build totals on the device: out-of-range atoms, entries, lower-index entries
    pg::PinnedBuf<int> h_totals;   // their host copy (one synchronisation per build)
    std::vector<double> h_cutoffs;  // cutoffs of the last engine build (rebuilds on the device coordinates)
    pg::SegGraph seg_g[6];          // captured stages of the list build (neighbor.cu)
    int list_kind = 0;              // PG_LIST_*: who built the lists

    // bond-order scratch
    pg::DevBuf<pg::F4> bo_fj;             // mixed precision: 4 records per short entry
    pg::DevBuf<pg::D4> bo_fj64;           // FP64: 4 records per short entry
    pg::DevBuf<double> bo_fc;             // centre-role forces per atom (3)
    pg::DevBuf<double> bo_zeta;           // per short entry (diagnostics)
    int lanes = 0;                        // 0: autotune
    int tuned_lanes[2] = {0, 0};

    // outputs
    pg::DevBuf<double> out_f;     // n x 3
    pg::DevBuf<double> out_chi;   // n
    pg::DevBuf<pg::FxAcc> out_acc;  // energy, virial[6], spare: exact fixed-point totals (fixed.cuh)

    // charge relaxation
    pg::DevBuf<double> rq_rate, rq_save, rq_stat;
    pg::DevBuf<int> rq_flag;
    pg::DevBuf<double> chi_k;   // relaxation loops: real-space Ewald kernel per full-list entry (R)
    pg::DevBuf<double> cg_buf;  // charge optimisation: q, r, p, H p, chi(0), partials, scalars
    pg::DevBuf<int> cg_flag;
    pg::DevBuf<double> md_p, md_m;  // dynamics: momenta (n x 3), masses
    pg::DevBuf<int> md_flag;
    bool md_ready = false, md_pending = false;  // state set; a step waits for its forces after a rebuild
    cudaGraphExec_t md_exec = nullptr;          // the captured step of the rebuilding loop
    unsigned long long md_sig = 0;              // what its kernel arguments were captured from

    int launches = 0;
    // device address of the no-allocation call's static scratch array in this
    // context's CUDA context (noalloc.cu), looked up on its first call
    void* noalloc_scratch = nullptr;

    // captured evaluation sequences (one per precision / flags / lanes)
    struct Graph {
        int precision, flags, lanes, launches;
        bool commit;  // begins with the check and commit of staged coordinates
        int pub;      // ends with the totals (2) and the update verdict (+1) written to h_tot
        unsigned long long state, alloc;
        cudaGraphExec_t exec;
    };
    std::vector<Graph> graphs;
    bool use_graphs = true;
    // optional CUDA events around the kernel groups: pair, bond pass, gather pass, k-space, reduce
    bool timing = false;
    cudaEvent_t tev[6] = {nullptr, nullptr, nullptr, nullptr, nullptr, nullptr};
    unsigned long long state_epoch = 1;  // bumped whenever kernel arguments change

    ~pg_context() {
        for (auto& g : graphs) cudaGraphExecDestroy(g.exec);
        if (md_exec) cudaGraphExecDestroy(md_exec);
        for (auto& e : tev)
            if (e) cudaEventDestroy(e);
    }
};

// The warm-start network (mlp.cu).
struct pg_mlp {
    int device = 0;
    int n_in = 0, n_h1 = 0, n_h2 = 0;
    long long n_params = 0;
    cudaStream_t stream = nullptr;
    pg::DevBuf<float> w, m, v, grad;   // FP32 master, Adam moments, gradient
    pg::DevBuf<__nv_bfloat16> wb;      // BF16 copy read by the forward pass
    pg::DevBuf<float> x, y;            // training samples
    long long n_samples = 0;
    pg::DevBuf<int> order;             // sample order of the current epoch
    pg::DevBuf<float> h1, h2, out, dz1, dz2, dy, lpart;  // per-batch activations
    pg::DevBuf<float> px, py;          // prediction scratch
    pg::DevBuf<float> gpart;           // tensor-core training: per-block partial gradients
    pg::DevBuf<double> dloss;          // summed squared error of an epoch, on the device
    long long step = 0;
    ~pg_mlp() {
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace pg {

// Fortran-style build of the cell arrays from the row-major cell and inverse.
void make_cell(const double* cell, const double* inv, const int32_t* pbc, Cell& C);
CellK cell_kernel_view(const Cell& C);

// neighbor.cu
void build_neighbor_lists(pg_context* ctx, const double* h_cutoffs);
// same_positions: pos0 holds the positions the cell-list build ran at (the
// list generation's reference positions were taken right after it)
void build_short_list(pg_context* ctx, bool same_positions = false);
void build_full_sep0(pg_context* ctx);
void launch_disp(pg_context* ctx, const int* skip, FxAcc* zero8 = nullptr, bool commit = false);
void build_allpairs_lists(pg_context* ctx, const double* h_cutoffs);
void install_neighbor_lists(pg_context* ctx, const int32_t* counts, const int32_t* idx, const int32_t* off);

// tables.cu
void fold_tables(pg_context* ctx);

// pair.cu, tersoff.cu, ewald.cu: energy and virial are added to the totals
// `acc` (null: not wanted); forces and electronegativities are written
// (first_*) or added to the per-atom outputs
int pair_kernel_blocks(int n, int G);
void launch_pair_kernel_impl(pg_context* ctx, int precision, int flags, bool first_f, bool first_chi, int G,
                             FxAcc* acc);
void launch_pair_kernel_skip(pg_context* ctx, int precision, int flags, bool first_f, bool first_chi, int G,
                             FxAcc* acc, const int* skip);

int bond_blocks(int n, int G);
void launch_bond_order_impl(pg_context* ctx, int precision, int flags, bool first_f, int G, FxAcc* acc,
                            const std::function<void()>& between, const int* skip = nullptr,
                            HostTotals* pub = nullptr, const int* pub_bad = nullptr);
void bond_zeta_diag(pg_context* ctx);
// noalloc.cu: the bond-order passes on static scratch (pg_bond_order_noalloc)
void bond_order_noalloc(pg_context* ctx, int precision, double* d_forces, double* d_totals);

// ewald.cu
void ewald_prepare(pg_context* ctx);
void launch_ewald_kspace(pg_context* ctx, int precision, int flags, bool first_f, bool first_chi, FxAcc* acc);
void launch_ewald_kspace_skip(pg_context* ctx, int precision, int flags, bool first_f, bool first_chi, FxAcc* acc,
                              const int* skip);

// mlp.cu: descriptors and the warm-start network (struct pg_mlp)
void descriptors(pg_context* ctx, int n_gauss, double r0, double r1, double width, double cutoff, float* out);
void mlp_create(pg_mlp** out, int n_in, int n_h1, int n_h2, int device);
void mlp_set_params(pg_mlp* M, const float* params, long long n);
void mlp_get_params(pg_mlp* M, float* params, long long n);
void mlp_add_samples(pg_mlp* M, const float* x, const float* y, long long n);
void mlp_clear_samples(pg_mlp* M);
void mlp_train(pg_mlp* M, int epochs, int batch, float lr, unsigned long long seed, float* epoch_loss);
void mlp_gradients(pg_mlp* M, const float* x, const float* y, long long n, float* grad, double* loss);
void mlp_predict(pg_mlp* M, const float* x, long long n, float* y);
// mlp_tc.cu: the tensor-core training step (two hidden layers of 64 units, <= 64 inputs)
bool mlp_tc_eligible(const pg_mlp* M);
void mlp_tc_batch_grad(pg_mlp* M, const float* x, const float* y, const int* rows, int nb, double* loss_dev);
void mlp_predict_charges(pg_mlp* M, pg_context* ctx, int n_gauss, double r0, double r1, double width, double cutoff,
                         int n_elements, const int* type_element, const float* x_mean, const float* x_scale,
                         double y_mean, double y_scale, double total_charge, double* charges);

// batch.cu: many systems per launch (struct pg_batch)
void batch_create(pg_batch** out, int device);
void batch_destroy(pg_batch* b);
void batch_add(pg_batch* b, pg_context* c);
void batch_set_lanes(pg_batch* b, int pair_lanes, int bond_lanes);
void batch_get_lanes(pg_batch* b, int precision, int* pair_lanes, int* bond_lanes);
void batch_set_tile_blocks(pg_batch* b, int blocks);
void batch_test_stall(pg_batch* b, int system, double wait_seconds);
void batch_get_tiles(pg_batch* b, int precision, int mode, int* pair_lanes, int* bond_lanes, int* blocks);
void batch_evaluate(pg_batch* b, int precision, int flags, int mode);
void batch_synchronize(pg_batch* b);
int batch_launches(const pg_batch* b);
cudaStream_t batch_stream(const pg_batch* b);

// relax.cu: mode PG_RELAX_DYNAMIC (damped, to a tolerance) or
// PG_RELAX_POTENTIOSTAT (undamped, fixed external potential, fixed step count)
constexpr int PG_RELAX_DYNAMIC = 0, PG_RELAX_POTENTIOSTAT = 1;
// md.cu: velocity Verlet on the device (pg_md_*)
void md_set_state(pg_context* ctx, const double* masses, const double* momenta);
void md_get_state(pg_context* ctx, double* momenta, double* positions);
void md_run(pg_context* ctx, int precision, int n_steps, double dt, double skin, int* steps_done, int* rebuild);
void md_run_rebuilding(pg_context* ctx, int precision, int n_steps, double dt, double skin, int* steps_done,
                       int* rebuilds);
void evaluate(pg_context* ctx, int precision, int flags);
// api.cu: lanes per atom of the pair kernel for this context's list lengths
int pair_lanes_for(const pg_context* ctx);
void launch_bond_b(pg_context* ctx, int precision, int G, const int* skip);
void launch_bond_chi(pg_context* ctx, int precision, bool first, const int* skip);
// pair.cu: the fixed real-space Ewald electronegativity matrix of a relaxation loop
bool chi_cache_prepare(pg_context* ctx, int precision);
void launch_chi_cache_apply(pg_context* ctx, int precision, const int* skip);
// atomfactor.cu: per-atom (level-1) bond-order factors; stage 0 computes the
// factors (before the pair kernel), stage 1 adds their forces and virial
void fold_atom_factors(pg_context* ctx, const std::map<int, int>& gmap);
void launch_atom_factors(pg_context* ctx, int precision, int stage, bool first_f, FxAcc* acc, const int* skip);
void atom_factor_gradients(pg_context* ctx, int precision, int group, int atom, int of_factor, double* out);
// triplet.cu: three-body potentials (bond_bend)
constexpr int PG_MAX_TRIPLET_RECORDS = 64;
constexpr int PG_MAX_QUAD_RECORDS = 64;
// origin of the neighbour lists
constexpr int PG_LIST_NONE = 0;
constexpr int PG_LIST_CELLS = 1;      // the engine's cell-list build
constexpr int PG_LIST_ALL_PAIRS = 2;  // the engine's all-pairs build
constexpr int PG_LIST_INSTALLED = 3;  // installed from the host
void launch_triplets(pg_context* ctx, int precision, int flags, bool first_f, FxAcc* acc, const int* skip);
// optimize.cu: the constrained energy minimum over the charges (quadratic energies)
void optimize_charges(pg_context* ctx, int precision, int max_iter, double tolerance, double* charges, int* iterations,
                      double* error);
void relax_charges(pg_context* ctx, int precision, int mode, int n_steps, double dt, double inertia, double friction,
                   double tolerance, double potential, double* rates, double* charges, int* steps, double* error,
                   double* max_dq);

// api.cu
void evaluate(pg_context* ctx, int precision, int flags);
void prepare(pg_context* ctx);  // fold tables, start a list generation, short list, Ewald tables
void settle_coordinates(pg_context* ctx);  // finish an outstanding coordinate update (may throw)

// peak.cu: FP32 rate of independent FMA chains on every SM (TFLOP/s, best launch ms)
void measure_fp32_peak(int device, double* tflops, double* ms);

// utilities
void exclusive_scan_int(const int* in, int* out, int n, cudaStream_t s, DevBuf<int>& tmp, int* total_host);

}  // namespace pg
