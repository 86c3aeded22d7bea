// args.cuh -- kernel argument records of the evaluation kernels, shared by
// the single-system launches (pair.cu, tersoff.cu) and the many-system launch
// (batch.cu), which uploads one record per system and walks a tile list.
#pragma once
#include "common.cuh"

namespace pg {

struct PairArgs {
    int n, T;
    const double* pos;
    const double* charge;
    const int* type;
    CellK C;
    const int* start;
    const int* idx;
    const int* off;
    const void* terms;  // PairT<R>
    const int2* index;
    const void* tab;    // tabulated potentials' rows (R)
    const SingleTerm* sterms;
    const int2* sindex;
    int ewald;
    int qpair;  // charge-dependent pair terms present: their electronegativities are wanted too
    double ew_rc, ew_is2, ew_k, ew_c2, ew_isq2;  // 1/(sqrt2 sigma), 1/(4 pi eps), 2/(sqrt(2 pi) sigma), 1/(2 sigma^2)
    int flags;
    int first_f, first_chi;
    double* out_f;
    double* out_chi;
    FxAcc* acc;       // global energy / virial totals (null: not wanted)
    const int* skip;  // optional device flag: nonzero = do nothing
    const F4* sep0;   // mixed path: bond vectors at list build
    const F4* disp;   // mixed path: displacements since the build (xyz) and FP32 charge (w)
    // per-atom (level-1) bond-order factors
    int ng;                // groups (0: none)
    const void* af;        // AfT<R>
    const int2* af_index;  // per (atom1 type, atom2 type)
    const void* af_post;   // AfPostT<R> per (group, type)
    const void* aff;       // AfT<R> force records
    const int2* aff_index; // per (type k, type j)
    void* afB;             // per (group, atom), R: factor
    void* afS;             // dB/dsum
    void* afW;             // prefactor times dB/dsum (written by the pair kernel, or by af_sum when fused)
    int af_fused;          // no scaled pair term: af_sum writes W, the pair kernel adds the factor forces
};

template <typename R>
struct Vec4T;
template <>
struct Vec4T<float> {
    using T = F4;
};
template <>
struct Vec4T<double> {
    using T = D4;
};

struct BondArgs {
    int n, T;
    const double* pos;
    const int* type;
    CellK C;
    const int* start;
    const int* idx;
    const int* off;
    const int* rev;
    const void* terms;  // PairT<R>
    const int2* index;
    const void* tab;    // tabulated potentials' rows (R)
    const void* trip;   // TripT<R>
    const void* post;   // PostT<R>
    const void* maxbr;  // R
    const void* bcut;   // per (ti, tk): rc, rs of bond ik (Vec2T<R>)
    int bcut_uniform;   // bcut holds for every tj
    const int* etype;   // per entry: partner type
    const int* order;   // lane-group slot -> atom (atoms grouped by list length)
    const int4* slot;   // per slot: atom, first short entry, entry count (one load instead of a chain)
    int n_terms;        // pair records in terms
    const F4* sep0;     // mixed path: bond vectors at list build
    const F4* disp;     // mixed path: per-atom displacement since the build
    float spf[SP_COUNT];  // single-species fast path parameters, FP32 copy
    double spd[SP_COUNT]; // and FP64
    int spec, spec_nterm, spec_bomask;
    int nblocks;          // blocks of this system in the bond and gather passes (many-system launch)
    int flags;
    int first_f;
    void* geo;         // per entry: bond geometry (atoms with more bonds than shared memory holds)
    void* fj;          // per entry m->x: the force of x's bonds on m, written by x through rev
    void* kacc;        // per entry i->k: the k parts of i's bonds on k
    void* bscr;        // per entry: running j parts of unstaged atoms' bonds
    void* fc;          // per atom: i part of the force (FP64, or 2^-32 fixed point in the mixed path)
    double* out_f;
    FxAcc* acc;        // global energy / virial totals (null: not wanted)
    double* zeta_out;
    const int* skip;   // optional device flag: nonzero = do nothing
    const double* q;   // FP64 charges (the mixed path reads the FP32 copy in disp .w)
    void* b_out;       // per entry: B of the bond (R; null: not kept), for the electronegativity pass
    // the gather pass as an evaluation's last kernel: its block 0 writes the
    // final totals and the verdict (pub_bad, may be null) of the coordinate
    // update into page-locked host memory (null: not this kernel's job)
    HostTotals* pub;
    const int* pub_bad;
};

struct DispArgs {
    int n;
    const double* pos;
    const double* pos0;
    const double* q;
    F4* d;             // null: only clear the totals
    const int* skip;
    FxAcc* zero8;
    // a staged coordinate update committed on the way (pos_in null: none): the
    // new coordinates from pos_in into pos_out, the old ones kept in pos_prev
    // until the verdict is read, bad set if any new value is not finite
    const double* pos_in;
    double* pos_out;
    double* pos_prev;
    int* bad;
};

// argument records of one system (pair.cu, tersoff.cu)
PairArgs make_pair_args(pg_context* ctx, int precision, int flags, bool first_f, bool first_chi, FxAcc* acc,
                        const int* skip);
BondArgs make_bond_args(pg_context* ctx, int precision, int flags, bool first_f, FxAcc* acc);
DispArgs make_disp_args(pg_context* ctx, F4* d, const int* skip, FxAcc* zero8);
void set_atom_factor_args(pg_context* ctx, int precision, PairArgs& A);  // atomfactor.cu
void prepare_bond_scratch(pg_context* ctx, int precision);
int pair_atoms_per_block(int n, int G);

// many-system launches: sys and tiles in device memory, tiles[t] = (system, block)
void launch_pair_batch(const PairArgs* sys, const int2* tiles, int ntiles, int grid, int threads, int precision, int G,
                       cudaStream_t st);
void launch_bond_batch(const BondArgs* sys, const int2* tiles, int ntiles, int grid, int precision, int G, bool spec,
                       bool forces, cudaStream_t st);
void launch_disp_batch(const DispArgs* sys, const int2* tiles, int ntiles, int grid, cudaStream_t st);

}  // namespace pg
