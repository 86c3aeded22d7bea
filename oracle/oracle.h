/*
 * oracle.h -- FP64 CPU restatement of the Pysic Fortran core (test infrastructure).
 *
 * This library is the parity oracle for the GB300 engine.  It is used only by
 * tests/, by __graft_entry__.smoke() and by bench.py's CPU baseline leg, always
 * as the checker and never as the thing measured or shipped.  Every routine
 * names the reference file:line it restates (paths relative to the Pysic
 * project root).
 *
 * Parity pins: the restatement is checked against the known-answer values in
 * doc/run examples.rst:106-145 and doc/pysic class.rst:88-157, against a
 * Tersoff (1988) silicon known answer, and against finite differences (the
 * reference's own check, pysic/calculator.py:1639-1832).  The reference core
 * itself is Fortran and cannot be compiled where these tests run, so the bit
 * pattern of the reference binary is not pinned directly.
 *
 * Conventions: 0-based atom indices, positions N x 3 C-order, cell rows are the
 * cell vectors (ASE layout), inv = numpy.linalg.inv(cell) (row-major).
 */
#ifndef PYSIC_ORACLE_H
#define PYSIC_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t n;
    const double* pos;      /* n x 3 */
    const double* charge;   /* n */
    const int32_t* type;    /* n, 0 .. n_types-1 */
    double cell[9];
    double inv[9];
    int32_t pbc[3];
} orc_system;

/* Interaction records in the order the reference core stores them
 * (pysic/calculator.py:1063-1447 permutes targets; Potentials.f90:2353-2472
 * builds each record). */
typedef struct {
    int32_t n_types;
    int32_t n_pair;
    const int32_t* pair_kind;     /* 0 LJ, 1 exponential, 2 Buckingham, 3 spring, 4 power, 5 shift_power,
                                     6 tabulated (params: first row, rows, range, scale),
                                     7 charge_pair (epsilon, n1, n2),
                                     8 charge_exp (first of 8 pair_table rows holding its 11 parameters
                                     and the derived eta1, eta2, beta1, beta2) */
    const double* pair_params;    /* 4 per record */
    const double* pair_cutoff;
    const double* pair_soft;      /* cutoff - cutoff_margin, as passed to add_potential */
    const uint64_t* pair_mask1;   /* type bitmask of target position 1 */
    const uint64_t* pair_mask2;   /* type bitmask of target position 2 */
    const int32_t* pair_group;    /* -1 = not scaled by a bond-order factor */
    int32_t n_single;
    const int32_t* single_kind;   /* 0 charge_self, 1 constant, 2 force */
    const double* single_params;  /* 4 per record: (epsilon, n) | (V) | (Fx, Fy, Fz) */
    const uint64_t* single_mask;
    int32_t n_bond;
    const double* bond_params;    /* 7 per record: beta, eta, a, c, d, h, mu */
    const double* bond_cutoff;
    const double* bond_soft;
    const uint64_t* bond_mask1;
    const uint64_t* bond_mask2;
    const uint64_t* bond_mask3;
    const int32_t* bond_group;
    int32_t ewald;
    double ewald_rc, ewald_kc, ewald_sigma, ewald_eps;
    int32_t ewald_kmax[3];
    const double* ewald_scaler;   /* n */
    const double* pair_table;     /* tabulated potentials: rows (V, d), concatenated */
    int64_t n_table_rows;
    int32_t n_tri;                /* three-body records (bond_bend), one per permutation */
    const int32_t* tri_kind;
    const double* tri_params;     /* 4 per record: epsilon, theta_0, n, m */
    const double* tri_cutoff;
    const double* tri_soft;
    const uint64_t* tri_mask1;
    const uint64_t* tri_mask2;
    const uint64_t* tri_mask3;
    const uint64_t* tri_center;   /* types that may be the middle atom */
    const uint64_t* pair_first;   /* per pair record: types of the unpermuted first target */
    /* per-atom (level-1) bond-order factors, one record per target tuple,
       unpermuted (calculator.py:1372-1430); they share the group numbering of
       pair_group / bond_group */
    int32_t n_afac;
    const int32_t* afac_kind;     /* 0 neighbors, 1 power_bond, 2 c_scale, 3 sqrt_scale, 4 table_bond,
                                     5 table_scale */
    const double* afac_params;    /* 5 per record: power_bond (a, n); c_scale (epsilon, N, C, gamma, min);
                                     sqrt_scale (epsilon); table_bond / table_scale (first row in
                                     pair_table, rows, range, scale) */
    const double* afac_cutoff;
    const double* afac_soft;
    const uint64_t* afac_mask1;
    const uint64_t* afac_mask2;   /* 0 for the one-target scalers */
    const int32_t* afac_group;
    const int32_t* single_group;  /* per single record: -1 or the group of its coordinator (null: all -1) */
    /* products of pair potentials (ProductPotential, pysic/interactions/local.py:7-283): per pair record
       the number of multiplying components (0: a plain record) and the index of its first component;
       per component its kind, 4 parameters (table rows as for pair records) and the types of the
       product's first target (null pair_nmul: no products) */
    const int32_t* pair_nmul;
    const int32_t* pair_mul0;
    const int32_t* mul_kind;
    const double* mul_params;
    const uint64_t* mul_first;
    /* four-body records (dihedral, Potentials.f90:3329-3611), one per distinct permutation of each
       target tuple: params (k, theta_0), cutoffs, the type masks of target positions 1-4 of the
       permuted record and of the unpermuted tuple (the evaluator's forward / reverse check) */
    int32_t n_quad;
    const double* quad_params;   /* 4 per record */
    const double* quad_cutoff;
    const double* quad_soft;
    const uint64_t* quad_mask;   /* 4 per record: positions 1-4 */
    const uint64_t* quad_orig;   /* 4 per record: unpermuted positions 1-4 */
} orc_model;

/* CSR neighbour list: entries of atom i are [start[i], start[i+1]). */
typedef struct {
    const int32_t* start;   /* n + 1 */
    const int32_t* idx;     /* neighbour atom */
    const int32_t* off;     /* 3 ints per entry: periodic image offset */
} orc_nblist;

/* FastNeighborList.build -> core_create_space_partitioning + core_build_neighbor_lists.
 * Writes counts[n]; if cap >= total also idx[total], off[3*total] in CSR order.
 * Returns total number of entries, or -1 on invalid input. */
int64_t orc_build_neighbors(const orc_system* sys, const double* cutoffs,
                            int32_t* counts, int32_t* idx, int32_t* off, int64_t cap);

/* core_calculate_energy / _forces / _electronegativities. what: 0 energy, 1 forces+stress, 2 enegs.
 * threads > 1 splits the outer atom loop (per-thread accumulators, summed in thread order). */
int orc_evaluate(const orc_system* sys, const orc_model* model, const orc_nblist* nb,
                 int what, int threads, double* energy, double* forces, double* stress, double* enegs);

/* Per ordered pair bond-order sums for group g: for entry e of atom i's list, zeta of (i -> j).
 * Helper used to validate the per-bond factors of the GPU path. */
/* Per-atom bond-order sums and factors of group g (core_calculate_bond_order_factors,
 * Core.f90:2015-2404, and core_post_process_bond_order_factors, 2671-2735): raw[n], factor[n]. */
int orc_atom_factors(const orc_system* sys, const orc_model* model, const orc_nblist* nb,
                     int group, double* raw, double* factor);

/* Gradients of the per-atom factors of group g (Core.f90:1157-1644, 2842-3080):
 * of_factor 0: of every atom's factor with respect to moving atom a; 1: of atom
 * a's factor with respect to moving every atom.  out: n x 3. */
int orc_atom_factor_gradients(const orc_system* sys, const orc_model* model, const orc_nblist* nb,
                              int group, int atom, int of_factor, double* out);

int orc_bond_zeta(const orc_system* sys, const orc_model* model, const orc_nblist* nb,
                  int group, double* zeta_per_entry);

#ifdef __cplusplus
}
#endif
#endif
