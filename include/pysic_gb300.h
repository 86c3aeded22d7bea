/*
 * pysic_gb300.h -- C ABI of the GB300 energy/force engine behind the Pysic API.
 *
 * The reference crosses from Python into its Fortran core through the f2py
 * module `pysic_interface` (fortran/PyInterface.f90), imported as
 * `pysic.pysic_fortran` (pysic/calculator.py:16).  This library replaces that
 * module.  Each entry point below names the f2py routine it stands in for.
 *
 * Conventions
 *  - Plain C types only; every function returns an int status (PG_OK = 0) and
 *    pg_last_error() returns a message for the calling thread's last failure.
 *  - Atom indices are 0-based; positions, forces and offsets are N x 3 in
 *    C order (the reference transposes (3,N) Fortran arrays in Python,
 *    calculator.py:941, 1496).
 *  - cell is 3 x 3 row-major with the cell vectors as rows (ASE layout); inv
 *    is its inverse (numpy.linalg.inv(cell)).
 *  - Stress/virial components are ordered xx, yy, zz, yz, xz, xy and hold the
 *    reference's potential part sum(r_a * F_b) (calculator.py:513-534 turns it
 *    into -(kinetic + virial)/V).
 *  - Interaction records are the reference's own records after the Python
 *    layer's target permutation (calculator.py:1063-1447); target filters are
 *    64-bit masks over atom types.
 *  - All state is owned by an opaque context; host arrays are only read or
 *    written during the call.  One context per thread; each context has its
 *    own CUDA stream on the current device.
 */
#ifndef PYSIC_GB300_H
#define PYSIC_GB300_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PG_OK 0
#define PG_ERR_INVALID 1        /* invalid argument                                   */
#define PG_ERR_CUDA 2           /* CUDA runtime error or device out of memory          */
#define PG_ERR_NOT_READY 3      /* cell / atoms / neighbour lists not set              */
#define PG_ERR_UNSUPPORTED 4    /* interaction the engine does not evaluate            */
#define PG_ERR_NOT_CONVERGED 5  /* charge relaxation hit its step limit                */
#define PG_ERR_TIMEOUT 6        /* a device-side wait ran out (bounded spin)           */
#define PG_ERR_SMALL_CELL 7     /* cell narrower than the cutoff: cell list not usable */

#define PG_PREC_FP64 0   /* every operation in FP64                                   */
#define PG_PREC_MIXED 1  /* FP32 per pair/triplet, FP64 (compensated) accumulation     */

#define PG_WANT_ENERGY 1
#define PG_WANT_FORCES 2  /* forces and virial */
#define PG_WANT_ENEGS 4   /* electronegativities */

typedef struct pg_context pg_context;
typedef struct pg_batch pg_batch;
typedef struct pg_mlp pg_mlp;

/* Thread-local message of the last failing call ("" if none). */
const char* pg_last_error(void);
/* Library version string. */
const char* pg_version(void);

/* Create / destroy an engine context.  Replaces the module-global state set up by
 * start_potentials / start_bond_order_factors (PyInterface.f90:51-80, called at
 * import, pysic/core.py:19-30) and torn down by release (PyInterface.f90:1023-1036). */
int pg_create(pg_context** ctx);
int pg_destroy(pg_context* ctx);
/* Same on an explicit CUDA device (one replica per GPU); device < 0 keeps the current one. */
int pg_create_on(pg_context** ctx, int32_t device);

/* create_cell(vectors, inverse, periodicity), PyInterface.f90:208-222 */
int pg_create_cell(pg_context* ctx, const double* cell, const double* inv, const int32_t* pbc);

/* create_atoms(masses, charges, positions, momenta, tags, elements), PyInterface.f90:250-268.
 * Elements and tags arrive already folded into atom types (0 .. 63). */
int pg_create_atoms(pg_context* ctx, int32_t n, const double* positions, const double* charges,
                    const int32_t* types);
/* update_atom_coordinates(positions, momenta), PyInterface.f90:277-286.
 * Enqueues the copy and a check for non-finite values without waiting; the
 * next evaluation commits the coordinates in front of its kernels.  A rejected
 * update (non-finite value) keeps the old coordinates and is reported by the
 * next call that waits on the device (pg_calculate* with PG_ERR_INVALID, or
 * any call that reads the coordinates).  The copy is cudaMemcpyAsync:
 * page-locked positions are read asynchronously and must stay unchanged until
 * that call; pageable memory is consumed before the function returns. */
int pg_update_atom_coordinates(pg_context* ctx, const double* positions);
/* update_atom_charges(charges), PyInterface.f90:295-302 */
int pg_update_atom_charges(pg_context* ctx, const double* charges);
/* Read back the engine's copy of the charges (used after pg_relax_charges). */
int pg_get_atom_charges(pg_context* ctx, double* charges);

/* allocate_potentials(n) + add_potential(...) for every pair record,
 * PyInterface.f90:370-380, 433-480.  kind: 0 LJ (epsilon, sigma), 1 exponential
 * (epsilon, zeta), 2 Buckingham (A, C, sigma), 3 spring (k, R_0; shifted by its
 * value at the cutoff), 4 power (epsilon, a, n), 5 shift_power (epsilon, r1, r2,
 * n), 6 tabulated (first row, row count, range, scale; rows set with
 * pg_set_pair_tables), 7 charge_pair (epsilon, n1, n2: epsilon q1^n1 q2^n2 with
 * the first-target types of pg_set_pair_first_targets), 10 step (e1, e2, r1, r2;
 * the reference's force, c (1, 1, 1) on the pair's atom 1 and -c (1, 1, 1) on
 * atom 2, Potentials.f90:4917-4967; unscaled, outside products); params: 4 per record
 * (unused tail zero); soft: cutoff - cutoff_margin; group: bond-order group
 * (-1 none). */
int pg_set_pair_potentials(pg_context* ctx, int32_t n_types, int32_t n_records, const int32_t* kind,
                           const double* params, const double* cutoff, const double* soft,
                           const uint64_t* mask1, const uint64_t* mask2, const int32_t* group);
/* add_potential(...) for three-body records (kind 0: bond_bend, params epsilon,
 * theta_0, n, m; V = epsilon (cos^n theta - cos^n theta_0)^m, Potentials.f90:
 * 3159-3314), one record per distinct permutation of each target tuple as
 * calculator.py adds them: type masks of target positions 1, 2, 3 and of the
 * types that may sit in the middle (the unpermuted tuple's second element).
 * At most 64 records.  Triplets are found as core_loop_over_local_interactions
 * finds them (Core.f90:3540-3943). */
int pg_set_triplet_potentials(pg_context* ctx, int32_t n_records, const int32_t* kind, const double* params,
                              const double* cutoff, const double* soft, const uint64_t* mask1,
                              const uint64_t* mask2, const uint64_t* mask3, const uint64_t* center);
/* add_potential(...) for four-body records (kind 0: dihedral, params k, phi_0;
 * V = k/2 (cos phi - cos phi_0)^2, Potentials.f90:3329-3611), one record per
 * distinct permutation of each target tuple as calculator.py adds them: per
 * record 4 type masks of target positions 1..4 (masks[4 r + t]) and 4 of the
 * unpermuted tuple (orig[4 r + t]), which the evaluator matches forwards or
 * backwards along the chain.  At most 64 records.  Chains are found as
 * core_loop_over_local_interactions finds them (Core.f90:3540-3943): from
 * every triplet, the fourth atom among the neighbours of either end. */
int pg_set_quad_potentials(pg_context* ctx, int32_t n_records, const int32_t* kind, const double* params,
                           const double* cutoff, const double* soft, const uint64_t* masks,
                           const uint64_t* orig);
/* Products of pair potentials (ProductPotential, pysic/interactions/local.py:7-283;
 * add_potential with is_multiplier, PyInterface.f90:433-480, Core.f90:909-953),
 * set after pg_set_pair_potentials (which clears them): per pair record the
 * number of factors besides the record itself (0: a plain record, at most 8)
 * and the index of its first factor; per factor its kind and 4 parameters (as
 * for pair records) and the types of the product's first target, which decide
 * the parameter order of charge-dependent factors.  Energy, forces and
 * electronegativities follow the product rule (Potentials.f90:2512-2700); the
 * record's own smooth cutoff multiplies the whole product.  Products cannot
 * carry a bond-order factor (PG_ERR_UNSUPPORTED). */
int pg_set_pair_products(pg_context* ctx, int32_t n_records, const int32_t* n_mul, const int32_t* mul0,
                         int32_t n_factors, const int32_t* kind, const double* params, const uint64_t* first);
/* Per pair record: the types of its unpermuted first target
 * (original_elements(1) of create_potential, Potentials.f90:2353-2472), which
 * decide charge_pair's exponent order (Potentials.f90:4415-4513). */
int pg_set_pair_first_targets(pg_context* ctx, int32_t n_records, const uint64_t* masks);
/* The tables of every tabulated pair record, concatenated: n_rows rows of (V,
 * d) as read_table (Utility.f90:384-433) reads table_XXXX.txt; evaluated as
 * evaluate_energy_table / _force_table (Potentials.f90:4227-4298). */
int pg_set_pair_tables(pg_context* ctx, int64_t n_rows, const double* rows);
/* add_potential(...) for single-atom records, params 4 per record: kind 0
 * charge_self (epsilon, n), 1 constant (V), 2 force (Fx, Fy, Fz; energy -F . r
 * at the absolute position).  Single-atom terms add nothing to the virial. */
int pg_set_single_potentials(pg_context* ctx, int32_t n_records, const int32_t* kind, const double* params,
                             const uint64_t* mask);
/* allocate_bond_order_factors(n) + add_bond_order_factor(...), PyInterface.f90:384-395, 482-526.
 * Tersoff records: params beta, eta, a, c, d, h, mu. */
int pg_set_bond_order_factors(pg_context* ctx, int32_t n_records, const double* params, const double* cutoff,
                              const double* soft, const uint64_t* mask1, const uint64_t* mask2,
                              const uint64_t* mask3, const int32_t* group);
/* add_bond_order_factor(...) (PyInterface.f90:482-526) for the per-atom
 * (level-1) factors, one record per target tuple, unpermuted: kind 0 neighbors,
 * 1 power_bond (params a, n), 2 c_scale (epsilon, N, C, gamma, min),
 * 3 sqrt_scale (epsilon), 4 table_bond and 5 table_scale (first row in the
 * rows of pg_set_pair_tables, rows, range, scale) (Potentials.f90:5581-5673,
 * 5972-6063, 6223-6765);
 * params 5 per record; mask2 is unused by the one-target scalers; group: the
 * Coordinator's group, shared with the pair and single-atom records.  At most 4
 * such groups; a group cannot also hold Tersoff factors. */
int pg_set_atom_factors(pg_context* ctx, int32_t n_records, const int32_t* kind, const double* params,
                        const double* cutoff, const double* soft, const uint64_t* mask1, const uint64_t* mask2,
                        const int32_t* group);
/* The Coordinator group of each record set by pg_set_single_potentials (-1:
 * none), whose per-atom factor scales the term (core_evaluate_local_singlet,
 * Core.f90:4095-4239); constant and force terms only.  pg_set_single_potentials
 * resets every group to -1. */
int pg_set_single_groups(pg_context* ctx, int32_t n_records, const int32_t* group);
/* set_ewald_parameters(real_cut, k_radius, reciprocal_cut, sigma, epsilon, scaler),
 * PyInterface.f90:1039-1046.  scaler has one entry per atom. */
int pg_set_ewald(pg_context* ctx, double real_cut, double k_radius, const int32_t* kmax, double sigma,
                 double epsilon, const double* scaler);
/* Switch Ewald summation off (the reference does this by re-initialising the core). */
int pg_clear_ewald(pg_context* ctx);

/* generate_neighbor_lists(n_atoms, cutoffs), PyInterface.f90:1062-1072: the cell-list
 * build of FastNeighborList (calculator.py:62-108).  cutoffs already include the
 * list skin; skin is passed separately so the engine can derive its short list
 * for bond-order terms.  The lists are bit-identical, order included, to
 * core_build_neighbor_lists (Core.f90:8148-8280).  Fails with PG_ERR_SMALL_CELL
 * when the cell is narrower than the largest cutoff (the reference then uses
 * ASE's list, calculator.py:829-848). */
int pg_generate_neighbor_lists(pg_context* ctx, const double* cutoffs, double skin);
/* The list the reference takes from ASE's NeighborList when the cell is narrower
 * than the cutoff (calculator.py:829-848, 905-915 -> create_neighbor_list,
 * PyInterface.f90:528-546), built on the device: both directions, no self pair,
 * i and j neighbours when |r_j + n.cell - r_i| < c_i + c_j.  Ordered by partner,
 * then image offset. */
int pg_generate_all_pairs_lists(pg_context* ctx, const double* cutoffs, double skin);
/* get_number_of_neighbors_of_atom, PyInterface.f90:1075-1082, for all atoms at once. */
int pg_get_neighbor_counts(pg_context* ctx, int32_t* counts);
/* get_neighbor_list_of_atom, PyInterface.f90:1085-1096, for all atoms at once:
 * neighbours (0-based) and offsets (3 per entry) in CSR order. */
int pg_get_neighbor_lists(pg_context* ctx, int32_t* neighbors, int32_t* offsets);
/* create_neighbor_list(atom, neighbors, offsets), PyInterface.f90:528-546, for all
 * atoms at once: install lists built elsewhere (ASE's list for small cells). */
int pg_create_neighbor_lists(pg_context* ctx, const int32_t* counts, const int32_t* neighbors,
                             const int32_t* offsets, double skin);

/* calculate_energy(energy), PyInterface.f90:652-660 */
int pg_calculate_energy(pg_context* ctx, int32_t precision, double* energy);
/* calculate_forces(n_atoms, forces, stress), PyInterface.f90:668-677 */
int pg_calculate_forces(pg_context* ctx, int32_t precision, double* forces, double* stress);
/* calculate_electronegativities(n_atoms, enegs), PyInterface.f90:684-692 */
int pg_calculate_electronegativities(pg_context* ctx, int32_t precision, double* enegs);
/* One fused evaluation of any of energy, forces + virial and electronegativities
 * (flags: PG_WANT_*).  The reference needs one full pass per quantity
 * (calculator.py:940, 968).  Null output pointers are skipped; one
 * synchronisation per call. */
int pg_calculate(pg_context* ctx, int32_t precision, int32_t flags, double* energy, double* forces,
                 double* stress, double* enegs);

/* Damped charge dynamics of ChargeRelaxation 'dynamic' (pysic/charges/relaxation.py:417-450)
 * run on the device: the loop calls the electronegativity kernels without host
 * round trips.  rates (q-dot) is read and written back so that successive calls
 * warm-start like the reference's persistent charge_rates (relaxation.py:431-432).
 * The stopping test is the reference's: max(chi - mean(chi)) < tolerance (signed
 * max, relaxation.py:449) or step count reached.  On return charges holds the
 * relaxed charges, *steps the steps taken, *error the final signed max and
 * *max_dq the largest |q change| of the last step. */
int pg_relax_charges(pg_context* ctx, int32_t precision, int32_t n_steps, double timestep, double inertia,
                     double friction, double tolerance, double* rates, double* charges, int32_t* steps,
                     double* error, double* max_dq);

/* ChargeRelaxation 'potentiostat' (pysic/charges/relaxation.py:453-481) on the
 * device: undamped charge dynamics driven by chi - potential (no mean
 * subtracted, so the total charge follows the external potential) for exactly
 * n_steps steps.  rates is read and written back as for pg_relax_charges;
 * charges receives the final charges and *max_dchi (may be null) the final
 * max(chi - potential).  PG_ERR_NOT_CONVERGED only when the dynamics diverge
 * (non-finite electronegativities). */
int pg_relax_charges_potentiostat(pg_context* ctx, int32_t precision, int32_t n_steps, double timestep,
                                  double inertia, double potential, double* rates, double* charges,
                                  double* max_dchi);

/* Velocity Verlet molecular dynamics on the device, step for step what ASE's
 * VelocityVerlet.step does around Pysic.get_forces (p += dt/2 F; r += dt p / m;
 * F(r); p += dt/2 F, each operation rounded once), without host round trips.
 * pg_md_set_state uploads masses (N) and momenta (N x 3); pg_md_verlet runs up
 * to n_steps steps on the context's coordinates and stops early when an atom
 * has moved more than skin/2 since the neighbour lists were built (*rebuild =
 * 1; the step is then left after its drift): rebuild the lists
 * (pg_generate_neighbor_lists reads the device coordinates) and call again,
 * which completes that step first.  *steps_done counts completed steps.
 * pg_md_get_state downloads momenta and positions (either may be null). */
int pg_md_set_state(pg_context* ctx, const double* masses, const double* momenta);
/* The same dynamics for exactly n_steps steps, the neighbour lists rebuilt on
 * the device whenever an atom has moved more than skin/2 since the last build
 * (the FastNeighborList policy, calculator.py:29-189), with the cutoffs and
 * the builder (cell list or all pairs) of the last pg_generate_neighbor_lists /
 * pg_generate_all_pairs_lists call; the host only launches and reads a flag
 * word per chunk of steps.  *rebuilds counts the rebuilds; the positions of the
 * last build are read with pg_get_list_positions.  Lists installed from the
 * host (pg_create_neighbor_lists) give PG_ERR_NOT_READY: use pg_md_verlet. */
int pg_md_run(pg_context* ctx, int32_t precision, int32_t n_steps, double timestep, double skin, int32_t* steps_done,
              int32_t* rebuilds);
/* The positions (N x 3) at which the current neighbour lists were built (the
 * reference positions of FastNeighborList's skin test). */
int pg_get_list_positions(pg_context* ctx, double* positions);
int pg_md_verlet(pg_context* ctx, int32_t precision, int32_t n_steps, double timestep, double skin,
                 int32_t* steps_done, int32_t* rebuild);
int pg_md_get_state(pg_context* ctx, double* momenta, double* positions);

/* ChargeRelaxation 'optimize' (pysic/charges/relaxation.py:483-488; the
 * reference calls SciPy's SLSQP on the energy and electronegativities) for
 * energies quadratic in the charges (Ewald and charge_self with n <= 2): the
 * constrained minimum at fixed total charge by projected conjugate gradients on
 * the device.  Stops when max |chi - mean(chi)| <= tolerance (recomputed from
 * the final charges) or after max_iterations; charges receives the result (the
 * context keeps it), *iterations and *error the count and the final max |chi -
 * mean(chi)|.  PG_ERR_UNSUPPORTED for other energies (the caller falls back to
 * SLSQP), PG_ERR_NOT_CONVERGED at the iteration limit or for a non-convex
 * energy. */
int pg_optimize_charges(pg_context* ctx, int32_t precision, int32_t max_iterations, double tolerance,
                        double* charges, int32_t* iterations, double* error);

/* Per-atom bond-order factors of a Coordinator group after an evaluation at the
 * current positions (core_get_bond_order_factors, Core.f90:759-783, behind
 * calculate_bond_order_factors, PyInterface.f90): B_i = post(sum), the sum
 * itself without a scaler; zeros for a group without per-atom factors.
 * n entries. */
int pg_get_atom_factors(pg_context* ctx, int32_t precision, int32_t group, double* factors);
/* Gradients of a Coordinator group's per-atom factors at the current positions
 * (calculate_bond_order_gradients / _of_factor, PyInterface.f90:605-650, over
 * core_calculate_bond_order_gradients, Core.f90:1157-1989): of_factor 0, the
 * gradient of every atom's factor with respect to moving `atom`; 1, of `atom`'s
 * factor with respect to moving every atom.  gradients: n x 3 (0-based atom). */
int pg_get_atom_factor_gradients(pg_context* ctx, int32_t precision, int32_t group, int32_t atom, int32_t of_factor,
                                 double* gradients);

/* Per ordered bond (CSR entry of the engine's short list) Tersoff sums zeta_ij of
 * group 0: the quantity core_calculate_pair_bond_order_factor (Core.f90:2439-2637)
 * accumulates.  Diagnostic; n_entries receives the short-list length. */
int pg_get_bond_zeta(pg_context* ctx, double* zeta, int64_t capacity, int64_t* n_entries);

/* Tile of the bond-order kernels: lanes per atom (4, 8, 16 or 32), one bond per
 * lane; PG_LANES_TRIPLET, 16 lanes per atom with one (bond, neighbour) pair per
 * lane; 0 lets the built-in autotuner choose on the next evaluation. */
#define PG_LANES_TRIPLET 64
int pg_set_lanes_per_atom(pg_context* ctx, int32_t lanes);
/* Tile size of the full-list kernels (pair, per-atom factors, cached Ewald
 * matrix): lanes per atom (8, 16 or 32); 0 chooses by list length and atom
 * count. */
int pg_set_pair_lanes(pg_context* ctx, int32_t lanes);
int pg_get_lanes_per_atom(pg_context* ctx, int32_t* lanes);

/* ---- device-resident evaluation (benchmarks, MD drivers) ----------------
 * pg_device_evaluate launches one evaluation on the context's stream using the
 * positions and charges already on the device and leaves energy, virial, forces
 * and electronegativities in device memory; pg_device_results copies them out.
 * pg_device_positions exposes the device position buffer (N x 3 doubles) so a
 * caller can update it in place. */
int pg_device_evaluate(pg_context* ctx, int32_t precision, int32_t flags);
int pg_device_synchronize(pg_context* ctx);
int pg_device_results(pg_context* ctx, double* energy, double* forces, double* stress, double* enegs);
int pg_device_positions(pg_context* ctx, double** device_ptr);
/* The CUDA stream the context launches on (cudaStream_t as void*). */
int pg_get_stream(pg_context* ctx, void** stream);

/* Bond-order (Tersoff) energy, virial and forces without any device allocation
 * during the call.  No counterpart in the reference, whose f2py calls always
 * allocate their NumPy outputs.
 * All per-call scratch comes from one static device array of
 * PG_NOALLOC_SCRATCH_BYTES; a system that needs more is rejected with
 * PG_ERR_INVALID and a message giving both sizes.  d_forces (N x 3 doubles) and
 * d_totals (7 doubles: energy, then the virial xx, yy, zz, yz, xz, xy) are device
 * pointers owned by the caller; the work is enqueued on the context's stream
 * (pg_get_stream) and the call returns without waiting.
 *  - Only contexts whose every term runs in the bond-order kernels (no Ewald,
 *    charge or out-of-bond pair terms): PG_ERR_UNSUPPORTED otherwise.
 *  - Tables and lists must be current: call pg_calculate once after the last
 *    change of potentials, lists or lanes (PG_ERR_NOT_READY otherwise).
 *  - The first call on each context looks up the static array's device
 *    address (in the CUDA context then current) and keeps it; make that call
 *    before any stream capture.  A pg_context created before a device reset
 *    (cudaDeviceReset) must not be used after it.
 *  - An empty system writes zero totals and launches nothing.
 *  - The array is shared by every context on the device: calls that overlap in
 *    time race on it and must be ordered by the caller. */
#define PG_NOALLOC_SCRATCH_BYTES (32u << 20)
int pg_bond_order_noalloc(pg_context* ctx, int32_t precision, double* d_forces, double* d_totals);

/* ---- learned warm start for charge relaxation ------------------------------
 * No counterpart in the reference, whose ChargeRelaxation starts from the
 * current charges (pysic/charges/relaxation.py:394-450).
 *
 * pg_descriptors: per atom, n_types x n_gauss radial features
 *   sum_j exp(-(r_ij - mu_k)^2 / (2 width^2)) (1 + cos(pi r_ij / cutoff)) / 2 over
 *   neighbours j of each type with r_ij < cutoff, mu_k evenly spaced on [r0, r1];
 *   out is N x (n_types * n_gauss) floats, type-major.  Needs lists at least as
 *   long as cutoff (built by pg_generate_neighbor_lists / _all_pairs_lists).
 * pg_mlp_*: a network n_in -> n_h1 -> n_h2 -> 1 with tanh activations, BF16
 *   weights and FP32 arithmetic, trained on the GPU (mean squared error, Adam).
 *   Parameters are FP32 in the order W1 (n_h1 x n_in, row-major), b1, W2
 *   (n_h2 x n_h1), b2, w3 (n_h2), b3.  pg_mlp_gradients returns the loss and
 *   its gradient for the given samples (no update), for gradient checks.
 * pg_mlp_predict_charges: the warm start of a context's structure without
 *   leaving the device: descriptors (as pg_descriptors), per-type columns added
 *   in type order into per-element columns (type_element[t] = element index
 *   of type t, n_types entries), the one-hot element code appended, inputs
 *   (x - x_mean) / x_scale, the network, q = y * y_scale + y_mean in FP64,
 *   then shifted by (sum q - total_charge) / N.  The charges replace the
 *   context's own; charges (N doubles, may be null) receives a copy.  The
 *   network needs n_in = n_elements x (n_gauss + 1). */
int pg_descriptors(pg_context* ctx, int32_t n_gauss, double r0, double r1, double width, double cutoff,
                   float* out);
int pg_mlp_create(pg_mlp** mlp, int32_t n_in, int32_t n_h1, int32_t n_h2, int32_t device);
int pg_mlp_destroy(pg_mlp* mlp);
int pg_mlp_param_count(pg_mlp* mlp, int64_t* count);
int pg_mlp_set_params(pg_mlp* mlp, const float* params, int64_t count);
int pg_mlp_get_params(pg_mlp* mlp, float* params, int64_t count);
int pg_mlp_add_samples(pg_mlp* mlp, const float* x, const float* y, int64_t n);
int pg_mlp_clear_samples(pg_mlp* mlp);
int pg_mlp_train(pg_mlp* mlp, int32_t epochs, int32_t batch, float learning_rate, uint64_t seed,
                 float* epoch_loss);
int pg_mlp_gradients(pg_mlp* mlp, const float* x, const float* y, int64_t n, float* grad, double* loss);
int pg_mlp_predict(pg_mlp* mlp, const float* x, int64_t n, float* y);
int pg_mlp_predict_charges(pg_mlp* mlp, pg_context* ctx, int32_t n_gauss, double r0, double r1, double width,
                           double cutoff, int32_t n_elements, const int32_t* type_element, const float* x_mean,
                           const float* x_scale, double y_mean, double y_scale, double total_charge,
                           double* charges);

/* ---- many independent systems ------------------------------------------------
 * No counterpart in the reference, which holds one system per process.  A batch
 * borrows fully set-up contexts (same device; pair and bond-order terms, no
 * Ewald) and evaluates them all
 *   mode 0: in ONE persistent launch, replayed from a CUDA graph: resident
 *           blocks take (phase, system, cells) tiles in dependency order
 *           (displacements, pair terms, bond pass, gather) with bounded
 *           per-system waits; a wait that runs out makes pg_batch_synchronize
 *           return PG_ERR_TIMEOUT;
 *   mode 1: each on its own (one pg_device_evaluate per context);
 *   mode 2: with one launch per phase over the tile list of all systems.
 * Results stay in each context: read them with pg_device_results after
 * pg_batch_synchronize.  Tiles -- lanes per atom of the pair body (8 or 16 in
 * mode 0; 8, 16 or 32 in mode 2), of the bond-order body (4, 8, or
 * PG_LANES_TRIPLET) and, in mode 0, the cells of 128 threads' atoms that one
 * ticket hands a block (1..64) -- are timed on the batch itself when left 0;
 * pg_batch_get_tiles reports the ones in use. */
int pg_batch_create(pg_batch** batch, int32_t device);
int pg_batch_destroy(pg_batch* batch);
int pg_batch_add(pg_batch* batch, pg_context* ctx);
int pg_batch_set_lanes(pg_batch* batch, int32_t pair_lanes, int32_t bond_lanes);
int pg_batch_get_lanes(pg_batch* batch, int32_t precision, int32_t* pair_lanes, int32_t* bond_lanes);
int pg_batch_set_tile_blocks(pg_batch* batch, int32_t blocks);
int pg_batch_get_tiles(pg_batch* batch, int32_t precision, int32_t mode, int32_t* pair_lanes, int32_t* bond_lanes,
                       int32_t* blocks);
int pg_batch_evaluate(pg_batch* batch, int32_t precision, int32_t flags, int32_t mode);
/* Test of the persistent launch's bounded waits: from the next mode-0
 * evaluation on, the pair and bond tiles of `system` wait for a displacement
 * tile that never comes, so every such wait runs out after wait_seconds (at
 * most 1 s) and pg_batch_synchronize returns PG_ERR_TIMEOUT; the kernel ends
 * normally and the context stays usable.  system = -1 ends the test (the wait
 * limit stays as given; the default is 0.5 s). */
int pg_batch_test_stall(pg_batch* batch, int32_t system, double wait_seconds);
int pg_batch_synchronize(pg_batch* batch);
int pg_batch_get_stream(pg_batch* batch, void** stream);
int pg_batch_last_launch_count(pg_batch* batch, int32_t* launches);

/* FP32 rate of this GPU: a kernel of independent fused multiply-add chains on
 * every SM (cudaDevAttrMultiProcessorCount), best of several timed launches.
 * *tflops receives TFLOP/s, *ms (may be null) the best launch's duration.  The
 * benchmark's roofline denominator for the FP32-bound bond-order kernels.  No
 * counterpart in the reference; device < 0 keeps the current device. */
int pg_measure_fp32_peak(int32_t device, double* tflops, double* ms);
/* Device allocations (cudaMalloc of a growing buffer) made by this library in
 * this process so far; diagnostic, so that a caller can check that a call
 * allocated nothing.  No counterpart in the reference. */
int pg_device_allocation_count(uint64_t* count);
/* Kernel launches issued by the last pg_device_evaluate / pg_calculate. */
int pg_last_launch_count(pg_context* ctx, int32_t* launches);
/* Record CUDA events around the kernel groups of each evaluation;
 * pg_get_kernel_times waits for the last evaluation and returns five durations
 * in ms: pair kernel, bond-order pass, gather pass, k-space Ewald, reduction. */
int pg_set_kernel_timing(pg_context* ctx, int32_t enable);
int pg_get_kernel_times(pg_context* ctx, float* ms);
/* Replay each evaluation sequence from a captured CUDA graph (default on). */
int pg_set_graphs(pg_context* ctx, int32_t enable);

#ifdef __cplusplus
}
#endif
#endif
