"""Python handle on one engine context (the GB300 replacement of the
reference's Fortran core state, fortran/Core.f90:13-98)."""
import ctypes
import os

import numpy as np

from . import _lib as L
from .error import EngineError


class Engine:
    """Owns one ``pg_context``: cell, atoms, interaction records, neighbour
    lists and device buffers.  Every method maps to one C-ABI call."""

    def __init__(self, device=None):
        self.lib = L.load()
        ctx = ctypes.c_void_p()
        if device is None:
            device = int(os.environ.get("PYSIC_GB300_DEVICE", "-1"))
        L.check(self.lib.pg_create_on(ctypes.byref(ctx), int(device)))
        self.ctx = ctx
        self.n = 0
        self._alib = L.addr_lib()
        self._addr = L.AddressCache()

    def close(self):
        if getattr(self, "ctx", None) is not None and self.ctx.value:
            self.lib.pg_destroy(self.ctx)
            self.ctx = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # --- state ------------------------------------------------------------
    def set_cell(self, cell, pbc):
        cell = L.as_f64(cell, (3, 3))
        inv = L.as_f64(np.linalg.inv(cell))
        pbc = L.as_i32(np.asarray(pbc, dtype=bool).astype(np.int32))
        L.check(self.lib.pg_create_cell(self.ctx, L.dptr(cell), L.dptr(inv), L.iptr(pbc)))

    def set_atoms(self, positions, charges, types):
        pos = L.as_f64(positions, (-1, 3))
        q = L.as_f64(charges)
        t = L.as_i32(types)
        self.n = len(pos)
        L.check(self.lib.pg_create_atoms(self.ctx, self.n, L.dptr(pos), L.dptr(q), L.iptr(t)))

    def update_positions(self, positions):
        if isinstance(positions, np.ndarray) and positions.dtype == np.float64 and positions.flags.c_contiguous \
                and positions.size == 3 * self.n:
            L.check(self._alib.pg_update_atom_coordinates(self.ctx, self._addr(positions)))
            return
        pos = L.as_f64(positions, (-1, 3))
        L.check(self.lib.pg_update_atom_coordinates(self.ctx, L.dptr(pos)))

    def update_charges(self, charges):
        q = L.as_f64(charges)
        L.check(self.lib.pg_update_atom_charges(self.ctx, L.dptr(q)))

    def get_charges(self):
        q = np.zeros(self.n)
        L.check(self.lib.pg_get_atom_charges(self.ctx, L.dptr(q)))
        return q

    def set_model(self, model):
        a = model.arrays()
        first = np.ascontiguousarray(a["pair_first"], dtype=np.uint64)
        L.check(self.lib.pg_set_pair_first_targets(self.ctx, len(first), L.u64ptr(first)))
        tab = L.as_f64(a["pair_table"])
        L.check(self.lib.pg_set_pair_tables(self.ctx, len(tab) // 2, L.dptr(tab)))
        L.check(self.lib.pg_set_triplet_potentials(
            self.ctx, len(a["tri_kind"]), L.iptr(a["tri_kind"]), L.dptr(a["tri_params"]), L.dptr(a["tri_cutoff"]),
            L.dptr(a["tri_soft"]), L.u64ptr(a["tri_mask1"]), L.u64ptr(a["tri_mask2"]), L.u64ptr(a["tri_mask3"]),
            L.u64ptr(a["tri_center"])))
        L.check(self.lib.pg_set_quad_potentials(
            self.ctx, len(a["quad_kind"]), L.iptr(a["quad_kind"]), L.dptr(a["quad_params"]),
            L.dptr(a["quad_cutoff"]), L.dptr(a["quad_soft"]), L.u64ptr(a["quad_mask"]), L.u64ptr(a["quad_orig"])))
        npair = len(a["pair_kind"])
        L.check(self.lib.pg_set_pair_potentials(
            self.ctx, model.n_types, npair, L.iptr(a["pair_kind"]), L.dptr(a["pair_params"]),
            L.dptr(a["pair_cutoff"]), L.dptr(a["pair_soft"]), L.u64ptr(a["pair_mask1"]), L.u64ptr(a["pair_mask2"]),
            L.iptr(a["pair_group"])))
        nm = L.as_i32(a["pair_nmul"]) if len(a["pair_nmul"]) else np.zeros(max(npair, 1), dtype=np.int32)
        m0 = L.as_i32(a["pair_mul0"]) if len(a["pair_mul0"]) else np.zeros(max(npair, 1), dtype=np.int32)
        mk = L.as_i32(a["mul_kind"]) if len(a["mul_kind"]) else np.zeros(1, dtype=np.int32)
        mp = L.as_f64(a["mul_params"]) if len(a["mul_params"]) else np.zeros(4)
        mf = L.as_u64(a["mul_first"]) if len(a["mul_first"]) else np.zeros(1, dtype=np.uint64)
        L.check(self.lib.pg_set_pair_products(self.ctx, npair, L.iptr(nm), L.iptr(m0), len(a["mul_kind"]), L.iptr(mk),
                                              L.dptr(mp), L.u64ptr(mf)))
        L.check(self.lib.pg_set_single_potentials(
            self.ctx, len(a["single_kind"]), L.iptr(a["single_kind"]), L.dptr(a["single_params"]),
            L.u64ptr(a["single_mask"])))
        L.check(self.lib.pg_set_single_groups(self.ctx, len(a["single_kind"]), L.iptr(a["single_group"])))
        L.check(self.lib.pg_set_atom_factors(
            self.ctx, len(a["afac_kind"]), L.iptr(a["afac_kind"]), L.dptr(a["afac_params"]),
            L.dptr(a["afac_cutoff"]), L.dptr(a["afac_soft"]), L.u64ptr(a["afac_mask1"]), L.u64ptr(a["afac_mask2"]),
            L.iptr(a["afac_group"])))
        L.check(self.lib.pg_set_bond_order_factors(
            self.ctx, len(a["bond_cutoff"]), L.dptr(a["bond_params"]), L.dptr(a["bond_cutoff"]),
            L.dptr(a["bond_soft"]), L.u64ptr(a["bond_mask1"]), L.u64ptr(a["bond_mask2"]), L.u64ptr(a["bond_mask3"]),
            L.iptr(a["bond_group"])))
        self.set_ewald(model.ewald)

    def set_ewald(self, ew):
        if ew is None:
            L.check(self.lib.pg_clear_ewald(self.ctx))
            return
        kmax = L.as_i32(ew["kmax"])
        sc = L.as_f64(ew["scaler"])
        L.check(self.lib.pg_set_ewald(self.ctx, ew["rc"], ew["kc"], L.iptr(kmax), ew["sigma"], ew["eps"],
                                      L.dptr(sc)))

    # --- neighbour lists ---------------------------------------------------
    def build_neighbors(self, cutoffs, skin):
        """Cell-list build (FastNeighborList); raises EngineError with status
        PG_ERR_SMALL_CELL when the cell is narrower than the cutoff."""
        c = L.as_f64(cutoffs)
        L.check(self.lib.pg_generate_neighbor_lists(self.ctx, L.dptr(c), float(skin)))

    def build_all_pairs(self, cutoffs, skin):
        c = L.as_f64(cutoffs)
        L.check(self.lib.pg_generate_all_pairs_lists(self.ctx, L.dptr(c), float(skin)))

    def install_neighbors(self, counts, idx, off, skin):
        counts = L.as_i32(counts)
        idx = L.as_i32(idx)
        off = L.as_i32(np.asarray(off).reshape(-1, 3))
        L.check(self.lib.pg_create_neighbor_lists(self.ctx, L.iptr(counts), L.iptr(idx), L.iptr(off),
                                                  float(skin)))

    def neighbor_lists(self):
        counts = np.zeros(self.n, dtype=np.int32)
        L.check(self.lib.pg_get_neighbor_counts(self.ctx, L.iptr(counts)))
        total = int(counts.sum())
        idx = np.zeros(max(total, 1), dtype=np.int32)
        off = np.zeros((max(total, 1), 3), dtype=np.int32)
        L.check(self.lib.pg_get_neighbor_lists(self.ctx, L.iptr(idx), L.iptr(off)))
        return counts, idx[:total], off[:total]

    # --- evaluation --------------------------------------------------------
    def calculate(self, precision=L.PREC_FP64, energy=True, forces=True, enegs=False):
        flags = (L.WANT_ENERGY if energy else 0) | (L.WANT_FORCES if forces else 0) | (L.WANT_ENEGS if enegs else 0)
        e = np.zeros(1)
        f = np.zeros((self.n, 3))
        s = np.zeros(6)
        c = np.zeros(self.n)
        L.check(self.lib.pg_calculate(self.ctx, precision, flags, L.dptr(e), L.dptr(f), L.dptr(s), L.dptr(c)))
        out = {}
        if energy:
            out["energy"] = float(e[0])
        if forces:
            out["forces"] = f
            out["stress"] = s
        if enegs:
            out["enegs"] = c
        return out

    def relax_charges(self, precision, n_steps, timestep, inertia, friction, tolerance, rates):
        rates = L.as_f64(rates).copy()
        q = np.zeros(self.n)
        steps = ctypes.c_int32(0)
        err = ctypes.c_double(0)
        dq = ctypes.c_double(0)
        st = self.lib.pg_relax_charges(self.ctx, precision, int(n_steps), float(timestep), float(inertia),
                                       float(friction), float(tolerance), L.dptr(rates), L.dptr(q),
                                       ctypes.byref(steps), ctypes.byref(err), ctypes.byref(dq))
        if st not in (L.PG_OK, L.PG_ERR_NOT_CONVERGED):
            L.check(st)
        return {"charges": q, "rates": rates, "steps": steps.value, "error": err.value, "max_dq": dq.value,
                "converged": st == L.PG_OK}

    # ---- molecular dynamics (pg_md_*) ------------------------------------------
    def md_set_state(self, masses, momenta):
        m = L.as_f64(masses)
        p = L.as_f64(momenta, (-1, 3))
        L.check(self.lib.pg_md_set_state(self.ctx, L.dptr(m), L.dptr(p)))

    def md_verlet(self, precision, n_steps, timestep, skin):
        """Up to n_steps velocity Verlet steps; (steps completed, rebuild needed)."""
        s = ctypes.c_int32(0)
        r = ctypes.c_int32(0)
        L.check(self.lib.pg_md_verlet(self.ctx, precision, int(n_steps), float(timestep), float(skin),
                                      ctypes.byref(s), ctypes.byref(r)))
        return s.value, bool(r.value)

    def md_run(self, precision, n_steps, timestep, skin):
        """Exactly n_steps velocity Verlet steps with the lists rebuilt on the
        device as needed; (steps completed, list rebuilds)."""
        s = ctypes.c_int32(0)
        r = ctypes.c_int32(0)
        L.check(self.lib.pg_md_run(self.ctx, precision, int(n_steps), float(timestep), float(skin), ctypes.byref(s),
                                   ctypes.byref(r)))
        return s.value, r.value

    def list_positions(self):
        """The positions at which the current lists were built."""
        r = np.zeros((self.n, 3))
        L.check(self.lib.pg_get_list_positions(self.ctx, L.dptr(r)))
        return r

    def md_get_state(self):
        p = np.zeros((self.n, 3))
        r = np.zeros((self.n, 3))
        L.check(self.lib.pg_md_get_state(self.ctx, L.dptr(p), L.dptr(r)))
        return p, r

    def optimize_charges(self, precision, max_iterations, tolerance):
        """Constrained energy minimum over the charges on the device
        (pg_optimize_charges).  Returns None when the energy is not quadratic
        in the charges (the caller then uses SLSQP)."""
        q = np.zeros(self.n)
        it = ctypes.c_int32(0)
        err = ctypes.c_double(0)
        st = self.lib.pg_optimize_charges(self.ctx, precision, int(max_iterations), float(tolerance), L.dptr(q),
                                          ctypes.byref(it), ctypes.byref(err))
        if st == L.PG_ERR_UNSUPPORTED:
            return None
        if st not in (L.PG_OK, L.PG_ERR_NOT_CONVERGED):
            L.check(st)
        return {"charges": q, "iterations": it.value, "error": err.value, "converged": st == L.PG_OK}

    def relax_charges_potentiostat(self, precision, n_steps, timestep, inertia, potential, rates):
        rates = L.as_f64(rates).copy()
        q = np.zeros(self.n)
        m = ctypes.c_double(0)
        L.check(self.lib.pg_relax_charges_potentiostat(self.ctx, precision, int(n_steps), float(timestep),
                                                       float(inertia), float(potential), L.dptr(rates), L.dptr(q),
                                                       ctypes.byref(m)))
        return {"charges": q, "rates": rates, "steps": int(n_steps), "max_dchi": m.value}

    def atom_factors(self, group, precision=L.PREC_FP64):
        """Per-atom bond-order factors of a Coordinator group at the current positions."""
        out = np.zeros(max(self.n, 1))
        L.check(self.lib.pg_get_atom_factors(self.ctx, int(precision), int(group), L.dptr(out)))
        return out[:self.n]

    def atom_factor_gradients(self, group, atom, of_factor=False, precision=L.PREC_FP64):
        """n x 3 gradients of a Coordinator group's per-atom factors."""
        out = np.zeros((max(self.n, 1), 3))
        L.check(self.lib.pg_get_atom_factor_gradients(self.ctx, int(precision), int(group), int(atom),
                                                      1 if of_factor else 0, L.dptr(out)))
        return out[:self.n]

    def bond_zeta(self):
        n = ctypes.c_int64(0)
        L.check(self.lib.pg_get_bond_zeta(self.ctx, None, 0, ctypes.byref(n)))
        z = np.zeros(max(n.value, 1))
        L.check(self.lib.pg_get_bond_zeta(self.ctx, L.dptr(z), n.value, ctypes.byref(n)))
        return z[:n.value]

    def set_pair_lanes(self, lanes):
        L.check(self.lib.pg_set_pair_lanes(self.ctx, int(lanes)))

    def set_lanes(self, lanes):
        L.check(self.lib.pg_set_lanes_per_atom(self.ctx, int(lanes)))

    def get_lanes(self):
        v = ctypes.c_int32(0)
        L.check(self.lib.pg_get_lanes_per_atom(self.ctx, ctypes.byref(v)))
        return v.value

    # --- device-resident use --------------------------------------------------
    def device_evaluate(self, precision, flags):
        L.check(self.lib.pg_device_evaluate(self.ctx, precision, flags))

    def device_synchronize(self):
        L.check(self.lib.pg_device_synchronize(self.ctx))

    def device_results(self):
        e = np.zeros(1)
        f = np.zeros((self.n, 3))
        s = np.zeros(6)
        c = np.zeros(self.n)
        L.check(self.lib.pg_device_results(self.ctx, L.dptr(e), L.dptr(f), L.dptr(s), L.dptr(c)))
        return {"energy": float(e[0]), "forces": f, "stress": s, "enegs": c}

    def device_positions_ptr(self):
        p = ctypes.POINTER(ctypes.c_double)()
        L.check(self.lib.pg_device_positions(self.ctx, ctypes.byref(p)))
        return ctypes.cast(p, ctypes.c_void_p).value

    def stream_handle(self):
        s = ctypes.c_void_p()
        L.check(self.lib.pg_get_stream(self.ctx, ctypes.byref(s)))
        return s.value or 0

    def launch_count(self):
        v = ctypes.c_int32(0)
        L.check(self.lib.pg_last_launch_count(self.ctx, ctypes.byref(v)))
        return v.value

    def descriptors(self, n_types, n_gauss, r0, r1, width, cutoff):
        """Per-atom radial descriptors (n_types * n_gauss floats per atom)."""
        out = np.zeros((self.n, n_types * n_gauss), dtype=np.float32)
        L.check(self.lib.pg_descriptors(self.ctx, int(n_gauss), float(r0), float(r1), float(width), float(cutoff),
                                        L.fptr(out)))
        return out

    def set_kernel_timing(self, enable):
        L.check(self.lib.pg_set_kernel_timing(self.ctx, 1 if enable else 0))

    def kernel_times(self):
        """Durations (ms) of the last evaluation's kernel groups: pair, bond
        pass, gather pass, k-space Ewald, reduction."""
        ms = (ctypes.c_float * 5)()
        L.check(self.lib.pg_get_kernel_times(self.ctx, ms))
        return dict(zip(("pair", "bond_pass", "gather_pass", "kspace", "reduce"), list(ms)))

    def set_graphs(self, enable):
        L.check(self.lib.pg_set_graphs(self.ctx, 1 if enable else 0))

    def calculate_into(self, precision, flags, energy, forces, stress, enegs):
        """pg_calculate into caller-provided (e.g. page-locked) C-contiguous
        float64 host arrays (any of them may be None)."""
        a = self._addr
        L.check(self._alib.pg_calculate(self.ctx, precision, flags, a(energy), a(forces), a(stress), a(enegs)))


__all__ = ["Engine", "EngineError"]
