"""Drop-in for the reference's f2py module: ``pysic_interface``.

The reference's Python package reaches its Fortran core through
``import pysic.pysic_fortran as pf`` and calls ``pf.pysic_interface.<routine>``
(routines in fortran/PyInterface.f90).  This module offers the same object,
with the same routine names, argument order, array layouts and return values
as f2py generates them, backed by the GB300 engine's C ABI:

    import pysic_gb300.pf_shim as pf
    pf.pysic_interface.create_atoms(masses, charges, positions, momenta, tags, elements)

Conventions kept from f2py:
- arrays of shape (3, N) in and out (positions, momenta, forces, offsets,
  gradients), element labels as (2, n) integer codes (pysic/utility/f2py.py:
  153-175), atom indices 0-based in Python and 1-based where the reference's
  Python passes them so (create_neighbor_list, calculate_bond_order_gradients);
- dimension arguments that f2py infers are optional (generate_neighbor_lists,
  set_ewald_parameters, create_atoms) and the ones it requires are required
  (calculate_forces(n_atoms), calculate_electronegativities(n_atoms));
- add_potential and add_bond_order_factor return a success flag.

The reference registers interaction records one at a time and then builds its
per-atom lists (create_potential_list, PyInterface.f90:548); the engine takes
the whole record set per kind, with target filters folded into atom types.
This module collects the records and commits them, together with the atoms,
before the first neighbour build or evaluation after a change.  The element
code of a label is used as it comes: atoms and records with the same code
pair are the same element.

Errors of the engine raise pysic_gb300.error.EngineError.  Evaluation runs in
FP64 unless ``pysic_interface.precision`` is set to PREC_MIXED.
"""
import numpy as np

from . import _lib as L
from . import core
from .engine import Engine
from .model import MAX_TYPES, Model, _charge_exp_record, _table_record

PREC_FP64 = L.PREC_FP64
PREC_MIXED = L.PREC_MIXED
NO_TARGET = -9  # the reference's "no tag / no index" marker (calculator.py:1239-1240)


def _codes(a, n):
    """(2, n) element codes as a list of n hashable pairs."""
    a = np.asarray(a, dtype=np.int64).reshape(2, -1) if n else np.zeros((2, 0), dtype=np.int64)
    return [(int(a[0, k]), int(a[1, k])) for k in range(a.shape[1])]


def _ints(a, n):
    a = np.asarray(a, dtype=np.int64).reshape(-1)
    return [int(x) for x in a[:n]]


class PysicInterface:
    """The routines of fortran/PyInterface.f90 that the reference's Python
    layer calls on the energy / force path, one engine context behind them
    (the reference keeps one system in module globals, Core.f90:22-91)."""

    skin = 0.5  # FastNeighborList.neighbor_marginal (calculator.py:48): generate_neighbor_lists gets cutoff + skin

    def __init__(self):
        self.precision = PREC_FP64
        self._engine = None
        self._gmap = {}
        self._reset_system()
        self._reset_records()

    # ---- life cycle (PyInterface.f90:51-200, 1023-1036) -------------------------
    def start_potentials(self):
        pass

    def start_bond_order_factors(self):
        pass

    def start_mpi(self):
        pass

    def finish_mpi(self):
        pass

    def start_rng(self, seed):
        pass

    def distribute_mpi(self, n_atoms):
        pass

    def release(self):
        if self._engine is not None:
            self._engine.close()
        self._engine = None
        self._reset_system()
        self._reset_records()

    def _reset_system(self):
        self._n = 0
        self._cell = None
        self._pbc = None
        self._pos = np.zeros((0, 3))
        self._charges = np.zeros(0)
        self._tags = []
        self._elements = []
        self._atoms_dirty = True
        self._lists = None  # (counts, idx, off) of the last built or installed lists
        self._pending_lists = None  # per-atom lists handed over with create_neighbor_list
        self._list_skin = self.skin

    def _reset_records(self):
        self._pots = []  # raw add_potential records
        self._multipliers = []  # factors of the next product record
        self._bonds = []  # raw add_bond_order_factor records
        self._ewald = None
        self._model = None
        self._records_dirty = True

    def _eng(self):
        if self._engine is None:
            self._engine = Engine()
        return self._engine

    # ---- system (PyInterface.f90:208-302) -------------------------------------
    def create_cell(self, vectors, inverse, periodicity):
        """vectors: the cell transposed, columns are the cell vectors
        (calculator.py:1555-1565)."""
        self._cell = np.ascontiguousarray(np.transpose(np.asarray(vectors, dtype=np.float64)))
        self._pbc = np.asarray(periodicity, dtype=bool).reshape(3)
        self._eng().set_cell(self._cell, self._pbc)
        self._lists = None

    def create_atoms(self, masses, charges, positions, momenta, tags, elements, n_atoms=None):
        """positions and momenta (3, N), elements (2, N) codes (calculator.py:1600-1626)."""
        pos = np.asarray(positions, dtype=np.float64)
        n = pos.shape[1] if pos.ndim == 2 else len(np.asarray(masses))
        self._n = int(n)
        self._pos = np.ascontiguousarray(pos.reshape(3, -1).T) if n else np.zeros((0, 3))
        self._charges = np.asarray(charges, dtype=np.float64).reshape(-1).copy()
        self._tags = _ints(tags, n)
        self._elements = _codes(elements, n)
        self._atoms_dirty = True
        self._lists = None
        self._model = None

    def get_number_of_atoms(self):
        return self._n

    def update_atom_coordinates(self, positions, momenta=None):
        pos = np.ascontiguousarray(np.asarray(positions, dtype=np.float64).reshape(3, -1).T)
        self._pos = pos
        if not self._atoms_dirty and self._engine is not None:
            self._engine.update_positions(pos)

    def update_atom_charges(self, charges):
        self._charges = np.asarray(charges, dtype=np.float64).reshape(-1).copy()
        if not self._atoms_dirty and self._engine is not None:
            self._engine.update_charges(self._charges)

    # ---- interaction records (PyInterface.f90:370-575) -------------------------
    def allocate_potentials(self, n_pots):
        self._pots = []
        self._records_dirty = True

    def allocate_bond_order_factors(self, n_bonds):
        self._bonds = []
        self._records_dirty = True

    def allocate_bond_order_storage(self, n_atoms, n_groups, n_factors):
        pass

    def clear_potential_multipliers(self):
        self._multipliers = []

    def add_potential(self, pot_name, parameters, cutoff, smooth_cut, elements, tags, indices, orig_elements,
                      orig_tags, orig_indices, pot_index, is_multiplier):
        """One interaction record, targets already permuted by the caller
        (calculator.py:1255-1360).  Returns the success flag.  Factors of a
        product (is_multiplier) are kept, in arrival order, and attached to
        every following record until clear_potential_multipliers."""
        name = str(pot_name)
        if name not in core.POTENTIALS:
            return False
        nt = core.POTENTIALS[name][0]
        rec = {"name": name, "params": [float(x) for x in np.asarray(parameters).reshape(-1)],
               "cutoff": float(cutoff), "soft": float(smooth_cut),
               "elements": _codes(elements, nt), "tags": _ints(tags, nt), "indices": _ints(indices, nt),
               "orig_elements": _codes(orig_elements, nt), "orig_tags": _ints(orig_tags, nt),
               "orig_indices": _ints(orig_indices, nt), "group": int(pot_index)}
        if bool(is_multiplier):
            # a factor of a product: kept until its leading record arrives (Core.f90:909-953)
            self._multipliers.append(rec)
            return True
        rec["multipliers"] = list(self._multipliers)
        self._pots.append(rec)
        self._records_dirty = True
        return True

    def add_bond_order_factor(self, bond_name, parameters, param_split, cutoff, smooth_cut, elements, orig_elements,
                              group_index):
        """One bond-order factor record (unpermuted targets, calculator.py:
        1397-1434).  Returns the success flag."""
        name = str(bond_name)
        if name not in core.BOND_ORDER_FACTORS:
            return False
        nt = core.BOND_ORDER_FACTORS[name][0]
        self._bonds.append({"name": name, "params": [float(x) for x in np.asarray(parameters).reshape(-1)],
                            "cutoff": float(cutoff), "soft": float(smooth_cut), "elements": _codes(elements, nt),
                            "group": int(group_index)})
        self._records_dirty = True
        return True

    def create_potential_list(self):
        self._records_dirty = True

    def create_bond_order_factor_list(self):
        self._records_dirty = True

    def set_ewald_parameters(self, real_cut, k_radius, reciprocal_cut, sigma, epsilon, scaler, n_atoms=None):
        self._ewald = {"rc": float(real_cut), "kc": float(k_radius),
                       "kmax": np.asarray(reciprocal_cut, dtype=np.int32).reshape(3).copy(),
                       "sigma": float(sigma), "eps": float(epsilon),
                       "scaler": np.asarray(scaler, dtype=np.float64).reshape(-1).copy()}
        if self._model is not None:
            self._model.ewald = self._ewald
            self._eng().set_ewald(self._ewald)

    # ---- records folded into types and masks -----------------------------------
    def build_model(self):
        """The collected records as the engine's Model: atom types from the
        element codes (and tags or indices where a record targets them), one
        64-bit type mask per target position, coordinator groups numbered in
        the order of the reference's group indices."""
        pots, bonds, n = self._pots, self._bonds, self._n
        use_tags = any(t != NO_TARGET for p in pots for t in p["tags"])
        targeted = {i for p in pots for i in p["indices"] if i != NO_TARGET}
        sig_of = {}
        types = np.zeros(n, dtype=np.int32)
        for i in range(n):
            sig = (self._elements[i], self._tags[i] if use_tags else None, i if i in targeted else None)
            if sig not in sig_of:
                sig_of[sig] = len(sig_of)
            types[i] = sig_of[sig]
        if len(sig_of) > MAX_TYPES:
            raise core.InvalidPotentialError("more than {0} distinguishable atom types".format(MAX_TYPES))
        sigs = [None] * len(sig_of)
        for s, t in sig_of.items():
            sigs[t] = s

        def mask(target):
            e, g, i = target
            m = 0
            for t, (se, sg, si) in enumerate(sigs):
                if (e is not None and se == e) or (g is not None and sg == g) or (i is not None and si == i):
                    m |= 1 << t
            return m

        def target(rec, k, orig=False):
            ind = rec["orig_indices" if orig else "indices"][k]
            tag = rec["orig_tags" if orig else "tags"][k]
            if ind != NO_TARGET:
                return (None, None, ind)
            if tag != NO_TARGET:
                return (None, tag, None)
            return (rec["orig_elements" if orig else "elements"][k], None, None)

        M = Model()
        M.types, M.type_signatures, M.n_types = types, sigs, len(sigs)
        gids = sorted({b["group"] for b in bonds})
        gmap = {g: k for k, g in enumerate(gids)}
        M.n_groups = len(gids)
        # groups of pair (Tersoff) factors only: the bond-order kernels scale any pair term with them
        pair_level = {gmap[g] for g in gids
                      if all(core.level_of_factor(b["name"]) == 2 for b in bonds if b["group"] == g)}
        mul_blocks = {}  # first factor record of each product's factor list
        for rec in pots:
            kind = rec["name"]
            core.check_engine_support(kind)
            params = list(rec["params"])
            grp = gmap.get(rec["group"], -1)
            nt = len(rec["elements"])
            if nt == 2:
                if kind not in core.PAIR_KIND:
                    raise core.InvalidPotentialError("'{0}' is not a pair potential of the GB300 engine".format(kind))
                if kind in ("charge_pair", "charge_exp", "charge_abs") and grp >= 0 and grp not in pair_level:
                    raise core.InvalidPotentialError("per-atom bond-order scaling of {0} is not evaluated by the GB300 "
                                                     "engine".format(kind))
                if kind == "tabulated":
                    params = _table_record(M, params)
                elif kind == "charge_exp":
                    params = _charge_exp_record(M, params)
                elif kind == "charge_abs":
                    first = len(M.pair_table) // 2
                    M.pair_table.extend([float(x) for x in params[:8]])
                    params = [float(first), 0.0, 0.0, 0.0]
                M.pair_first.append(mask(target(rec, 0, orig=True)))
                M.pair_kind.append(core.PAIR_KIND[kind])
                M.pair_params.append((params + [0.0] * 4)[:4])
                M.pair_cutoff.append(rec["cutoff"])
                M.pair_soft.append(rec["soft"])
                M.pair_mask1.append(mask(target(rec, 0)))
                M.pair_mask2.append(mask(target(rec, 1)))
                M.pair_group.append(grp)
                muls = rec.get("multipliers", [])
                key = tuple(id(mr) for mr in muls)
                shared = key in mul_blocks  # every permuted record of one product shares its factors
                M.pair_nmul.append(len(muls))
                M.pair_mul0.append(mul_blocks[key] if shared else len(M.mul_kind))
                if muls and not shared:
                    mul_blocks[key] = len(M.mul_kind)
                if muls and grp >= 0 and grp not in pair_level:
                    raise core.InvalidPotentialError("products scaled by per-atom bond-order factors are not evaluated by "
                                                     "the GB300 engine")
                for mr in ([] if shared else muls):
                    mk = mr["name"]
                    core.check_engine_support(mk)
                    if mk not in core.PAIR_KIND:
                        raise core.InvalidPotentialError("'{0}' is not a pair potential of the GB300 engine".format(mk))
                    mp = list(mr["params"])
                    if mk == "tabulated":
                        mp = _table_record(M, mp)
                    elif mk == "charge_exp":
                        mp = _charge_exp_record(M, mp)
                    elif mk == "charge_abs":
                        first = len(M.pair_table) // 2
                        M.pair_table.extend([float(x) for x in mp[:8]])
                        mp = [float(first), 0.0, 0.0, 0.0]
                    M.mul_kind.append(core.PAIR_KIND[mk])
                    M.mul_params.append((mp + [0.0] * 4)[:4])
                    M.mul_first.append(mask(target(mr, 0, orig=True)))
            elif nt == 1:
                if kind not in core.SINGLE_KIND:
                    raise core.InvalidPotentialError("'{0}' is not a single-atom term of the GB300 engine".format(kind))
                if grp >= 0 and kind == "charge_self":
                    raise core.InvalidPotentialError("bond-order scaling of charge_self is not evaluated by the "
                                                     "GB300 engine")
                M.single_kind.append(core.SINGLE_KIND[kind])
                M.single_params.append((params + [0.0] * 4)[:4])
                M.single_mask.append(mask(target(rec, 0)))
                M.single_group.append(grp)
            elif nt == 3:
                if kind not in core.TRIPLET_KIND:
                    raise core.InvalidPotentialError("'{0}' is not a three-body potential of the GB300 engine"
                                                     .format(kind))
                if grp >= 0:
                    raise core.InvalidPotentialError("bond-order scaling of three-body potentials is not evaluated "
                                                     "by the GB300 engine")
                M.tri_kind.append(core.TRIPLET_KIND[kind])
                M.tri_params.append((params + [0.0] * 4)[:4])
                M.tri_cutoff.append(rec["cutoff"])
                M.tri_soft.append(rec["soft"])
                M.tri_mask1.append(mask(target(rec, 0)))
                M.tri_mask2.append(mask(target(rec, 1)))
                M.tri_mask3.append(mask(target(rec, 2)))
                M.tri_center.append(mask(target(rec, 1, orig=True)))
            elif nt == 4:
                if kind not in core.QUAD_KIND:
                    raise core.InvalidPotentialError("'{0}' is not a four-body potential of the GB300 engine"
                                                     .format(kind))
                if grp >= 0:
                    raise core.InvalidPotentialError("bond-order scaling of four-body potentials is not evaluated "
                                                     "by the GB300 engine")
                M.quad_kind.append(core.QUAD_KIND[kind])
                M.quad_params.append((params + [0.0] * 4)[:4])
                M.quad_cutoff.append(rec["cutoff"])
                M.quad_soft.append(rec["soft"])
                M.quad_mask.append([mask(target(rec, t)) for t in range(4)])
                M.quad_orig.append([mask(target(rec, t, orig=True)) for t in range(4)])
            else:
                raise core.InvalidPotentialError("{0}-body potentials are not evaluated by the GB300 engine".format(nt))
        for rec in bonds:
            kind = rec["name"]
            core.check_engine_support(kind)
            flat = list(rec["params"])
            g = gmap[rec["group"]]
            el = rec["elements"]
            if kind in core.ATOM_FACTOR_KIND:
                if kind in ("table_bond", "table_scale"):
                    flat = _table_record(M, flat)
                M.afac_kind.append(core.ATOM_FACTOR_KIND[kind])
                M.afac_params.append((flat + [0.0] * 5)[:5])
                M.afac_cutoff.append(rec["cutoff"])
                M.afac_soft.append(rec["soft"])
                M.afac_mask1.append(mask((el[0], None, None)))
                M.afac_mask2.append(mask((el[1], None, None)) if len(el) > 1 else 0)
                M.afac_group.append(g)
            else:
                M.bond_params.append(flat)
                M.bond_cutoff.append(rec["cutoff"])
                M.bond_soft.append(rec["soft"])
                M.bond_mask1.append(mask((el[0], None, None)))
                M.bond_mask2.append(mask((el[1], None, None)))
                M.bond_mask3.append(mask((el[2], None, None)))
                M.bond_group.append(g)
        M.ewald = self._ewald
        self._gmap = gmap
        return M

    def _commit(self):
        """Atoms and records into the engine, if either changed since the last commit."""
        if self._cell is None:
            raise core.InvalidParametersError("no cell: create_cell first")
        if not (self._atoms_dirty or self._records_dirty):
            return
        eng = self._eng()
        M = self.build_model()
        old = self._model
        if self._atoms_dirty or old is None or not np.array_equal(old.types, M.types):
            eng.set_atoms(self._pos, self._charges, M.types)
            if self._lists is not None:  # lists stay valid for the same positions
                eng.install_neighbors(*self._lists, self._list_skin)
        eng.set_model(M)
        self._model = M
        self._atoms_dirty = self._records_dirty = False

    # ---- neighbour lists (PyInterface.f90:528-546, 1062-1096) ---------------------
    def generate_neighbor_lists(self, cutoffs, n_atoms=None):
        """The cell-list build of FastNeighborList.build (calculator.py:62-108);
        cutoffs include the list skin, as ASE's NeighborList hands them over."""
        self._commit()
        eng = self._eng()
        eng.build_neighbors(np.asarray(cutoffs, dtype=np.float64).reshape(-1), self.skin)
        self._lists = eng.neighbor_lists()
        self._list_skin = self.skin
        self._pending_lists = None

    def get_number_of_neighbors_of_atom(self, atom_index):
        if self._lists is None:
            return 0
        return int(self._lists[0][int(atom_index)])

    def get_neighbor_list_of_atom(self, atom_index, n_neighbors):
        """(neighbours, 0-based; offsets, (3, n)) like f2py returns them."""
        counts, idx, off = self._lists
        s = int(np.sum(counts[:int(atom_index)]))
        k = int(n_neighbors)
        return idx[s:s + k].copy(), np.ascontiguousarray(off[s:s + k].T)

    def create_neighbor_list(self, atom_index, neighbors, offsets, n_nbs=None):
        """The list of one atom built elsewhere (ASE's NeighborList for small
        cells, calculator.py:1582-1590): atom_index 1-based, neighbours 0-based,
        offsets (3, n).  Installed on the device before the next evaluation."""
        if self._pending_lists is None:
            self._pending_lists = [None] * self._n
        nb = np.asarray(neighbors, dtype=np.int32).reshape(-1)
        off = np.asarray(offsets, dtype=np.int32).reshape(3, -1).T if len(nb) else np.zeros((0, 3), np.int32)
        self._pending_lists[int(atom_index) - 1] = (nb, off)

    def _ready(self):
        self._commit()
        if self._pending_lists is not None:
            parts = [p if p is not None else (np.zeros(0, np.int32), np.zeros((0, 3), np.int32))
                     for p in self._pending_lists]
            counts = np.array([len(p[0]) for p in parts], dtype=np.int32)
            idx = np.concatenate([p[0] for p in parts]) if parts else np.zeros(0, np.int32)
            off = np.concatenate([p[1] for p in parts]) if parts else np.zeros((0, 3), np.int32)
            self._lists = (counts, idx, off)
            self._list_skin = self.skin
            self._eng().install_neighbors(counts, idx, off, self.skin)
            self._pending_lists = None
        if self._lists is None and self._n > 0:
            raise core.InvalidParametersError("no neighbour lists: generate_neighbor_lists or create_neighbor_list first")
        return self._eng()

    # ---- evaluation (PyInterface.f90:579-692) -------------------------------------
    def calculate_energy(self):
        return float(self._ready().calculate(self.precision, energy=True, forces=False)["energy"])

    def calculate_forces(self, n_atoms):
        """(forces (3, N), stress [xx, yy, zz, yz, xz, xy]) like f2py returns them."""
        r = self._ready().calculate(self.precision, energy=False, forces=True)
        return np.ascontiguousarray(r["forces"].T), r["stress"]

    def calculate_electronegativities(self, n_atoms):
        return self._ready().calculate(self.precision, energy=False, forces=False, enegs=True)["enegs"]

    def calculate_bond_order_factors(self, n_atoms, group_index):
        eng = self._ready()
        g = self._gmap.get(int(group_index))
        if g is None:
            return np.zeros(self._n)
        return eng.atom_factors(g, self.precision)

    def calculate_bond_order_gradients(self, n_atoms, group_index, atom_index):
        """(3, N) gradients of every factor with respect to moving atom_index (1-based)."""
        eng = self._ready()
        g = self._gmap.get(int(group_index))
        if g is None:
            return np.zeros((3, self._n))
        return np.ascontiguousarray(eng.atom_factor_gradients(g, int(atom_index) - 1, False, self.precision).T)

    def calculate_bond_order_gradients_of_factor(self, n_atoms, group_index, atom_index):
        """(3, N) gradients of atom_index's (1-based) factor with respect to moving every atom."""
        eng = self._ready()
        g = self._gmap.get(int(group_index))
        if g is None:
            return np.zeros((3, self._n))
        return np.ascontiguousarray(eng.atom_factor_gradients(g, int(atom_index) - 1, True, self.precision).T)

    # ---- descriptor queries (PyInterface.f90:706-1021), names as plain strings ------
    def number_of_potentials(self):
        return len(core.POTENTIALS)

    def number_of_bond_order_factors(self):
        return len(core.BOND_ORDER_FACTORS)

    def is_potential(self, potential_name):
        return str(potential_name) in core.POTENTIALS

    def is_bond_order_factor(self, bond_order_name):
        return str(bond_order_name) in core.BOND_ORDER_FACTORS

    def number_of_targets_of_potential(self, potential_name):
        return core.POTENTIALS[str(potential_name)][0]

    def number_of_targets_of_bond_order_factor(self, bond_order_name):
        return core.BOND_ORDER_FACTORS[str(bond_order_name)][0]

    def level_of_bond_order_factor(self, bond_order_name):
        return core.BOND_ORDER_FACTORS[str(bond_order_name)][1]

    def number_of_parameters_of_potential(self, potential_name):
        return len(core.POTENTIALS[str(potential_name)][1])

    def number_of_parameters_of_bond_order_factor(self, bond_order_name, n_targets):
        return len(core.BOND_ORDER_FACTORS[str(bond_order_name)][2][int(n_targets) - 1])


pysic_interface = PysicInterface()

__all__ = ["PysicInterface", "pysic_interface", "PREC_FP64", "PREC_MIXED", "NO_TARGET"]
