"""The Pysic calculator on the GB300 engine.

Mirrors pysic/calculator.py:192-1832 of the reference: an ASE calculator
(``get_potential_energy``, ``get_forces``, ``get_stress``) plus Pysic's own
queries (``get_electronegativities``, ``get_charges``, numerical-derivative
helpers), with the same caching rules and the same neighbour-list policy
(FastNeighborList when every cell width exceeds the largest cutoff plus skin,
calculator.py:798-858; otherwise an all-pairs list with ASE NeighborList
semantics).  Where the reference keeps one global Fortran core
(``Pysic.core``, calculator.py:221), each calculator here owns an engine
context; ``precision='mixed'`` selects the FP32-per-term kernels.
"""
import copy
import math

import numpy as np

from . import _lib as L
from .engine import Engine
from .error import EngineError, InvalidPotentialError, MissingAtomsError, warn
from .interactions import CompoundPotential, CoulombSummation, Potential  # noqa: F401  (re-exported API)
from .model import compile_model, individual_cutoffs


def _charges_of(atoms):
    try:
        return np.asarray(atoms.get_initial_charges(), dtype=np.float64)
    except AttributeError:
        return np.asarray(atoms.get_charges(), dtype=np.float64)


def _set_charges(atoms, q):
    try:
        atoms.set_initial_charges(q)
    except AttributeError:
        atoms.set_charges(q)


def _fast_list_applies(cell, pbc, max_cut):
    """calculator.py:829-848: every perpendicular cell width >= max cutoff."""
    cell = np.asarray(cell, dtype=np.float64)
    for i in range(3):
        normal = np.cross(cell[(i + 1) % 3], cell[(i + 2) % 3])
        nn = math.sqrt(np.dot(normal, normal))
        if nn == 0.0:
            return False
        if math.fabs(np.dot(cell[i], normal)) / nn < max_cut:
            return False
    return True


class FastNeighborList:
    """Cell-list neighbour list (pysic/calculator.py:29-189).

    ``cutoffs`` are per-atom interaction ranges; the list radius of atom i is
    cutoffs[i] + skin, and the list of atom i holds every image of every atom
    closer than that (one atom may appear with several offsets in small cells).
    The build runs on the GPU and reproduces the reference's lists entry for
    entry, order included."""

    neighbor_marginal = 0.5

    def __init__(self, cutoffs, skin=None):
        if skin is None:
            skin = FastNeighborList.neighbor_marginal
        self.skin = float(skin)
        self.cutoffs = np.asarray(cutoffs, dtype=np.float64) + self.skin
        self.nupdates = 0
        self._flat = None       # (counts, neighbour indices, offsets) as the engine returns them
        self._lists = None      # per-atom arrays, made from _flat on first use
        self._source = None     # engine whose lists have not been downloaded yet
        self.positions = None
        self.pbc = None
        self.cell = None
        self.all_pairs = False

    def _store(self, counts, idx, off):
        self._flat = (counts, idx, off)
        self._lists = None
        self._source = None

    def _per_atom(self):
        """The per-atom neighbour and offset arrays, downloaded and split on
        first use (a long run of device rebuilds needs none of them)."""
        if self._source is not None:
            self._store(*self._source.neighbor_lists())
        if self._lists is None:
            if self._flat is None:
                return [], []
            counts, idx, off = self._flat
            starts = np.concatenate([[0], np.cumsum(counts)])
            self._lists = ([idx[starts[i]:starts[i + 1]].copy() for i in range(len(counts))],
                           [off[starts[i]:starts[i + 1]].copy() for i in range(len(counts))])
        return self._lists

    @property
    def counts(self):
        self._per_atom()
        return None if self._flat is None else self._flat[0]

    @property
    def neighbors(self):
        return self._per_atom()[0]

    @property
    def displacements(self):
        return self._per_atom()[1]

    def build(self, atoms, engine=None):
        """Build the list for ``atoms`` (calculator.py:62-108).  With no engine
        given, a private engine context holds the structure."""
        own = engine is None
        if own:
            engine = Engine()
            engine.set_cell(atoms.get_cell(), atoms.get_pbc())
            engine.set_atoms(atoms.get_positions(), np.zeros(len(atoms)), np.zeros(len(atoms), dtype=np.int32))
        if self.all_pairs:
            engine.build_all_pairs(self.cutoffs, self.skin)
        else:
            engine.build_neighbors(self.cutoffs, self.skin)
        if own:
            self._store(*engine.neighbor_lists())
        else:
            self._source = engine  # downloaded when first asked for
            self._lists = None
        self.positions = np.array(atoms.get_positions())
        self.pbc = np.array(atoms.get_pbc())
        self.cell = np.array(atoms.get_cell())
        self.nupdates += 1
        if own:
            engine.close()

    def needs_update(self, atoms):
        """ASE NeighborList.update policy: rebuild when the cell, periodicity or
        atom count changed, or some atom moved more than skin/2."""
        if self.positions is None or len(atoms) != len(self.positions):
            return True
        if not np.array_equal(self.pbc, atoms.get_pbc()) or not np.array_equal(self.cell, atoms.get_cell()):
            return True
        if len(atoms) == 0:
            return False
        d2 = ((np.asarray(atoms.get_positions()) - self.positions) ** 2).sum(axis=1)
        return bool(d2.max() > (0.5 * self.skin) ** 2)

    def rebuild_on_device(self, engine, positions):
        """Rebuild the engine's lists from its own (device) coordinates, as the
        device dynamics loop asks; ``positions`` are those coordinates.  The
        host copy of the lists is refreshed by ``refresh_from(engine)``."""
        if self.all_pairs:
            engine.build_all_pairs(self.cutoffs, self.skin)
        else:
            engine.build_neighbors(self.cutoffs, self.skin)
        self.positions = np.array(positions)
        self.nupdates += 1

    def refresh_from(self, engine):
        """The engine's current lists become this list's (downloaded when
        first asked for)."""
        self._source = engine
        self._lists = None

    def update(self, atoms, engine=None):
        if self.needs_update(atoms):
            self.build(atoms, engine)
            return True
        return False

    def get_neighbors(self, index, atoms=None, sort=False):
        nbors = self.neighbors[index]
        displ = self.displacements[index]
        if sort and atoms is not None and len(nbors) > 0:
            d = self.get_neighbor_distances(index, atoms)
            order = np.argsort(d, kind="stable")
            return nbors[order], displ[order]
        return nbors, displ

    def get_neighbor_separations(self, index, atoms, sort=False):
        indices, offsets = self.get_neighbors(index)
        pos = np.asarray(atoms.get_positions())
        cell = np.asarray(atoms.get_cell())
        seps = pos[indices] + offsets @ cell - pos[index]
        if sort:
            order = np.argsort(np.sqrt((seps ** 2).sum(axis=1)), kind="stable")
            return seps[order]
        return seps

    def get_neighbor_distances(self, index, atoms, sort=False):
        d = np.sqrt((self.get_neighbor_separations(index, atoms) ** 2).sum(axis=1))
        return np.sort(d) if sort else d


class Pysic:
    """ASE calculator on the GB300 engine (pysic/calculator.py:192-1832)."""

    def __init__(self, atoms=None, potentials=None, charge_relaxation=None, coulomb=None, full_initialization=False,
                 precision="fp64"):
        self.structure = None
        self.neighbor_list = None
        self.potentials = []
        self.charge_relaxation = None
        self.coulomb = None
        self.charges = None
        self.forces = None
        self.stress = None
        self.energy = None
        self.electronegativities = None
        self.extra_calculators = []
        self.force_core_initialization = full_initialization
        self.set_precision(precision)
        self._engine = None
        self._pushed = None
        self.set_atoms(atoms)
        self.set_potentials(potentials)
        self.set_charge_relaxation(charge_relaxation)
        self.set_coulomb_summation(coulomb)

    # --- configuration ------------------------------------------------------
    def set_precision(self, precision):
        """'fp64' (default: every operation in FP64) or 'mixed' (FP32 per pair
        and triplet, FP64 accumulation)."""
        if precision not in ("fp64", "mixed"):
            raise ValueError("precision must be 'fp64' or 'mixed'")
        self.precision = precision
        self._invalidate()

    def _prec(self):
        return L.PREC_FP64 if self.precision == "fp64" else L.PREC_MIXED

    def _invalidate(self):
        self.forces = None
        self.energy = None
        self.stress = None
        self.electronegativities = None

    def __repr__(self):
        return "Pysic(atoms={0},potentials={1},full_initialization={2})".format(
            self.structure, self.potentials, self.force_core_initialization)

    def core_initialization_is_forced(self):
        return self.force_core_initialization

    def set_atoms(self, atoms=None):
        """Keep a copy of the structure; results are dropped when it changes
        (calculator.py:537-601)."""
        if atoms is None:
            return
        changed = self.structure is None or self.structure != atoms or \
            not np.array_equal(_charges_of(self.structure), _charges_of(atoms))
        if changed:
            self._invalidate()
            self.structure = atoms.copy()

    def get_atoms(self):
        return self.structure

    def set_potentials(self, potentials):
        self.potentials = []
        if potentials is None:
            return
        self._invalidate()
        for p in (potentials if isinstance(potentials, list) else [potentials]):
            self.add_potential(p)

    def add_potential(self, potential):
        for p in (potential if isinstance(potential, list) else [potential]):
            if isinstance(p, CompoundPotential):
                p.build(self)
            else:
                self.potentials.append(p)
                # Coordinator queries (calculate_bond_order_factors) go to this calculator
                if p.get_coordinator() is not None:
                    p.get_coordinator()._calculator = self
        self._invalidate()

    def remove_potential(self, potential):
        if isinstance(potential, CompoundPotential):
            potential.remove(self)
            return
        pots = list(self.potentials)
        pots.remove(potential)
        self.set_potentials(pots)

    def get_potentials(self):
        return self.potentials

    def add_calculator(self, calculator):
        for c in (calculator if isinstance(calculator, list) else [calculator]):
            self.extra_calculators.append(c)
        self._invalidate()

    def remove_calculator(self, calculator):
        self.extra_calculators.remove(calculator)
        self._invalidate()

    def get_calculators(self):
        return self.extra_calculators

    def set_coulomb_summation(self, coulomb):
        self.coulomb = coulomb
        self._invalidate()

    def get_coulomb_summation(self):
        return self.coulomb

    def set_charge_relaxation(self, charge_relaxation):
        try:
            charge_relaxation.set_calculator(self, reciprocal=False)
        except AttributeError:
            pass
        self.charge_relaxation = charge_relaxation

    def get_charge_relaxation(self):
        return self.charge_relaxation

    def get_individual_cutoffs(self, scaler=1.0):
        if self.structure is None:
            return None
        return individual_cutoffs(self.structure, self.potentials, self.coulomb, scaler)

    def get_neighbor_lists(self):
        return self.neighbor_list

    get_neighbor_list = get_neighbor_lists

    def create_neighbor_lists(self, cutoffs=None, marginal=None):
        """Choose the list type and create it (calculator.py:798-858)."""
        if marginal is None:
            marginal = FastNeighborList.neighbor_marginal
        if cutoffs is None:
            cutoffs = self.get_individual_cutoffs(1.0)
        max_cut = (max(cutoffs) if len(cutoffs) else 0.0) + marginal
        self.neighbor_list = FastNeighborList(cutoffs, skin=marginal)
        self.neighbor_list.all_pairs = not _fast_list_applies(self.structure.get_cell(), self.structure.get_pbc(),
                                                              max_cut)
        self._pushed = None if self._pushed is None else dict(self._pushed, lists=False)

    def calculation_required(self, atoms=None, quantities=("forces", "energy", "stress", "electronegativities")):
        if isinstance(quantities, str):
            quantities = [quantities]
        attr = {"energy": "energy", "forces": "forces", "stress": "stress",
                "electronegativities": "electronegativities"}
        # the structure changed in place since the last evaluation (charges set
        # through get_atoms(), as the relaxations do): every cached result is stale
        if self._engine_stale():
            self._invalidate()
            return True
        need = [getattr(self, attr[q]) is None for q in quantities if q in attr]
        return any(need)

    # --- engine synchronisation (set_core, calculator.py:998-1637) ------------
    def _engine_stale(self):
        if self._pushed is None or self.structure is None:
            return True
        s = self.structure
        p = self._pushed
        return not (p["n"] == len(s) and np.array_equal(p["positions"], s.get_positions())
                    and np.array_equal(p["charges"], _charges_of(s)) and np.array_equal(p["cell"], s.get_cell())
                    and np.array_equal(p["pbc"], s.get_pbc()) and p["symbols"] == s.get_chemical_symbols()
                    and np.array_equal(p["tags"], s.get_tags()) and p["potentials"] == self.potentials
                    and p["coulomb"] == self.coulomb and p.get("lists", False))

    def set_core(self):
        if self.structure is None:
            raise MissingAtomsError("No atoms assigned to the calculator.")
        s = self.structure
        p = self._pushed
        full = (self._engine is None or p is None or self.force_core_initialization or p["n"] != len(s)
                or p["symbols"] != s.get_chemical_symbols() or not np.array_equal(p["tags"], s.get_tags())
                or p["potentials"] != self.potentials or p["coulomb"] != self.coulomb)
        if full:
            if self._engine is None:
                self._engine = Engine()
            model = compile_model(s, self.potentials, self.coulomb)
            self._model = model
            q = _charges_of(s)
            tq = float(np.sum(q))
            if abs(tq) > 0.001:
                warn("There is non-zero total charge in the system: {0}".format(tq), 5)
            self._engine.set_cell(s.get_cell(), s.get_pbc())
            self._engine.set_atoms(s.get_positions(), q, model.types)
            self._engine.set_model(model)
            self.create_neighbor_lists()
            self.neighbor_list.build(s, self._engine)
        else:
            cell, pbc = s.get_cell(), s.get_pbc()
            cell_changed = not (np.array_equal(p["cell"], cell) and np.array_equal(p["pbc"], pbc))
            if cell_changed:
                self._engine.set_cell(cell, pbc)
                if self.coulomb is not None:
                    self._model.ewald = None
                    from .model import ewald_settings
                    self._engine.set_ewald(ewald_settings(s, self.coulomb))
            pos = s.get_positions()
            if not np.array_equal(p["positions"], pos) or cell_changed:
                self._engine.update_positions(pos)
            q = _charges_of(s)
            if not np.array_equal(p["charges"], q):
                self._engine.update_charges(q)
            if self.neighbor_list is None or not p.get("lists", False) or cell_changed:
                self.create_neighbor_lists()
                self.neighbor_list.build(s, self._engine)
            else:
                self.neighbor_list.update(s, self._engine)
            # the interaction set compared equal above: its stored copy stays
            self.charges = q
            # get_positions / get_cell / ... hand out copies: kept as they are
            p.update({"positions": np.asarray(pos, dtype=np.float64), "charges": np.array(q, dtype=np.float64),
                      "cell": cell, "pbc": pbc, "lists": True})
            return
        self.charges = _charges_of(s)
        self._pushed = {"n": len(s), "positions": s.get_positions(), "charges": _charges_of(s),
                        "cell": s.get_cell(), "pbc": s.get_pbc(), "symbols": s.get_chemical_symbols(),
                        "tags": s.get_tags(), "potentials": copy.deepcopy(self.potentials),
                        "coulomb": copy.deepcopy(self.coulomb), "lists": True}

    @property
    def engine(self):
        return self._engine

    # --- calculations (calculator.py:918-996) -----------------------------------
    def _run(self, energy=False, forces=False, enegs=False):
        self.set_core()
        return self._engine.calculate(self._prec(), energy=energy, forces=forces, enegs=enegs)

    def calculate_electronegativities(self):
        self.electronegativities = self._run(enegs=True)["enegs"]

    def calculate_forces(self, skip_charge_relaxation=False):
        if self.charge_relaxation is not None and not skip_charge_relaxation:
            self.charge_relaxation.charge_relaxation()
        r = self._run(energy=True, forces=True)
        self.forces, self.stress, self.energy = r["forces"], r["stress"], r["energy"]
        self._add_extra("forces")

    def calculate_energy(self, skip_charge_relaxation=False):
        if self.charge_relaxation is not None and not skip_charge_relaxation:
            self.charge_relaxation.charge_relaxation()
        self.energy = self._run(energy=True)["energy"]
        self._add_extra("energy")

    def calculate_stress(self, skip_charge_relaxation=False):
        self.calculate_forces(skip_charge_relaxation)

    def _add_extra(self, what):
        if not self.extra_calculators:
            return
        system_copy = self.structure.copy()
        for calc in self.extra_calculators:
            if what == "energy":
                self.energy = self.energy + calc.get_potential_energy(system_copy)
            else:
                self.forces = self.forces + calc.get_forces(system_copy)
                self.stress = self.stress + calc.get_stress(system_copy)

    def get_electronegativities(self, atoms=None):
        self.set_atoms(atoms)
        if self.calculation_required(atoms, "electronegativities"):
            self.calculate_electronegativities()
        return np.copy(self.electronegativities)

    def get_electronegativity_differences(self, atoms=None):
        """chi - mean(chi), calculator.py:411-416"""
        enegs = self.get_electronegativities(atoms)
        return enegs - enegs.sum() / len(enegs)

    def get_forces(self, atoms=None, skip_charge_relaxation=False):
        self.set_atoms(atoms)
        if self.calculation_required(atoms, "forces"):
            self.calculate_forces(skip_charge_relaxation=skip_charge_relaxation)
        return np.copy(self.forces)

    def get_potential_energy(self, atoms=None, force_consistent=False, skip_charge_relaxation=False):
        self.set_atoms(atoms)
        if self.calculation_required(atoms, "energy"):
            self.calculate_energy(skip_charge_relaxation=skip_charge_relaxation)
        return self.energy

    def get_stress(self, atoms=None, skip_charge_relaxation=False):
        """-(kinetic + virial)/V in the order xx, yy, zz, yz, xz, xy
        (calculator.py:468-534)."""
        self.set_atoms(atoms)
        if self.calculation_required(atoms, "stress"):
            self.calculate_stress(skip_charge_relaxation=skip_charge_relaxation)
        mom = np.asarray(self.structure.get_momenta())
        masses = np.asarray(self.structure.get_masses())
        vel = mom / masses[:, None] if len(masses) else mom
        kin = np.array([np.dot(mom[:, 0], vel[:, 0]), np.dot(mom[:, 1], vel[:, 1]), np.dot(mom[:, 2], vel[:, 2]),
                        np.dot(mom[:, 1], vel[:, 2]), np.dot(mom[:, 0], vel[:, 2]), np.dot(mom[:, 0], vel[:, 1])])
        return np.copy(-(kin + self.stress) / self.structure.get_volume())

    def get_charges(self, system=None):
        if self.charges is not None:
            return self.charges
        src = system if system is not None else self.structure
        return _charges_of(src)

    # --- numerical checks (calculator.py:1639-1832) ----------------------------------
    def get_numerical_energy_gradient(self, atom_index, shift=0.0001, atoms=None):
        """Central-difference -dE/dr of one atom (calculator.py:1639-1677)."""
        system = self.structure.copy() if atoms is None else atoms.copy()
        orig = system.copy()
        out = []
        for c in range(3):
            pos = system.get_positions()
            pos[atom_index, c] += shift
            system.set_positions(pos)
            ep = self.get_potential_energy(system)
            pos[atom_index, c] -= 2.0 * shift
            system.set_positions(pos)
            em = self.get_potential_energy(system)
            pos[atom_index, c] += shift
            system.set_positions(pos)
            out.append(-(ep - em) / (2.0 * shift))
        self.get_potential_energy(orig)
        return out

    def get_numerical_electronegativity(self, atom_index, shift=0.001, atoms=None):
        """Central-difference -dE/dq of one atom (calculator.py:1782-1832)."""
        system = self.structure.copy() if atoms is None else atoms.copy()
        orig = self.structure.copy()
        q = _charges_of(system).copy()
        q[atom_index] += shift
        _set_charges(system, q)
        ep = self.get_potential_energy(system)
        q[atom_index] -= 2.0 * shift
        _set_charges(system, q)
        em = self.get_potential_energy(system)
        self.set_atoms(orig)
        return (em - ep) / (2.0 * shift)

    def get_bond_zeta(self):
        """Tersoff sums zeta_ij of every ordered bond of the engine's short list
        (the quantity core_calculate_pair_bond_order_factor accumulates)."""
        self.set_core()
        return self._engine.bond_zeta()


__all__ = ["Pysic", "FastNeighborList", "InvalidPotentialError", "EngineError"]
