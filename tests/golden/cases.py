"""Seeded small structures and interaction sets of the golden fixtures.

Each case is small enough for the FP64 oracle to evaluate in well under a
second; `make_golden.py` stores the oracle's neighbour lists, energies, forces,
virials, electronegativities and relaxed charges for them in
`oracle_cases.npz`.  The stored positions, cells and charges are what the
tests read back, so a later change to a structure generator cannot move a
fixture silently.
"""
import numpy as np

from pysic_gb300 import workloads as W
from pysic_gb300.atoms import Atoms


def _tersoff_si64():
    return W.diamond_si(2, noise=0.10, seed=11), W.tersoff_si_potentials(), None


def _lj_fcc108():
    return W.lj_fcc(3, noise=0.05, seed=12), W.lj_potentials(cutoff=6.0), None


def _nacl64_ewald():
    atoms = W.rocksalt_nacl(2, noise=0.05, seed=13)
    pots, coul = W.nacl_potentials(cutoff=5.0, sigma=1.4, real_cutoff=5.0)
    return atoms, pots, coul


def _sio2_120():
    atoms = W.sio2_box(40, seed=14)
    pots, coul = W.sio2_potentials(real_cutoff=5.5, sigma=1.6)
    q = np.where(np.array(atoms.get_chemical_symbols()) == "Si", 0.4, -0.2)
    atoms.set_initial_charges(q)
    return atoms, pots, coul


def _triclinic_si():
    """Sheared Si cell: the neighbour build on a non-orthogonal cell."""
    atoms = W.diamond_si(2, noise=0.10, seed=15)
    cell = atoms.get_cell().copy()
    cell[1, 0] += 2.1
    cell[2, 0] -= 1.3
    cell[2, 1] += 0.9
    atoms.set_cell(cell, scale_atoms=True)
    return atoms, W.tersoff_si_potentials(), None


CASES = {
    "tersoff_si64": _tersoff_si64,
    "lj_fcc108": _lj_fcc108,
    "nacl64_ewald": _nacl64_ewald,
    "sio2_120": _sio2_120,
    "triclinic_si64": _triclinic_si,
}

# charge relaxation settings of the relaxed-charge fixture (sio2_120)
RELAX = {"n_steps": 400, "timestep": 0.1, "inertia": 1.0, "friction": 4.0, "tolerance": 1e-4}


def restore(name, arrays):
    """The case's atoms as stored in the fixture, with its interaction set."""
    _, pots, coul = CASES[name]()
    symbols = [str(s) for s in arrays[name + "/symbols"]]
    atoms = Atoms(symbols, arrays[name + "/positions"], cell=arrays[name + "/cell"],
                  pbc=arrays[name + "/pbc"].astype(bool), charges=arrays[name + "/charges"])
    return atoms, pots, coul
