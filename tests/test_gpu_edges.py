"""Edge cases of the evaluation path on the GPU: an empty system, atoms without
neighbours, a ragged cluster in vacuum (non-periodic, list lengths from zero
to full), a lone ion under Ewald (non-neutral: background term), each against
the oracle where it has something to say."""
import numpy as np
import pytest

import pysic_gb300 as pysic
from helpers import engine_all, oracle_all
from pysic_gb300 import workloads as W

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_empty_system(precision):
    atoms = pysic.Atoms([], np.zeros((0, 3)), cell=np.eye(3) * 10.0, pbc=True)
    for pots, coul in ((W.lj_potentials(), None), (W.tersoff_si_potentials(), None),
                       W.nacl_potentials(cutoff=4.0, sigma=1.2, real_cutoff=4.0)):
        calc = pysic.Pysic(atoms.copy(), pots, coulomb=coul, precision=precision)
        assert calc.get_potential_energy() == 0.0
        assert calc.get_forces().shape == (0, 3)
        assert np.array_equal(calc.get_stress(), np.zeros(6))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_atoms_without_neighbours(precision):
    pos = np.array([[1.0, 1.0, 1.0], [21.0, 1.0, 1.0], [1.0, 21.0, 1.0], [11.0, 11.0, 31.0]])
    atoms = pysic.Atoms(["X"] * 4, pos, cell=np.eye(3) * 40.0, pbc=True)
    got = engine_all(atoms, W.lj_potentials(cutoff=8.5), None, precision)
    assert got["energy"] == 0.0
    assert np.array_equal(got["forces"], np.zeros((4, 3)))


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_ragged_cluster_in_vacuum(precision):
    """A 64-atom Si crystallite, non-periodic, with three far atoms: list
    lengths 0 to 4 and bonds cut at the surface."""
    core = W.diamond_si(2, noise=0.08, seed=41)
    pos = np.vstack([core.get_positions() + 5.0, [[40.0, 5.0, 5.0], [5.0, 40.0, 5.0], [42.0, 42.0, 42.0]]])
    atoms = pysic.Atoms(["Si"] * len(pos), pos, cell=np.eye(3) * 50.0, pbc=False)
    pots = W.tersoff_si_potentials()
    ref = oracle_all(atoms, pots)
    got = engine_all(atoms, pots, None, precision)
    n = len(atoms)
    if precision == "fp64":
        assert got["energy"] == pytest.approx(ref["energy"], rel=1e-12)
        assert np.abs(got["forces"] - ref["forces"]).max() < 1e-10 * max(1.0, np.abs(ref["forces"]).max())
    else:
        assert abs(got["energy"] - ref["energy"]) / n <= 1e-5
        assert np.abs(got["forces"] - ref["forces"]).max() <= 1e-4
    assert np.array_equal(got["forces"][-3:], np.zeros((3, 3)))


def test_lone_ion_under_ewald():
    """One charged ion in a periodic box: only self, background and its own
    images contribute (Potentials.f90:1428-1653)."""
    atoms = pysic.Atoms(["Na"], [[1.0, 2.0, 3.0]], cell=np.eye(3) * 12.0, pbc=True, charges=[1.0])
    pots, coul = W.nacl_potentials(cutoff=5.0, sigma=1.4, real_cutoff=5.0)
    ref = oracle_all(atoms, pots, coul)
    got = engine_all(atoms, pots, coul, "fp64")
    assert got["energy"] == pytest.approx(ref["energy"], rel=1e-11)
    assert np.abs(got["forces"]).max() < 1e-12
    assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-10
