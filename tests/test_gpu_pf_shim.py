"""The f2py drop-in (pysic_gb300.pf_shim) driven in the reference's call order
(create_atoms, create_cell, add_potential / add_bond_order_factor, the lists,
then separate energy, force and electronegativity passes, as pysic/
calculator.py:918-996, 1063-1447 and 1595-1637 do), against the oracle.
Tolerances as in the parity tests: neighbour lists bit-identical; FP64 energy
1e-12 relative, forces 1e-10 of the largest force, electronegativities 1e-9;
mixed path 1e-5 eV/atom and 1e-4 eV/A."""
import numpy as np
import pytest

import oracle
import pf_driver
import pysic_gb300 as pysic
from helpers import oracle_all, oracle_lists
from pysic_gb300 import pf_shim
from pysic_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _check(atoms, pots, coul=None, precision=pf_shim.PREC_FP64):
    pi = pf_shim.PysicInterface()
    pi.precision = precision
    pf_driver.load(pi, atoms, pots, coul)
    lists = pf_driver.neighbors(pi, atoms, pots, coul)
    c, i, o = oracle_lists(atoms, pots, coul)
    assert np.array_equal([len(x[0]) for x in lists], c)
    assert np.array_equal(np.concatenate([x[0] for x in lists]), i)
    assert np.array_equal(np.concatenate([x[1].T for x in lists]), o)
    n = pi.get_number_of_atoms()
    assert n == len(atoms)
    e = pi.calculate_energy()
    f, s = pi.calculate_forces(n)
    chi = pi.calculate_electronegativities(n)
    assert f.shape == (3, n) and s.shape == (6,)
    ref = oracle_all(atoms, pots, coul)
    if precision == pf_shim.PREC_FP64:
        assert e == pytest.approx(ref["energy"], rel=1e-12, abs=1e-11)
        assert np.abs(f.T - ref["forces"]).max() < 1e-10 * max(1.0, np.abs(ref["forces"]).max())
        np.testing.assert_allclose(s, ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())
        assert np.abs(chi - ref["enegs"]).max() < 1e-9
    else:
        assert abs(e - ref["energy"]) / n < 1e-5
        assert np.abs(f.T - ref["forces"]).max() < 1e-4
    return pi, ref


@pytest.mark.parametrize("precision", [pf_shim.PREC_FP64, pf_shim.PREC_MIXED])
def test_shim_tersoff_silicon(precision):
    _check(W.diamond_si(3, seed=31), W.tersoff_si_potentials(), precision=precision)


def test_shim_ewald_buckingham():
    pots, coul = W.nacl_potentials(cutoff=6.0, sigma=1.6, real_cutoff=6.0)
    _check(W.rocksalt_nacl(3, noise=0.1, seed=32), pots, coul)


def test_shim_moves_atoms_and_keeps_lists():
    atoms = W.diamond_si(3, seed=33)
    pots = W.tersoff_si_potentials()
    pi, _ = _check(atoms, pots)
    moved = atoms.get_positions() + np.random.default_rng(2).normal(0, 0.03, (len(atoms), 3))
    pi.update_atom_coordinates(moved.T, np.zeros((3, len(atoms))))
    f, _ = pi.calculate_forces(len(atoms))
    m = pysic.Atoms(atoms.get_chemical_symbols(), moved, cell=atoms.get_cell(), pbc=True)
    ref = oracle_all(m, pots, lists=oracle_lists(atoms, pots))  # the same (skin-covered) lists
    assert np.abs(f.T - ref["forces"]).max() < 1e-10 * max(1.0, np.abs(ref["forces"]).max())


def test_shim_lists_installed_atom_by_atom():
    """The small-cell route: ASE's list handed over with create_neighbor_list
    (calculator.py:1582-1590)."""
    atoms = W.lj_fcc(2, noise=0.05, seed=34)
    pots = W.lj_potentials(cutoff=5.0)
    pi = pf_shim.PysicInterface()
    pf_driver.load(pi, atoms, pots)
    c, i, o = oracle_lists(atoms, pots)
    start = np.concatenate([[0], np.cumsum(c)])
    for a in range(len(atoms)):
        pi.create_neighbor_list(a + 1, i[start[a]:start[a + 1]], o[start[a]:start[a + 1]].T)
    e = pi.calculate_energy()
    ref = oracle_all(atoms, pots, lists=(c, i, o))
    assert e == pytest.approx(ref["energy"], rel=1e-12)


def test_shim_coordinator_queries():
    atoms = W.fcc_alloy(3, symbols=("Cu",), noise=0.05, seed=35)
    calc = pysic.Pysic()
    calc.add_potential(W.sutton_chen_potentials(("Cu",)))
    pots = calc.get_potentials()
    pi = pf_shim.PysicInterface()
    coords = pf_driver.load(pi, atoms, pots)
    pf_driver.neighbors(pi, atoms, pots)
    n = len(atoms)
    group = coords[0][1]
    fac = pi.calculate_bond_order_factors(n, group)
    ref = oracle_all(atoms, pots)
    c, i, o = ref["lists"]
    _, rfac = oracle.atom_factors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), ref["model"], c, i, o, 0)
    np.testing.assert_allclose(fac, rfac, rtol=1e-12)
    g = pi.calculate_bond_order_gradients(n, group, 5)  # 1-based atom index, (3, N)
    rg = oracle.atom_factor_gradients(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), ref["model"],
                                      c, i, o, 0, 4, of_factor=False)
    assert g.shape == (3, n)
    np.testing.assert_allclose(g.T, rg, rtol=1e-10, atol=1e-12)


@pytest.mark.parametrize("precision", [pf_shim.PREC_FP64, pf_shim.PREC_MIXED])
def test_shim_dihedral_and_bend(precision):
    """Four-body records through add_potential (four-element targets and
    originals, as calculator.py passes them) with bond_bend and a pair term."""
    _, atoms, pots = list(W.dihedral_cases())[1]
    _check(atoms, pots, precision=precision)


@pytest.mark.parametrize("case", [c[0] for c in W.comb_style_cases()])
def test_shim_tersoff_scaled_charge_products(case):
    """Products registered as the reference does (factors last to first with
    is_multiplier, then the lead's permuted records, clear_potential_multipliers)
    under a Tersoff Coordinator: energy, forces and electronegativities against
    the oracle."""
    _, atoms, pots = next(c for c in W.comb_style_cases() if c[0] == case)
    _check(atoms, pots)
