"""GPU parity of the per-atom (level-1) bond-order factors: neighbors,
power_bond, c_scale, sqrt_scale (Potentials.f90:5581-6436) scaling single-atom
and pair potentials (Core.f90:2015-2404, 2671-2735, 4095-4239, 4745-4933),
and the Sutton-Chen compound built from them (suttonchen.py:68-176).

Tolerances as in test_gpu_parity.py: FP64 energy 1e-12 relative, forces
1e-10 eV/A, virial 1e-9 relative against the oracle; mixed 1e-5 eV/atom and
1e-4 eV/A against the FP64 result.
"""
import numpy as np
import pytest

import oracle
import pysic_gb300 as pysic
from helpers import engine_all, oracle_all, oracle_lists
from pysic_gb300 import workloads as W
from pysic_gb300.error import EngineError
from pysic_gb300.model import compile_model

pytestmark = pytest.mark.gpu


def _pieces(compounds):
    calc = pysic.Pysic()
    for p in compounds:
        calc.add_potential(p)
    return calc.get_potentials()


def _check_fp64(atoms, pots, lanes=0):
    ref = oracle_all(atoms, pots)
    got = engine_all(atoms, pots, None, "fp64", lanes)
    assert got["energy"] == pytest.approx(ref["energy"], rel=1e-12, abs=1e-11)
    assert np.abs(got["forces"] - ref["forces"]).max() < 1e-10 * max(1.0, np.abs(ref["forces"]).max())
    np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())
    return ref, got


def _scaled_pair_pots():
    count = pysic.BondOrderParameters("neighbors", cutoff=3.2, cutoff_margin=0.7, symbols=[["Cu", "Cu"], ["Cu", "Ag"]])
    scale = pysic.BondOrderParameters("c_scale", parameters=[[0.8, 11.0, 0.5, 0.3, -50.0], []], symbols=[["Cu"]])
    dens = pysic.BondOrderParameters("power_bond", parameters=[[], [2.6, 4.0]], cutoff=4.2, cutoff_margin=0.4,
                                     symbols=[["Ag", "Ag"], ["Ag", "Cu"]])
    P = pysic.Potential
    return [P("exponential", symbols=[["Cu", "Cu"], ["Cu", "Ag"]], parameters=[1.5, 1.2], cutoff=4.0,
              cutoff_margin=0.5, coordinator=pysic.Coordinator([scale, count])),
            P("LJ", symbols=[["Cu", "Ag"], ["Ag", "Ag"]], parameters=[0.05, 2.5], cutoff=4.5),
            P("constant", parameters=[-0.3], symbols=[["Ag"]], coordinator=pysic.Coordinator([dens])),
            P("force", parameters=[0.1, -0.2, 0.05], symbols=[["Ag"]], coordinator=pysic.Coordinator([dens]))]


@pytest.mark.parametrize("lanes", [8, 32])
def test_sutton_chen_fp64_parity(lanes):
    atoms = W.fcc_alloy(4, symbols=("Cu",), noise=0.06, seed=11)
    ref, got = _check_fp64(atoms, _pieces(W.sutton_chen_potentials(("Cu",))), lanes)
    assert np.abs(ref["forces"]).max() > 0.05


def test_sutton_chen_alloy_fp64_parity():
    """Two elements: one density group per element, and each mixed pair counted
    only from the atom the reference's pick makes atom1."""
    atoms = W.fcc_alloy(4, symbols=("Cu", "Ag"), noise=0.06, seed=12)
    _check_fp64(atoms, _pieces(W.sutton_chen_potentials(("Cu", "Ag"))))


def test_scaled_pair_and_single_terms_fp64_parity():
    """A pair potential scaled by a c_scale-processed neighbour count, an
    unscaled pair potential beside it, and constant / force terms scaled by an
    unprocessed power_bond sum (the scaled force term loses its own force, as in
    core_evaluate_local_singlet)."""
    atoms = W.fcc_alloy(4, symbols=("Cu", "Ag"), noise=0.08, seed=13)
    _check_fp64(atoms, _scaled_pair_pots())


def test_sutton_chen_mixed_accuracy():
    atoms = W.fcc_alloy(8, symbols=("Cu", "Ag"), noise=0.06, seed=14)
    pots = _pieces(W.sutton_chen_potentials(("Cu", "Ag")))
    ref = engine_all(atoms, pots, None, "fp64")
    got = engine_all(atoms, pots, None, "mixed")
    n = len(atoms)
    assert abs(got["energy"] - ref["energy"]) / n <= 1e-5
    assert np.abs(got["forces"] - ref["forces"]).max() <= 1e-4 * max(1.0, np.abs(ref["forces"]).max())
    np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-4, atol=1e-4 * np.abs(ref["stress"]).max())


def test_sutton_chen_bit_reproducible():
    atoms = W.fcc_alloy(5, symbols=("Cu", "Ag"), noise=0.06, seed=15)
    pots = _pieces(W.sutton_chen_potentials(("Cu", "Ag")))
    for prec in ("fp64", "mixed"):
        a = engine_all(atoms, pots, None, prec, lanes=8)
        b = engine_all(atoms, pots, None, prec, lanes=8)
        assert a["energy"] == b["energy"]
        assert np.array_equal(a["forces"], b["forces"])


def test_coordinator_factors_match_the_oracle():
    """Coordinator.calculate_bond_order_factors (bondorder.py:493-506) on the
    device: the post-processed per-atom factors of each group."""
    atoms = W.fcc_alloy(4, symbols=("Cu", "Ag"), noise=0.06, seed=16)
    pots = _pieces(W.sutton_chen_potentials(("Cu", "Ag")))
    calc = pysic.Pysic(atoms, pots, precision="fp64")
    atoms.set_calculator(calc)
    model = compile_model(atoms, pots)
    lists = oracle_lists(atoms, pots)
    coords = [p.get_coordinator() for p in pots if p.get_coordinator() is not None]
    assert len(coords) == 2
    for c in coords:
        c.calculate_bond_order_factors()
        got = c.get_bond_order_factors()
        _, want = oracle.atom_factors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), model, *lists,
                                      group=c.get_group_index())
        assert np.abs(want).max() > 1.0
        np.testing.assert_allclose(got, want, rtol=1e-12, atol=1e-12)


def test_sutton_chen_device_md_conserves_energy():
    """Device velocity Verlet on the Sutton-Chen forces: the total energy drifts
    by less than 1e-4 eV/atom over 200 fs at 600 K."""
    atoms = W.fcc_alloy(5, symbols=("Cu",), noise=0.0, seed=17)
    rng = np.random.default_rng(17)
    m = atoms.get_masses()[:, None]
    kT = 8.617333e-5 * 600.0
    p = rng.normal(0.0, 1.0, (len(atoms), 3)) * np.sqrt(m * kT)
    p -= p.mean(axis=0)
    atoms.set_momenta(p)
    calc = pysic.Pysic(atoms, _pieces(W.sutton_chen_potentials(("Cu",))), precision="fp64")
    atoms.set_calculator(calc)

    def total():
        pm = atoms.get_momenta()
        return atoms.get_potential_energy() + 0.5 * np.sum(pm * pm / m)

    e0 = total()
    dyn = pysic.VelocityVerlet(atoms, 1.0 * 0.09822694788464063)  # 1 fs in ASE time units
    dyn.run(200)
    assert abs(total() - e0) / len(atoms) < 1e-4


def test_many_system_launch_rejects_per_atom_factors():
    atoms = W.fcc_alloy(4, symbols=("Cu",), noise=0.05, seed=18)
    from pysic_gb300.batch import BatchedPysic

    calc = pysic.Pysic(atoms, _pieces(W.sutton_chen_potentials(("Cu",))))
    with pytest.raises(EngineError):
        BatchedPysic([calc]).evaluate("fp64")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tabulated_factors_parity(precision, tmp_path, monkeypatch):
    """table_bond summed per atom and post-processed by table_scale
    (Potentials.f90:6496-6765), scaling a constant and a pair potential, on
    two elements, against the oracle."""
    monkeypatch.chdir(tmp_path)
    r = np.linspace(0.0, 6.0, 161)
    v = np.exp(-r / 1.1)
    np.savetxt(str(tmp_path / "table_0011.txt"), np.column_stack([v, 6.0 * (-v / 1.1)]))
    x = np.linspace(0.0, 3.0, 121)
    np.savetxt(str(tmp_path / "table_0012.txt"), np.column_stack([np.sqrt(x + 0.2), 1.5 / np.sqrt(x + 0.2)]))
    atoms = W.fcc_alloy(4, symbols=("Cu", "Ag"), noise=0.08, seed=19)
    bond = pysic.BondOrderParameters("table_bond", parameters=[[], [11, 6.0, 0.9]], cutoff=4.0, cutoff_margin=0.6,
                                     symbols=[["Cu", "Cu"], ["Cu", "Ag"], ["Ag", "Ag"]])
    scale = pysic.BondOrderParameters("table_scale", parameters=[[12, 3.0, -1.3], []], symbols=[["Cu"]])
    P = pysic.Potential
    pots = [P("constant", parameters=[0.7], symbols=[["Cu"], ["Ag"]], coordinator=pysic.Coordinator([scale, bond])),
            P("exponential", symbols=[["Ag", "Ag"]], parameters=[0.4, 1.3], cutoff=4.2,
              coordinator=pysic.Coordinator([scale, bond]))]
    if precision == "fp64":
        _check_fp64(atoms, pots)
        return
    ref = oracle_all(atoms, pots)
    got = engine_all(atoms, pots, None, "mixed")
    assert abs(got["energy"] - ref["energy"]) / len(atoms) <= 1e-5
    assert np.abs(got["forces"] - ref["forces"]).max() <= 1e-4 * max(1.0, np.abs(ref["forces"]).max())


def test_coordinator_gradients_match_the_oracle():
    """Coordinator.get_bond_order_gradients / _of_factor (bondorder.py:508-534)
    on the device against the oracle's restatement of
    core_calculate_bond_order_gradients (Core.f90:1157-1989), two elements."""
    atoms = W.fcc_alloy(4, symbols=("Cu", "Ag"), noise=0.06, seed=20)
    pots = _pieces(W.sutton_chen_potentials(("Cu", "Ag")))
    calc = pysic.Pysic(atoms, pots, precision="fp64")
    atoms.set_calculator(calc)
    model = compile_model(atoms, pots)
    lists = oracle_lists(atoms, pots)
    args = (atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), model) + tuple(lists)
    for c in [p.get_coordinator() for p in pots if p.get_coordinator() is not None]:
        g = c.get_group_index()
        for a in (0, 33, 101):
            got = c.get_bond_order_gradients(a)
            want = oracle.atom_factor_gradients(*args, group=g, atom=a)
            np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-12)
            got = c.get_bond_order_gradients_of_factor(a)
            want = oracle.atom_factor_gradients(*args, group=g, atom=a, of_factor=True)
            np.testing.assert_allclose(got, want, rtol=1e-10, atol=1e-12)
