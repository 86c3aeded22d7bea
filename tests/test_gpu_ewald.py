"""GPU parity of Ewald summation, charge terms and device-resident charge relaxation.

Tolerances: FP64 path within 1e-11 relative (energy), 1e-9 eV/A (forces),
1e-9 eV/e (electronegativities) of the oracle; mixed path within 1e-5 eV/atom
and 1e-3 eV/A of the FP64 path; relaxation: same step count and charges
within 1e-8 e (FP64).
"""
import numpy as np
import pytest

import oracle
import pysic_gb300 as pysic
from helpers import engine_all, oracle_all, oracle_lists
from pysic_gb300 import workloads as W
from pysic_gb300.model import compile_model

pytestmark = pytest.mark.gpu


def _nacl_small():
    atoms = W.rocksalt_nacl(3, noise=0.1, seed=21)
    pots, coul = W.nacl_potentials(sigma=1.6, real_cutoff=6.0, cutoff=6.0)
    return atoms, pots, coul


def test_ewald_fp64_parity():
    atoms, pots, coul = _nacl_small()
    ref = oracle_all(atoms, pots, coul)
    got = engine_all(atoms, pots, coul, "fp64")
    assert got["energy"] == pytest.approx(ref["energy"], rel=1e-11)
    assert np.abs(got["forces"] - ref["forces"]).max() < 1e-9
    assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-9
    np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())


def test_ewald_triclinic_and_scaler_fp64_parity():
    rng = np.random.default_rng(3)
    cell = np.array([[11.0, 0.0, 0.0], [2.5, 10.5, 0.0], [-1.0, 1.5, 12.0]])
    n = 60
    pos = rng.uniform(0, 1, (n, 3)) @ cell
    q = rng.normal(0, 0.5, n)
    q -= q.mean()
    atoms = pysic.Atoms(["Na"] * (n // 2) + ["Cl"] * (n // 2), pos, cell=cell, pbc=True, charges=q)
    scaler = list(rng.uniform(0.5, 1.5, n))
    coul = pysic.CoulombSummation("ewald", [4.0, W.ewald_kcut(1.3), 1.3, W.EPS0], scaler=scaler)
    pots = [pysic.Potential("Buckingham", symbols=[["Na", "Cl"]], parameters=[1000.0, 13717.42, 0.3], cutoff=4.0)]
    ref = oracle_all(atoms, pots, coul)
    got = engine_all(atoms, pots, coul, "fp64")
    assert got["energy"] == pytest.approx(ref["energy"], rel=1e-11)
    # random positions without rejection: some Buckingham forces reach 1e7 eV/A
    assert np.abs(got["forces"] - ref["forces"]).max() < 1e-12 * max(1.0, np.abs(ref["forces"]).max())
    assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-9


def test_ewald_nacl_8000_mixed_vs_fp64():
    atoms = W.rocksalt_nacl()
    pots, coul = W.nacl_potentials()
    a64 = engine_all(atoms, pots, coul, "fp64")
    am = engine_all(atoms, pots, coul, "mixed")
    n = len(atoms)
    print("NaCl 8000 mixed-fp64: dE/atom", abs(am["energy"] - a64["energy"]) / n, "max dF",
          np.abs(am["forces"] - a64["forces"]).max())
    assert abs(am["energy"] - a64["energy"]) / n < 1e-5
    assert np.abs(am["forces"] - a64["forces"]).max() < 1e-3


def test_charge_self_and_ewald_enegs_fp64():
    atoms = W.sio2_box(100, seed=4)
    pots, coul = W.sio2_potentials(real_cutoff=6.0, sigma=1.8)
    q = np.random.default_rng(1).normal(0, 0.4, len(atoms))
    q -= q.mean()
    atoms.set_initial_charges(q)
    ref = oracle_all(atoms, pots, coul)
    got = engine_all(atoms, pots, coul, "fp64")
    assert got["energy"] == pytest.approx(ref["energy"], rel=1e-11)
    assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-9


def test_charge_relaxation_matches_oracle_loop():
    atoms = W.sio2_box(100, seed=5)
    pots, coul = W.sio2_potentials(real_cutoff=6.0, sigma=1.8)
    params = dict(n_steps=400, timestep=0.1, inertia=1.0, friction=4.0, tolerance=1e-4)
    calc = pysic.Pysic(atoms, pots, coulomb=coul, precision="fp64")
    rel = pysic.ChargeRelaxation("dynamic", calculator=calc,
                                 parameters=[params[k] for k in ("n_steps", "timestep", "inertia", "friction",
                                                                 "tolerance")])
    q_gpu = rel.charge_relaxation()
    model = compile_model(atoms, pots, coul)
    lists = oracle_lists(atoms, pots, coul)
    r = oracle.relax_charges(atoms.get_positions(), np.zeros(len(atoms)), atoms.get_cell(), atoms.get_pbc(), model,
                             *lists, **params)
    assert rel.last_steps == r["steps"]
    assert r["steps"] < params["n_steps"]
    np.testing.assert_allclose(q_gpu, r["charges"], atol=1e-8)
    assert abs(q_gpu.sum()) < 1e-9


def test_charge_relaxation_warm_rates_persist():
    atoms = W.sio2_box(60, seed=6)
    pots, coul = W.sio2_potentials(real_cutoff=5.0, sigma=1.6)
    calc = pysic.Pysic(atoms, pots, coulomb=coul)
    rel = pysic.ChargeRelaxation("dynamic", calculator=calc, parameters=[5, 0.1, 1.0, 4.0, 1e-12])
    rel.charge_relaxation()
    assert rel.last_steps == 5 and rel.last_converged is False
    assert np.abs(rel.charge_rates).max() > 0


def test_graph_replay_matches_direct_launches():
    atoms, pots, coul = _nacl_small()
    calc = pysic.Pysic(atoms, pots, coulomb=coul, precision="mixed")
    calc.set_core()
    eng = calc.engine
    a = eng.calculate(1, energy=True, forces=True, enegs=True)
    b = eng.calculate(1, energy=True, forces=True, enegs=True)  # graph replay
    eng.set_graphs(False)
    c = eng.calculate(1, energy=True, forces=True, enegs=True)
    for x in (b, c):
        assert x["energy"] == a["energy"]
        assert np.array_equal(x["forces"], a["forces"])
        assert np.array_equal(x["enegs"], a["enegs"])


def test_potentiostat_matches_oracle_loop():
    """'potentiostat' (relaxation.py:453-481) on the device against the oracle:
    undamped dynamics under a fixed external potential, total charge free."""
    atoms = W.sio2_box(60, seed=8)
    pots, coul = W.sio2_potentials(real_cutoff=5.5, sigma=1.6)
    q0 = np.where(np.array(atoms.get_chemical_symbols()) == "Si", 0.3, -0.15)
    atoms.set_initial_charges(q0)
    params = dict(n_steps=25, timestep=0.02, inertia=1.0, potential=6.0)
    calc = pysic.Pysic(atoms, pots, coulomb=coul, precision="fp64")
    rel = pysic.ChargeRelaxation("potentiostat", calculator=calc,
                                 parameters=[params[k] for k in ("n_steps", "timestep", "inertia", "potential")])
    q_gpu = rel.charge_relaxation()
    model = compile_model(atoms, pots, coul)
    lists = oracle_lists(atoms, pots, coul)
    r = oracle.relax_potentiostat(atoms.get_positions(), q0, atoms.get_cell(), atoms.get_pbc(), model, *lists,
                                  **params)
    assert rel.last_steps == 25
    np.testing.assert_allclose(q_gpu, r["charges"], atol=1e-9)
    np.testing.assert_allclose(rel.charge_rates, r["rates"], atol=1e-9)
    assert abs(q_gpu.sum() - q0.sum()) > 1e-3  # the potentiostat moves the total charge


def test_observers_see_every_due_step_and_do_not_change_the_run():
    """Observers are called at the steps their intervals name, with the atoms
    holding that step's charges; cutting the device loop for them leaves the
    relaxation's steps and charges as they are without observers."""
    atoms = W.sio2_box(60, seed=9)
    pots, coul = W.sio2_potentials(real_cutoff=5.5, sigma=1.6)
    params = [400, 0.1, 1.0, 4.0, 1e-4]

    def make():
        a = atoms.copy()
        a.set_initial_charges(np.zeros(len(a)))
        calc = pysic.Pysic(a, pots, coulomb=coul, precision="fp64")
        return calc, pysic.ChargeRelaxation("dynamic", calculator=calc, parameters=params)

    calc0, plain = make()
    q_plain = plain.charge_relaxation()
    calc1, watched = make()
    seen = []
    watched.add_observer(lambda: seen.append((watched.last_steps, calc1.get_atoms().get_initial_charges())),
                         interval=7)
    seen_steps = []
    watched.add_observer(lambda: seen_steps.append(1), interval=21)
    q_watched = watched.charge_relaxation()
    assert watched.last_steps == plain.last_steps
    assert np.array_equal(q_watched, q_plain)
    assert len(seen) == plain.last_steps // 7
    assert len(seen_steps) == plain.last_steps // 21
    # the charges an observer saw at step 14 are the oracle's after 14 steps
    model = compile_model(atoms, pots, coul)
    lists = oracle_lists(atoms, pots, coul)
    r = oracle.relax_charges(atoms.get_positions(), np.zeros(len(atoms)), atoms.get_cell(), atoms.get_pbc(), model,
                             *lists, n_steps=14, timestep=0.1, inertia=1.0, friction=4.0, tolerance=1e-4)
    np.testing.assert_allclose(seen[1][1], r["charges"], atol=1e-9)


def _optimize_case():
    atoms = W.sio2_box(60, seed=10)
    atoms.set_initial_charges(np.zeros(len(atoms)))
    pots, coul = W.sio2_potentials(real_cutoff=5.5, sigma=1.6)
    return atoms, pots, coul


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_optimize_on_device_reaches_the_dynamic_minimum(precision):
    """'optimize' (relaxation.py:483-488) by projected conjugate gradients on
    the device: the constrained minimum the damped dynamics converge to, in far
    fewer electronegativity evaluations, total charge unchanged."""
    atoms, pots, coul = _optimize_case()
    calc = pysic.Pysic(atoms.copy(), pots, coulomb=coul, precision="fp64")
    dyn = pysic.ChargeRelaxation("dynamic", calculator=calc, parameters=[4000, 0.05, 1.0, 3.0, 1e-9])
    q_dyn = dyn.charge_relaxation()
    assert dyn.last_converged
    calc2 = pysic.Pysic(atoms.copy(), pots, coulomb=coul, precision=precision)
    tol = 1e-9 if precision == "fp64" else 1e-4
    opt = pysic.ChargeRelaxation("optimize", calculator=calc2, parameters=[500, tol])
    q_opt = opt.charge_relaxation()
    assert opt.last_converged and opt.last_error <= tol
    assert opt.last_steps < dyn.last_steps / 3
    np.testing.assert_allclose(q_opt, q_dyn, atol=1e-8 if precision == "fp64" else 2e-5)
    assert abs(q_opt.sum()) < 1e-9
    # the engine keeps the optimised charges
    np.testing.assert_array_equal(calc2.engine.get_charges(), q_opt)


def test_optimize_falls_back_to_slsqp_for_non_quadratic_energies():
    pytest.importorskip("scipy")
    atoms, pots, coul = _optimize_case()
    pots = pots + [pysic.Potential("charge_self", symbols=[["O"]], parameters=[0.05, 4])]
    calc = pysic.Pysic(atoms.copy(), pots, coulomb=coul, precision="fp64")
    calc.set_core()
    assert calc.engine.optimize_charges(0, 100, 1e-6) is None
    opt = pysic.ChargeRelaxation("optimize", calculator=calc, parameters=[200, 1e-8])
    q = opt.charge_relaxation()
    chi = calc.get_electronegativities()
    assert np.abs(chi - chi.mean()).max() < 1e-3
    assert abs(q.sum()) < 1e-6


def _qpair_case():
    atoms = W.sio2_box(100, seed=26)
    q = np.where(np.array(atoms.get_chemical_symbols()) == "Si", 0.5, -0.25)
    atoms.set_initial_charges(q + np.random.default_rng(4).normal(0.0, 0.05, len(q)))
    pots, coul = W.sio2_potentials(real_cutoff=5.5, sigma=1.6)
    P = pysic.Potential
    pots = pots + [P("charge_pair", symbols=[["Si", "O"]], parameters=[0.4, 2, 1], cutoff=3.0, cutoff_margin=0.8),
                   P("charge_pair", symbols=[["O", "O"]], parameters=[0.3, 1, 1], cutoff=2.8, cutoff_margin=0.5)]
    return atoms, pots, coul


def test_charge_pair_fp64_parity():
    """charge_pair (Potentials.f90:4415-4513) beside Ewald and charge_self:
    energy, smooth-cutoff forces, virial and electronegativities."""
    atoms, pots, coul = _qpair_case()
    ref = oracle_all(atoms, pots, coul)
    got = engine_all(atoms, pots, coul, "fp64")
    assert got["energy"] == pytest.approx(ref["energy"], rel=1e-11)
    assert np.abs(got["forces"] - ref["forces"]).max() < 1e-9 * max(1.0, np.abs(ref["forces"]).max())
    np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())
    assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-9


def test_charge_pair_mixed_and_relaxation():
    atoms, pots, coul = _qpair_case()
    ref = oracle_all(atoms, pots, coul)
    got = engine_all(atoms, pots, coul, "mixed")
    assert abs(got["energy"] - ref["energy"]) / len(atoms) <= 1e-5
    assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-4
    # the damped relaxation sees the charge_pair electronegativities
    params = dict(n_steps=600, timestep=0.05, inertia=1.0, friction=3.0, tolerance=1e-4)
    calc = pysic.Pysic(atoms.copy(), pots, coulomb=coul, precision="fp64")
    rel = pysic.ChargeRelaxation("dynamic", calculator=calc,
                                 parameters=[params[k] for k in ("n_steps", "timestep", "inertia", "friction",
                                                                 "tolerance")])
    q_gpu = rel.charge_relaxation()
    model = compile_model(atoms, pots, coul)
    r = oracle.relax_charges(atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(),
                             model, *oracle_lists(atoms, pots, coul), **params)
    assert rel.last_steps == r["steps"]
    np.testing.assert_allclose(q_gpu, r["charges"], atol=1e-8)
    # not quadratic in the charges: 'optimize' leaves the device solver
    assert calc.engine.optimize_charges(0, 10, 1e-4) is None


def _qexp_case():
    atoms = W.sio2_box(100, seed=27)
    q = np.where(np.array(atoms.get_chemical_symbols()) == "Si", 0.5, -0.25)
    atoms.set_initial_charges(q + np.random.default_rng(5).normal(0.0, 0.05, len(q)))
    pots, coul = W.sio2_potentials(real_cutoff=5.5, sigma=1.6)
    P = pysic.Potential
    # Rmax / (Rmax - Rmin) = Qmax / (Qmax - Qmin): eta = 1, a finite beta
    pots = pots + [P("charge_exp", symbols=[["Si", "O"]],
                     parameters=[0.3, 2.0, 1.0, 2.0, 1.0, 3.0, 1.5, 2.4, 1.2, 0.6, 0.4], cutoff=3.0,
                     cutoff_margin=0.8),
                   P("charge_exp", symbols=[["O", "O"]],
                     parameters=[0.2, 2.5, 1.25, 1.8, 0.9, 2.5, 1.25, 1.8, 0.9, 0.5, 0.5], cutoff=2.6,
                     cutoff_margin=0.5)]
    return atoms, pots, coul


def test_charge_exp_parity_and_relaxation():
    """charge_exp (Potentials.f90:3691-3903) beside Ewald and charge_self:
    FP64 energy, smooth-cutoff forces, virial and electronegativities against
    the oracle, the mixed path within its tolerance, and the damped relaxation
    on its electronegativities."""
    atoms, pots, coul = _qexp_case()
    ref = oracle_all(atoms, pots, coul)
    got = engine_all(atoms, pots, coul, "fp64")
    assert got["energy"] == pytest.approx(ref["energy"], rel=1e-11)
    assert np.abs(got["forces"] - ref["forces"]).max() < 1e-9 * max(1.0, np.abs(ref["forces"]).max())
    np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())
    assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-9
    mixed = engine_all(atoms, pots, coul, "mixed")
    assert abs(mixed["energy"] - ref["energy"]) / len(atoms) <= 1e-5
    assert np.abs(mixed["enegs"] - ref["enegs"]).max() < 1e-4
    params = dict(n_steps=600, timestep=0.05, inertia=1.0, friction=3.0, tolerance=1e-4)
    calc = pysic.Pysic(atoms.copy(), pots, coulomb=coul, precision="fp64")
    rel = pysic.ChargeRelaxation("dynamic", calculator=calc,
                                 parameters=[params[k] for k in ("n_steps", "timestep", "inertia", "friction",
                                                                 "tolerance")])
    q_gpu = rel.charge_relaxation()
    model = compile_model(atoms, pots, coul)
    r = oracle.relax_charges(atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(),
                             model, *oracle_lists(atoms, pots, coul), **params)
    assert rel.last_steps == r["steps"]
    np.testing.assert_allclose(q_gpu, r["charges"], atol=1e-8)


def test_charge_abs_parity():
    """charge_abs (Potentials.f90:4525-4728) beside Ewald and charge_self: FP64
    energy, cut-factor forces, virial and electronegativities against the
    oracle; the mixed path within its tolerance."""
    atoms = W.sio2_box(100, seed=29)
    q = np.where(np.array(atoms.get_chemical_symbols()) == "Si", 0.5, -0.25)
    atoms.set_initial_charges(q + np.random.default_rng(7).normal(0.0, 0.05, len(q)))
    pots, coul = W.sio2_potentials(real_cutoff=5.5, sigma=1.6)
    P = pysic.Potential
    pots = pots + [P("charge_abs", symbols=[["Si", "O"]], parameters=[1.0, 0.5, 0.3, 2.0, 0.8, 0.7, -0.2, 1.5],
                     cutoff=3.0, cutoff_margin=0.8),
                   P("charge_abs", symbols=[["O", "O"]], parameters=[0.6, 0.4, -0.1, 2.5, 0.6, 0.4, -0.1, 2.5],
                     cutoff=2.6, cutoff_margin=0.5)]
    ref = oracle_all(atoms, pots, coul)
    got = engine_all(atoms, pots, coul, "fp64")
    assert got["energy"] == pytest.approx(ref["energy"], rel=1e-11)
    assert np.abs(got["forces"] - ref["forces"]).max() < 1e-9 * max(1.0, np.abs(ref["forces"]).max())
    np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())
    assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-9
    mixed = engine_all(atoms, pots, coul, "mixed")
    assert abs(mixed["energy"] - ref["energy"]) / len(atoms) <= 1e-5
    assert np.abs(mixed["enegs"] - ref["enegs"]).max() < 1e-4


@pytest.mark.parametrize("case", [c[0] for c in W.comb_style_cases()])
def test_tersoff_scaled_charge_products_parity_and_relaxation(case):
    """A Tersoff Coordinator on charge-dependent products and on a charge_exp
    (COMB's attraction form, comb.py:660-900), evaluated in the bond-order
    kernels: FP64 energy, forces, virial and electronegativities against the
    oracle (energy 1e-11 relative, forces 1e-9 of the largest, virial 1e-9,
    electronegativities 1e-9), mixed precision within 1e-5 eV/atom, 1e-4 of
    the largest force and 1e-4 eV/e, and the damped relaxation on these
    electronegativities (bond orders fixed with the positions) against the
    oracle's loop: same steps, charges within 1e-8 e.  The second case has
    COMB's layout: one Coordinator per element pair."""
    _, atoms, pots = next(c for c in W.comb_style_cases() if c[0] == case)
    ref = oracle_all(atoms, pots)
    for lanes in (4, 8, 64):
        got = engine_all(atoms, pots, None, "fp64", lanes)
        assert got["energy"] == pytest.approx(ref["energy"], rel=1e-11)
        assert np.abs(got["forces"] - ref["forces"]).max() < 1e-9 * max(1.0, np.abs(ref["forces"]).max())
        np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())
        assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-9
    mixed = engine_all(atoms, pots, None, "mixed")
    fmax = max(1.0, np.abs(ref["forces"]).max())
    assert abs(mixed["energy"] - ref["energy"]) / len(atoms) <= 1e-5
    assert np.abs(mixed["forces"] - ref["forces"]).max() < 1e-4 * fmax
    assert np.abs(mixed["enegs"] - ref["enegs"]).max() < 1e-4
    # the charges' self-energies (the SiO2 workload's chi q + J q^2) give the
    # relaxation its minimum
    pots = pots + [pysic.Potential("charge_self", symbols=[[e]], parameters=[c, n])
                   for e, (chi, hard) in W.SIO2_CHARGE_PARAMS.items() for c, n in ((chi, 1), (hard, 2))]
    params = dict(n_steps=400, timestep=0.05, inertia=1.0, friction=3.0, tolerance=1e-4)
    calc = pysic.Pysic(atoms.copy(), pots, precision="fp64")
    rel = pysic.ChargeRelaxation("dynamic", calculator=calc,
                                 parameters=[params[k] for k in ("n_steps", "timestep", "inertia", "friction",
                                                                 "tolerance")])
    q_gpu = rel.charge_relaxation()
    model = compile_model(atoms, pots)
    r = oracle.relax_charges(atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(),
                             model, *oracle_lists(atoms, pots), **params)
    assert rel.last_steps == r["steps"] > 1
    np.testing.assert_allclose(q_gpu, r["charges"], atol=1e-8)
