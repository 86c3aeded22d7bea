"""The COMB potential (CombPotential, pysic/interactions/comb.py) on the GPU
against the oracle, with its full 12 A Coulomb and field ranges on a random
600-atom SiO2 box with random charges.

Every COMB piece at once: bond bending (triplet kernel), Tersoff-scaled
charge_exp x charge_abs x exponential attraction with one Coordinator per
element pair (bond-order kernels), charge_exp x exponential repulsion, field
and Slater-Coulomb products (pair kernel), charge self energies up to q^4
(single-atom kernel) and the Ewald summation the compound puts on the
calculator.  Tolerances: FP64 energy 1e-11 relative, forces 1e-9 of the
largest, virial 1e-9 relative, electronegativities 1e-9 eV/e; mixed
precision 1e-5 eV/atom, 1e-4 of the largest force, 1e-4 eV/e; the damped
charge relaxation: same step count as the oracle's loop and charges within
1e-8 e (FP64).
"""
import numpy as np
import pytest

import oracle
import pysic_gb300 as pysic
from helpers import engine_all, oracle_all, oracle_lists
from pysic_gb300 import workloads as W
from pysic_gb300.model import compile_model

pytestmark = pytest.mark.gpu

VARIANTS = {
    "screened": [],  # the default: real-space Ewald only (k cutoff 0)
    "long_coulomb": ["long_coulomb"],  # k-space Ewald as well
    "direct_coulomb": ["direct_coulomb"],  # bare Coulomb products, no Ewald
}


def _comb_box(variant):
    atoms = W.sio2_box(200, seed=71)
    q = np.random.default_rng(72).normal(0.0, 0.4, len(atoms))
    atoms.set_initial_charges(q - q.mean())
    calc = pysic.Pysic()
    pot = pysic.CombPotential()
    for ex in VARIANTS[variant]:
        pot.include(ex)
    pot.set_calculator(calc, True)
    return atoms, calc.get_potentials(), calc.get_coulomb_summation()


@pytest.mark.parametrize("variant", list(VARIANTS))
def test_comb_parity(variant):
    atoms, pots, coul = _comb_box(variant)
    assert (coul is None) == (variant == "direct_coulomb")
    ref = oracle_all(atoms, pots, coul, threads=8)
    for lanes in (0, 8):
        got = engine_all(atoms, pots, coul, "fp64", lanes)
        assert got["energy"] == pytest.approx(ref["energy"], rel=1e-11)
        assert np.abs(got["forces"] - ref["forces"]).max() < 1e-9 * max(1.0, np.abs(ref["forces"]).max())
        np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())
        assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-9
    mixed = engine_all(atoms, pots, coul, "mixed")
    assert abs(mixed["energy"] - ref["energy"]) / len(atoms) <= 1e-5
    assert np.abs(mixed["forces"] - ref["forces"]).max() < 1e-4 * max(1.0, np.abs(ref["forces"]).max())
    assert np.abs(mixed["enegs"] - ref["enegs"]).max() < 1e-4


def test_comb_dynamic_relaxation_matches_oracle_loop():
    atoms, pots, coul = _comb_box("screened")
    params = dict(n_steps=150, timestep=0.02, inertia=1.0, friction=3.0, tolerance=1e-4)
    calc = pysic.Pysic(atoms.copy(), pots, coulomb=coul, precision="fp64")
    rel = pysic.ChargeRelaxation("dynamic", calculator=calc,
                                 parameters=[params[k] for k in ("n_steps", "timestep", "inertia", "friction",
                                                                 "tolerance")])
    q_gpu = rel.charge_relaxation()
    model = compile_model(atoms, pots, coul)
    r = oracle.relax_charges(atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(),
                             model, *oracle_lists(atoms, pots, coul), threads=8, **params)
    assert rel.last_steps == r["steps"] > 1
    assert np.all(np.isfinite(q_gpu))
    np.testing.assert_allclose(q_gpu, r["charges"], atol=1e-8)
