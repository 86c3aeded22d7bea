"""GPU path against the stored golden fixtures (tests/golden/).

No oracle call at run time: the numbers compared against are the documented
values of the reference (reference_docs.json) and the oracle outputs stored in
oracle_cases.npz.  Tolerances as in the parity tests: neighbour lists
bit-identical; FP64 energy 1e-12 relative, forces 1e-10 relative to the largest
force, virial 1e-9 relative; mixed precision 1e-5 eV/atom and 1e-4 eV/A;
relaxed charges 1e-8 e with the same number of steps.
"""
import json
import os
import sys

import numpy as np
import pytest

import pysic_gb300 as pysic
from pysic_gb300 import _lib as L

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
sys.path.insert(0, GOLDEN)
import cases  # noqa: E402

G = np.load(os.path.join(GOLDEN, "oracle_cases.npz"))
NAMES = list(cases.CASES)


def _calc(name, precision="fp64"):
    atoms, pots, coul = cases.restore(name, G)
    calc = pysic.Pysic(atoms, pots, coulomb=coul, precision=precision)
    calc.set_core()
    return atoms, calc


@pytest.mark.parametrize("name", NAMES)
def test_neighbor_lists_match_fixture(name):
    _, calc = _calc(name)
    c, i, o = calc.engine.neighbor_lists()
    p = name + "/"
    np.testing.assert_array_equal(c, G[p + "nb_counts"])
    np.testing.assert_array_equal(i, G[p + "nb_index"])
    np.testing.assert_array_equal(o, G[p + "nb_offset"])


@pytest.mark.parametrize("name", NAMES)
def test_fp64_matches_fixture(name):
    _, calc = _calc(name)
    r = calc.engine.calculate(L.PREC_FP64, energy=True, forces=True, enegs=True)
    p = name + "/"
    e = float(G[p + "energy"])
    assert abs(r["energy"] - e) <= 1e-12 * max(1.0, abs(e))
    f = G[p + "forces"]
    assert np.abs(r["forces"] - f).max() <= 1e-10 * max(1.0, np.abs(f).max())
    s = G[p + "stress"]
    assert np.abs(r["stress"] - s).max() <= 1e-9 * max(1.0, np.abs(s).max())
    chi = G[p + "enegs"]
    assert np.abs(r["enegs"] - chi).max() <= 1e-10 * max(1.0, np.abs(chi).max())


@pytest.mark.parametrize("name", NAMES)
def test_mixed_matches_fixture(name):
    atoms, calc = _calc(name, "mixed")
    r = calc.engine.calculate(L.PREC_MIXED, energy=True, forces=True)
    p = name + "/"
    assert abs(r["energy"] - float(G[p + "energy"])) / len(atoms) <= 1e-5
    assert np.abs(r["forces"] - G[p + "forces"]).max() <= 1e-4


def test_relaxed_charges_match_fixture():
    atoms, calc = _calc("sio2_120")
    rx = cases.RELAX
    rel = pysic.ChargeRelaxation("dynamic", calculator=calc,
                                 parameters=[rx[k] for k in ("n_steps", "timestep", "inertia", "friction", "tolerance")])
    q = rel.charge_relaxation()
    assert rel.last_steps == int(G["sio2_120/relax_steps"])
    np.testing.assert_allclose(q, G["sio2_120/relaxed_charges"], atol=1e-8)
    np.testing.assert_allclose(rel.charge_rates, G["sio2_120/relaxed_rates"], atol=1e-8)


def test_documented_values():
    d = json.load(open(os.path.join(GOLDEN, "reference_docs.json")))
    he = d["he2_lj"]
    pot = pysic.Potential("LJ", symbols=[he["potential"]["symbols"]],
                          parameters=[he["potential"]["epsilon"], he["potential"]["sigma"]],
                          cutoff=he["potential"]["cutoff"])
    calc = pysic.Pysic(pysic.Atoms(he["symbols"], he["positions"]), [pot])
    assert calc.get_potential_energy() == pytest.approx(he["energy"], rel=1e-14)
    np.testing.assert_allclose(calc.get_forces(), he["forces"], atol=0.6e-8)
    coh = d["coh_lj"]
    pots = [pysic.Potential("LJ", symbols=coh[k]["symbols"], parameters=coh[k]["parameters"],
                            cutoff=coh[k]["cutoff"]) for k in ("pot1", "pot2")]
    calc = pysic.Pysic(pysic.Atoms(coh["symbols"], coh["positions"]), pots)
    assert calc.get_potential_energy() == pytest.approx(coh["energy_both"], rel=1e-11)
    np.testing.assert_allclose(calc.get_forces(), coh["forces_both"], atol=0.6e-8)
