"""GPU checks of the many-system launch (csrc/batch.cu): every system of a
batch of uneven silicon boxes (Tersoff + Lennard-Jones) must get the results
its own calculator gives.  Tolerances as in the parity tests: FP64 energies
1e-12 relative and forces 1e-10 relative to the largest force; mixed precision
1e-5 eV/atom and 1e-4 of the largest force against the FP64 results."""
import numpy as np
import pytest

import pysic_gb300 as pysic
from pysic_gb300 import _lib as L
from pysic_gb300 import workloads as W
from pysic_gb300.batch import BatchedPysic

pytestmark = pytest.mark.gpu


def _systems(precision, counts=(64, 97, 150, 211, 300, 73), seed=3):
    pots = W.batched_potentials()
    out = []
    for k, n in enumerate(counts):
        atoms = W.random_box(["Si"] * n, W.SI_DENSITY, 2.0, seed * 1000 + k)
        calc = pysic.Pysic(atoms, pots, precision=precision)
        calc.set_core()
        out.append(calc)
    return out


def _single(calcs, precision):
    prec = L.PREC_FP64 if precision == "fp64" else L.PREC_MIXED
    return [c.engine.calculate(prec, energy=True, forces=True) for c in calcs]


@pytest.mark.parametrize("lanes", [(0, 0), (8, 4), (32, 8), (16, 64)])  # 64: the triplet tile
def test_batch_matches_each_system_fp64(lanes):
    calcs = _systems("fp64")
    ref = _single(calcs, "fp64")
    batch = BatchedPysic(calcs, pair_lanes=lanes[0], bond_lanes=lanes[1])
    for _ in range(2):  # captured graph, then its replay
        batch.evaluate("fp64")
        got = batch.results()
        for g, r in zip(got, ref):
            assert g["energy"] == pytest.approx(r["energy"], rel=1e-12, abs=1e-11)
            assert np.abs(g["forces"] - r["forces"]).max() <= 1e-10 * max(1.0, np.abs(r["forces"]).max())
            np.testing.assert_allclose(g["stress"], r["stress"], rtol=1e-9, atol=1e-9 * np.abs(r["stress"]).max())


def test_batch_mixed_accuracy_and_per_system_mode():
    # random boxes with atoms down to 2.0 A carry forces of tens of eV/A, so the
    # mixed-precision force bound is taken relative to the largest force
    calcs = _systems("mixed")
    ref64 = _single(calcs, "fp64")
    ref32 = _single(calcs, "mixed")
    batch = BatchedPysic(calcs)
    batch.evaluate("mixed")
    got = batch.results()
    for c, g, r, m in zip(calcs, got, ref64, ref32):
        n = len(c.get_atoms())
        fmax = max(1.0, np.abs(r["forces"]).max())
        assert abs(g["energy"] - r["energy"]) / n < 1e-5
        assert np.abs(g["forces"] - r["forces"]).max() < 1e-4 * fmax
        assert abs(g["energy"] - m["energy"]) / n < 1e-6
        assert np.abs(g["forces"] - m["forces"]).max() < 1e-5 * fmax
    batch.evaluate("mixed", mode="each")
    each = batch.results()
    for g, e in zip(got, each):
        assert abs(g["energy"] - e["energy"]) < 1e-6 * max(1.0, abs(e["energy"]))
    assert batch.launch_count() > 3 * len(calcs) - 1


def test_batch_follows_position_updates():
    calcs = _systems("fp64", counts=(80, 120))
    batch = BatchedPysic(calcs)
    batch.evaluate("fp64")
    batch.results()
    rng = np.random.default_rng(9)
    for c in calcs:
        a = c.get_atoms()
        a.set_positions(a.get_positions() + rng.normal(0, 0.02, (len(a), 3)))
        c.set_core()  # uploads the new positions (lists stay valid within the skin)
    ref = _single(calcs, "fp64")
    batch.evaluate("fp64")
    for g, r in zip(batch.results(), ref):
        assert g["energy"] == pytest.approx(r["energy"], rel=1e-12, abs=1e-11)
