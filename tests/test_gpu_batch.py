"""GPU checks of the many-system launches (csrc/batch.cu, csrc/persist.cuh):
every system of a batch of uneven silicon boxes (Tersoff + Lennard-Jones)
must get the results its own calculator gives, in the one persistent launch
over every tile shape and in the per-phase launches.  Tolerances as in the parity tests: FP64 energies
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


# (pair lanes, bond lanes, cells per tile, mode); bond lanes 64: the triplet tile
TILES = [(0, 0, 0, "batched"), (8, 4, 1, "batched"), (16, 8, 2, "batched"), (8, 64, 4, "batched"),
         (16, 4, 64, "batched"), (32, 8, 0, "phases"), (16, 64, 0, "phases")]


@pytest.mark.parametrize("tiles", TILES, ids=lambda t: "{3}-{0}-{1}-{2}".format(*t))
def test_batch_matches_each_system_fp64(tiles):
    pl, bl, cells, mode = tiles
    calcs = _systems("fp64")
    ref = _single(calcs, "fp64")
    batch = BatchedPysic(calcs, pair_lanes=pl, bond_lanes=bl)
    batch.set_tile_blocks(cells)
    for _ in range(2):  # captured graph, then its replay
        batch.evaluate("fp64", mode=mode)
        got = batch.results()
        for g, r in zip(got, ref):
            assert g["energy"] == pytest.approx(r["energy"], rel=1e-12, abs=1e-11)
            assert np.abs(g["forces"] - r["forces"]).max() <= 1e-10 * max(1.0, np.abs(r["forces"]).max())
            np.testing.assert_allclose(g["stress"], r["stress"], rtol=1e-9, atol=1e-9 * np.abs(r["stress"]).max())
    assert batch.launch_count() == (1 if mode == "batched" else 4)
    p, q, c = batch.get_tiles("fp64", mode)
    assert p in (8, 16, 32) and q in (4, 8, 64) and c >= 1
    if pl:
        assert (p, q) == (pl, bl)


def test_persistent_launch_is_bit_reproducible():
    """The exact fixed-point totals and gather forces make the one-launch
    results independent of which block takes which tile."""
    calcs = _systems("mixed", counts=(64, 300, 150, 97, 211, 73, 128))
    batch = BatchedPysic(calcs, pair_lanes=8, bond_lanes=4)
    batch.set_tile_blocks(1)
    batch.evaluate("mixed")
    a = batch.results()
    batch.evaluate("mixed")
    b = batch.results()
    for x, y in zip(a, b):
        assert x["energy"] == y["energy"] and np.array_equal(x["forces"], y["forces"])


def test_persistent_wait_runs_out_and_reports_timeout():
    """A system whose tiles wait for work that never comes: every wait ends at
    its limit, the launch ends, synchronize reports PG_ERR_TIMEOUT, and the
    next evaluation (test hook off) is correct again."""
    calcs = _systems("fp64", counts=(64, 97, 150))
    ref = _single(calcs, "fp64")
    batch = BatchedPysic(calcs, pair_lanes=8, bond_lanes=4)
    batch.set_tile_blocks(1)
    batch.test_stall(1, wait_seconds=0.05)
    batch.evaluate("fp64")
    with pytest.raises(L.EngineError) as err:
        batch.results()
    assert err.value.status == L.PG_ERR_TIMEOUT
    batch.test_stall(-1, wait_seconds=0.5)
    batch.evaluate("fp64")
    for g, r in zip(batch.results(), ref):
        assert g["energy"] == pytest.approx(r["energy"], rel=1e-12, abs=1e-11)


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
    batch.evaluate("mixed", mode="phases")
    for g, e in zip(got, batch.results()):
        assert abs(g["energy"] - e["energy"]) < 1e-6 * max(1.0, abs(e["energy"]))


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
