"""GPU parity against the FP64 oracle at the full sizes of the benchmark
configurations (the oracle runs on every host core):

- Tersoff silicon, 16x16x16 diamond cells (32768 atoms, 24 subcells per axis);
- rock-salt NaCl, 10x10x10 cells (8000 ions), Buckingham + Ewald with the
  configuration's own parameters (real-space cutoff 10 A, sigma 2.5 A, k cutoff
  for a 1e-6 reciprocal tail);
- 'dynamic' charge relaxation of a 3000-atom SiO2-like box;
- the many-system launch on systems of the 512-box workload, the largest
  (2028 atoms) and smallest (64 atoms) included.

Tolerances (the same as the small-case parity tests):
- neighbour lists: bit-identical, entry order included;
- FP64 path: energy 1e-12 relative (Ewald 1e-11), forces 1e-10 relative to the
  largest force (Ewald 1e-9 eV/A per unit of the largest force), virial 1e-9
  relative, electronegativities 1e-9 eV/e;
- mixed path against the oracle: 1e-5 eV/atom; forces 1e-4 eV/A for Tersoff
  silicon, 1e-3 eV/A for Ewald, 1e-4 of the largest force for the random boxes
  of the many-system workload (atoms down to 2.0 A apart carry forces of tens
  of eV/A);
- relaxation (FP64): the same number of steps and charges within 1e-8 e.
"""
import math
import os

import numpy as np
import pytest

import oracle
import pysic_gb300 as pysic
from helpers import engine_all, oracle_all, oracle_lists
from pysic_gb300 import _lib as L
from pysic_gb300 import workloads as W
from pysic_gb300.model import compile_model

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 1


def _same_lists(calc, atoms, pots, coul=None):
    c, i, o = calc.engine.neighbor_lists()
    rc, ri, ro = oracle_lists(atoms, pots, coul)
    assert np.array_equal(c, rc)
    assert np.array_equal(i, ri)
    assert np.array_equal(o, ro)
    return rc, ri, ro


@pytest.fixture(scope="module")
def tersoff_32768():
    atoms = W.diamond_si(16, seed=0)
    pots = W.tersoff_si_potentials()
    lists = oracle_lists(atoms, pots)
    return atoms, pots, oracle_all(atoms, pots, lists=lists, threads=THREADS)


def test_tersoff_32768_lists_bit_exact(tersoff_32768):
    atoms, pots, ref = tersoff_32768
    calc = pysic.Pysic(atoms, pots)
    calc.set_core()
    c, _, _ = _same_lists(calc, atoms, pots)
    assert len(atoms) == 32768 and 3.9 < c.mean() < 5.0


def test_tersoff_32768_fp64_parity(tersoff_32768):
    atoms, pots, ref = tersoff_32768
    got = engine_all(atoms, pots, None, "fp64")
    assert got["energy"] == pytest.approx(ref["energy"], rel=1e-12)
    assert np.abs(got["forces"] - ref["forces"]).max() < 1e-10 * max(1.0, np.abs(ref["forces"]).max())
    np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())


def test_tersoff_32768_mixed_against_oracle(tersoff_32768):
    atoms, pots, ref = tersoff_32768
    got = engine_all(atoms, pots, None, "mixed")
    n = len(atoms)
    de = abs(got["energy"] - ref["energy"]) / n
    df = np.abs(got["forces"] - ref["forces"]).max()
    print("Tersoff 32768 mixed - oracle: dE/atom %.3e eV, max dF %.3e eV/A" % (de, df))
    assert de <= 1e-5
    assert df <= 1e-4


@pytest.fixture(scope="module")
def nacl_8000():
    atoms = W.rocksalt_nacl()
    pots, coul = W.nacl_potentials()
    lists = oracle_lists(atoms, pots, coul)
    return atoms, pots, coul, oracle_all(atoms, pots, coul, lists=lists, threads=THREADS)


def test_nacl_8000_lists_bit_exact(nacl_8000):
    atoms, pots, coul, ref = nacl_8000
    calc = pysic.Pysic(atoms, pots, coulomb=coul)
    calc.set_core()
    c, _, _ = _same_lists(calc, atoms, pots, coul)
    assert len(atoms) == 8000 and c.mean() > 150


def test_nacl_8000_fp64_parity(nacl_8000):
    atoms, pots, coul, ref = nacl_8000
    # the configuration's Ewald: ~14.6k half-space k vectors
    kmax = compile_model(atoms, pots, coul).ewald["kmax"]
    assert all(k >= 18 for k in kmax)
    got = engine_all(atoms, pots, coul, "fp64")
    assert got["energy"] == pytest.approx(ref["energy"], rel=1e-11)
    assert np.abs(got["forces"] - ref["forces"]).max() < 1e-9 * max(1.0, np.abs(ref["forces"]).max())
    assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-9
    np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())


def test_nacl_8000_mixed_against_oracle(nacl_8000):
    atoms, pots, coul, ref = nacl_8000
    got = engine_all(atoms, pots, coul, "mixed")
    n = len(atoms)
    de = abs(got["energy"] - ref["energy"]) / n
    df = np.abs(got["forces"] - ref["forces"]).max()
    dchi = np.abs(got["enegs"] - ref["enegs"]).max()
    print("NaCl 8000 mixed - oracle: dE/atom %.3e eV, max dF %.3e eV/A, max dchi %.3e eV/e" % (de, df, dchi))
    assert de <= 1e-5
    assert df <= 1e-3
    assert dchi <= 1e-3


RELAX = dict(n_steps=4000, timestep=0.05, inertia=1.0, friction=3.0, tolerance=1e-4)


def test_sio2_3000_relaxation_matches_oracle_loop():
    atoms = W.sio2_box(1000, seed=0)
    pots, coul = W.sio2_potentials()
    calc = pysic.Pysic(atoms, pots, coulomb=coul, precision="fp64")
    rel = pysic.ChargeRelaxation("dynamic", calculator=calc,
                                 parameters=[RELAX[k] for k in ("n_steps", "timestep", "inertia", "friction",
                                                                "tolerance")])
    q_gpu = rel.charge_relaxation()
    model = compile_model(atoms, pots, coul)
    lists = oracle_lists(atoms, pots, coul)
    r = oracle.relax_charges(atoms.get_positions(), np.zeros(len(atoms)), atoms.get_cell(), atoms.get_pbc(), model,
                             *lists, threads=THREADS, **RELAX)
    print("SiO2 3000 relaxation: %d steps (oracle %d), max |dq| %.3e e" % (rel.last_steps, r["steps"],
                                                                          np.abs(q_gpu - r["charges"]).max()))
    assert len(atoms) == 3000
    assert r["steps"] < RELAX["n_steps"]
    assert rel.last_steps == r["steps"]
    np.testing.assert_allclose(q_gpu, r["charges"], atol=1e-8)
    assert abs(q_gpu.sum()) < 1e-9


# systems of the 512-box workload: counts log-uniform in [64, 2048] from seed 0,
# box k from random_box(..., seed=k), as the benchmark builds them
def _batched_counts():
    rng = np.random.default_rng(0)
    return np.floor(np.exp(rng.uniform(math.log(64), math.log(2048), 512))).astype(int)


def _batched_systems(precision):
    counts = _batched_counts()
    order = np.argsort(counts, kind="stable")
    pick = sorted(set(order[-3:].tolist() + order[:2].tolist() + [0, 1, 100, 255, 400]))
    pots = W.batched_potentials()
    out = []
    for k in pick:
        atoms = W.random_box(["Si"] * int(counts[k]), W.SI_DENSITY, 2.0, int(k))
        calc = pysic.Pysic(atoms, pots, precision=precision)
        calc.set_core()
        out.append((k, atoms, calc))
    return pots, out


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batched_systems_against_oracle(precision):
    from pysic_gb300.batch import BatchedPysic

    pots, systems = _batched_systems(precision)
    assert max(len(a) for _, a, _ in systems) == _batched_counts().max()
    assert min(len(a) for _, a, _ in systems) == 64
    batch = BatchedPysic([c for _, _, c in systems])
    batch.evaluate(precision)
    got = batch.results()
    for (k, atoms, calc), g in zip(systems, got):
        ref = oracle_all(atoms, pots, threads=THREADS)
        n = len(atoms)
        fmax = max(1.0, np.abs(ref["forces"]).max())
        if precision == "fp64":
            assert g["energy"] == pytest.approx(ref["energy"], rel=1e-12, abs=1e-11), k
            assert np.abs(g["forces"] - ref["forces"]).max() <= 1e-10 * fmax, k
            np.testing.assert_allclose(g["stress"], ref["stress"], rtol=1e-9,
                                       atol=1e-9 * np.abs(ref["stress"]).max())
        else:
            assert abs(g["energy"] - ref["energy"]) / n <= 1e-5, k
            assert np.abs(g["forces"] - ref["forces"]).max() <= 1e-4 * fmax, k
