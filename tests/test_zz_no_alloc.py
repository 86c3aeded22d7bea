"""pg_bond_order_noalloc: the bond-order evaluation on static device scratch.

Kept in its own file, named to be collected last, so that it runs both alone
and after every other GPU test in the same process.  The output buffers are
allocated here by the test; the entry point itself allocates nothing.
"""
import ctypes

import numpy as np
import pytest

import pysic_gb300 as pysic
from pysic_gb300 import _lib as L
from pysic_gb300 import workloads as W

pytestmark = pytest.mark.gpu

# tolerances of the parity tests: FP64 path against itself, mixed path against FP64
TOL = {"fp64": (1e-10, 1e-10), "mixed": (1e-5, 1e-4)}  # (eV/atom, eV/A)


def _calc(n_cells, precision):
    atoms = W.diamond_si(n_cells, noise=0.10, seed=21)
    calc = pysic.Pysic(atoms, W.tersoff_si_potentials(), precision=precision)
    calc.set_core()
    return atoms, calc


def _allocations(lib):
    count = ctypes.c_uint64(0)
    assert lib.pg_device_allocation_count(ctypes.byref(count)) == L.PG_OK
    return count.value


def _noalloc(calc, prec, n):
    """One call through the C ABI; the library's allocation count must not move."""
    import torch

    f = torch.full((max(n, 1), 3), float("nan"), dtype=torch.float64, device="cuda")
    t = torch.full((7,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    eng = calc.engine
    before = _allocations(eng.lib)
    st = eng.lib.pg_bond_order_noalloc(eng.ctx, prec, ctypes.c_void_p(f.data_ptr()), ctypes.c_void_p(t.data_ptr()))
    msg = eng.lib.pg_last_error().decode() if st else ""
    if st == L.PG_OK:
        eng.device_synchronize()
    assert _allocations(eng.lib) == before, "the no-allocation call allocated device memory"
    return st, msg, f.cpu().numpy()[:n], t.cpu().numpy()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_matches_regular_call_twice(precision):
    atoms, calc = _calc(3, precision)
    prec = calc._prec()
    ref = calc.engine.calculate(prec, energy=True, forces=True)
    e_tol, f_tol = TOL[precision]
    n = len(atoms)
    results = []
    for _ in range(2):  # two calls in a row
        st, msg, f, t = _noalloc(calc, prec, n)
        assert st == L.PG_OK, msg
        assert abs(t[0] - ref["energy"]) / n <= e_tol
        assert np.abs(f - ref["forces"]).max() <= f_tol
        np.testing.assert_allclose(t[1:], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())
        results.append((f, t))
    assert np.array_equal(results[0][0], results[1][0])
    assert np.array_equal(results[0][1], results[1][1])


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_noalloc_empty_system(precision):
    atoms = pysic.Atoms([], np.zeros((0, 3)), cell=np.eye(3) * 10.0, pbc=True)
    calc = pysic.Pysic(atoms, W.tersoff_si_potentials(), precision=precision)
    assert calc.get_potential_energy() == 0.0
    for _ in range(2):
        st, msg, f, t = _noalloc(calc, calc._prec(), 0)
        assert st == L.PG_OK, msg
        assert f.shape == (0, 3)
        assert np.array_equal(t, np.zeros(7))


def test_noalloc_rejects_systems_beyond_the_static_limit():
    # 110592 atoms at ~4.1 short-list entries each: 4 x 32 B per entry plus
    # 24 B per atom, about 61 MB of FP64 scratch against the 32 MiB array
    atoms, calc = _calc(24, "fp64")
    calc.engine.calculate(L.PREC_FP64, energy=True, forces=False)
    st, msg, _, _ = _noalloc(calc, L.PREC_FP64, len(atoms))
    assert st == L.PG_ERR_INVALID
    assert "static limit" in msg


def test_noalloc_rejects_terms_outside_the_bond_order_kernels():
    atoms = W.lj_fcc(3, noise=0.05, seed=2)
    calc = pysic.Pysic(atoms, W.lj_potentials(cutoff=6.0))
    calc.get_potential_energy()
    st, msg, _, _ = _noalloc(calc, L.PREC_FP64, len(atoms))
    assert st in (L.PG_ERR_UNSUPPORTED, L.PG_ERR_NOT_READY)
