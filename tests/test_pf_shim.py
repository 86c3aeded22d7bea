"""The f2py drop-in (pysic_gb300.pf_shim) on the CPU: records registered one
at a time in the reference's order fold into the same engine records as the
package's own compile step."""
import numpy as np
import pytest

import pf_driver
import pysic_gb300 as pysic
from pysic_gb300 import pf_shim
from pysic_gb300 import workloads as W
from pysic_gb300.model import compile_model


class _NoEngine(pf_shim.PysicInterface):
    """the record bookkeeping only: no device context"""

    def _eng(self):
        class Null:
            def __getattr__(self, name):
                return lambda *a, **k: None
        return Null()


def _cases():
    yield "tersoff", W.diamond_si(2, seed=1), W.tersoff_si_potentials(), None
    pots, coul = W.nacl_potentials(cutoff=5.0, sigma=1.4, real_cutoff=5.0)
    yield "ewald", W.rocksalt_nacl(2, seed=2), pots, coul
    pots, coul = W.sio2_potentials(real_cutoff=5.0, sigma=1.5)
    yield "sio2", W.sio2_box(20, seed=3), pots, coul
    a = W.fcc_alloy(2, symbols=("Cu", "Ag"), seed=4)
    calc = pysic.Pysic()
    calc.add_potential(W.sutton_chen_potentials(("Cu", "Ag")))
    yield "sutton_chen", a, calc.get_potentials(), None
    a = W.lj_fcc(2, seed=5)
    a.set_tags(np.arange(len(a)) % 3)
    yield "tags_indices", a, [pysic.Potential("LJ", tags=[[0, 1]], parameters=[0.01, 3.0], cutoff=5.0),
                             pysic.Potential("LJ", indices=[[2, 7]], parameters=[0.02, 2.5], cutoff=5.0),
                             pysic.Potential("LJ", symbols=[["X", "X"]], parameters=[0.005, 3.2], cutoff=5.0)], None
    _, a, pots = list(W.dihedral_cases())[1]
    yield "dihedral_bend", a, pots, None
    for name, a, pots in W.comb_style_cases():
        yield name, a, pots, None


# rows of the table array behind a record's first parameter: tabulated
# (rows, count in p1), charge_exp (8 rows), charge_abs (4 rows)
_TABLE_ROWS = {6: None, 8: 8, 9: 4}


def _resolved(a, kind, params):
    """a record's parameters with table offsets replaced by the rows they
    point to (the two builders lay the shared table out in another order)"""
    p = [float(x) for x in params]
    if kind in _TABLE_ROWS:
        rows = int(p[1]) if _TABLE_ROWS[kind] is None else _TABLE_ROWS[kind]
        first = int(p[0])
        p = [tuple(np.asarray(a["pair_table"])[2 * first:2 * (first + rows)].tolist())] + p[1:]
        if _TABLE_ROWS[kind] is not None:
            p = p[:1]
    return tuple(p)


def _pair_rows(a):
    """the same records, each with its factors resolved; the reference's own
    set() of permutations fixes no order"""
    n = len(a["pair_kind"])
    rows = []
    for r in range(n):
        kind = int(a["pair_kind"][r])
        nm = int(a["pair_nmul"][r]) if len(a["pair_nmul"]) else 0
        m0 = int(a["pair_mul0"][r]) if len(a["pair_mul0"]) else 0
        factors = tuple((int(a["mul_kind"][c]), _resolved(a, int(a["mul_kind"][c]), a["mul_params"][c]),
                         int(a["mul_first"][c])) for c in range(m0, m0 + nm))
        rows.append((kind, int(a["pair_group"][r]), int(a["pair_mask1"][r]), int(a["pair_mask2"][r]),
                     int(a["pair_first"][r]), float(a["pair_cutoff"][r]), float(a["pair_soft"][r]),
                     _resolved(a, kind, a["pair_params"][r]), factors))
    return sorted(rows, key=repr)


@pytest.mark.parametrize("case", list(_cases()), ids=lambda c: c[0])
def test_shim_records_equal_compiled_records(case):
    _, atoms, pots, coul = case
    pi = _NoEngine()
    pf_driver.load(pi, atoms, pots, coul)
    got = pi.build_model()
    ref = compile_model(atoms, pots, coul)
    assert got.n_types == ref.n_types
    assert np.array_equal(got.types, ref.types)
    ga, ra = got.arrays(), ref.arrays()
    assert _pair_rows(ga) == _pair_rows(ra)
    for key in ra:
        if not key.startswith("pair_") and not key.startswith("mul_"):
            assert np.array_equal(ga[key], ra[key]), key
    if coul is not None:
        for k in ("rc", "kc", "sigma", "eps"):
            assert got.ewald[k] == ref.ewald[k]
        assert np.array_equal(got.ewald["kmax"], ref.ewald["kmax"])


def test_shim_signature_conventions():
    pi = _NoEngine()
    assert pi.is_potential("LJ") and not pi.is_potential("nonsense")
    assert pi.number_of_targets_of_bond_order_factor("tersoff") == 3
    assert pi.level_of_bond_order_factor("tersoff") == 2
    assert pi.number_of_parameters_of_bond_order_factor("tersoff", 2) == 5
    # a factor of a product waits for its leading record, which takes it (Core.f90:909-953)
    none, xx = np.array([-9, -9]), np.array([pf_driver.codes("X")] * 2).T
    assert pi.add_potential("exponential", np.array([2.0, 0.5]), 5.0, 5.0, xx, none, none, xx, none, none, -1, True)
    assert pi.add_potential("LJ", np.array([1.0, 1.0]), 5.0, 5.0, xx, none, none, xx, none, none, -1, False)
    pi.clear_potential_multipliers()
    assert [m["name"] for m in pi._pots[-1]["multipliers"]] == ["exponential"]
    assert pi.add_potential("nonsense", np.array([1.0]), 5.0, 5.0, xx, none, none, xx, none, none, -1, False) is False
