"""CPU checks of the golden fixtures in tests/golden/.

- The documented known answers (reference_docs.json, parsed from the
  reference's documentation by tests/golden/make_golden.py) against the
  oracle, to the digits the documentation prints.
- The oracle's stored outputs for the seeded cases (oracle_cases.npz) against
  a fresh oracle run: any drift of the oracle is caught here.
"""
import json
import os

import numpy as np
import pytest

import oracle
import pysic_gb300 as pysic
from helpers import oracle_all
from pysic_gb300.model import compile_model, individual_cutoffs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _docs():
    with open(os.path.join(GOLDEN, "reference_docs.json")) as fh:
        return json.load(fh)


def _cases():
    import sys

    sys.path.insert(0, GOLDEN)
    import cases

    return cases, np.load(os.path.join(GOLDEN, "oracle_cases.npz"))


def _allpairs_lists(atoms, cuts):
    n = len(atoms)
    pos = atoms.get_positions()
    c, idx = [], []
    for a in range(n):
        row = [b for b in range(n) if b != a and np.linalg.norm(pos[b] - pos[a]) < cuts[a] + cuts[b]]
        c.append(len(row))
        idx += row
    return np.array(c), np.array(idx), np.zeros((len(idx), 3), dtype=int)


def _lj(spec):
    p = pysic.Potential("LJ", cutoff=spec["cutoff"])
    p.set_symbols(spec["symbols"])
    if "parameters" in spec:
        p.set_parameters(spec["parameters"])
    else:
        p.set_parameter_value("epsilon", spec["epsilon"])
        p.set_parameter_value("sigma", spec["sigma"])
    return p


def _run(symbols, positions, pots):
    atoms = pysic.Atoms(symbols, positions)
    cuts = np.array(individual_cutoffs(atoms, pots)) + 0.5
    return oracle_all(atoms, pots, lists=_allpairs_lists(atoms, cuts))


def test_documented_he2():
    d = _docs()["he2_lj"]
    r = _run(d["symbols"], d["positions"], [_lj(d["potential"])])
    assert r["energy"] == pytest.approx(d["energy"], rel=1e-15, abs=1e-17)
    np.testing.assert_allclose(r["forces"], d["forces"], atol=0.6 * 10.0 ** -d["printed_digits"])


@pytest.mark.parametrize("which", ["pot1", "pot2", "both"])
def test_documented_coh(which):
    d = _docs()["coh_lj"]
    pots = [_lj(d["pot1"]), _lj(d["pot2"])] if which == "both" else [_lj(d[which])]
    r = _run(d["symbols"], d["positions"], pots)
    # the documentation prints 12 significant digits for these energies
    assert r["energy"] == pytest.approx(d["energy_" + which], rel=1e-11)
    np.testing.assert_allclose(r["forces"], d["forces_" + which], atol=0.6 * 10.0 ** -d["printed_digits"])


@pytest.mark.parametrize("name", ["tersoff_si64", "lj_fcc108", "nacl64_ewald", "sio2_120", "triclinic_si64"])
def test_oracle_reproduces_fixture(name):
    cases, g = _cases()
    atoms, pots, coul = cases.restore(name, g)
    p = name + "/"
    cuts = np.array(individual_cutoffs(atoms, pots, coul)) + 0.5
    np.testing.assert_array_equal(cuts, g[p + "cutoffs"])
    c, i, o = oracle.neighbors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), cuts)
    np.testing.assert_array_equal(c, g[p + "nb_counts"])
    np.testing.assert_array_equal(i, g[p + "nb_index"])
    np.testing.assert_array_equal(o, g[p + "nb_offset"])
    r = oracle_all(atoms, pots, coul, lists=(c, i, o))
    scale = max(1.0, abs(float(g[p + "energy"])))
    assert abs(r["energy"] - float(g[p + "energy"])) <= 1e-12 * scale
    np.testing.assert_allclose(r["forces"], g[p + "forces"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(r["stress"], g[p + "stress"], rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(r["enegs"], g[p + "enegs"], rtol=1e-10, atol=1e-10)


def test_oracle_relaxation_reproduces_fixture():
    cases, g = _cases()
    atoms, pots, coul = cases.restore("sio2_120", g)
    model = compile_model(atoms, pots, coul)
    lists = (g["sio2_120/nb_counts"], g["sio2_120/nb_index"], g["sio2_120/nb_offset"])
    r = oracle.relax_charges(atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(),
                             model, *lists, **cases.RELAX)
    assert r["steps"] == int(g["sio2_120/relax_steps"])
    np.testing.assert_allclose(r["charges"], g["sio2_120/relaxed_charges"], atol=1e-10)
