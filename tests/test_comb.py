"""CombPotential on the CPU: its parameter table against the reference's
(reference_docs.json, parsed from pysic/interactions/comb.py), the pieces it
builds and their order, the component switches, and the oracle's COMB energy
against finite differences (forces, electronegativities)."""
import json
import os

import numpy as np
import pytest

import oracle
import pysic_gb300 as pysic
from pysic_gb300 import workloads as W
from pysic_gb300.comb import POSSIBLE_EXCLUDES
from pysic_gb300.model import compile_model, individual_cutoffs

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _reference_table():
    with open(os.path.join(GOLDEN, "reference_docs.json")) as fh:
        return json.load(fh)["comb10_parameters"]["values"]


def test_parameter_table_is_the_references():
    ref = _reference_table()
    pot = pysic.CombPotential()
    assert set(pot.params) == set(ref)
    for name, value in ref.items():
        assert pot.get_parameter_value(name) == value, name


def _kinds(pieces):
    out = []
    for p in pieces:
        if isinstance(p, pysic.ProductPotential):
            out.append(tuple(q.get_potential_type() for q in p.get_potentials()))
        else:
            out.append(p.get_potential_type())
    return out


def test_pieces_in_the_references_order():
    calc = pysic.Pysic()
    pot = pysic.CombPotential()
    pot.set_calculator(calc, True)
    kinds = _kinds(pot.get_elements())
    assert len(kinds) == 40
    assert kinds[:2] == ["bond_bend", "bond_bend"]
    assert kinds[2:5] == [("charge_exp", "charge_abs", "exponential")] * 3
    assert kinds[5:8] == [("charge_exp", "exponential")] * 3
    assert kinds[8:16] == ["charge_self"] * 8
    assert kinds[16:28] == [("charge_pair", "power")] * 12
    assert kinds[28:32] == [("charge_pair", "power", "exponential")] + [
        ("charge_pair", "power", "exponential", "shift_power")] * 3
    # attraction pieces carry one Coordinator each (Si-Si, O-O, Si-O)
    coords = [p.get_coordinator() for p in pot.get_elements()[2:5]]
    assert [len(c.get_bond_order_parameters()) for c in coords] == [2, 2, 4]
    # the O-O Coulomb corrections keep the reference's double set_cutoff
    for p in pot.get_elements()[32:36]:
        assert p.get_symbols() == [["O", "O"]]
        assert p.get_cutoff() == 0.1 and p.get_cutoff_margin() == 0.0
    # default exclusions: screened real-space Ewald on the calculator
    ew = calc.get_coulomb_summation().get_parameters()
    assert ew["k_cutoff"] == 0.0 and ew["real_cutoff"] == 12.0 and ew["sigma"] == 3.535533906
    assert len(calc.get_potentials()) == 40


def test_component_switches():
    pot = pysic.CombPotential()
    assert pot.list_possible_excludes() == list(POSSIBLE_EXCLUDES)
    assert pot.is_excluded("direct_coulomb") and pot.is_included("si_self")
    pot.include("direct_coulomb")
    pot.define_elements()  # no Ewald needed, so no calculator needed
    assert len(pot.get_elements()) == 43
    pot.exclude("si_self")
    pot.toggle_exclude("osio_bend")
    pot.define_elements()
    assert len(pot.get_elements()) == 38
    pot.exclude_all()
    with pytest.raises(Exception):
        pot.define_elements()  # the Ewald summation needs the calculator
    calc = pysic.Pysic()
    pot.set_calculator(calc)
    pot.define_elements()
    assert pot.get_elements() == []
    pot.include("long_coulomb")
    pot.define_elements()
    rc, kc, sigma, _ = pysic.estimate_ewald_parameters(12.0)
    assert calc.get_coulomb_summation().get_parameters()["k_cutoff"] == kc
    pot.include_all()
    assert pot.list_excludes() == ["direct_coulomb", "long_coulomb"]


def _short_comb():
    """COMB with its 12 A Coulomb and field ranges cut to 5 A, so that a small
    random SiO2 box holds it (every piece kept)."""
    calc = pysic.Pysic()
    pot = pysic.CombPotential()
    for name in ("coulomb cutoff", "field cutoff"):
        pot.set_parameter_value(name, 5.0)
    pot.set_calculator(calc, True)
    return calc.get_potentials(), calc.get_coulomb_summation()


def _oracle(atoms, pots, coul, what):
    cuts = np.array(individual_cutoffs(atoms, pots, coul)) + 0.5
    c, i, o = oracle.neighbors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), cuts)
    model = compile_model(atoms, pots, coul)
    return oracle.evaluate(atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(),
                           model, c, i, o, what)


def test_oracle_comb_forces_and_electronegativities_are_gradients():
    oracle.build()
    atoms = W.sio2_box(40, seed=73)
    q = np.random.default_rng(74).normal(0.0, 0.4, len(atoms))
    atoms.set_initial_charges(q - q.mean())
    pots, coul = _short_comb()
    f, _ = _oracle(atoms, pots, coul, "forces")
    chi = _oracle(atoms, pots, coul, "enegs")
    h = 1e-5
    for a in (0, 7, 55, 101):
        for c in range(3):
            e = []
            for s in (1, -1):
                b = atoms.copy()
                p = b.get_positions()
                p[a, c] += s * h
                b.set_positions(p)
                e.append(_oracle(b, pots, coul, "energy"))
            assert f[a, c] == pytest.approx(-(e[0] - e[1]) / (2 * h), rel=1e-5, abs=1e-5)
        e = []
        for s in (1, -1):
            b = atoms.copy()
            qq = b.get_initial_charges().copy()
            qq[a] += s * h
            b.set_initial_charges(qq)
            e.append(_oracle(b, pots, coul, "energy"))
        assert chi[a] == pytest.approx(-(e[0] - e[1]) / (2 * h), rel=1e-5, abs=1e-5)
