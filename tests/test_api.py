"""CPU tests of the host side: the C ABI library, descriptor tables, record
compilation and the API objects (no GPU calls)."""
import ctypes
import os
import re

import numpy as np
import pytest

import pysic_gb300 as pysic
from pysic_gb300 import _lib, core
from pysic_gb300 import workloads as W
from pysic_gb300.model import compile_model, individual_cutoffs

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _header_functions():
    text = open(os.path.join(ROOT, "include", "pysic_gb300.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|const char\*)\s+(pg_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol(engine_lib):
    declared = _header_functions()
    assert len(declared) >= 30
    for name in declared:
        assert hasattr(engine_lib, name), name
        assert name in _lib.exported_symbols(), name
    assert engine_lib.pg_version().decode().startswith("pysic_gb300")


def test_errors_without_context(engine_lib):
    st = engine_lib.pg_calculate_energy(None, 0, None)
    assert st == _lib.PG_ERR_INVALID
    assert b"null context" in engine_lib.pg_last_error()


def test_descriptors_match_reference_tables():
    assert core.names_of_parameters("LJ") == ["epsilon", "sigma"]
    assert core.names_of_parameters("tersoff") == [["beta", "eta"], ["a", "c", "d", "h", "mu"]]
    assert core.number_of_targets("tersoff") == 3
    assert core.level_of_factor("tersoff") == 2
    assert core.index_of_parameter("Buckingham", "sigma") == 2
    assert core.index_of_parameter("tersoff", "mu") == [1, 4]
    assert "charge_self" in core.list_valid_potentials()


def test_potential_api():
    p = pysic.Potential("LJ", cutoff=10.0)
    p.set_symbols(["He", "He"])
    p.set_parameter_value("epsilon", 0.1)
    assert p.get_symbols() == [["He", "He"]]
    assert p.get_parameter_values() == [0.1, 0.0]
    with pytest.raises(pysic.InvalidPotentialError):
        pysic.Potential("nope")
    with pytest.raises(pysic.InvalidPotentialError):
        p.set_cutoff_margin(11.0)
    p.set_cutoff_margin(1.0)
    assert p.get_soft_cutoff() == 9.0


def test_bond_order_parameters_api():
    b = pysic.BondOrderParameters("tersoff", cutoff=3.0, cutoff_margin=0.6, symbols=[["Si", "Si", "Si"]])
    b.set_parameter_value("beta", 1.1e-6)
    b.set_parameter_value("mu", 3.0)
    assert b.get_parameters_as_list() == [1.1e-6, 0.0, 0.0, 0.0, 0.0, 0.0, 3.0]
    assert b.get_soft_cutoff() == pytest.approx(2.4)


def test_record_compilation_permutes_like_the_reference():
    atoms = W.rocksalt_nacl(1)
    pots, coul = W.nacl_potentials()
    M = compile_model(atoms, pots, coul)
    # Na-Cl becomes the records Na-Cl and Cl-Na (calculator.py:1256-1276)
    assert len(M.pair_kind) == 2
    assert M.pair_mask1[0] == M.pair_mask2[1] and M.pair_mask2[0] == M.pair_mask1[1]
    assert M.ewald["kmax"].tolist() == [int(M.ewald["kc"] * 5.64 / (2 * np.pi) + 0.5)] * 3


def test_tersoff_records_and_groups():
    atoms = W.diamond_si(1)
    M = compile_model(atoms, W.tersoff_si_potentials())
    assert M.n_groups == 1
    assert M.pair_group == [-1, 0]
    assert len(M.bond_params) == 1


def test_individual_cutoffs():
    atoms = W.diamond_si(1)
    cuts = individual_cutoffs(atoms, W.tersoff_si_potentials())
    assert cuts == [3.0] * len(atoms)


def test_types_fold_tags_and_indices():
    atoms = pysic.Atoms(["Si", "Si", "O"], np.zeros((3, 3)), tags=[0, 1, 1])
    pots = [pysic.Potential("LJ", tags=[[1, 1]], parameters=[1, 1], cutoff=3.0),
            pysic.Potential("LJ", indices=[[0, 2]], parameters=[1, 1], cutoff=3.0)]
    M = compile_model(atoms, pots)
    assert M.n_types == 3
    assert len(M.pair_kind) == 3  # (1,1) once, (0,2) and (2,0)


def test_unsupported_factor_rejected_at_compile():
    """The three-target per-atom 'triplet' factor (whose forces the reference
    itself does not evaluate, Core.f90:4908-4912) is refused when compiled."""
    atoms = W.diamond_si(1)
    pot = pysic.Potential("constant", symbols=[["Si"]], parameters=[1.0])
    pot.set_coordinator(pysic.Coordinator([pysic.BondOrderParameters("triplet", cutoff=3.0,
                                                                     symbols=[["Si", "Si", "Si"]])]))
    with pytest.raises((pysic.InvalidPotentialError, pysic.InvalidCoordinatorError)):
        compile_model(atoms, [pot])


def test_four_body_records_compile():
    """dihedral: one record per distinct permutation of each target tuple, the
    unpermuted tuple kept for the evaluator's forward / backward match; tag
    targets are refused."""
    atoms = W.sio2_box(6, seed=1)
    M = compile_model(atoms, [pysic.Potential("dihedral", symbols=[["Si", "O", "O", "Si"]], parameters=[0.5, 1.2],
                                              cutoff=3.0)])
    assert len(M.quad_kind) == 6  # 4! / (2! 2!)
    assert all(list(o) == list(M.quad_orig[0]) for o in M.quad_orig)
    with pytest.raises(pysic.InvalidPotentialError):
        compile_model(atoms, [pysic.Potential("dihedral", tags=[[0, 0, 0, 0]], parameters=[0.5, 1.2], cutoff=3.0)])


def test_new_pair_and_single_kinds_compile():
    atoms = W.diamond_si(1)
    pots = [pysic.Potential("spring", symbols=[["Si", "Si"]], parameters=[2.0, 2.3], cutoff=3.0),
            pysic.Potential("power", symbols=[["Si", "Si"]], parameters=[0.5, 2.0, 3.0], cutoff=3.0),
            pysic.Potential("shift_power", symbols=[["Si", "Si"]], parameters=[0.5, 3.2, 2.0, 2.0], cutoff=3.0),
            pysic.Potential("constant", symbols=[["Si"]], parameters=[-0.25]),
            pysic.Potential("force", symbols=[["Si"]], parameters=[0.1, -0.2, 0.3])]
    M = compile_model(atoms, pots)
    assert list(M.pair_kind) == [3, 4, 5]
    assert list(M.single_kind) == [1, 2]
    a = M.arrays()
    assert a["single_params"].shape == (2, 4)
    np.testing.assert_array_equal(a["single_params"][1], [0.1, -0.2, 0.3, 0.0])
    np.testing.assert_array_equal(a["pair_params"][2], [0.5, 3.2, 2.0, 2.0])


def test_charge_relaxation_api():
    r = pysic.ChargeRelaxation("dynamic", parameters=[100, 0.1, 1.0, 0.5, 1e-4])
    assert r.get_parameters()["tolerance"] == 1e-4
    with pytest.raises(pysic.InvalidRelaxationError):
        pysic.ChargeRelaxation("nope")


def test_workloads_shapes():
    assert len(W.lj_fcc()) == 864
    assert len(W.diamond_si(8)) == 4096
    a = W.rocksalt_nacl()
    assert len(a) == 8000 and a.get_initial_charges().sum() == 0
    assert W.ewald_kcut(2.5) == pytest.approx(2.1, abs=0.03)


def test_sutton_chen_pieces_and_factor_records():
    """SuttonChenPotential builds the reference's pieces (suttonchen.py:68-176):
    a power pair potential and, per element, a constant scaled by sqrt_scale
    over power_bond on the element pairs that element leads; the factor records
    keep the unpermuted targets in the reference's order."""
    atoms = W.fcc_alloy(2, symbols=("Cu", "Ag"), seed=1)
    calc = pysic.Pysic()
    calc.add_potential(W.sutton_chen_potentials(("Cu", "Ag")))
    pots = calc.get_potentials()
    assert [p.get_potential_type() for p in pots] == ["power", "constant", "constant"]
    assert pots[0].get_symbols() == [["Cu", "Cu"], ["Cu", "Ag"], ["Ag", "Ag"]]
    dens = pots[2].get_coordinator().get_bond_order_parameters()
    assert [b.get_bond_order_type() for b in dens] == ["sqrt_scale", "power_bond"]
    assert dens[0].get_parameter_value("epsilon") == -W.SUTTON_CHEN_CU[2]
    assert dens[1].get_symbols() == [["Ag", "Cu"], ["Ag", "Ag"]]
    M = compile_model(atoms, pots)
    assert M.afac_kind == [3, 1, 1, 3, 1, 1]
    assert M.afac_group == [0, 0, 0, 1, 1, 1]
    assert M.single_group == [0, 1]
    assert M.pair_group == [-1] * len(M.pair_group)


def test_scaled_charge_self_rejected():
    atoms = W.fcc_alloy(2, symbols=("Cu",))
    count = pysic.BondOrderParameters("neighbors", cutoff=3.0, symbols=[["Cu", "Cu"]])
    pot = pysic.Potential("charge_self", symbols=[["Cu"]], parameters=[1.0, 2], coordinator=pysic.Coordinator([count]))
    with pytest.raises(pysic.InvalidPotentialError):
        compile_model(atoms, [pot])


def test_coordinator_copies_share_their_calculator():
    """A Coordinator attached to a calculator (engine handles inside) deep-copies
    with the calculator shared, as the calculator's change tracking needs."""
    import copy
    import ctypes

    class _Calc:
        handle = ctypes.pointer(ctypes.c_int(1))

    count = pysic.BondOrderParameters("neighbors", cutoff=3.0, symbols=[["Cu", "Cu"]])
    pot = pysic.Potential("constant", symbols=[["Cu"]], parameters=[1.0], coordinator=pysic.Coordinator([count]))
    calc = _Calc()
    pot.get_coordinator()._calculator = calc
    dup = copy.deepcopy(pot)
    assert dup == pot
    assert dup.get_coordinator()._calculator is calc
    assert dup.get_coordinator().get_bond_order_parameters()[0] is not count
