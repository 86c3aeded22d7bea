"""GPU parity: the engine against the FP64 oracle on the same seeded inputs.

Tolerances:
- neighbour lists: bit-identical (indices, offsets and order);
- FP64 path: energy within 1e-12 relative, forces within 1e-10 eV/A,
  virial within 1e-9 relative (summation order differs from the oracle);
- mixed path: energy within 1e-5 eV/atom, forces within 1e-4 eV/A of the
  FP64 result (the spec accuracy target).
"""
import numpy as np
import pytest

import pysic_gb300 as pysic
from helpers import engine_all, oracle_all, oracle_lists
from pysic_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def _lists_equal(atoms, pots, coulomb=None, skin=0.5):
    calc = pysic.Pysic(atoms, pots, coulomb=coulomb)
    calc.set_core()
    c, i, o = calc.engine.neighbor_lists()
    rc, ri, ro = oracle_lists(atoms, pots, coulomb, skin)
    assert np.array_equal(c, rc)
    assert np.array_equal(i, ri)
    assert np.array_equal(o, ro)
    return c


def _rand_cell(seed, scale=10.0):
    rng = np.random.default_rng(seed)
    cell = np.eye(3) * scale + rng.uniform(-0.25, 0.25, (3, 3)) * scale
    return cell


def test_neighbor_lists_bit_exact_lj_fcc():
    c = _lists_equal(W.lj_fcc(), W.lj_potentials())
    assert 70 < c.mean() < 90


def test_neighbor_lists_bit_exact_silicon():
    _lists_equal(W.diamond_si(8, seed=1), W.tersoff_si_potentials())


@pytest.mark.parametrize("seed", [0, 1, 2, 3])
def test_neighbor_lists_bit_exact_triclinic(seed):
    rng = np.random.default_rng(100 + seed)
    cell = _rand_cell(seed, 12.0)
    n = 150
    frac = rng.uniform(-0.3, 1.3, (n, 3))  # also atoms outside the cell
    atoms = pysic.Atoms(["Ar"] * n, frac @ cell, cell=cell, pbc=[True, seed % 2 == 0, True])
    pots = [pysic.Potential("LJ", symbols=[["Ar", "Ar"]], parameters=[0.01, 3.0], cutoff=2.5 + 0.5 * seed)]
    _lists_equal(atoms, pots)


def test_neighbor_lists_bit_exact_small_cells():
    # one and two subcells per axis: periodic images of the same atom appear
    rng = np.random.default_rng(5)
    for L, rc in ((4.5, 2.5), (7.5, 3.0), (9.0, 3.9), (12.0, 3.2)):
        n = 40
        atoms = pysic.Atoms(["Ar"] * n, rng.uniform(0, L, (n, 3)), cell=np.eye(3) * L, pbc=True)
        pots = [pysic.Potential("LJ", symbols=[["Ar", "Ar"]], parameters=[0.01, 2.0], cutoff=rc)]
        _lists_equal(atoms, pots)


def test_neighbor_lists_lattice_sites_on_boundaries():
    # perfect lattice in a sheared cell: wrapped fractional coordinates land on 0
    cell = np.array([[5.0, 0, 0], [2.5, 4.33, 0], [0, 0, 5.0]])
    g = np.array([[i, j, k] for i in range(3) for j in range(3) for k in range(3)], dtype=float) / 3.0
    big = cell * 3
    atoms = pysic.Atoms(["Ar"] * len(g), g @ big, cell=big, pbc=True)
    pots = [pysic.Potential("LJ", symbols=[["Ar", "Ar"]], parameters=[0.01, 2.0], cutoff=4.0)]
    _lists_equal(atoms, pots)


def test_neighbor_lists_nonperiodic():
    rng = np.random.default_rng(8)
    atoms = pysic.Atoms(["Ar"] * 200, rng.uniform(-2, 22, (200, 3)), cell=np.eye(3) * 20.0, pbc=False)
    pots = [pysic.Potential("LJ", symbols=[["Ar", "Ar"]], parameters=[0.01, 2.0], cutoff=4.0)]
    _lists_equal(atoms, pots)


def test_golden_vectors_on_gpu():
    atoms = pysic.Atoms("He2", [[0.0, 0.0, 0.0], [0.0, 0.0, 3.0]])
    pot = pysic.Potential("LJ", symbols=[["He", "He"]], parameters=[0.1, 2.5], cutoff=10.0)
    calc = pysic.Pysic(atoms, [pot])
    assert calc.get_potential_energy() == pytest.approx(-0.022274132189576905, rel=1e-14)
    np.testing.assert_allclose(calc.get_forces(), [[0, 0, 0.02211693], [0, 0, -0.02211693]], atol=5e-9)
    atoms = pysic.Atoms("COH", [[0.0, 0.0, 0.0], [2.0, 0.0, 0.0], [2.0, 2.0, 2.0]])
    p1 = pysic.Potential("LJ", symbols=["C", "O"], parameters=[1, 1], cutoff=10.0)
    p2 = pysic.Potential("LJ", symbols=["O", "H"], parameters=[1, 1], cutoff=10.0)
    calc = pysic.Pysic(atoms, [p1, p2])
    assert calc.get_potential_energy() == pytest.approx(-0.0173301696777, abs=5e-14)
    np.testing.assert_allclose(calc.get_forces(), [[0.04541016, 0, 0], [-0.04541016, 0.00291824, 0.00291824],
                                                   [0, -0.00291824, -0.00291824]], atol=5e-9)


def _check_fp64(atoms, pots, coulomb=None, lanes=0):
    ref = oracle_all(atoms, pots, coulomb)
    got = engine_all(atoms, pots, coulomb, "fp64", lanes)
    assert got["energy"] == pytest.approx(ref["energy"], rel=1e-12, abs=1e-11)
    assert np.abs(got["forces"] - ref["forces"]).max() < 1e-10 * max(1.0, np.abs(ref["forces"]).max())
    np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())
    return ref, got


def test_lj_fcc_fp64_parity():
    _check_fp64(W.lj_fcc(), W.lj_potentials())


@pytest.mark.parametrize("lanes", [4, 8, 16, 32, 64])  # 64: the triplet tile
def test_tersoff_fp64_parity(lanes):
    _check_fp64(W.diamond_si(3, seed=11), W.tersoff_si_potentials(), lanes=lanes)


def _two_species_tersoff():
    """Silicon parameters on two element labels: the kernels take their table
    path (two atom types) instead of the single-species fast path, for the
    same physics."""
    p = W.TERSOFF_SI
    rc, margin = p["R"] + p["D"], 2.0 * p["D"]
    els = ["Si", "Ge"]
    triples = [[a, b, c] for a in els for b in els for c in els]
    pairs = [["Si", "Si"], ["Si", "Ge"], ["Ge", "Ge"]]
    bo = pysic.BondOrderParameters("tersoff", cutoff=rc, cutoff_margin=margin, symbols=triples,
                                   parameters=[[p["beta"], p["n"]], [0.0, p["c"], p["d"], p["h"], 3.0]])
    crd = pysic.Coordinator([bo])
    rep = pysic.Potential("exponential", symbols=pairs, parameters=[p["A"], p["lambda1"]], cutoff=rc,
                          cutoff_margin=margin)
    att = pysic.Potential("exponential", symbols=pairs, parameters=[-p["B"], p["lambda2"]], cutoff=rc,
                          cutoff_margin=margin, coordinator=crd)
    return [rep, att]


@pytest.mark.parametrize("lanes", [4, 8, 64])
def test_tersoff_table_path_matches_fast_path(lanes):
    atoms = W.diamond_si(3, seed=14)
    mixed_atoms = atoms.copy()
    symbols = ["Si" if k % 3 else "Ge" for k in range(len(atoms))]
    mixed_atoms = pysic.Atoms(symbols, atoms.get_positions(), cell=atoms.get_cell(), pbc=atoms.get_pbc())
    ref, got = _check_fp64(mixed_atoms, _two_species_tersoff(), lanes=lanes)
    fast = engine_all(atoms, W.tersoff_si_potentials(), precision="fp64", lanes=lanes)
    assert got["energy"] == pytest.approx(fast["energy"], rel=1e-12)
    assert np.abs(got["forces"] - fast["forces"]).max() < 1e-10
    mixed = engine_all(mixed_atoms, _two_species_tersoff(), precision="mixed", lanes=lanes)
    assert abs(mixed["energy"] - got["energy"]) / len(atoms) < 1e-5
    assert np.abs(mixed["forces"] - got["forces"]).max() < 1e-4


def _long_range_tersoff(R=3.6):
    """Silicon Tersoff with the cutoff moved out to R + D = 3.9 A: 11 to 24
    bonds per atom in a random box, so the triplet tile runs several blocks of
    4 bonds and keeps atoms with more than 16 bonds in global memory."""
    p = dict(W.TERSOFF_SI)
    p["R"] = R
    return W.tersoff_si_potentials(p)


@pytest.mark.parametrize("lanes", [8, 64])
def test_tersoff_many_bonds_fp64_parity(lanes):
    atoms = W.random_box(["Si"] * 120, W.SI_DENSITY, 2.0, 9)
    ref, got = _check_fp64(atoms, _long_range_tersoff(), lanes=lanes)
    c = ref["lists"][0]
    assert c.max() > 16 and c.min() < 16
    mixed = engine_all(atoms, _long_range_tersoff(), precision="mixed", lanes=lanes)
    fmax = max(1.0, np.abs(got["forces"]).max())
    assert abs(mixed["energy"] - got["energy"]) / len(atoms) < 1e-5
    assert np.abs(mixed["forces"] - got["forces"]).max() < 1e-4 * fmax


@pytest.mark.parametrize("lanes", [0, 4, 64])
def test_tersoff_mixed_accuracy_32768_each_tile(lanes):
    atoms = W.diamond_si(16, seed=0)
    pots = W.tersoff_si_potentials()
    m = engine_all(atoms, pots, precision="mixed", lanes=lanes)
    d = engine_all(atoms, pots, precision="fp64", lanes=lanes)
    n = len(atoms)
    assert abs(m["energy"] - d["energy"]) / n < 1e-5
    assert np.abs(m["forces"] - d["forces"]).max() < 1e-4


def test_tersoff_mixed_accuracy_4096():
    atoms = W.diamond_si(8, seed=12)
    pots = W.tersoff_si_potentials()
    ref, got64 = _check_fp64(atoms, pots)
    mixed = engine_all(atoms, pots, precision="mixed")
    n = len(atoms)
    assert abs(mixed["energy"] - got64["energy"]) / n < 1e-5
    assert np.abs(mixed["forces"] - got64["forces"]).max() < 1e-4


def test_tersoff_zeta_matches_oracle():
    import oracle

    atoms = W.diamond_si(2, seed=13)
    pots = W.tersoff_si_potentials()
    calc = pysic.Pysic(atoms, pots)
    z = calc.get_bond_zeta()
    ref = oracle_all(atoms, pots)
    c, i, o = ref["lists"]
    zr = oracle.bond_zeta(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), ref["model"], c, i, o)
    # g(theta) is evaluated in a cancellation-free form: ~1e-12 relative from the oracle's
    np.testing.assert_allclose(z, zr, rtol=1e-11, atol=1e-9)


@pytest.mark.parametrize("lanes", [0, 64])
def test_results_are_bit_reproducible(lanes):
    atoms = W.diamond_si(4, seed=14)
    pots = W.tersoff_si_potentials()
    calc = pysic.Pysic(atoms, pots, precision="mixed")
    calc.set_core()
    if lanes:
        calc.engine.set_lanes(lanes)
    a = calc.engine.calculate(calc._prec())
    b = calc.engine.calculate(calc._prec())
    assert a["energy"] == b["energy"]
    assert np.array_equal(a["forces"], b["forces"])


def test_md_style_position_update():
    """positions move less than skin/2: the list is reused, offsets stay valid"""
    atoms = W.diamond_si(3, seed=15)
    pots = W.tersoff_si_potentials()
    calc = pysic.Pysic(atoms, pots)
    calc.get_forces()
    nl = calc.get_neighbor_lists()
    moved = atoms.copy()
    moved.set_positions(atoms.get_positions() + np.random.default_rng(1).normal(0, 0.05, (len(atoms), 3)))
    f = calc.get_forces(moved)
    assert calc.get_neighbor_lists().nupdates == nl.nupdates
    ref = oracle_all(moved, pots, lists=oracle_lists(atoms, pots))
    assert np.abs(f - ref["forces"]).max() < 1e-10


def test_rejected_coordinate_update_keeps_the_old_positions():
    """pg_update_atom_coordinates stages the new coordinates; the device checks
    them in front of the next evaluation (or before any other call that reads
    them) and moves them into place only when every value is finite.  The
    verdict comes with the next call that waits on the device."""
    from pysic_gb300 import _lib as L

    atoms = W.diamond_si(2, noise=0.1, seed=3)
    calc = pysic.Pysic(atoms, W.tersoff_si_potentials())
    e0 = calc.get_potential_energy()
    f0 = calc.get_forces()
    eng = calc.engine
    # the mixed path commits an update inside its displacement pass and puts
    # the old coordinates back when the verdict is read
    m0 = eng.calculate(L.PREC_MIXED, energy=True, forces=True)
    for bad in (np.nan, np.inf, -np.inf):
        pos = atoms.get_positions()
        pos[5, 1] = bad
        for precision in (L.PREC_FP64, L.PREC_MIXED):  # a fresh graph and its replay
            with pytest.raises(L.EngineError) as err:
                eng.update_positions(pos)
                eng.calculate(precision, energy=True, forces=True)
            assert err.value.status == L.PG_ERR_INVALID
        r = eng.calculate(L.PREC_FP64, energy=True, forces=True)
        assert r["energy"] == e0
        assert np.array_equal(r["forces"], f0)
        r = eng.calculate(L.PREC_MIXED, energy=True, forces=True)
        assert r["energy"] == m0["energy"]
        assert np.array_equal(r["forces"], m0["forces"])
        # a call that reads the coordinates outside an evaluation reports it too
        eng.update_positions(pos)
        with pytest.raises(L.EngineError) as err:
            eng.neighbor_lists()
        assert err.value.status == L.PG_ERR_INVALID
        # and so does the device-resident route, with the results
        for precision in (L.PREC_FP64, L.PREC_MIXED):
            eng.update_positions(pos)
            eng.device_evaluate(precision, L.WANT_ENERGY | L.WANT_FORCES)
            with pytest.raises(L.EngineError):
                eng.device_results()
        r = eng.calculate(L.PREC_FP64, energy=True, forces=True)
        assert r["energy"] == e0
        # an update committed by the displacement pass whose verdict is read by
        # a call outside an evaluation
        eng.update_positions(pos)
        eng.device_evaluate(L.PREC_MIXED, L.WANT_ENERGY | L.WANT_FORCES)
        with pytest.raises(L.EngineError):
            eng.neighbor_lists()
        r = eng.calculate(L.PREC_FP64, energy=True, forces=True)
        assert r["energy"] == e0
    # a valid update afterwards is taken
    moved = atoms.get_positions() + 0.01
    eng.update_positions(moved)
    r = eng.calculate(L.PREC_FP64, energy=True, forces=True)
    ref = oracle_all(pysic.Atoms(atoms.get_chemical_symbols(), moved, cell=atoms.get_cell(), pbc=atoms.get_pbc()),
                     W.tersoff_si_potentials(), lists=oracle_lists(atoms, W.tersoff_si_potentials()))
    assert np.abs(r["forces"] - ref["forces"]).max() < 1e-10


def _more_kinds():
    P = pysic.Potential
    atoms = W.lj_fcc(3, noise=0.08, seed=31)
    pots = [P("spring", symbols=[["X", "X"]], parameters=[0.3, 3.7], cutoff=5.0),
            P("power", symbols=[["X", "X"]], parameters=[0.05, 3.0, 6.5], cutoff=6.0, cutoff_margin=0.5),
            P("shift_power", symbols=[["X", "X"]], parameters=[0.02, 6.5, 3.0, 3.0], cutoff=6.0),
            P("constant", symbols=[["X"]], parameters=[-0.1]),
            P("force", symbols=[["X"]], parameters=[0.05, -0.02, 0.01])]
    return atoms, pots


def test_spring_power_shift_power_constant_force_fp64_parity():
    """The pair kinds spring, power, shift_power (Potentials.f90:3042-3085,
    4119-4152, 4803-4842) and the single-atom constant and constant-force terms
    (3122-3147, 3942-3966) against the oracle."""
    atoms, pots = _more_kinds()
    ref, got = _check_fp64(atoms, pots)
    # the constant forces show in the forces and leave the virial alone
    assert abs(ref["forces"][:, 0].sum() - 0.05 * len(atoms)) < 1e-9


def test_spring_power_shift_power_constant_force_mixed():
    atoms, pots = _more_kinds()
    ref = oracle_all(atoms, pots)
    got = engine_all(atoms, pots, None, "mixed")
    n = len(atoms)
    assert abs(got["energy"] - ref["energy"]) / n <= 1e-5
    assert np.abs(got["forces"] - ref["forces"]).max() <= 1e-4 * max(1.0, np.abs(ref["forces"]).max())


@pytest.mark.parametrize("margin", [0.0, 1.0])
def test_step_potential_parity(margin):
    """step (Potentials.f90:4858-4967) with the reference's force (the same
    value on all three components, +c on the pair's atom 1 and -c on atom 2,
    as the reference's loop picks them) and its stress terms, beside LJ, with
    and without a smooth cut: FP64 against the oracle, mixed precision within
    1e-5 eV/atom and 1e-4 of the largest force, over pair-kernel lane counts."""
    P = pysic.Potential
    atoms = W.lj_fcc(3, noise=0.08, seed=37)
    pots = [P("step", symbols=[["X", "X"]], parameters=[0.04, -0.01, 3.0, 5.0], cutoff=5.5, cutoff_margin=margin),
            P("LJ", symbols=[["X", "X"]], parameters=[0.0104, 3.4], cutoff=6.0)]
    ref, got = _check_fp64(atoms, pots)
    assert abs(ref["forces"].sum(axis=0)).max() < 1e-9  # third law holds pair by pair
    n = len(atoms)
    for lanes in (8, 32):
        calc = pysic.Pysic(atoms, pots, precision="fp64")
        calc.set_core()
        calc.engine.set_pair_lanes(lanes)
        r = calc.engine.calculate(calc._prec(), energy=True, forces=True)
        assert r["energy"] == pytest.approx(ref["energy"], rel=1e-12, abs=1e-11)
        assert np.abs(r["forces"] - ref["forces"]).max() < 1e-10
        np.testing.assert_allclose(r["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())
    mixed = engine_all(atoms, pots, None, "mixed")
    assert abs(mixed["energy"] - ref["energy"]) / n <= 1e-5
    assert np.abs(mixed["forces"] - ref["forces"]).max() <= 1e-4 * max(1.0, np.abs(ref["forces"]).max())
    np.testing.assert_allclose(mixed["stress"], ref["stress"], rtol=1e-4, atol=1e-4 * np.abs(ref["stress"]).max())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_tabulated_potential_parity(precision, tmp_path, monkeypatch):
    """'tabulated' (Potentials.f90:4227-4298) from table_0003.txt, smoothed at
    its cutoff, with LJ on the side, against the oracle."""
    monkeypatch.chdir(tmp_path)
    r = np.linspace(0.0, 6.0, 121)
    v = 0.3 * np.exp(-r / 0.8) - 0.05 * np.exp(-((r - 3.4) ** 2))
    dvdr = -0.3 / 0.8 * np.exp(-r / 0.8) + 0.1 * (r - 3.4) * np.exp(-((r - 3.4) ** 2))
    np.savetxt(str(tmp_path / "table_0003.txt"), np.column_stack([v, 6.0 * dvdr]))
    P = pysic.Potential
    atoms = W.lj_fcc(3, noise=0.1, seed=33)
    pots = [P("tabulated", symbols=[["X", "X"]], parameters=[3, 6.0, 1.2], cutoff=5.5, cutoff_margin=0.5),
            P("LJ", symbols=[["X", "X"]], parameters=[0.0104, 3.4], cutoff=7.0)]
    ref = oracle_all(atoms, pots)
    got = engine_all(atoms, pots, None, precision)
    n = len(atoms)
    if precision == "fp64":
        assert got["energy"] == pytest.approx(ref["energy"], rel=1e-12, abs=1e-11)
        assert np.abs(got["forces"] - ref["forces"]).max() < 1e-10 * max(1.0, np.abs(ref["forces"]).max())
        np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-9, atol=1e-9 * np.abs(ref["stress"]).max())
    else:
        assert abs(got["energy"] - ref["energy"]) / n <= 1e-5
        assert np.abs(got["forces"] - ref["forces"]).max() <= 1e-4 * max(1.0, np.abs(ref["forces"]).max())


def _bend_pots():
    P = pysic.Potential
    return [P("bond_bend", symbols=[["O", "Si", "O"]], parameters=[1.3, 1.9106, 1, 2], cutoff=2.4, cutoff_margin=0.4),
            P("bond_bend", symbols=[["Si", "O", "Si"]], parameters=[0.7, 2.6, 2, 2], cutoff=2.2),
            P("exponential", symbols=[["Si", "O"]], parameters=[40.0, 3.0], cutoff=3.0, cutoff_margin=0.5)]


@pytest.mark.parametrize("n_si", [12, 200])
def test_bond_bend_fp64_parity(n_si):
    """Three-body bond_bend (Potentials.f90:3159-3314) found as the reference's
    triplet loops find it (Core.f90:3540-3943), against the oracle."""
    _check_fp64(W.sio2_box(n_si, seed=22), _bend_pots())


def test_bond_bend_mixed_accuracy():
    atoms = W.sio2_box(200, seed=23)
    pots = _bend_pots()
    ref = oracle_all(atoms, pots)
    got = engine_all(atoms, pots, None, "mixed")
    n = len(atoms)
    assert abs(got["energy"] - ref["energy"]) / n <= 1e-5
    assert np.abs(got["forces"] - ref["forces"]).max() <= 1e-4 * max(1.0, np.abs(ref["forces"]).max())
    np.testing.assert_allclose(got["stress"], ref["stress"], rtol=1e-4, atol=1e-4 * np.abs(ref["stress"]).max())


def test_bond_bend_results_are_bit_reproducible():
    atoms = W.sio2_box(200, seed=24)
    a = engine_all(atoms, _bend_pots(), None, "fp64")
    b = engine_all(atoms, _bend_pots(), None, "fp64")
    assert a["energy"] == b["energy"]
    assert np.array_equal(a["forces"], b["forces"])


def test_page_locked_buffers_match_pageable_ones():
    """Page-locked host arrays (read and written asynchronously) give the
    results of pageable ones, and a non-finite coordinate in a page-locked
    update is rejected the same way."""
    import torch

    from pysic_gb300 import _lib as L

    atoms = W.diamond_si(3, noise=0.1, seed=13)
    calc = pysic.Pysic(atoms, W.tersoff_si_potentials())
    calc.get_potential_energy()
    eng = calc.engine
    n = len(atoms)
    flags = L.WANT_ENERGY | L.WANT_FORCES | L.WANT_ENEGS

    def pinned(shape):
        return torch.zeros(shape, dtype=torch.float64, pin_memory=True).numpy()

    moved = atoms.get_positions() + np.random.default_rng(4).normal(0, 0.02, (n, 3))
    for prec in (L.PREC_FP64, L.PREC_MIXED):
        eng.update_positions(moved)
        ref = eng.calculate(prec, energy=True, forces=True, enegs=True)
        pos = pinned((n, 3))
        pos[:] = moved
        e, f, s, c = pinned(1), pinned((n, 3)), pinned(6), pinned(n)
        for _ in range(2):
            eng.update_positions(pos)
            eng.calculate_into(prec, flags, e, f, s, c)
            assert e[0] == ref["energy"]
            assert np.array_equal(f, ref["forces"])
            assert np.array_equal(s, ref["stress"])
        pos[7, 2] = np.nan
        with pytest.raises(L.EngineError) as err:
            eng.update_positions(pos)
            eng.calculate_into(prec, flags, e, f, s, c)
        assert err.value.status == L.PG_ERR_INVALID
        eng.calculate_into(prec, flags, e, f, s, c)
        assert e[0] == ref["energy"] and np.array_equal(f, ref["forces"])


def test_page_locked_step_buffers_in_every_combination():
    """Page-locked coordinates are read asynchronously after the update call
    returns: a page-locked coordinate buffer rewritten in place gives each new
    configuration's results, page-locked and pageable inputs and outputs mix
    freely, a page-locked update is committed by calls that are not
    evaluations, and a non-finite value in it is rejected there too, with the
    old coordinates kept.  Every result is bit-identical to the pageable
    path's."""
    import torch

    from pysic_gb300 import _lib as L

    atoms = W.diamond_si(3, noise=0.1, seed=17)
    calc = pysic.Pysic(atoms, W.tersoff_si_potentials())
    calc.get_potential_energy()
    eng = calc.engine
    n = len(atoms)
    flags = L.WANT_ENERGY | L.WANT_FORCES | L.WANT_ENEGS

    def pinned(shape):
        return torch.zeros(shape, dtype=torch.float64, pin_memory=True).numpy()

    rng = np.random.default_rng(5)
    configs = [atoms.get_positions() + rng.normal(0, 0.03, (n, 3)) for _ in range(4)]
    for prec in (L.PREC_FP64, L.PREC_MIXED):
        refs = []
        for x in configs:
            eng.update_positions(x.copy())
            refs.append(eng.calculate(prec, energy=True, forces=True, enegs=True))
        pos = pinned((n, 3))
        outs = {"pinned": (pinned(1), pinned((n, 3)), pinned(6), pinned(n)),
                "pageable": (np.zeros(1), np.zeros((n, 3)), np.zeros(6), np.zeros(n))}
        for step, (x, ref) in enumerate(zip(configs, refs)):
            for src in ("pinned", "pageable"):
                for dst in ("pinned", "pageable"):
                    e, f, s, c = outs[dst]
                    if src == "pinned":
                        pos[:] = x  # the same buffer, new values
                        eng.update_positions(pos)
                    else:
                        eng.update_positions(x.copy())
                    eng.calculate_into(prec, flags, e, f, s, c)
                    assert e[0] == ref["energy"], (step, src, dst)
                    assert np.array_equal(f, ref["forces"]) and np.array_equal(s, ref["stress"])
                    assert np.array_equal(c, ref["enegs"])
        # a page-locked update committed by a call that is not an evaluation
        # (the list-positions query settles outstanding updates first)
        pos[:] = configs[1]
        eng.update_positions(pos)
        eng.list_positions()
        r = eng.calculate(prec, energy=True, forces=True, enegs=True)
        assert r["energy"] == refs[1]["energy"] and np.array_equal(r["forces"], refs[1]["forces"])
        # rejected: when settled outside an evaluation, with results copied by
        # the copy engine, and with results published
        pos[3, 0] = np.inf
        eng.update_positions(pos)
        with pytest.raises(L.EngineError) as err:
            eng.list_positions()
        assert err.value.status == L.PG_ERR_INVALID
        eng.update_positions(pos)
        with pytest.raises(L.EngineError) as err:
            eng.calculate(prec, energy=True, forces=True, enegs=True)
        assert err.value.status == L.PG_ERR_INVALID
        r = eng.calculate(prec, energy=True, forces=True, enegs=True)
        assert r["energy"] == refs[1]["energy"] and np.array_equal(r["forces"], refs[1]["forces"])
        pos[3, 0] = np.nan
        e, f, s, c = outs["pinned"]
        with pytest.raises(L.EngineError) as err:
            eng.update_positions(pos)
            eng.calculate_into(prec, flags, e, f, s, c)
        assert err.value.status == L.PG_ERR_INVALID
        eng.calculate_into(prec, flags, e, f, s, c)
        assert e[0] == refs[1]["energy"] and np.array_equal(f, refs[1]["forces"])


@pytest.mark.parametrize("case", [c[0] for c in W.product_cases()])
def test_product_potentials_parity(case):
    """Products of pair potentials (ProductPotential): FP64 against the oracle
    (energy 1e-12 relative, forces 1e-10 of the largest force, virial 1e-9,
    electronegativities 1e-9), mixed precision against FP64 (1e-5 eV/atom,
    1e-4 of the largest force)."""
    _, atoms, pots = next(c for c in W.product_cases() if c[0] == case)
    ref, got = _check_fp64(atoms, pots)
    assert np.abs(got["enegs"] - ref["enegs"]).max() < 1e-9
    if case == "comb_repulsion":
        assert np.abs(ref["enegs"]).max() > 1e-3
    m = engine_all(atoms, pots, None, "mixed")
    fmax = max(1.0, np.abs(got["forces"]).max())
    assert abs(m["energy"] - got["energy"]) / len(atoms) < 1e-5
    assert np.abs(m["forces"] - got["forces"]).max() < 1e-4 * fmax


@pytest.mark.parametrize("case", [c[0] for c in W.dihedral_cases()])
def test_dihedral_parity(case):
    """Four-body dihedral (Potentials.f90:3329-3611) on the chains the
    reference's loops find (Core.f90:3614-3940): FP64 against the oracle
    (energy 1e-12 relative, forces 1e-10 of the largest force, virial 1e-9),
    mixed precision against the oracle (1e-5 eV/atom, 1e-4 of the largest
    force), and run to run bit-identical."""
    _, atoms, pots = next(c for c in W.dihedral_cases() if c[0] == case)
    ref, got = _check_fp64(atoms, pots)
    assert np.abs(ref["forces"]).max() > 1e-3
    m = engine_all(atoms, pots, None, "mixed")
    fmax = max(1.0, np.abs(ref["forces"]).max())
    assert abs(m["energy"] - ref["energy"]) / len(atoms) < 1e-5
    assert np.abs(m["forces"] - ref["forces"]).max() < 1e-4 * fmax
    again = engine_all(atoms, pots, None, "fp64")
    assert again["energy"] == got["energy"] and np.array_equal(again["forces"], got["forces"])


def test_dihedral_larger_box_parity():
    """A 1500-atom Si / O box with dihedral, bond_bend and pair terms: many
    warps, every chain loop populated."""
    _, _, pots = list(W.dihedral_cases())[1]
    _check_fp64(W.sio2_box(500, seed=53), pots)
