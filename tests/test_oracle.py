"""CPU tests of the oracle: the pins that make it trustworthy.

- known-answer values from the reference's documentation
  (doc/run examples.rst:106-145, doc/pysic class.rst:88-157),
- the published Tersoff (1988) silicon cohesive energy, -4.63 eV/atom at a = 5.432 A,
- finite-difference forces and electronegativities, the reference's own
  self-check (pysic/calculator.py:1639-1832),
- Newton's third law and translation invariance,
- neighbour-list invariants of the restated FastNeighborList.
"""
import os

import numpy as np
import pytest

import oracle
import pysic_gb300 as pysic
from helpers import oracle_all, oracle_lists
from pysic_gb300 import workloads as W
from pysic_gb300.model import compile_model, individual_cutoffs


def _allpairs(atoms, cuts):
    n = len(atoms)
    pos = atoms.get_positions()
    c, i, o = [], [], []
    for a in range(n):
        k = 0
        for b in range(n):
            if a != b and np.linalg.norm(pos[b] - pos[a]) < cuts[a] + cuts[b]:
                i.append(b)
                o.append([0, 0, 0])
                k += 1
        c.append(k)
    return np.array(c), np.array(i), np.array(o).reshape(-1, 3)


def _nonperiodic(atoms, pots):
    cuts = np.array(individual_cutoffs(atoms, pots)) + 0.5
    return oracle_all(atoms, pots, lists=_allpairs(atoms, cuts))


def test_he2_golden():
    """doc/run examples.rst:106-145"""
    atoms = pysic.Atoms("He2", [[0.0, 0.0, 0.0], [0.0, 0.0, 3.0]])
    pot = pysic.Potential("LJ", cutoff=10.0)
    pot.set_symbols(["He", "He"])
    pot.set_parameter_value("epsilon", 0.1)
    pot.set_parameter_value("sigma", 2.5)
    r = _nonperiodic(atoms, [pot])
    assert r["energy"] == -0.022274132189576905
    np.testing.assert_allclose(r["forces"], [[0, 0, 0.02211693], [0, 0, -0.02211693]], atol=5e-9)


def test_coh_golden():
    """doc/pysic class.rst:88-157"""
    atoms = pysic.Atoms("COH", [[0.0, 0.0, 0.0], [2.0, 0.0, 0.0], [2.0, 2.0, 2.0]])
    p1 = pysic.Potential("LJ", symbols=["C", "O"], parameters=[1, 1], cutoff=10.0)
    p2 = pysic.Potential("LJ", symbols=["O", "H"], parameters=[1, 1], cutoff=10.0)
    assert _nonperiodic(atoms, [p1])["energy"] == pytest.approx(-0.015380859375, abs=1e-15)
    assert _nonperiodic(atoms, [p2])["energy"] == pytest.approx(-0.00194931030273, abs=5e-15)
    r = _nonperiodic(atoms, [p1, p2])
    assert r["energy"] == pytest.approx(-0.0173301696777, abs=5e-14)
    np.testing.assert_allclose(r["forces"], [[0.04541016, 0, 0], [-0.04541016, 0.00291824, 0.00291824],
                                             [0, -0.00291824, -0.00291824]], atol=5e-9)


def test_tersoff_silicon_known_answer():
    """Tersoff, Phys. Rev. B 38, 9902 (1988): E_coh = -4.63 eV/atom at a = 5.432 A."""
    atoms = W.diamond_si(2, a0=5.432, noise=0.0)
    r = oracle_all(atoms, W.tersoff_si_potentials())
    assert r["energy"] / len(atoms) == pytest.approx(-4.63, abs=5e-3)
    assert np.abs(r["forces"]).max() < 1e-10


def _fd_forces(atoms, pots, idx, h=1e-4, coulomb=None):
    lists = oracle_lists(atoms, pots, coulomb, skin=1.0)
    model = compile_model(atoms, pots, coulomb)
    out = []
    for c in range(3):
        e = []
        for s in (+h, -h):
            pos = atoms.get_positions()
            pos[idx, c] += s
            e.append(oracle.evaluate(pos, atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(), model,
                                     *lists, what="energy"))
        out.append(-(e[0] - e[1]) / (2 * h))
    f, _ = oracle.evaluate(atoms.get_positions(), atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(),
                           model, *lists, what="forces")
    return np.array(out), f[idx]


@pytest.mark.parametrize("idx", [0, 5, 11])
def test_tersoff_forces_match_finite_differences(idx):
    atoms = W.diamond_si(2, noise=0.12, seed=3)
    fd, f = _fd_forces(atoms, W.tersoff_si_potentials(), idx)
    np.testing.assert_allclose(f, fd, atol=2e-6, rtol=1e-6)


def test_tersoff_stress_matches_strain_derivative():
    """virial W = -dE/d(strain) for a homogeneous deformation."""
    atoms = W.diamond_si(2, noise=0.08, seed=4)
    pots = W.tersoff_si_potentials()
    r = oracle_all(atoms, pots)
    model = compile_model(atoms, pots)
    h = 1e-6
    e = []
    for s in (+h, -h):
        eps = np.eye(3)
        eps[0, 0] += s
        a2 = atoms.copy()
        a2.set_cell(atoms.get_cell() @ eps, scale_atoms=True)
        lists = oracle_lists(a2, pots)
        e.append(oracle.evaluate(a2.get_positions(), a2.get_initial_charges(), a2.get_cell(), a2.get_pbc(), model,
                                 *lists, what="energy"))
    dE = (e[0] - e[1]) / (2 * h)
    assert r["stress"][0] == pytest.approx(-dE, rel=1e-6, abs=1e-6)


def test_lj_newton_and_translation():
    atoms = W.lj_fcc(3, noise=0.1, seed=1)
    pots = W.lj_potentials(cutoff=6.0)
    r = oracle_all(atoms, pots)
    assert np.abs(r["forces"].sum(axis=0)).max() < 1e-12
    a2 = atoms.copy()
    a2.set_positions(atoms.get_positions() + np.array([0.3, -1.1, 2.7]))
    r2 = oracle_all(a2, pots)
    assert r2["energy"] == pytest.approx(r["energy"], rel=1e-12)


def test_neighbor_list_symmetry_and_cutoff():
    atoms = W.diamond_si(3, noise=0.1, seed=2)
    pots = W.tersoff_si_potentials()
    c, idx, off = oracle_lists(atoms, pots)
    start = np.concatenate([[0], np.cumsum(c)])
    pos, cell = atoms.get_positions(), atoms.get_cell()
    entries = set()
    for a in range(len(atoms)):
        for e in range(start[a], start[a + 1]):
            d = np.linalg.norm(pos[idx[e]] + off[e] @ cell - pos[a])
            assert d < 3.5
            entries.add((a, idx[e], tuple(off[e])))
    for (a, b, o) in entries:
        assert (b, a, tuple(-np.array(o))) in entries
    # completeness against brute force over images
    for a in range(0, len(atoms), 17):
        want = set()
        for b in range(len(atoms)):
            for n1 in (-1, 0, 1):
                for n2 in (-1, 0, 1):
                    for n3 in (-1, 0, 1):
                        if a == b and n1 == n2 == n3 == 0:
                            continue
                        d = np.linalg.norm(pos[b] + np.array([n1, n2, n3]) @ cell - pos[a])
                        if d < 3.5:
                            want.add(b)
        got = set(idx[start[a]:start[a + 1]].tolist())
        assert got == want


def test_electronegativity_matches_charge_derivative():
    atoms = W.sio2_box(40, seed=5)
    pots, coul = W.sio2_potentials(real_cutoff=5.0, sigma=1.6)
    q = np.random.default_rng(0).normal(0, 0.3, len(atoms))
    q -= q.mean()
    atoms.set_initial_charges(q)
    model = compile_model(atoms, pots, coul)
    lists = oracle_lists(atoms, pots, coul)
    chi = oracle.evaluate(atoms.get_positions(), q, atoms.get_cell(), atoms.get_pbc(), model, *lists, what="enegs")
    for i in (0, 7, 50):
        e = []
        for s in (1e-4, -1e-4):
            qq = q.copy()
            qq[i] += s
            e.append(oracle.evaluate(atoms.get_positions(), qq, atoms.get_cell(), atoms.get_pbc(), model, *lists,
                                     what="energy"))
        assert chi[i] == pytest.approx(-(e[0] - e[1]) / 2e-4, rel=1e-6, abs=1e-7)


def test_ewald_forces_match_finite_differences():
    atoms = W.rocksalt_nacl(2, noise=0.1, seed=6)
    pots, coul = W.nacl_potentials(sigma=1.4, real_cutoff=5.0, cutoff=5.0)
    fd, f = _fd_forces(atoms, pots, 3, h=1e-5, coulomb=coul)
    np.testing.assert_allclose(f, fd, atol=1e-5, rtol=1e-5)


def test_threaded_oracle_matches_serial():
    atoms = W.diamond_si(3, noise=0.1, seed=9)
    pots = W.tersoff_si_potentials()
    a = oracle_all(atoms, pots, threads=1)
    b = oracle_all(atoms, pots, threads=4)
    assert b["energy"] == pytest.approx(a["energy"], rel=1e-13)
    np.testing.assert_allclose(b["forces"], a["forces"], atol=1e-11)


def _write_exp_table(path, ident, max_r, n, A=2.0, rho=0.6):
    """A table of V = A exp(-r/rho) with d = max_r dV/dr (the derivative with
    respect to r / max_r, as the Hermite form of evaluate_energy_table uses
    it)."""
    r = np.linspace(0.0, max_r, n)
    v = A * np.exp(-r / rho)
    d = max_r * (-v / rho)
    np.savetxt(os.path.join(path, "table_{0:04d}.txt".format(ident)), np.column_stack([v, d]))
    return A, rho


def test_oracle_tabulated_potential_interpolates_its_table(tmp_path, monkeypatch):
    """evaluate_energy_table / _force_table (Potentials.f90:4227-4298) in the
    oracle: a fine table of an exponential reproduces it (cubic Hermite), and
    beyond the range the energy is the last tabulated value, unscaled, and the
    force zero -- as the reference writes it."""
    monkeypatch.chdir(tmp_path)
    A, rho = _write_exp_table(str(tmp_path), 7, 5.0, 401)
    scale = 1.5
    pos = np.array([[0.0, 0.0, 0.0], [1.37, 0.4, -0.2], [7.5, 7.5, 7.5]])
    atoms = pysic.Atoms(["X"] * 3, pos, cell=np.eye(3) * 30.0, pbc=False)
    pot = pysic.Potential("tabulated", symbols=[["X", "X"]], parameters=[7, 5.0, scale], cutoff=14.0)
    model = compile_model(atoms, [pot])
    cuts = np.full(3, 14.0)
    c, i, o = oracle.neighbors(pos, atoms.get_cell(), atoms.get_pbc(), cuts)
    args = (pos, np.zeros(3), atoms.get_cell(), atoms.get_pbc(), model, c, i, o)
    e = oracle.evaluate(*args, what="energy")
    f, _ = oracle.evaluate(*args, what="forces")
    d01 = np.linalg.norm(pos[1] - pos[0])
    # pair 0-1 inside the range; pairs with atom 2 beyond it: each adds the last
    # row's V unscaled
    expect = scale * A * np.exp(-d01 / rho) + 2 * A * np.exp(-5.0 / rho)
    assert e == pytest.approx(expect, rel=1e-9)
    fmag = scale * A / rho * np.exp(-d01 / rho)
    np.testing.assert_allclose(f[1], fmag * (pos[1] - pos[0]) / d01, rtol=1e-7)
    np.testing.assert_array_equal(f[2], np.zeros(3))


def _bend_case():
    atoms = W.sio2_box(12, seed=21)
    P = pysic.Potential
    pots = [P("bond_bend", symbols=[["O", "Si", "O"]], parameters=[1.3, 1.9106, 1, 2], cutoff=2.4,
              cutoff_margin=0.4),
            P("bond_bend", symbols=[["Si", "O", "Si"]], parameters=[0.7, 2.6, 2, 2], cutoff=2.2)]
    return atoms, pots


def test_oracle_bond_bend_forces_are_the_energy_gradient():
    """bond_bend (Potentials.f90:3159-3314) in the oracle's triplet loops:
    forces equal minus the finite-difference gradient of the energy, smooth
    cutoff included."""
    atoms, pots = _bend_case()
    model = compile_model(atoms, pots)
    lists = oracle_lists(atoms, pots)
    pos0 = atoms.get_positions()

    def energy(p):
        return oracle.evaluate(p, atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(), model, *lists,
                               what="energy")

    f, _ = oracle.evaluate(pos0, atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(), model, *lists,
                           what="forces")
    assert np.abs(f).max() > 0.1
    h = 1e-6
    rng = np.random.default_rng(0)
    for a in rng.choice(len(atoms), 6, replace=False):
        for c in range(3):
            p1, p2 = pos0.copy(), pos0.copy()
            p1[a, c] += h
            p2[a, c] -= h
            num = -(energy(p1) - energy(p2)) / (2 * h)
            assert f[a, c] == pytest.approx(num, abs=2e-5)


def test_oracle_charge_pair_derivatives():
    """charge_pair (Potentials.f90:4415-4513) in the oracle: electronegativities
    are minus the charge derivatives of the energy and forces minus its position
    gradient (the smooth cutoff's), with the exponent order of the unpermuted
    first target."""
    atoms = W.sio2_box(12, seed=25)
    q = np.random.default_rng(3).normal(0.0, 0.5, len(atoms))
    atoms.set_initial_charges(q)
    P = pysic.Potential
    pots = [P("charge_pair", symbols=[["Si", "O"]], parameters=[0.4, 2, 1], cutoff=3.0, cutoff_margin=0.8),
            P("charge_pair", symbols=[["O", "O"]], parameters=[-0.2, 1, 3], cutoff=2.6, cutoff_margin=0.5)]
    model = compile_model(atoms, pots)
    lists = oracle_lists(atoms, pots)
    pos = atoms.get_positions()

    def ev(p, qq, what):
        return oracle.evaluate(p, qq, atoms.get_cell(), atoms.get_pbc(), model, *lists, what=what)

    chi = ev(pos, q, "enegs")
    f, _ = ev(pos, q, "forces")
    assert np.abs(chi).max() > 0.05 and np.abs(f).max() > 0.01
    h = 1e-6
    for a in (0, 5, 17, 30):
        dq = np.zeros(len(q))
        dq[a] = h
        num = -(ev(pos, q + dq, "energy") - ev(pos, q - dq, "energy")) / (2 * h)
        assert chi[a] == pytest.approx(num, abs=1e-6)
        for c in range(3):
            p1, p2 = pos.copy(), pos.copy()
            p1[a, c] += h
            p2[a, c] -= h
            numf = -(ev(p1, q, "energy") - ev(p2, q, "energy")) / (2 * h)
            assert f[a, c] == pytest.approx(numf, abs=1e-6)


# ---- per-atom (level-1) bond-order factors ----------------------------------

def _sc_closed_form(atoms, p, cutoff, margin):
    """Sutton-Chen energy from its formula (minimum image, cutoff < L/2), with the
    reference's smooth cutoff on both the pair and the density terms."""
    eps, a, c, n, m = p
    pos = atoms.get_positions()
    L = np.diag(atoms.get_cell())
    soft = cutoff - margin
    e_pair, rho = 0.0, np.zeros(len(atoms))
    for i in range(len(atoms)):
        d = pos - pos[i]
        d -= L * np.round(d / L)
        r = np.linalg.norm(d, axis=1)
        r[i] = np.inf
        sel = r < cutoff
        rr = r[sel]
        f = np.where(rr < soft, 1.0, 0.5 * (1 + np.cos(np.pi * (rr - soft) / (cutoff - soft))))
        e_pair += 0.5 * np.sum(eps * f * (a / rr) ** n)
        rho[i] = np.sum(f * (a / rr) ** m)
    return e_pair - eps * c * np.sum(np.sqrt(rho))


def test_oracle_sutton_chen_closed_form_and_gradient():
    """Sutton-Chen as the reference assembles it (suttonchen.py:68-176: a power
    pair potential plus a constant scaled by sqrt_scale over power_bond) in the
    oracle's per-atom factor loops (Core.f90:2015-2404, 2671-2735, 4745-4933):
    energy equal to the closed form, forces minus its gradient, virial minus
    its strain derivative."""
    atoms = W.fcc_alloy(4, a0=3.61, symbols=("Cu",), noise=0.06, seed=5)
    pots = W.sutton_chen_potentials(("Cu",), cutoff=5.0, cutoff_margin=0.6)
    calc = pysic.Pysic()
    for p in pots:
        calc.add_potential(p)
    pots = calc.get_potentials()
    assert [q.get_potential_type() for q in pots] == ["power", "constant"]
    r = oracle_all(atoms, pots)
    assert r["energy"] == pytest.approx(_sc_closed_form(atoms, W.SUTTON_CHEN_CU, 5.0, 0.6), rel=1e-12)
    # cohesive energy of the perfect crystal in the known range for this cutoff
    perfect = W.fcc_alloy(4, a0=3.61, symbols=("Cu",), noise=0.0)
    assert oracle_all(perfect, pots)["energy"] / len(perfect) == pytest.approx(-3.2, abs=0.4)
    fd, f = _fd_forces(atoms, pots, 7, h=1e-5)
    np.testing.assert_allclose(f, fd, atol=2e-7, rtol=1e-6)
    model = compile_model(atoms, pots)
    h = 1e-6
    e = []
    for s in (+h, -h):
        eps = np.eye(3)
        eps[1, 1] += s
        a2 = atoms.copy()
        a2.set_cell(atoms.get_cell() @ eps, scale_atoms=True)
        e.append(oracle.evaluate(a2.get_positions(), a2.get_initial_charges(), a2.get_cell(), a2.get_pbc(), model,
                                 *oracle_lists(a2, pots), what="energy"))
    assert r["stress"][1] == pytest.approx(-(e[0] - e[1]) / (2 * h), rel=1e-6, abs=1e-7)


def test_oracle_scaled_pair_potential_gradient():
    """A pair potential scaled by a c_scale-processed neighbour count (the
    doublet's (B_i + B_j)/2, Core.f90:4345-4350, 5486-5560): forces are minus the
    energy gradient for a single element."""
    atoms = W.fcc_alloy(4, a0=3.61, symbols=("Cu",), noise=0.08, seed=6)
    count = pysic.BondOrderParameters("neighbors", cutoff=3.2, cutoff_margin=0.7, symbols=[["Cu", "Cu"]])
    scale = pysic.BondOrderParameters("c_scale", parameters=[[0.8, 11.0, 0.5, 0.3, -50.0], []], symbols=[["Cu"]])
    pot = pysic.Potential("exponential", symbols=[["Cu", "Cu"]], parameters=[1.5, 1.2], cutoff=4.0,
                          cutoff_margin=0.5, coordinator=pysic.Coordinator([scale, count]))
    raw, fac = oracle.atom_factors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(),
                                   compile_model(atoms, [pot]), *oracle_lists(atoms, [pot]))
    assert raw.min() > 8 and raw.max() < 16 and np.ptp(fac) > 0.05
    for idx in (3, 50):
        fd, f = _fd_forces(atoms, [pot], idx, h=1e-5)
        np.testing.assert_allclose(f, fd, atol=2e-7, rtol=1e-6)


def test_oracle_atom_factor_sums_follow_the_picked_pair():
    """For an element pair A-B the reference adds a factor record only from the
    atom that pick makes atom1 (Core.f90:2040-2095): with the record [Cu, Ag]
    alone, each Cu-Ag pair counts once in both atoms' sums when the Cu atom is
    atom1 and not at all otherwise."""
    atoms = W.fcc_alloy(3, a0=3.61, symbols=("Cu", "Ag"), noise=0.05, seed=7)
    count = pysic.BondOrderParameters("neighbors", cutoff=3.0, symbols=[["Cu", "Ag"]])
    pot = pysic.Potential("constant", parameters=[1.0], symbols=[["Cu"]], coordinator=pysic.Coordinator([count]))
    model = compile_model(atoms, [pot])
    c, idx, off = oracle_lists(atoms, [pot])
    raw, fac = oracle.atom_factors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), model, c, idx, off)
    sym = np.array(atoms.get_chemical_symbols())
    pos, cell = atoms.get_positions(), atoms.get_cell()
    expect = np.zeros(len(atoms))
    start = np.concatenate([[0], np.cumsum(c)])
    for i in range(len(atoms)):
        for e in range(start[i], start[i + 1]):
            j, o = idx[e], off[e]
            d = np.linalg.norm(pos[j] + o @ cell - pos[i])
            # pick, Geometry.f90:648-676: atom1 is the lower index; an atom and
            # its own image by the sign of the first nonzero offset
            if i == j:
                first = next(x for x in o if x != 0) > 0
            else:
                first = i < j
            if first and sym[i] == "Cu" and sym[j] == "Ag" and d < 3.0:
                expect[i] += 1
                expect[j] += 1
    np.testing.assert_array_equal(raw, expect)
    np.testing.assert_array_equal(fac, expect)
    assert oracle_all(atoms, [pot])["energy"] == pytest.approx(expect[sym == "Cu"].sum(), abs=1e-12)


def test_oracle_tabulated_factors_gradient(tmp_path, monkeypatch):
    """table_bond (Potentials.f90:6663-6765) summed per atom and post-processed
    by table_scale (6496-6576), scaling a constant: forces are minus the energy
    gradient (one element), and a sum beyond table_scale's range gives the last
    tabulated value, unscaled."""
    monkeypatch.chdir(tmp_path)
    _write_exp_table(str(tmp_path), 11, 6.0, 161, A=1.0, rho=1.1)
    x = np.linspace(0.0, 3.0, 121)
    np.savetxt(str(tmp_path / "table_0012.txt"), np.column_stack([np.sqrt(x + 0.2), 3.0 * 0.5 / np.sqrt(x + 0.2)]))
    atoms = W.fcc_alloy(4, a0=3.61, symbols=("Cu",), noise=0.08, seed=8)
    bond = pysic.BondOrderParameters("table_bond", parameters=[[], [11, 6.0, 0.9]], cutoff=4.0, cutoff_margin=0.6,
                                     symbols=[["Cu", "Cu"]])
    scale = pysic.BondOrderParameters("table_scale", parameters=[[12, 3.0, -1.3], []], symbols=[["Cu"]])
    pot = pysic.Potential("constant", parameters=[0.7], symbols=[["Cu"]], coordinator=pysic.Coordinator([scale, bond]))
    model = compile_model(atoms, [pot])
    lists = oracle_lists(atoms, [pot])
    raw, fac = oracle.atom_factors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(), model, *lists)
    assert 0.5 < raw.min() and raw.max() < 3.0
    np.testing.assert_allclose(fac, -1.3 * np.sqrt(raw + 0.2), rtol=1e-6)
    for idx in (2, 40):
        fd, f = _fd_forces(atoms, [pot], idx, h=1e-5)
        np.testing.assert_allclose(f, fd, atol=2e-7, rtol=1e-6)
    # a range the sums exceed: the last row's value, unscaled
    short = pysic.BondOrderParameters("table_scale", parameters=[[12, 0.5, -1.3], []], symbols=[["Cu"]])
    pot2 = pysic.Potential("constant", parameters=[0.7], symbols=[["Cu"]],
                           coordinator=pysic.Coordinator([short, bond]))
    _, fac2 = oracle.atom_factors(atoms.get_positions(), atoms.get_cell(), atoms.get_pbc(),
                                  compile_model(atoms, [pot2]), *lists)
    np.testing.assert_allclose(fac2, np.sqrt(3.0 + 0.2), rtol=1e-15)


def test_oracle_atom_factor_gradients_match_finite_differences():
    """core_calculate_bond_order_gradients and _of_factor (Core.f90:1157-1989)
    restated: for one element, the gradient of every atom's Sutton-Chen density
    factor with respect to one atom, and of one atom's factor with respect to
    every atom, equal finite differences of the factors."""
    atoms = W.fcc_alloy(4, a0=3.61, symbols=("Cu",), noise=0.07, seed=9)
    calc = pysic.Pysic()
    calc.add_potential(W.sutton_chen_potentials(("Cu",)))
    pots = calc.get_potentials()
    model = compile_model(atoms, pots)
    lists = oracle_lists(atoms, pots)
    cell, pbc = atoms.get_cell(), atoms.get_pbc()
    pos0 = atoms.get_positions()
    a, h = 17, 1e-6
    g_all = oracle.atom_factor_gradients(pos0, cell, pbc, model, *lists, group=0, atom=a)
    g_of = oracle.atom_factor_gradients(pos0, cell, pbc, model, *lists, group=0, atom=a, of_factor=True)
    num_all = np.zeros((len(atoms), 3))
    for c in range(3):
        p1, p2 = pos0.copy(), pos0.copy()
        p1[a, c] += h
        p2[a, c] -= h
        f1 = oracle.atom_factors(p1, cell, pbc, model, *lists)[1]
        f2 = oracle.atom_factors(p2, cell, pbc, model, *lists)[1]
        num_all[:, c] = (f1 - f2) / (2 * h)
    np.testing.assert_allclose(g_all, num_all, atol=1e-6)
    for b in [a] + list(np.nonzero(np.abs(g_of).sum(axis=1))[0][:4]):
        for c in range(3):
            p1, p2 = pos0.copy(), pos0.copy()
            p1[b, c] += h
            p2[b, c] -= h
            d = (oracle.atom_factors(p1, cell, pbc, model, *lists)[1][a] -
                 oracle.atom_factors(p2, cell, pbc, model, *lists)[1][a]) / (2 * h)
            assert g_of[b, c] == pytest.approx(d, abs=1e-6)


def _charge_exp_case():
    atoms = W.sio2_box(12, seed=26)
    q = np.random.default_rng(4).normal(0.0, 0.4, len(atoms))
    atoms.set_initial_charges(q)
    # Rmax / (Rmax - Rmin) = Qmax / (Qmax - Qmin) gives eta = 1 (a finite beta)
    pots = [pysic.Potential("charge_exp", symbols=[["Si", "O"]],
                            parameters=[0.3, 2.0, 1.0, 2.0, 1.0, 3.0, 1.5, 2.4, 1.2, 0.6, 0.4],
                            cutoff=3.0, cutoff_margin=0.8),
            pysic.Potential("charge_exp", symbols=[["O", "O"]],
                            parameters=[0.2, 2.5, 1.25, 1.8, 0.9, 2.5, 1.25, 1.8, 0.9, 0.5, 0.5],
                            cutoff=2.6, cutoff_margin=0.5)]
    return atoms, pots


def test_oracle_charge_exp_derivatives():
    """charge_exp (Potentials.f90:3691-3903) in the oracle: electronegativities
    are minus the charge derivatives of the energy (with the parameter swap of
    the unpermuted first target), forces minus the position gradient (the cut
    factor's only)."""
    atoms, pots = _charge_exp_case()
    model = compile_model(atoms, pots)
    lists = oracle_lists(atoms, pots)
    pos, q = atoms.get_positions(), atoms.get_initial_charges()

    def ev(p, qq, what):
        return oracle.evaluate(p, qq, atoms.get_cell(), atoms.get_pbc(), model, *lists, what=what)

    chi = ev(pos, q, "enegs")
    f, _ = ev(pos, q, "forces")
    assert np.abs(chi).max() > 0.01 and np.abs(f).max() > 1e-3
    h = 1e-6
    for a in (0, 5, 17):
        q1, q2 = q.copy(), q.copy()
        q1[a] += h
        q2[a] -= h
        assert chi[a] == pytest.approx(-(ev(pos, q1, "energy") - ev(pos, q2, "energy")) / (2 * h), abs=1e-7)
        for c in range(3):
            p1, p2 = pos.copy(), pos.copy()
            p1[a, c] += h
            p2[a, c] -= h
            assert f[a, c] == pytest.approx(-(ev(p1, q, "energy") - ev(p2, q, "energy")) / (2 * h), abs=1e-7)


def test_oracle_charge_abs_derivatives():
    """charge_abs (Potentials.f90:4525-4728) in the oracle: electronegativities
    are minus the charge derivatives of the energy, forces minus the position
    gradient (the cut factor's only), exponents swapped with the unpermuted
    first target."""
    atoms = W.sio2_box(12, seed=28)
    q = np.random.default_rng(6).normal(0.0, 0.4, len(atoms))
    atoms.set_initial_charges(q)
    pots = [pysic.Potential("charge_abs", symbols=[["Si", "O"]], parameters=[1.0, 0.5, 0.3, 2.0, 0.8, 0.7, -0.2, 1.5],
                            cutoff=3.0, cutoff_margin=0.8),
            pysic.Potential("charge_abs", symbols=[["O", "O"]], parameters=[0.6, 0.4, -0.1, 2.5, 0.6, 0.4, -0.1, 2.5],
                            cutoff=2.6, cutoff_margin=0.5)]
    model = compile_model(atoms, pots)
    lists = oracle_lists(atoms, pots)
    pos = atoms.get_positions()

    def ev(p, qq, what):
        return oracle.evaluate(p, qq, atoms.get_cell(), atoms.get_pbc(), model, *lists, what=what)

    chi = ev(pos, q, "enegs")
    f, _ = ev(pos, q, "forces")
    assert np.abs(chi).max() > 0.01 and np.abs(f).max() > 1e-3
    h = 1e-6
    for a in (0, 5, 17):
        q1, q2 = q.copy(), q.copy()
        q1[a] += h
        q2[a] -= h
        assert chi[a] == pytest.approx(-(ev(pos, q1, "energy") - ev(pos, q2, "energy")) / (2 * h), abs=1e-7)
        for c in range(3):
            p1, p2 = pos.copy(), pos.copy()
            p1[a, c] += h
            p2[a, c] -= h
            assert f[a, c] == pytest.approx(-(ev(p1, q, "energy") - ev(p2, q, "energy")) / (2 * h), abs=1e-7)


# ---- products of potentials ---------------------------------------------------

@pytest.mark.parametrize("case", [c[0] for c in W.product_cases()])
def test_oracle_product_derivatives(case):
    """Products of pair potentials in the oracle (Potentials.f90:2512-2700):
    forces are minus the position gradient of the energy and electronegativities
    minus its charge derivatives, by finite differences."""
    _, atoms, pots = next(c for c in W.product_cases() if c[0] == case)
    model = compile_model(atoms, pots)
    assert max(model.pair_nmul) > 0
    lists = oracle_lists(atoms, pots)
    pos, q = atoms.get_positions(), atoms.get_initial_charges()

    def ev(p, qq, what):
        return oracle.evaluate(p, qq, atoms.get_cell(), atoms.get_pbc(), model, *lists, what=what)

    f, _ = ev(pos, q, "forces")
    chi = ev(pos, q, "enegs")
    assert np.abs(f).max() > 1e-3
    h = 1e-6
    scale = max(1.0, np.abs(f).max())
    for a in (0, 5, 17):
        for c in range(3):
            p1, p2 = pos.copy(), pos.copy()
            p1[a, c] += h
            p2[a, c] -= h
            assert f[a, c] == pytest.approx(-(ev(p1, q, "energy") - ev(p2, q, "energy")) / (2 * h), abs=1e-6 * scale)
        if case == "comb_repulsion":
            q1, q2 = q.copy(), q.copy()
            q1[a] += h
            q2[a] -= h
            assert chi[a] == pytest.approx(-(ev(pos, q1, "energy") - ev(pos, q2, "energy")) / (2 * h), abs=1e-6)


@pytest.mark.parametrize("case", [c[0] for c in W.dihedral_cases()])
def test_oracle_dihedral_forces_and_stress(case):
    """dihedral in the oracle (Potentials.f90:3329-3611 evaluated on the
    chains of Core.f90:3540-3943): forces minus the position gradient of the
    energy, the virial the strain derivative, by finite differences."""
    _, atoms, pots = next(c for c in W.dihedral_cases() if c[0] == case)
    model = compile_model(atoms, pots)
    lists = oracle_lists(atoms, pots, skin=1.0)
    pos = atoms.get_positions()

    def energy(p, cell=None):
        return oracle.evaluate(p, atoms.get_initial_charges(), atoms.get_cell() if cell is None else cell,
                               atoms.get_pbc(), model, *lists, what="energy")

    e0 = energy(pos)
    f, st = oracle.evaluate(pos, atoms.get_initial_charges(), atoms.get_cell(), atoms.get_pbc(), model, *lists,
                            what="forces")
    assert np.abs(f).max() > 1e-3
    h = 1e-6
    for a in (0, 3, 11, 20):
        for c in range(3):
            p1, p2 = pos.copy(), pos.copy()
            p1[a, c] += h
            p2[a, c] -= h
            assert f[a, c] == pytest.approx(-(energy(p1) - energy(p2)) / (2 * h), abs=1e-6 * max(1, abs(f).max()))
    # virial sum(r_a F_b): minus the energy's derivative with respect to a homogeneous strain
    cell = np.asarray(atoms.get_cell())
    for (a, b), k in (((0, 0), 0), ((1, 1), 1), ((2, 2), 2)):
        eps = np.eye(3)
        eps[a, b] += h
        em = np.eye(3)
        em[a, b] -= h
        de = (energy(pos @ eps.T, cell @ eps.T) - energy(pos @ em.T, cell @ em.T)) / (2 * h)
        assert st[k] == pytest.approx(-de, abs=1e-6 * max(1.0, abs(e0)))


@pytest.mark.parametrize("case", [c[0] for c in W.comb_style_cases()])
def test_oracle_tersoff_scaled_charge_products(case):
    """A Tersoff Coordinator on charge-dependent products (COMB's attraction
    form, comb.py:660-900) in the oracle: forces minus the position gradient
    of the energy, the virial its strain derivative and the electronegativities
    minus its charge derivatives, by finite differences (the bond-order factors
    depend on the positions only)."""
    _, atoms, pots = next(c for c in W.comb_style_cases() if c[0] == case)
    model = compile_model(atoms, pots)
    assert max(model.pair_nmul) > 0 and max(model.pair_group) >= 0
    lists = oracle_lists(atoms, pots)
    pos, q, cell = atoms.get_positions(), atoms.get_initial_charges(), np.asarray(atoms.get_cell())

    def ev(p, qq, what, c=None):
        return oracle.evaluate(p, qq, cell if c is None else c, atoms.get_pbc(), model, *lists, what=what)

    e0 = ev(pos, q, "energy")
    f, st = ev(pos, q, "forces")
    chi = ev(pos, q, "enegs")
    assert np.abs(f).max() > 1e-2 and np.abs(chi).max() > 1e-2
    h = 1e-6
    scale = max(1.0, np.abs(f).max())
    for a in (0, 4, 13, 30):
        for c in range(3):
            p1, p2 = pos.copy(), pos.copy()
            p1[a, c] += h
            p2[a, c] -= h
            assert f[a, c] == pytest.approx(-(ev(p1, q, "energy") - ev(p2, q, "energy")) / (2 * h), abs=1e-6 * scale)
        q1, q2 = q.copy(), q.copy()
        q1[a] += h
        q2[a] -= h
        assert chi[a] == pytest.approx(-(ev(pos, q1, "energy") - ev(pos, q2, "energy")) / (2 * h), abs=1e-6)
    for k, (a, b) in enumerate(((0, 0), (1, 1), (2, 2))):
        ep, em = np.eye(3), np.eye(3)
        ep[a, b] += h
        em[a, b] -= h
        de = (ev(pos @ ep.T, q, "energy", cell @ ep.T) - ev(pos @ em.T, q, "energy", cell @ em.T)) / (2 * h)
        assert st[k] == pytest.approx(-de, abs=1e-6 * max(1.0, abs(e0)))


def test_oracle_step_potential_is_the_references_formula():
    """step (Potentials.f90:4858-4967): e1 below r1, e2 above r2 and
    (e1 + e2)/2 (1 + cos(pi t)/2) between, t = (r - r1)/(r2 - r1); its force
    on the pair's atom 1 is c (1, 1, 1), c = (e1 + e2) pi/(4 (r2 - r1))
    sin(pi t), and -c (1, 1, 1) on atom 2 -- the reference's own force, which is
    neither the energy's gradient nor along the bond.  Without a margin there
    is no cut factor; with one, the smooth cut's radial term is added
    (Core.f90:5530-5560)."""
    e1, e2, r1, r2 = 0.3, -0.1, 2.0, 4.0
    u = np.array([0.48, -0.6, 0.64])
    u /= np.linalg.norm(u)
    for d, margin in ((1.5, 0.0), (3.0, 0.0), (3.3, 0.0), (4.5, 0.0), (3.3, 1.5)):
        atoms = pysic.Atoms("He2", [[0.0, 0.0, 0.0], list(d * u)])
        pot = pysic.Potential("step", symbols=[["He", "He"]], parameters=[e1, e2, r1, r2], cutoff=6.0,
                              cutoff_margin=margin)
        r = _nonperiodic(atoms, [pot])
        t = (d - r1) / (r2 - r1)
        v = e1 if d < r1 else e2 if d > r2 else (e1 + e2) * 0.5 * (1 + 0.5 * np.cos(np.pi * t))
        c = 0.0 if (d < r1 or d > r2) else (e1 + e2) * 0.25 * np.pi / (r2 - r1) * np.sin(np.pi * t)
        f, fp = 1.0, 0.0
        if margin > 0.0 and d > 6.0 - margin:
            w = (d - (6.0 - margin)) / margin
            f, fp = 0.5 * (1 + np.cos(np.pi * w)), -0.5 * np.pi / margin * np.sin(np.pi * w)
        assert r["energy"] == pytest.approx(v * f, rel=1e-12, abs=1e-15)
        f1 = c * f * np.ones(3) + v * fp * u  # atom 1 (index 0): u points from it to atom 2
        np.testing.assert_allclose(r["forces"][0], f1, rtol=1e-12, atol=1e-15)
        np.testing.assert_allclose(r["forces"][1], -f1, rtol=1e-12, atol=1e-15)


def test_step_potential_refused_where_its_force_cannot_be_carried():
    """The engine evaluates step as a plain pair term: a Coordinator or a
    product around it is refused at compile time (its force is not radial)."""
    atoms = W.lj_fcc(2, noise=0.05, seed=3)
    step = pysic.Potential("step", symbols=[["X", "X"]], parameters=[0.1, 0.0, 3.0, 4.0], cutoff=5.0)
    lj = pysic.Potential("LJ", symbols=[["X", "X"]], parameters=[0.01, 3.4], cutoff=5.0)
    compile_model(atoms, [step, lj])
    with pytest.raises(pysic.InvalidPotentialError):
        compile_model(atoms, [pysic.ProductPotential([step, lj])])
    with pytest.raises(pysic.InvalidPotentialError):
        compile_model(atoms, [pysic.ProductPotential([lj, step])])
    scaled = pysic.Potential("step", symbols=[["X", "X"]], parameters=[0.1, 0.0, 3.0, 4.0], cutoff=5.0)
    scaled.set_coordinator(pysic.Coordinator([pysic.BondOrderParameters("neighbors", cutoff=4.0,
                                                                        symbols=[["X", "X"]])]))
    with pytest.raises(pysic.InvalidPotentialError):
        compile_model(atoms, [scaled])
