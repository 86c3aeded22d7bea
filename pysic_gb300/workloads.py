"""Seeded synthetic structures and interaction sets of the benchmark workloads.

The reference publishes no benchmark inputs, so every workload is a seeded
synthetic structure with the shapes and parameters of the five benchmark
configurations:

1. ``lj_fcc``        Lennard-Jones fcc crystal, 6x6x6 cells, a = 5.26 A (864 atoms)
2. ``tersoff_si``    diamond silicon, a = 5.431 A, 8^3 (4096) or 16^3 (32768) atoms
3. ``ewald_nacl``    rock salt 10^3 cells (8000 ions) with Ewald + Buckingham
4. ``batched_si``    512 periodic Si boxes with log-uniform atom counts
5. ``sio2_relax``    SiO2-like boxes for charge relaxation

Noise is Gaussian with the stated sigma from ``numpy.random.default_rng(seed)``.
"""
import math

import numpy as np

from .atoms import Atoms
from .interactions import BondOrderParameters, Coordinator, CoulombSummation, Potential

EPS0 = 0.00552635  # e^2/(eV A), pysic/interactions/coulomb.py:201


def _lattice(basis, n, a0):
    g = np.array([[i, j, k] for i in range(n) for j in range(n) for k in range(n)], dtype=np.float64)
    return ((g[:, None, :] + np.asarray(basis)[None, :, :]).reshape(-1, 3)) * a0


def lj_fcc(n=6, a0=5.26, noise=0.05, seed=0, symbol="X"):
    basis = [[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]]
    pos = _lattice(basis, n, a0)
    pos = pos + np.random.default_rng(seed).normal(0.0, noise, pos.shape)
    return Atoms([symbol] * len(pos), pos, cell=np.eye(3) * a0 * n, pbc=True)


def lj_potentials(symbol="X", epsilon=0.0104, sigma=3.40, cutoff=8.5):
    """pysic LJ is epsilon[(s/r)^12 - (s/r)^6] (no factor 4, Potentials.f90:3003):
    epsilon is taken literally."""
    return [Potential("LJ", symbols=[[symbol, symbol]], parameters=[epsilon, sigma], cutoff=cutoff)]


# Sutton & Chen, Phil. Mag. Lett. 61, 139 (1990): copper (eps eV, a A, c, n, m)
SUTTON_CHEN_CU = (1.2382e-2, 3.61, 39.432, 9.0, 6.0)


def fcc_alloy(n=4, a0=3.61, symbols=("Cu", "Ag"), fraction=0.5, noise=0.05, seed=0):
    """fcc crystal with the sites of the second element drawn at the given fraction."""
    atoms = lj_fcc(n=n, a0=a0, noise=noise, seed=seed, symbol=symbols[0])
    if len(symbols) == 1:
        return atoms
    rng = np.random.default_rng(seed + 1)
    sym = np.where(rng.random(len(atoms)) < fraction, symbols[1], symbols[0])
    return Atoms(list(sym), atoms.get_positions(), cell=atoms.get_cell(), pbc=True)


def sutton_chen_potentials(symbols=("Cu",), p=SUTTON_CHEN_CU, cutoff=5.0, cutoff_margin=0.5):
    """One Sutton-Chen compound on every element pair of the given elements."""
    from .interactions import SuttonChenPotential

    pairs = [[a, b] for i, a in enumerate(symbols) for b in symbols[i:]]
    return [SuttonChenPotential(symbols=pairs, parameters=list(p), cutoff=cutoff, cutoff_margin=cutoff_margin)]


def diamond_si(n=8, a0=5.431, noise=0.10, seed=0):
    basis = [[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0], [0.25, 0.25, 0.25], [0.25, 0.75, 0.75],
             [0.75, 0.25, 0.75], [0.75, 0.75, 0.25]]
    pos = _lattice(basis, n, a0)
    if noise > 0:
        pos = pos + np.random.default_rng(seed).normal(0.0, noise, pos.shape)
    return Atoms(["Si"] * len(pos), pos, cell=np.eye(3) * a0 * n, pbc=True)


TERSOFF_SI = {"A": 1830.8, "B": 471.18, "lambda1": 2.4799, "lambda2": 1.7322, "beta": 1.1e-6, "n": 0.78734,
              "c": 100390.0, "d": 16.217, "h": -0.59825, "R": 2.7, "D": 0.3}


def tersoff_si_potentials(p=TERSOFF_SI):
    """Tersoff (1988) silicon in pysic terms: repulsive and attractive
    'exponential' pair potentials, the attractive one scaled by a 'tersoff'
    bond-order factor; cutoff R + D with margin 2D, so pysic's smooth cutoff
    1/2(1 + cos) on [R - D, R + D] equals Tersoff's 1/2 - 1/2 sin(pi/2 (r - R)/D)."""
    rc, margin = p["R"] + p["D"], 2.0 * p["D"]
    bo = BondOrderParameters("tersoff", cutoff=rc, cutoff_margin=margin, symbols=[["Si", "Si", "Si"]],
                             parameters=[[p["beta"], p["n"]], [0.0, p["c"], p["d"], p["h"], 3.0]])
    crd = Coordinator([bo])
    rep = Potential("exponential", symbols=[["Si", "Si"]], parameters=[p["A"], p["lambda1"]], cutoff=rc,
                    cutoff_margin=margin)
    att = Potential("exponential", symbols=[["Si", "Si"]], parameters=[-p["B"], p["lambda2"]], cutoff=rc,
                    cutoff_margin=margin, coordinator=crd)
    return [rep, att]


def rocksalt_nacl(n=10, a0=5.64, noise=0.05, seed=0):
    na = [[0, 0, 0], [0, 0.5, 0.5], [0.5, 0, 0.5], [0.5, 0.5, 0]]
    cl = [[0.5, 0, 0], [0.5, 0.5, 0.5], [0, 0, 0.5], [0, 0.5, 0]]
    pos = _lattice(na + cl, n, a0)
    symbols = (["Na"] * 4 + ["Cl"] * 4) * (len(pos) // 8)
    charges = np.tile(np.array([1.0] * 4 + [-1.0] * 4), len(pos) // 8)
    pos = pos + np.random.default_rng(seed).normal(0.0, noise, pos.shape)
    return Atoms(symbols, pos, cell=np.eye(3) * a0 * n, pbc=True, charges=charges)


def ewald_kcut(sigma, rel_tail=1e-6):
    """Reciprocal cutoff where exp(-sigma^2 k^2 / 2) falls to rel_tail."""
    return math.sqrt(-2.0 * math.log(rel_tail)) / sigma


def nacl_potentials(A=1000.0, rho=0.30, C=10.0, cutoff=10.0, sigma=2.5, real_cutoff=10.0, k_cutoff=None):
    """Buckingham A e^(-r/rho) - C/r^6 on unlike pairs: pysic's Buckingham is
    A e^(-r/sigma) - C' (sigma/r)^6 (Potentials.f90:3990-3998), so C' = C / rho^6."""
    buck = Potential("Buckingham", symbols=[["Na", "Cl"]], parameters=[A, C / rho ** 6, rho], cutoff=cutoff)
    if k_cutoff is None:
        k_cutoff = ewald_kcut(sigma)
    coul = CoulombSummation("ewald", [real_cutoff, k_cutoff, sigma, EPS0])
    return [buck], coul


def random_box(symbols, density_per_a3, min_dist, seed, max_tries=200000):
    """Uniform random positions in a cubic periodic box with rejection below
    min_dist (minimum image): random sequential addition, with candidates
    drawn in batches and tested against a cell grid, and the candidates of a
    batch accepted in draw order."""
    n = len(symbols)
    L = (n / density_per_a3) ** (1.0 / 3.0)
    rng = np.random.default_rng(seed)
    md2 = min_dist * min_dist
    nc = max(1, int(L // min_dist))
    cw = L / nc
    K = int(max(4, math.ceil(3.0 * density_per_a3 * cw ** 3) + 2))  # slots per grid cell, grown on demand
    occ = np.full((nc, nc, nc, K), -1, dtype=np.int64)
    cnt = np.zeros((nc, nc, nc), dtype=np.int64)
    offs = np.array([[a, b, c] for a in (-1, 0, 1) for b in (-1, 0, 1) for c in (-1, 0, 1)])
    if nc < 3:  # every cell is a neighbour of every other: one shared cell list
        offs = np.array([[a, b, c] for a in range(nc) for b in range(nc) for c in range(nc)])
    pos = np.zeros((n, 3))
    placed = 0
    tries = 0
    while placed < n:
        if tries > max_tries * max(1, n // 1000):
            raise RuntimeError("random packing failed")
        m = int(min(768, max(64, 2 * (n - placed))))
        cand = rng.uniform(0.0, L, (m, 3))
        tries += m
        cell = (cand // cw).astype(np.int64) % nc
        near = (cell[:, None, :] + offs[None, :, :]) % nc
        nb = occ[near[..., 0], near[..., 1], near[..., 2]].reshape(m, -1)
        d = pos[np.maximum(nb, 0)] - cand[:, None, :]
        d -= L * np.round(d / L)
        clash = (nb >= 0) & ((d * d).sum(-1) < md2)
        idx = np.nonzero(~clash.any(axis=1))[0]
        if len(idx) == 0:
            continue
        p = cand[idx]
        dd = p[:, None, :] - p[None, :, :]
        dd -= L * np.round(dd / L)
        conflict = (dd * dd).sum(-1) < md2
        keep = np.ones(len(idx), dtype=bool)
        for a in range(len(idx)):
            if keep[a]:
                keep[a + 1:] &= ~conflict[a, a + 1:]
        for q in idx[keep][: n - placed]:
            cx, cy, cz = cell[q]
            k = cnt[cx, cy, cz]
            if k >= K:
                occ = np.concatenate([occ, np.full((nc, nc, nc, K), -1, dtype=np.int64)], axis=3)
                K *= 2
            occ[cx, cy, cz, k] = placed
            cnt[cx, cy, cz] = k + 1
            pos[placed] = cand[q]
            placed += 1
    return Atoms(list(symbols), pos, cell=np.eye(3) * L, pbc=True)


SI_DENSITY = 2.33 * 6.02214076e23 / 28.0855 * 1e-24  # atoms per A^3 (0.04996)


def batched_si(n_systems=512, lo=64, hi=2048, seed=0):
    """Atom counts log-uniform in [lo, hi], cubic boxes at 2.33 g/cm^3, uniform
    random positions with rejection below 2.0 A."""
    rng = np.random.default_rng(seed)
    counts = np.floor(np.exp(rng.uniform(math.log(lo), math.log(hi), n_systems))).astype(int)
    return [random_box(["Si"] * int(c), SI_DENSITY, 2.0, seed * 100003 + k) for k, c in enumerate(counts)]


def batched_potentials():
    return tersoff_si_potentials() + [Potential("LJ", symbols=[["Si", "Si"]], parameters=[0.01, 2.1], cutoff=5.0)]


SIO2_DENSITY = 2.2 * 6.02214076e23 / 60.0843 * 3 * 1e-24  # atoms per A^3


def sio2_box(n_si=1000, seed=0):
    symbols = ["Si"] * n_si + ["O"] * (2 * n_si)
    return random_box(symbols, SIO2_DENSITY, 1.5, seed)


SIO2_CHARGE_PARAMS = {"Si": (4.17, 6.97), "O": (8.74, 13.36)}


def sio2_potentials(real_cutoff=10.0, sigma=2.5, k_cutoff=None, half_hardness=False):
    """Charge self energy chi q + J q^2 per element as two 'charge_self'
    terms (epsilon q^n, n = 1 and 2).  With J as the quadratic coefficient the
    charge Hessian of these random structures (Si-O pairs down to 1.5 A, point
    charges) is positive definite; with J/2 (half_hardness=True) the close
    Si-O Coulomb coupling (14.4/1.5 = 9.6 eV) exceeds the hardness and the
    energy has no minimum in q, so damped dynamics diverge."""
    pots = []
    for el, (chi, J) in SIO2_CHARGE_PARAMS.items():
        pots.append(Potential("charge_self", symbols=[[el]], parameters=[chi, 1]))
        pots.append(Potential("charge_self", symbols=[[el]], parameters=[J / 2.0 if half_hardness else J, 2]))
    if k_cutoff is None:
        k_cutoff = ewald_kcut(sigma)
    coul = CoulombSummation("ewald", [real_cutoff, k_cutoff, sigma, EPS0])
    return pots, coul


def product_cases():
    """Small structures with products of pair potentials (ProductPotential,
    pysic/interactions/local.py:7-283): a smooth-cut LJ x exponential x
    Buckingham product on an fcc crystal, and on random SiO2 boxes with
    charges the charge-dependent products of the COMB repulsion (charge_exp x
    exponential, the pysic COMB compound's form, pysic/interactions/comb.py:
    901-977) and a charge_pair x power product, next to plain terms."""
    P = Potential
    from .interactions import ProductPotential

    a1 = lj_fcc(2, noise=0.08, seed=41)
    prod1 = ProductPotential([P("LJ", symbols=[["X", "X"]], parameters=[0.02, 2.9], cutoff=5.0, cutoff_margin=0.7),
                              P("exponential", symbols=[["X", "X"]], parameters=[1.5, 0.3]),
                              P("Buckingham", symbols=[["X", "X"]], parameters=[2.0, 0.5, 1.1])])
    yield "lj_exp_buck", a1, [prod1, P("LJ", symbols=[["X", "X"]], parameters=[0.01, 3.1], cutoff=4.5)]
    a2 = sio2_box(12, seed=42)
    q = np.random.default_rng(5).normal(0.0, 0.4, len(a2))
    a2.set_initial_charges(q - q.mean())
    cexp = P("charge_exp", symbols=[["Si", "O"], ["O", "O"]],
             parameters=[0.3, 2.0, 1.0, 2.0, 1.0, 3.0, 1.5, 2.4, 1.2, 0.6, 0.4], cutoff=3.2, cutoff_margin=0.6)
    prod2 = ProductPotential([cexp, P("exponential", symbols=[["Si", "O"]], parameters=[40.0, 1.8])])
    prod3 = ProductPotential([P("charge_pair", symbols=[["Si", "Si"], ["Si", "O"]], parameters=[0.4, 2, 1],
                                cutoff=3.0, cutoff_margin=0.5),
                              P("power", symbols=[["Si", "Si"]], parameters=[0.8, 2.0, 3.0])])
    yield "comb_repulsion", a2, [prod2, prod3, P("exponential", symbols=[["O", "O"]], parameters=[10.0, 2.0],
                                                   cutoff=2.8, cutoff_margin=0.4)]


def dihedral_cases():
    """Structures with four-body dihedral terms (Potentials.f90:3329-3611):
    a single-element chain network (a distorted diamond crystal, every
    permutation of the one-element tuple the same record) and a two-element
    random box with an unsymmetric target tuple (several distinct
    permutations, the forward / backward element match) next to a bond_bend
    and a pair term, both with smooth cutoffs."""
    P = Potential
    a1 = diamond_si(2, noise=0.12, seed=51)
    yield "si_dihedral", a1, [P("dihedral", symbols=[["Si", "Si", "Si", "Si"]], parameters=[0.3, 1.1],
                                 cutoff=2.9, cutoff_margin=0.4)]
    a2 = sio2_box(10, seed=52)
    yield "sio_dihedral", a2, [P("dihedral", symbols=[["Si", "O", "O", "Si"], ["O", "Si", "O", "O"]],
                                  parameters=[0.4, 2.0], cutoff=2.6, cutoff_margin=0.5),
                               P("bond_bend", symbols=[["O", "Si", "O"]], parameters=[0.2, 1.9, 1, 2], cutoff=2.6,
                                 cutoff_margin=0.4),
                               P("exponential", symbols=[["Si", "O"]], parameters=[5.0, 1.5], cutoff=2.6)]


def comb_style_cases():
    """Tersoff bond-order factors scaling charge-dependent products, the form
    of COMB's attraction (pysic/interactions/comb.py:660-900: charge_exp x
    charge_abs x exponential with a Coordinator of 'tersoff' factors), on
    random SiO2 boxes with random charges: first one Coordinator over every
    Si / O triplet (the post-processing beta, eta shared by each centre
    element), the scaled product on Si-O and O-O pairs, a scaled charge_exp on
    Si-Si pairs, and an unscaled repulsion; then COMB's layout of one
    Coordinator per element pair with its own factors and post-processing.
    Energies, forces, virial and electronegativities all depend on the bond
    orders and the charges."""
    P = Potential
    from .interactions import ProductPotential

    a = sio2_box(12, seed=61)
    q = np.random.default_rng(62).normal(0.0, 0.5, len(a))
    a.set_initial_charges(q - q.mean())
    sio = [[x, y, z] for x in ("Si", "O") for y in ("Si", "O") for z in ("Si", "O")]
    bo = BondOrderParameters("tersoff", cutoff=3.0, cutoff_margin=0.6, symbols=sio,
                             parameters=[[0.8, 0.9], [0.0, 2.0, 1.5, -0.4, 1.0]])
    crd = Coordinator([bo])
    cexp = P("charge_exp", symbols=[["Si", "O"], ["O", "O"]],
             parameters=[0.3, 2.0, 1.0, 2.0, 1.0, 3.0, 1.5, 2.4, 1.2, 0.6, 0.4], cutoff=3.0, cutoff_margin=0.6)
    cabs = P("charge_abs", symbols=[["Si", "O"], ["O", "O"]], parameters=[1.2, 0.3, 0.2, 2.0, 1.5, 0.4, -0.3, 2.0])
    expo = P("exponential", symbols=[["Si", "O"], ["O", "O"]], parameters=[-8.0, 1.2])
    prod = ProductPotential([cexp, cabs, expo])
    prod.set_coordinator(crd)
    si = P("charge_exp", symbols=[["Si", "Si"]], parameters=[-0.5, 2.0, 1.0, 2.0, 1.0, 3.0, 1.5, 2.4, 1.2, 0.6, 0.4],
           cutoff=3.0, cutoff_margin=0.6, coordinator=crd)
    rep = P("exponential", symbols=[["Si", "O"], ["O", "O"], ["Si", "Si"]], parameters=[30.0, 2.5], cutoff=3.0,
            cutoff_margin=0.6)
    yield "comb_attraction", a, [prod, si, rep]
    # COMB's layout: one Coordinator per element pair (comb.py:700-900), each
    # with its own Tersoff factors and post-processing, on Si-Si, O-O and Si-O
    a2 = sio2_box(14, seed=63)
    q2 = np.random.default_rng(64).normal(0.0, 0.5, len(a2))
    a2.set_initial_charges(q2 - q2.mean())

    def crd(triples, beta, eta, h):
        return Coordinator([BondOrderParameters("tersoff", cutoff=3.0, cutoff_margin=0.6, symbols=triples,
                                                parameters=[[beta, eta], [0.0, 2.0, 1.5, h, 1.0]])])

    pots = []
    for pair, triples, beta, eta, h in (
            (["Si", "Si"], [["Si", "Si", "Si"], ["Si", "Si", "O"]], 0.8, 0.9, -0.4),
            (["O", "O"], [["O", "O", "O"], ["O", "O", "Si"]], 0.5, 1.3, 0.2),
            (["Si", "O"], [["Si", "O", "O"], ["Si", "O", "Si"], ["O", "Si", "Si"], ["O", "Si", "O"]], 1.1, 0.7,
             -0.1)):
        f1 = P("charge_exp", symbols=[pair], parameters=[0.3, 2.0, 1.0, 2.0, 1.0, 3.0, 1.5, 2.4, 1.2, 0.6, 0.4],
               cutoff=3.0, cutoff_margin=0.6)
        f2 = P("charge_abs", symbols=[pair], parameters=[1.2, 0.3, 0.2, 2.0, 1.5, 0.4, -0.3, 2.0])
        f3 = P("exponential", symbols=[pair], parameters=[-8.0, 1.2])
        prod = ProductPotential([f1, f2, f3])
        prod.set_coordinator(crd(triples, beta, eta, h))
        pots.append(prod)
    pots.append(rep)
    yield "comb_groups", a2, pots
