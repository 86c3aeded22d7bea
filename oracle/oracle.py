"""ctypes wrapper of the FP64 CPU oracle (oracle/oracle.c).

TEST INFRASTRUCTURE.  Imported only by tests/, by __graft_entry__.smoke() and
by bench.py's CPU-baseline leg, always as the checker (or, for the CPU
baseline, as the timed restatement of the reference's CPU path).  The product
package ``pysic_gb300`` never imports this module.

Takes the same interaction records as the engine (pysic_gb300.model.Model),
so parity tests compare the GPU and the restatement on identical input.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liborc.so")

_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int32)
_up = ctypes.POINTER(ctypes.c_uint64)


class _System(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("pos", _dp), ("charge", _dp), ("type", _ip),
                ("cell", ctypes.c_double * 9), ("inv", ctypes.c_double * 9), ("pbc", ctypes.c_int32 * 3)]


class _Model(ctypes.Structure):
    _fields_ = [("n_types", ctypes.c_int32), ("n_pair", ctypes.c_int32), ("pair_kind", _ip), ("pair_params", _dp),
                ("pair_cutoff", _dp), ("pair_soft", _dp), ("pair_mask1", _up), ("pair_mask2", _up),
                ("pair_group", _ip), ("n_single", ctypes.c_int32), ("single_kind", _ip), ("single_params", _dp),
                ("single_mask", _up), ("n_bond", ctypes.c_int32), ("bond_params", _dp), ("bond_cutoff", _dp),
                ("bond_soft", _dp), ("bond_mask1", _up), ("bond_mask2", _up), ("bond_mask3", _up),
                ("bond_group", _ip), ("ewald", ctypes.c_int32), ("ewald_rc", ctypes.c_double),
                ("ewald_kc", ctypes.c_double), ("ewald_sigma", ctypes.c_double), ("ewald_eps", ctypes.c_double),
                ("ewald_kmax", ctypes.c_int32 * 3), ("ewald_scaler", _dp), ("pair_table", _dp),
                ("n_table_rows", ctypes.c_int64), ("n_tri", ctypes.c_int32), ("tri_kind", _ip), ("tri_params", _dp),
                ("tri_cutoff", _dp), ("tri_soft", _dp), ("tri_mask1", _up), ("tri_mask2", _up), ("tri_mask3", _up),
                ("tri_center", _up), ("pair_first", _up), ("n_afac", ctypes.c_int32), ("afac_kind", _ip),
                ("afac_params", _dp), ("afac_cutoff", _dp), ("afac_soft", _dp), ("afac_mask1", _up),
                ("afac_mask2", _up), ("afac_group", _ip), ("single_group", _ip), ("pair_nmul", _ip),
                ("pair_mul0", _ip), ("mul_kind", _ip), ("mul_params", _dp), ("mul_first", _up),
                ("n_quad", ctypes.c_int32), ("quad_params", _dp), ("quad_cutoff", _dp), ("quad_soft", _dp),
                ("quad_mask", _up), ("quad_orig", _up)]


class _NbList(ctypes.Structure):
    _fields_ = [("start", _ip), ("idx", _ip), ("off", _ip)]


def build():
    """Compile liborc.so with the recipe in oracle/Makefile."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(os.path.join(HERE, "oracle.c")):
            build()
        L = ctypes.CDLL(LIB)
        L.orc_build_neighbors.restype = ctypes.c_int64
        L.orc_build_neighbors.argtypes = [ctypes.POINTER(_System), _dp, _ip, _ip, _ip, ctypes.c_int64]
        L.orc_evaluate.restype = ctypes.c_int
        L.orc_evaluate.argtypes = [ctypes.POINTER(_System), ctypes.POINTER(_Model), ctypes.POINTER(_NbList),
                                   ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, _dp]
        L.orc_bond_zeta.restype = ctypes.c_int
        L.orc_bond_zeta.argtypes = [ctypes.POINTER(_System), ctypes.POINTER(_Model), ctypes.POINTER(_NbList),
                                    ctypes.c_int, _dp]
        _lib = L
    return _lib


def _d(a):
    return a.ctypes.data_as(_dp)


def _i(a):
    return a.ctypes.data_as(_ip)


def _u(a):
    return a.ctypes.data_as(_up)


class _Keep:
    """holds the numpy arrays a ctypes structure points into"""

    def __init__(self):
        self.items = []

    def f64(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.items.append(a)
        return a

    def i32(self, a):
        a = np.ascontiguousarray(a, dtype=np.int32)
        self.items.append(a)
        return a

    def u64(self, a):
        a = np.ascontiguousarray(a, dtype=np.uint64)
        self.items.append(a)
        return a


def _system(keep, positions, charges, types, cell, pbc):
    s = _System()
    pos = keep.f64(np.asarray(positions).reshape(-1, 3))
    s.n = len(pos)
    s.pos = _d(pos)
    s.charge = _d(keep.f64(charges if charges is not None else np.zeros(len(pos))))
    s.type = _i(keep.i32(types if types is not None else np.zeros(len(pos))))
    cell = np.asarray(cell, dtype=np.float64).reshape(3, 3)
    inv = np.linalg.inv(cell)
    for k in range(9):
        s.cell[k] = cell.flat[k]
        s.inv[k] = inv.flat[k]
    for k in range(3):
        s.pbc[k] = int(bool(np.asarray(pbc).reshape(-1)[k] if np.ndim(pbc) else pbc))
    return s


def _model(keep, M, n):
    a = M.arrays()
    m = _Model()
    m.n_types = M.n_types
    m.n_pair = len(a["pair_kind"])
    m.pair_kind = _i(keep.i32(a["pair_kind"]))
    m.pair_params = _d(keep.f64(a["pair_params"]))
    m.pair_cutoff = _d(keep.f64(a["pair_cutoff"]))
    m.pair_soft = _d(keep.f64(a["pair_soft"]))
    m.pair_mask1 = _u(keep.u64(a["pair_mask1"]))
    m.pair_mask2 = _u(keep.u64(a["pair_mask2"]))
    m.pair_group = _i(keep.i32(a["pair_group"]))
    m.pair_table = _d(keep.f64(a["pair_table"]))
    m.n_table_rows = len(a["pair_table"]) // 2
    m.n_tri = len(a["tri_kind"])
    m.tri_kind = _i(keep.i32(a["tri_kind"]))
    m.tri_params = _d(keep.f64(a["tri_params"]))
    m.tri_cutoff = _d(keep.f64(a["tri_cutoff"]))
    m.tri_soft = _d(keep.f64(a["tri_soft"]))
    m.tri_mask1 = _u(keep.u64(a["tri_mask1"]))
    m.tri_mask2 = _u(keep.u64(a["tri_mask2"]))
    m.tri_mask3 = _u(keep.u64(a["tri_mask3"]))
    m.tri_center = _u(keep.u64(a["tri_center"]))
    m.pair_first = _u(keep.u64(a["pair_first"]))
    m.n_single = len(a["single_kind"])
    m.single_kind = _i(keep.i32(a["single_kind"]))
    m.single_params = _d(keep.f64(a["single_params"]))
    m.single_mask = _u(keep.u64(a["single_mask"]))
    m.single_group = _i(keep.i32(a["single_group"]))
    m.pair_nmul = _i(keep.i32(a["pair_nmul"] if len(a["pair_nmul"]) else np.zeros(1)))
    m.pair_mul0 = _i(keep.i32(a["pair_mul0"] if len(a["pair_mul0"]) else np.zeros(1)))
    m.mul_kind = _i(keep.i32(a["mul_kind"] if len(a["mul_kind"]) else np.zeros(1)))
    m.mul_params = _d(keep.f64(a["mul_params"] if len(a["mul_params"]) else np.zeros((1, 4))))
    m.mul_first = _u(keep.u64(a["mul_first"] if len(a["mul_first"]) else np.zeros(1)))
    m.n_quad = len(a["quad_kind"])
    m.quad_params = _d(keep.f64(a["quad_params"] if len(a["quad_kind"]) else np.zeros((1, 4))))
    m.quad_cutoff = _d(keep.f64(a["quad_cutoff"] if len(a["quad_kind"]) else np.zeros(1)))
    m.quad_soft = _d(keep.f64(a["quad_soft"] if len(a["quad_kind"]) else np.zeros(1)))
    m.quad_mask = _u(keep.u64(a["quad_mask"] if len(a["quad_kind"]) else np.zeros((1, 4))))
    m.quad_orig = _u(keep.u64(a["quad_orig"] if len(a["quad_kind"]) else np.zeros((1, 4))))
    m.n_afac = len(a["afac_kind"])
    m.afac_kind = _i(keep.i32(a["afac_kind"]))
    m.afac_params = _d(keep.f64(a["afac_params"]))
    m.afac_cutoff = _d(keep.f64(a["afac_cutoff"]))
    m.afac_soft = _d(keep.f64(a["afac_soft"]))
    m.afac_mask1 = _u(keep.u64(a["afac_mask1"]))
    m.afac_mask2 = _u(keep.u64(a["afac_mask2"]))
    m.afac_group = _i(keep.i32(a["afac_group"]))
    m.n_bond = len(a["bond_cutoff"])
    m.bond_params = _d(keep.f64(a["bond_params"]))
    m.bond_cutoff = _d(keep.f64(a["bond_cutoff"]))
    m.bond_soft = _d(keep.f64(a["bond_soft"]))
    m.bond_mask1 = _u(keep.u64(a["bond_mask1"]))
    m.bond_mask2 = _u(keep.u64(a["bond_mask2"]))
    m.bond_mask3 = _u(keep.u64(a["bond_mask3"]))
    m.bond_group = _i(keep.i32(a["bond_group"]))
    ew = M.ewald
    if ew is not None:
        m.ewald = 1
        m.ewald_rc = ew["rc"]
        m.ewald_kc = ew["kc"]
        m.ewald_sigma = ew["sigma"]
        m.ewald_eps = ew["eps"]
        for k in range(3):
            m.ewald_kmax[k] = int(ew["kmax"][k])
        m.ewald_scaler = _d(keep.f64(ew["scaler"]))
    else:
        m.ewald = 0
        m.ewald_scaler = _d(keep.f64(np.ones(max(n, 1))))
    return m


def _nblist(keep, counts, idx, off):
    nb = _NbList()
    start = np.concatenate([[0], np.cumsum(np.asarray(counts, dtype=np.int64))]).astype(np.int32)
    nb.start = _i(keep.i32(start))
    nb.idx = _i(keep.i32(idx if len(idx) else np.zeros(1)))
    nb.off = _i(keep.i32(np.asarray(off).reshape(-1, 3) if len(idx) else np.zeros((1, 3))))
    return nb


def neighbors(positions, cell, pbc, cutoffs):
    """Restated FastNeighborList build: (counts, neighbours, offsets) in CSR order."""
    keep = _Keep()
    s = _system(keep, positions, None, None, cell, pbc)
    cut = keep.f64(cutoffs)
    n = s.n
    counts = np.zeros(max(n, 1), dtype=np.int32)
    total = lib().orc_build_neighbors(ctypes.byref(s), _d(cut), _i(counts), None, None, 0)
    if total < 0:
        raise ValueError("cell narrower than the cutoff")
    idx = np.zeros(max(total, 1), dtype=np.int32)
    off = np.zeros((max(total, 1), 3), dtype=np.int32)
    lib().orc_build_neighbors(ctypes.byref(s), _d(cut), _i(counts), _i(idx), _i(off), total)
    return counts[:n], idx[:total], off[:total]


def evaluate(positions, charges, cell, pbc, model, counts, idx, off, what="energy", threads=1):
    """core_calculate_energy / _forces / _electronegativities restated.
    Returns the energy, (forces, stress) or the electronegativities."""
    keep = _Keep()
    s = _system(keep, positions, charges, model.types, cell, pbc)
    m = _model(keep, model, s.n)
    nb = _nblist(keep, counts, idx, off)
    code = {"energy": 0, "forces": 1, "enegs": 2}[what]
    e = np.zeros(1)
    f = np.zeros((max(s.n, 1), 3))
    st = np.zeros(6)
    c = np.zeros(max(s.n, 1))
    rc = lib().orc_evaluate(ctypes.byref(s), ctypes.byref(m), ctypes.byref(nb), code, int(threads), _d(e), _d(f),
                            _d(st), _d(c))
    if rc != 0:
        raise RuntimeError("oracle evaluation failed")
    if what == "energy":
        return float(e[0])
    if what == "forces":
        return f[:s.n], st
    return c[:s.n]


def atom_factors(positions, cell, pbc, model, counts, idx, off, group=0):
    """Per-atom bond-order sums and factors of one Coordinator group."""
    keep = _Keep()
    s = _system(keep, positions, None, model.types, cell, pbc)
    m = _model(keep, model, s.n)
    nb = _nblist(keep, counts, idx, off)
    raw = np.zeros(max(s.n, 1))
    fac = np.zeros(max(s.n, 1))
    lib().orc_atom_factors(ctypes.byref(s), ctypes.byref(m), ctypes.byref(nb), int(group), _d(raw), _d(fac))
    return raw[:s.n], fac[:s.n]


def atom_factor_gradients(positions, cell, pbc, model, counts, idx, off, group, atom, of_factor=False):
    """Gradients of one group's per-atom factors (n x 3): of every factor with
    respect to moving `atom`, or of `atom`'s factor with respect to every atom."""
    keep = _Keep()
    s = _system(keep, positions, None, model.types, cell, pbc)
    m = _model(keep, model, s.n)
    nb = _nblist(keep, counts, idx, off)
    out = np.zeros((max(s.n, 1), 3))
    rc = lib().orc_atom_factor_gradients(ctypes.byref(s), ctypes.byref(m), ctypes.byref(nb), int(group), int(atom),
                                         1 if of_factor else 0, _d(out))
    if rc != 0:
        raise ValueError("atom index out of range")
    return out[:s.n]


def bond_zeta(positions, cell, pbc, model, counts, idx, off, group=0):
    keep = _Keep()
    s = _system(keep, positions, None, model.types, cell, pbc)
    m = _model(keep, model, s.n)
    nb = _nblist(keep, counts, idx, off)
    z = np.zeros(max(len(idx), 1))
    lib().orc_bond_zeta(ctypes.byref(s), ctypes.byref(m), ctypes.byref(nb), int(group), _d(z))
    return z[:len(idx)]


def relax_charges(positions, charges, cell, pbc, model, counts, idx, off, n_steps, timestep, inertia, friction,
                  tolerance, rates=None, threads=1):
    """ChargeRelaxation 'dynamic', pysic/charges/relaxation.py:417-450, on the
    restated electronegativities."""
    q = np.array(charges, dtype=np.float64)
    n = len(q)
    rates = np.zeros(n) if rates is None else np.array(rates, dtype=np.float64)
    dt = timestep
    dt2 = dt * dt
    inv_mq = 1.0 / inertia
    future = 1.0 / (1.0 + 0.5 * friction * dt)

    def dchi(qq):
        c = evaluate(positions, qq, cell, pbc, model, counts, idx, off, "enegs", threads)
        return c - c.sum() / len(c)

    error = 2.0 * tolerance
    step = 0
    force = dchi(q)
    max_dq = 0.0
    while error > tolerance and step < n_steps:
        dq = rates * dt + (force - friction * rates) * inv_mq * dt2
        q = q + dq
        rates = (1.0 - 0.5 * friction * dt) * rates + force * 0.5 * inv_mq * dt
        force = dchi(q)
        rates = future * (rates + force * 0.5 * inv_mq * dt)
        step += 1
        error = force.max()
        max_dq = float(np.abs(dq).max())
    return {"charges": q, "rates": rates, "steps": step, "error": float(error), "max_dq": max_dq}


def relax_potentiostat(positions, charges, cell, pbc, model, counts, idx, off, n_steps, timestep, inertia,
                       potential, rates=None, threads=1):
    """ChargeRelaxation 'potentiostat', pysic/charges/relaxation.py:453-481:
    undamped charge dynamics driven by chi - potential for n_steps steps."""
    q = np.array(charges, dtype=np.float64)
    rates = np.zeros(len(q)) if rates is None else np.array(rates, dtype=np.float64)
    dt = timestep
    dt2 = dt * dt
    inv_mq = 1.0 / inertia

    def force_of(qq):
        return evaluate(positions, qq, cell, pbc, model, counts, idx, off, "enegs", threads) - potential

    force = force_of(q)
    for _ in range(int(n_steps)):
        q = q + (rates * dt + force * inv_mq * dt2)
        rates = rates + force * 0.5 * inv_mq * dt
        force = force_of(q)
        rates = rates + force * 0.5 * inv_mq * dt
    return {"charges": q, "rates": rates, "steps": int(n_steps), "max_dchi": float(force.max())}
