"""Compile Pysic interaction objects into the flat interaction records the
engine consumes.

The reference pushes potentials into its Fortran core one record at a time:
pysic/calculator.py:1063-1447 permutes every target tuple (an A-B pair
potential becomes the records A-B and B-A, an A-A potential one record),
leaves bond-order factor symbols unpermuted (calculator.py:1372, 1410-1416),
assigns one group index per distinct Coordinator (1217-1233) and calls
add_potential / add_bond_order_factor (PyInterface.f90:433-526).  The core
then filters records per atom by element, tag or index
(potential_affects_atom, Potentials.f90:1195-1259).

Here the same record list is built once, and the per-atom filters are turned
into *types*: atoms that no filter can tell apart share a type, and every
record carries one 64-bit type mask per target position.  The records keep
the reference's order, so the oracle can walk them exactly like the core,
while the GPU kernels fold them into dense per-type-pair tables.
"""
from itertools import permutations

import numpy as np

from . import core
from .error import InvalidParametersError, InvalidPotentialError

MAX_TYPES = 64


# The reference's step force is not the gradient of its energy and not along
# the bond (Potentials.f90:4917-4937); the engine evaluates it for plain
# records only.
_STEP_ONLY_PLAIN = ("the step potential is evaluated by the GB300 engine as a plain pair term only "
                    "(no bond-order scaling, no products): its force is not radial")

def _distinct_permutations(targets):
    return list(dict.fromkeys(permutations(targets)))


class Model:
    """Interaction records of one calculator for one atomic structure."""

    def __init__(self):
        self.n_types = 0
        self.types = np.zeros(0, dtype=np.int32)
        self.type_signatures = []
        self.pair_kind = []
        self.pair_params = []
        self.pair_table = []  # tabulated potentials: rows (V, d), concatenated
        self.pair_first = []  # types of each record's unpermuted first target
        self.pair_cutoff = []
        self.pair_soft = []
        self.pair_mask1 = []
        self.pair_mask2 = []
        self.pair_group = []
        # products of pair potentials: per pair record the number of multiplying
        # components and the index of its first one; per component its kind,
        # parameters and the types of the product's first target
        self.pair_nmul = []
        self.pair_mul0 = []
        self.mul_kind = []
        self.mul_params = []
        self.mul_first = []
        self.single_kind = []
        self.single_params = []
        self.single_mask = []
        self.single_group = []
        # per-atom (level-1) bond-order factors, one record per target tuple
        self.afac_kind = []
        self.afac_params = []
        self.afac_cutoff = []
        self.afac_soft = []
        self.afac_mask1 = []
        self.afac_mask2 = []
        self.afac_group = []
        self.bond_params = []
        self.bond_cutoff = []
        self.bond_soft = []
        self.bond_mask1 = []
        self.bond_mask2 = []
        self.bond_mask3 = []
        self.bond_group = []
        # three-body potentials (bond_bend), one record per distinct permutation
        # of each target tuple, as the reference adds them
        self.tri_kind = []
        self.tri_params = []
        self.tri_cutoff = []
        self.tri_soft = []
        self.tri_mask1 = []
        self.tri_mask2 = []
        self.tri_mask3 = []
        self.tri_center = []  # types whose element is the tuple's middle one (original_elements(2))
        # four-body potentials (dihedral), one record per distinct permutation of
        # each target tuple: masks of positions 1-4 of the permuted record and of
        # the unpermuted tuple
        self.quad_kind = []
        self.quad_params = []
        self.quad_cutoff = []
        self.quad_soft = []
        self.quad_mask = []
        self.quad_orig = []
        self.n_groups = 0
        self.coordinators = []
        self.ewald = None

    # arrays in the layout of the C ABI
    def arrays(self):
        d = {}
        d["pair_kind"] = np.array(self.pair_kind, dtype=np.int32)
        d["pair_params"] = np.array(self.pair_params, dtype=np.float64).reshape(-1, 4)
        d["pair_table"] = np.array(self.pair_table, dtype=np.float64).reshape(-1)
        d["pair_first"] = np.array(self.pair_first, dtype=np.uint64)
        d["pair_cutoff"] = np.array(self.pair_cutoff, dtype=np.float64)
        d["pair_soft"] = np.array(self.pair_soft, dtype=np.float64)
        d["pair_mask1"] = np.array(self.pair_mask1, dtype=np.uint64)
        d["pair_mask2"] = np.array(self.pair_mask2, dtype=np.uint64)
        d["pair_group"] = np.array(self.pair_group, dtype=np.int32)
        d["pair_nmul"] = np.array(self.pair_nmul, dtype=np.int32)
        d["pair_mul0"] = np.array(self.pair_mul0, dtype=np.int32)
        d["mul_kind"] = np.array(self.mul_kind, dtype=np.int32)
        d["mul_params"] = np.array(self.mul_params, dtype=np.float64).reshape(-1, 4)
        d["mul_first"] = np.array(self.mul_first, dtype=np.uint64)
        d["single_kind"] = np.array(self.single_kind, dtype=np.int32)
        d["single_params"] = np.array(self.single_params, dtype=np.float64).reshape(-1, 4)
        d["single_mask"] = np.array(self.single_mask, dtype=np.uint64)
        d["single_group"] = np.array(self.single_group, dtype=np.int32)
        d["afac_kind"] = np.array(self.afac_kind, dtype=np.int32)
        d["afac_params"] = np.array(self.afac_params, dtype=np.float64).reshape(-1, 5)
        d["afac_cutoff"] = np.array(self.afac_cutoff, dtype=np.float64)
        d["afac_soft"] = np.array(self.afac_soft, dtype=np.float64)
        d["afac_mask1"] = np.array(self.afac_mask1, dtype=np.uint64)
        d["afac_mask2"] = np.array(self.afac_mask2, dtype=np.uint64)
        d["afac_group"] = np.array(self.afac_group, dtype=np.int32)
        d["bond_params"] = np.array(self.bond_params, dtype=np.float64).reshape(-1, 7)
        d["bond_cutoff"] = np.array(self.bond_cutoff, dtype=np.float64)
        d["bond_soft"] = np.array(self.bond_soft, dtype=np.float64)
        d["bond_mask1"] = np.array(self.bond_mask1, dtype=np.uint64)
        d["bond_mask2"] = np.array(self.bond_mask2, dtype=np.uint64)
        d["bond_mask3"] = np.array(self.bond_mask3, dtype=np.uint64)
        d["bond_group"] = np.array(self.bond_group, dtype=np.int32)
        d["tri_kind"] = np.array(self.tri_kind, dtype=np.int32)
        d["tri_params"] = np.array(self.tri_params, dtype=np.float64).reshape(-1, 4)
        d["tri_cutoff"] = np.array(self.tri_cutoff, dtype=np.float64)
        d["tri_soft"] = np.array(self.tri_soft, dtype=np.float64)
        d["tri_mask1"] = np.array(self.tri_mask1, dtype=np.uint64)
        d["tri_mask2"] = np.array(self.tri_mask2, dtype=np.uint64)
        d["tri_mask3"] = np.array(self.tri_mask3, dtype=np.uint64)
        d["tri_center"] = np.array(self.tri_center, dtype=np.uint64)
        d["quad_kind"] = np.array(self.quad_kind, dtype=np.int32)
        d["quad_params"] = np.array(self.quad_params, dtype=np.float64).reshape(-1, 4)
        d["quad_cutoff"] = np.array(self.quad_cutoff, dtype=np.float64)
        d["quad_soft"] = np.array(self.quad_soft, dtype=np.float64)
        d["quad_mask"] = np.array(self.quad_mask, dtype=np.uint64).reshape(-1, 4)
        d["quad_orig"] = np.array(self.quad_orig, dtype=np.uint64).reshape(-1, 4)
        return d


def assign_types(atoms, potentials):
    """Group atoms into types: element, plus tag if any potential targets tags,
    plus index if some potential targets that index."""
    symbols = list(atoms.get_chemical_symbols())
    tags = np.asarray(atoms.get_tags())
    use_tags = any(p.get_tags() for p in potentials)
    targeted = set()
    for p in potentials:
        for t in p.get_indices() or []:
            targeted.update(int(x) for x in t)
    sig_of = {}
    types = np.zeros(len(symbols), dtype=np.int32)
    for i, s in enumerate(symbols):
        sig = (s, int(tags[i]) if use_tags else None, i if i in targeted else None)
        if sig not in sig_of:
            sig_of[sig] = len(sig_of)
        types[i] = sig_of[sig]
    if len(sig_of) > MAX_TYPES:
        raise InvalidPotentialError("more than {0} distinguishable atom types".format(MAX_TYPES))
    sigs = [None] * len(sig_of)
    for s, t in sig_of.items():
        sigs[t] = s
    return types, sigs


def _mask(sigs, element=None, tag=None, index=None):
    m = 0
    for t, (e, g, i) in enumerate(sigs):
        if (element is not None and e == element) or (tag is not None and g is not None and g == tag) or \
                (index is not None and i is not None and i == index):
            m |= 1 << t
    return m


def read_table(ident):
    """Rows (V, d) of table_XXXX.txt in the working directory, XXXX the id in
    four digits (read_table, Utility.f90:384-433; file name as in
    create_potential, Potentials.f90:2460-2466)."""
    name = "table_{0:04d}.txt".format(int(ident))
    try:
        rows = np.loadtxt(name, ndmin=2, dtype=np.float64)
    except OSError:
        raise InvalidPotentialError("tabulated potential: no table file " + name)
    if rows.shape[1] < 2 or rows.shape[0] < 2:
        raise InvalidPotentialError("tabulated potential: " + name + " needs at least two rows of V and d")
    return rows[:, :2]


def _table_record(M, params):
    """[id, range, scale] -> [first row, rows, range, scale] with the rows
    appended to the model's table."""
    rows = read_table(params[0])
    first = len(M.pair_table) // 2
    M.pair_table.extend(rows.reshape(-1).tolist())
    return [float(first), float(len(rows)), float(params[1]), float(params[2])]


def _charge_exp_record(M, params):
    """charge_exp's 11 parameters and the derived eta1, eta2, beta1, beta2
    (calculate_derived_parameters_charge_exp, Potentials.f90:3751-3766) as 8
    rows of the table array; the record keeps the first row."""
    p = [np.float64(x) for x in params]
    with np.errstate(all="ignore"):  # C pow semantics: a negative base needs an integral exponent
        eta1 = np.log(p[1] / (p[1] - p[2])) / np.log(p[3] / (p[3] - p[4]))
        eta2 = np.log(p[5] / (p[5] - p[6])) / np.log(p[7] / (p[7] - p[8]))
        beta1 = np.power(p[2] - p[1], 1.0 / eta1) / (p[3] - p[4])
        beta2 = np.power(p[6] - p[5], 1.0 / eta2) / (p[7] - p[8])
    p = [float(x) for x in p]
    block = p + [float(eta1), float(eta2), float(beta1), float(beta2), 0.0]
    if not all(np.isfinite(block)):
        raise InvalidParametersError("charge_exp: parameters give no finite eta / beta")
    first = len(M.pair_table) // 2
    M.pair_table.extend(block)
    return [float(first), 0.0, 0.0, 0.0]


def compile_model(atoms, potentials, coulomb=None):
    potentials = list(potentials or [])
    M = Model()
    M.types, M.type_signatures = assign_types(atoms, potentials)
    M.n_types = len(M.type_signatures)
    sigs = M.type_signatures

    # distinct coordinators -> groups (calculator.py:1077-1090, 1217-1233)
    coords = []
    for pot in potentials:
        c = pot.get_coordinator()
        if c is None:
            continue
        if not any(c.get_bond_order_parameters() == k.get_bond_order_parameters() for k in coords):
            coords.append(c)
    M.coordinators = coords
    M.n_groups = len(coords)

    def group_of(pot):
        c = pot.get_coordinator()
        if c is None:
            return -1
        for g, k in enumerate(coords):
            if c.get_bond_order_parameters() == k.get_bond_order_parameters():
                c.set_group_index(g)
                return g
        return -1

    def pair_level(g):
        """a group of pair (Tersoff) bond-order factors, which the bond-order
        kernels evaluate with any pair term they scale"""
        return g >= 0 and all(core.level_of_factor(b.get_bond_order_type()) == 2
                              for b in coords[g].get_bond_order_parameters())

    def pair_params_of(kind, params):
        """the parameters of one pair term as the engine stores them"""
        if kind == "tabulated":
            return _table_record(M, params)
        if kind == "charge_exp":
            return _charge_exp_record(M, params)
        if kind == "charge_abs":  # (a, b, Q, n) of both targets as 4 rows of the table array
            first = len(M.pair_table) // 2
            M.pair_table.extend([float(x) for x in params[:8]])
            return [float(first), 0.0, 0.0, 0.0]
        return params

    for pot in potentials:
        factors = pot.get_potentials()
        lead = factors[0]
        kind = lead.get_potential_type()
        core.check_engine_support(kind)
        nt = pot.get_number_of_targets()
        params = [float(x) for x in lead.get_parameter_values()]
        grp = group_of(pot)
        # a product: the leading potential's records carry the other factors
        # (calculator.py:1208-1360; the factors take the product's first target
        # tuple as their own, unpermuted)
        mul0, nmul = len(M.mul_kind), len(factors) - 1
        if nmul:
            if nt != 2:
                raise InvalidPotentialError("products of {0}-body potentials are not evaluated by the GB300 engine"
                                            .format(nt))
            if grp >= 0 and not pair_level(grp):
                raise InvalidPotentialError("products scaled by per-atom bond-order factors are not evaluated by the "
                                            "GB300 engine")
            lead_first = next((t for t in (pot.get_symbols(), pot.get_tags(), pot.get_indices()) if t), None)
            if lead_first is None:
                raise InvalidPotentialError("a product of potentials without targets")
            t0 = lead_first[0][0]
            fmask = _mask(sigs, *((t0, None, None) if pot.get_symbols() else
                                  (None, int(t0), None) if pot.get_tags() else (None, None, int(t0))))
            # the reference registers a product's factors last to first and the core
            # keeps them in that order (calculator.py:1208-1213, Core.f90:925-944)
            for fac in reversed(factors[1:]):
                fk = fac.get_potential_type()
                core.check_engine_support(fk)
                if fk == "step":
                    raise InvalidPotentialError(_STEP_ONLY_PLAIN)
                if fk not in core.PAIR_KIND:
                    raise InvalidPotentialError("'{0}' is not a pair potential of the GB300 engine".format(fk))
                M.mul_kind.append(core.PAIR_KIND[fk])
                M.mul_params.append((pair_params_of(fk, [float(x) for x in fac.get_parameter_values()]) +
                                     [0.0] * 4)[:4])
                M.mul_first.append(fmask)
        targets = []  # (position filters) tuples of (element, tag, index) per position
        firsts = []   # the unpermuted tuple's first target of each record (original_elements(1))
        for t in pot.get_symbols() or []:
            for perm in _distinct_permutations(t):
                targets.append([(e, None, None) for e in perm])
                firsts.append((t[0], None, None))
        for t in pot.get_tags() or []:
            for perm in _distinct_permutations(t):
                targets.append([(None, int(g), None) for g in perm])
                firsts.append((None, int(t[0]), None))
        for t in pot.get_indices() or []:
            for perm in _distinct_permutations(t):
                targets.append([(None, None, int(i)) for i in perm])
                firsts.append((None, None, int(t[0])))
        if nt == 2:
            if kind not in core.PAIR_KIND:
                raise InvalidPotentialError("'{0}' is not a pair potential of the GB300 engine".format(kind))
            params = pair_params_of(kind, params)
            if kind == "step" and (grp >= 0 or nmul):
                raise InvalidPotentialError(_STEP_ONLY_PLAIN)
            if kind in ("charge_pair", "charge_exp", "charge_abs") and grp >= 0 and not pair_level(grp):
                raise InvalidPotentialError("per-atom bond-order scaling of {0} is not evaluated by the GB300 engine"
                                            .format(kind))
            for tg, first in zip(targets, firsts):
                M.pair_first.append(_mask(sigs, *first))
                M.pair_kind.append(core.PAIR_KIND[kind])
                M.pair_params.append((params + [0.0] * 4)[:4])
                M.pair_cutoff.append(float(pot.get_cutoff()))
                M.pair_soft.append(float(pot.get_soft_cutoff()))
                M.pair_mask1.append(_mask(sigs, *tg[0]))
                M.pair_mask2.append(_mask(sigs, *tg[1]))
                M.pair_group.append(grp)
                M.pair_nmul.append(nmul)
                M.pair_mul0.append(mul0)
        elif nt == 1:
            if kind not in core.SINGLE_KIND:
                raise InvalidPotentialError("'{0}' is not a single-atom term of the GB300 engine".format(kind))
            if grp >= 0 and kind == "charge_self":
                raise InvalidPotentialError("bond-order scaling of charge_self is not evaluated by the GB300 engine")
            for tg in targets:
                M.single_kind.append(core.SINGLE_KIND[kind])
                M.single_params.append((params + [0.0] * 4)[:4])
                M.single_mask.append(_mask(sigs, *tg[0]))
                M.single_group.append(grp)
        elif nt == 3:
            if kind not in core.TRIPLET_KIND:
                raise InvalidPotentialError("'{0}' is not a three-body potential of the GB300 engine".format(kind))
            if grp >= 0:
                raise InvalidPotentialError("bond-order scaling of three-body potentials is not evaluated by the "
                                            "GB300 engine")
            if pot.get_tags() or pot.get_indices():
                raise InvalidPotentialError("three-body potentials are evaluated for element targets only")
            # create_potential (Potentials.f90:2353-2472) keeps the unpermuted
            # tuple as original_elements; the evaluator requires its middle
            # element at the centre atom (Potentials.f90:3206-3314)
            for t in pot.get_symbols() or []:
                centre = _mask(sigs, t[1], None, None)
                for perm in _distinct_permutations(t):
                    M.tri_kind.append(core.TRIPLET_KIND[kind])
                    M.tri_params.append((params + [0.0] * 4)[:4])
                    M.tri_cutoff.append(float(pot.get_cutoff()))
                    M.tri_soft.append(float(pot.get_soft_cutoff()))
                    M.tri_mask1.append(_mask(sigs, perm[0], None, None))
                    M.tri_mask2.append(_mask(sigs, perm[1], None, None))
                    M.tri_mask3.append(_mask(sigs, perm[2], None, None))
                    M.tri_center.append(centre)
        elif nt == 4:
            if kind not in core.QUAD_KIND:
                raise InvalidPotentialError("'{0}' is not a four-body potential of the GB300 engine".format(kind))
            if grp >= 0:
                raise InvalidPotentialError("bond-order scaling of four-body potentials is not evaluated by the "
                                            "GB300 engine")
            if pot.get_tags() or pot.get_indices():
                raise InvalidPotentialError("four-body potentials are evaluated for element targets only")
            # create_potential keeps the unpermuted tuple (original_elements), which the
            # dihedral evaluator matches forwards or backwards (Potentials.f90:3380-3611)
            for t in pot.get_symbols() or []:
                orig = [_mask(sigs, e, None, None) for e in t]
                for perm in _distinct_permutations(t):
                    M.quad_kind.append(core.QUAD_KIND[kind])
                    M.quad_params.append((params + [0.0] * 4)[:4])
                    M.quad_cutoff.append(float(pot.get_cutoff()))
                    M.quad_soft.append(float(pot.get_soft_cutoff()))
                    M.quad_mask.append([_mask(sigs, e, None, None) for e in perm])
                    M.quad_orig.append(orig)
        else:
            raise InvalidPotentialError("{0}-body potentials are not evaluated by the GB300 engine".format(nt))

    for g, c in enumerate(coords):
        for bond in c.get_bond_order_parameters():
            bkind = bond.get_bond_order_type()
            core.check_engine_support(bkind)
            flat = [float(x) for x in bond.get_parameters_as_list()]
            if bkind in core.ATOM_FACTOR_KIND:
                # per-atom factors keep the reference's global order (coordinator,
                # factor, target tuple): the first scaler of an element wins
                # (core_post_process_bond_order_factors, Core.f90:2697-2712)
                if bkind in ("table_bond", "table_scale"):
                    # [id, range, scale] -> [first row, rows, range, scale] (create_bond_order_factor
                    # reads table_XXXX.txt like the tabulated potential, Potentials.f90:5200-5213)
                    flat = _table_record(M, flat)
                for tg in bond.get_symbols() or []:
                    M.afac_kind.append(core.ATOM_FACTOR_KIND[bkind])
                    M.afac_params.append((flat + [0.0] * 5)[:5])
                    M.afac_cutoff.append(float(bond.get_cutoff()))
                    M.afac_soft.append(float(bond.get_soft_cutoff()))
                    M.afac_mask1.append(_mask(sigs, element=tg[0]))
                    M.afac_mask2.append(_mask(sigs, element=tg[1]) if len(tg) > 1 else 0)
                    M.afac_group.append(g)
                continue
            for tg in bond.get_symbols() or []:
                M.bond_params.append(flat)
                M.bond_cutoff.append(float(bond.get_cutoff()))
                M.bond_soft.append(float(bond.get_soft_cutoff()))
                M.bond_mask1.append(_mask(sigs, element=tg[0]))
                M.bond_mask2.append(_mask(sigs, element=tg[1]))
                M.bond_mask3.append(_mask(sigs, element=tg[2]))
                M.bond_group.append(g)

    if coulomb is not None:
        M.ewald = ewald_settings(atoms, coulomb)
    return M


def ewald_settings(atoms, coulomb):
    """k-space truncation of pysic/calculator.py:1450-1482."""
    p = coulomb.get_parameters()
    rcut, kcut, sigma, eps = p["real_cutoff"], p["k_cutoff"], p["sigma"], p["epsilon"]
    reci = 2.0 * np.pi * np.asarray(atoms.get_reciprocal_cell())
    volume = np.dot(reci[0], np.cross(reci[1], reci[2]))
    k1 = int(kcut * np.linalg.norm(np.cross(reci[1], reci[2])) / volume + 0.5)
    k2 = int(kcut * np.linalg.norm(np.cross(reci[0], reci[2])) / volume + 0.5)
    k3 = int(kcut * np.linalg.norm(np.cross(reci[0], reci[1])) / volume + 0.5)
    n = len(atoms)
    scaler = coulomb.get_scaling_factors()
    if scaler is None:
        scaler = np.ones(n)
    elif len(scaler) != n:
        raise InvalidParametersError("Length of the scaling factor vector does not match the number of atoms.")
    return {"rc": float(rcut), "kc": float(kcut), "kmax": np.array([k1, k2, k3], dtype=np.int32),
            "sigma": float(sigma), "eps": float(eps), "scaler": np.asarray(scaler, dtype=np.float64)}


def individual_cutoffs(atoms, potentials, coulomb=None, scaler=1.0):
    """Per-atom interaction range, pysic/calculator.py:860-915."""
    potentials = list(potentials or [])
    symbols = atoms.get_chemical_symbols()
    tags = atoms.get_tags()
    base = coulomb.get_realspace_cutoff() if coulomb is not None else 0.0
    cuts = []
    for index, (sym, tag) in enumerate(zip(symbols, tags)):
        mc = base
        for pot in potentials:
            active = sym in pot.get_different_symbols() or tag in pot.get_different_tags() or \
                index in pot.get_different_indices()
            if active and pot.get_cutoff() > mc:
                mc = pot.get_cutoff()
            c = pot.get_coordinator()
            if c is not None:
                for bond in c.get_bond_order_parameters():
                    if sym in bond.get_different_symbols() and bond.get_cutoff() > mc:
                        mc = bond.get_cutoff()
        cuts.append(mc * scaler)
    return cuts
