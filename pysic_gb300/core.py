"""Descriptor queries of the Pysic API.

The reference asks its Fortran core for the names, target counts, levels and
parameter names of every potential and bond-order factor at import time
(pysic/core.py:19-30, 44-486, answered by Potentials.f90:2264-2350 and the
create_*_characterizer_* routines).  This module holds the same table
statically.  Names, orders and levels match the reference so that
``Potential('LJ', parameters=[eps, sigma])`` and ``names_of_parameters`` behave
identically.  ``ENGINE_SUPPORTED`` lists what the GB300 engine evaluates; the
others can be constructed but are rejected when a calculation is requested.
"""
from .error import InvalidPotentialError, InvalidParametersError

# name -> (n_targets, [parameter names]) ; Potentials.f90:2916-5076
POTENTIALS = {
    "LJ": (2, ["epsilon", "sigma"]),
    "spring": (2, ["k", "R_0"]),
    "force": (1, ["Fx", "Fy", "Fz"]),
    "bond_bend": (3, ["epsilon", "theta_0", "n", "m"]),
    "dihedral": (4, ["k", "theta_0"]),
    "exponential": (2, ["epsilon", "zeta"]),
    "charge_exp": (2, ["epsilon", "Rmax1", "Rmin1", "Qmax1", "Qmin1", "Rmax2", "Rmin2", "Qmax2",
                       "Qmin2", "xi1", "xi2"]),
    "constant": (1, ["V"]),
    "Buckingham": (2, ["A", "C", "sigma"]),
    "power": (2, ["epsilon", "a", "n"]),
    "tabulated": (2, ["id", "range", "scale"]),
    "charge_self": (1, ["epsilon", "n"]),
    "charge_pair": (2, ["epsilon", "n1", "n2"]),
    "charge_abs": (2, ["a1", "b1", "Q1", "n1", "a2", "b2", "Q2", "n2"]),
    "shift_power": (2, ["epsilon", "r1", "r2", "n"]),
    "step": (2, ["e1", "e2", "r1", "r2"]),
}

# name -> (n_targets, level, [[scaling parameter names], [local parameter names]])
# Potentials.f90:5077-6769
BOND_ORDER_FACTORS = {
    "neighbors": (2, 1, [[], []]),
    "tersoff": (3, 2, [["beta", "eta"], ["a", "c", "d", "h", "mu"]]),
    "c_scale": (1, 1, [["epsilon", "N", "C", "gamma", "min"], []]),
    "triplet": (3, 1, [[], []]),
    "power_bond": (2, 1, [[], ["a", "n"]]),
    "sqrt_scale": (1, 1, [["epsilon"], []]),
    "table_scale": (1, 1, [["id", "range", "scale"], []]),
    "table_bond": (2, 1, [[], ["id", "range", "scale"]]),
}

# kinds understood by the GB300 engine (codes of the C ABI, include/pysic_gb300.h)
PAIR_KIND = {"LJ": 0, "exponential": 1, "Buckingham": 2, "spring": 3, "power": 4, "shift_power": 5, "tabulated": 6,
             "charge_pair": 7, "charge_exp": 8, "charge_abs": 9, "step": 10}
SINGLE_KIND = {"charge_self": 0, "constant": 1, "force": 2}
TRIPLET_KIND = {"bond_bend": 0}
QUAD_KIND = {"dihedral": 0}
BOND_KIND = {"tersoff": 0}
ATOM_FACTOR_KIND = {"neighbors": 0, "power_bond": 1, "c_scale": 2, "sqrt_scale": 3, "table_bond": 4,
                    "table_scale": 5}
ENGINE_SUPPORTED = (set(PAIR_KIND) | set(SINGLE_KIND) | set(TRIPLET_KIND) | set(QUAD_KIND) | set(BOND_KIND) |
                    set(ATOM_FACTOR_KIND))


def list_potentials():
    return list_valid_potentials()


def list_valid_potentials():
    """Names of the potentials the API knows (pysic/core.py:49-63)."""
    return list(POTENTIALS.keys())


def list_bond_order_factors():
    return list_valid_bond_order_factors()


def list_valid_bond_order_factors():
    return list(BOND_ORDER_FACTORS.keys())


def is_potential(potential_name):
    return is_valid_potential(potential_name)


def is_valid_potential(potential_name):
    return potential_name in POTENTIALS


def is_bond_order_factor(bond_order_name):
    return is_valid_bond_order_factor(bond_order_name)


def is_valid_bond_order_factor(bond_order_name):
    return bond_order_name in BOND_ORDER_FACTORS


def is_charge_relaxation(relaxation_name):
    return is_valid_charge_relaxation(relaxation_name)


def is_valid_charge_relaxation(relaxation_name):
    from .relaxation import ChargeRelaxation
    return relaxation_name in ChargeRelaxation.relaxation_modes


def is_coulomb_summation(summation_name):
    return is_valid_coulomb_summation(summation_name)


def is_valid_coulomb_summation(summation_name):
    from .coulomb import CoulombSummation
    return summation_name in CoulombSummation.summation_modes


def number_of_targets(potential_name):
    """pysic/core.py:187-202"""
    if potential_name in POTENTIALS:
        return POTENTIALS[potential_name][0]
    if potential_name in BOND_ORDER_FACTORS:
        return BOND_ORDER_FACTORS[potential_name][0]
    return 0


def level_of_factor(bond_order_name):
    """pysic/core.py:204-216"""
    if bond_order_name in BOND_ORDER_FACTORS:
        return BOND_ORDER_FACTORS[bond_order_name][1]
    return 0


def number_of_parameters(potential_name, as_list=False):
    """pysic/core.py:218-261: an int for potentials, [n_scaling, n_local] for factors."""
    if potential_name in POTENTIALS:
        n = len(POTENTIALS[potential_name][1])
        return [n] if as_list else n
    if potential_name in BOND_ORDER_FACTORS:
        names = BOND_ORDER_FACTORS[potential_name][2]
        return [len(names[0]), len(names[1])]
    return 0


def names_of_parameters(potential_name):
    """pysic/core.py:263-321"""
    if potential_name in POTENTIALS:
        return list(POTENTIALS[potential_name][1])
    if potential_name in BOND_ORDER_FACTORS:
        names = BOND_ORDER_FACTORS[potential_name][2]
        return [list(names[0]), list(names[1])]
    return []


def index_of_parameter(potential_name, parameter_name):
    """pysic/core.py:323-364: an int for potentials, [list, position] for factors."""
    if potential_name in POTENTIALS:
        names = POTENTIALS[potential_name][1]
        return names.index(parameter_name) if parameter_name in names else -1
    if potential_name in BOND_ORDER_FACTORS:
        names = BOND_ORDER_FACTORS[potential_name][2]
        for k in range(2):
            if parameter_name in names[k]:
                return [k, names[k].index(parameter_name)]
        return None
    return -1


def descriptions_of_parameters(potential_name):
    return names_of_parameters(potential_name)


def description_of_potential(potential_name, parameter_values=None, cutoff=None, elements=None, tags=None,
                             indices=None):
    lines = ["potential '{0}'".format(potential_name),
             "parameters: {0}".format(names_of_parameters(potential_name))]
    if parameter_values is not None:
        lines.append("values: {0}".format(parameter_values))
    if cutoff is not None:
        lines.append("cutoff: {0}".format(cutoff))
    print("\n".join(lines))


def check_engine_support(kind):
    if kind not in ENGINE_SUPPORTED:
        raise InvalidPotentialError(
            "'{0}' is part of the Pysic API but is not evaluated by the GB300 engine".format(kind))


__all__ = [
    "list_potentials", "list_valid_potentials", "list_bond_order_factors", "list_valid_bond_order_factors",
    "is_potential", "is_valid_potential", "is_bond_order_factor", "is_valid_bond_order_factor",
    "is_charge_relaxation", "is_valid_charge_relaxation", "is_coulomb_summation", "is_valid_coulomb_summation",
    "number_of_targets", "level_of_factor", "number_of_parameters", "names_of_parameters",
    "index_of_parameter", "descriptions_of_parameters", "description_of_potential", "InvalidParametersError",
]
