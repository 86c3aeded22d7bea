"""The reference's calls into its core, in its order, restated for the tests:
pysic/calculator.py initialize_fortran_core (1595-1637: create_atoms,
create_cell), update_core_potentials (1063-1447: one add_potential per
distinct permutation of every target tuple, unpermuted bond-order factor
records, group indices of the first potential that names each coordinator),
update_core_coulomb (1450-1482), the neighbour build of FastNeighborList
(62-108) and the separate energy / force / electronegativity passes (918-996).
Element labels are coded as two integers per label; any injective code works
since the core only compares codes."""
from itertools import permutations

import numpy as np

from pysic_gb300.model import ewald_settings, individual_cutoffs


def codes(label):
    s = (label + "  ")[:2]
    return [ord(s[0]), ord(s[1])]


def _perms(t):
    return list(dict.fromkeys(permutations(t)))


def load(pi, atoms, pots, coulomb=None):
    n = len(atoms)
    pi.create_atoms(atoms.get_masses(), atoms.get_initial_charges(), atoms.get_positions().T,
                    np.zeros((3, n)), np.asarray(atoms.get_tags()),
                    np.array([codes(s) for s in atoms.get_chemical_symbols()]).T)
    cell = np.asarray(atoms.get_cell())
    pi.create_cell(cell.T, np.linalg.inv(cell).T, np.asarray(atoms.get_pbc()))
    coords = []  # (coordinator, group index)
    for k, p in enumerate(pots):
        c = p.get_coordinator()
        if c is not None and not any(c is x for x, _ in coords):
            coords.append((c, k))
    pi.allocate_potentials(0)
    for p in pots:
        c = p.get_coordinator()
        grp = next((g for x, g in coords if x.get_bond_order_parameters() == c.get_bond_order_parameters()), -1) \
            if c is not None else -1
        nt = p.get_number_of_targets()
        none = np.array(nt * [-9])
        # a product's factors first, last to first, once each with the first
        # unpermuted target tuple (calculator.py:1208-1213, 1255-1280)
        for fac in reversed(p.get_potentials()[1:]):
            t = p.get_symbols()[0]
            assert pi.add_potential(fac.get_potential_type(), np.array(fac.get_parameter_values()), p.get_cutoff(),
                                    p.get_soft_cutoff(), np.array([codes(s) for s in t]).T, none, none,
                                    np.array([codes(s) for s in t]).T, none, none, grp, True)
        p = p.get_potentials()[0] if len(p.get_potentials()) > 1 else p
        for t in p.get_symbols() or []:
            for perm in _perms(t):
                assert pi.add_potential(p.get_potential_type(), np.array(p.get_parameter_values()), p.get_cutoff(),
                                        p.get_soft_cutoff(), np.array([codes(s) for s in perm]).T, none, none,
                                        np.array([codes(s) for s in t]).T, none, none, grp, False)
        for t in p.get_tags() or []:
            for perm in _perms(t):
                assert pi.add_potential(p.get_potential_type(), np.array(p.get_parameter_values()), p.get_cutoff(),
                                        p.get_soft_cutoff(), np.array(nt * [codes("xx")]).T, np.array(perm), none,
                                        np.array(nt * [codes("xx")]).T, np.array(t), none, grp, False)
        for t in p.get_indices() or []:
            for perm in _perms(t):
                assert pi.add_potential(p.get_potential_type(), np.array(p.get_parameter_values()), p.get_cutoff(),
                                        p.get_soft_cutoff(), np.array(nt * [codes("xx")]).T, none, np.array(perm),
                                        np.array(nt * [codes("xx")]).T, none, np.array(t), grp, False)
        pi.clear_potential_multipliers()
    pi.allocate_bond_order_factors(0)
    for c, g in coords:
        for b in c.get_bond_order_parameters():
            for t in b.get_symbols():
                assert pi.add_bond_order_factor(b.get_bond_order_type(), np.array(b.get_parameters_as_list()),
                                                np.array(b.get_number_of_parameters()), b.get_cutoff(),
                                                b.get_soft_cutoff(), np.array([codes(s) for s in t]).T,
                                                np.array([codes(s) for s in t]).T, g)
    pi.allocate_bond_order_storage(n, 0, len(coords))
    pi.create_potential_list()
    pi.create_bond_order_factor_list()
    if coulomb is not None:
        ew = ewald_settings(atoms, coulomb)
        pi.set_ewald_parameters(ew["rc"], ew["kc"], ew["kmax"], ew["sigma"], ew["eps"], ew["scaler"])
    return coords


def neighbors(pi, atoms, pots, coulomb=None, skin=0.5):
    cuts = np.array(individual_cutoffs(atoms, pots, coulomb)) + skin
    pi.generate_neighbor_lists(cuts)
    lists = []
    for i in range(len(atoms)):
        k = pi.get_number_of_neighbors_of_atom(i)
        lists.append(pi.get_neighbor_list_of_atom(i, k) if k else (np.zeros(0, int), np.zeros((3, 0), int)))
    return lists
