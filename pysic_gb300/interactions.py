"""User-facing interaction objects: Potential, BondOrderParameters, Coordinator,
CoulombSummation.

These mirror pysic/interactions/local.py:284-776, bondorder.py:7-534 and
coulomb.py:6-218 of the reference: same constructor arguments, parameter
orders, target-list format ([[a, b], [c, d]]), cutoff / cutoff-margin
semantics (soft cutoff = cutoff - margin) and equality rules.  They hold no
engine state; the calculator compiles them into interaction records when a
calculation is requested (pysic_gb300/model.py).
"""
import copy

from . import core
from .error import InvalidCoordinatorError, InvalidParametersError, InvalidPotentialError, InvalidSummationError, warn


def _accepts_target_list(targets, n_targets):
    try:
        for a_set in targets:
            if not isinstance(a_set, (list, tuple)) or len(a_set) != n_targets:
                return False
        return True
    except TypeError:
        return False


def _normalise_targets(targets, n_targets, err):
    if targets is None:
        return None
    if _accepts_target_list(targets, n_targets):
        return [list(t) for t in targets]
    if _accepts_target_list([targets], n_targets):
        return [list(targets)]
    raise err("Invalid number of targets.")


def _different(lists):
    out = []
    for group in lists or []:
        for x in group:
            if x not in out:
                out.append(x)
    return out


class Potential(object):
    """A local potential acting on 1-4 targets (pysic/interactions/local.py:284-776)."""

    def __init__(self, potential_type, symbols=None, tags=None, indices=None, parameters=None, cutoff=0.0,
                 cutoff_margin=0.0, coordinator=None):
        if not core.is_valid_potential(potential_type):
            raise InvalidPotentialError('There is no potential called "{0}".'.format(potential_type))
        self.potential_type = potential_type
        self.symbols = None
        self.tags = None
        self.indices = None
        self.cutoff = cutoff
        self.cutoff_margin = 0.0
        self.coordinator = None
        self.set_cutoff_margin(cutoff_margin)
        self.n_targets = core.number_of_targets(potential_type)
        self.names_of_params = core.names_of_parameters(potential_type)
        self.set_symbols(symbols)
        self.set_tags(tags)
        self.set_indices(indices)
        self.parameters = [0.0] * len(self.names_of_params) if parameters is None else list(parameters)
        if len(self.parameters) != len(self.names_of_params):
            raise InvalidPotentialError('The potential "{0}" requires {1} parameters: {2}'.format(
                potential_type, len(self.names_of_params), self.names_of_params))
        self.set_coordinator(coordinator)

    def __eq__(self, other):
        try:
            return (self.symbols == other.symbols and self.tags == other.tags and self.indices == other.indices
                    and self.potential_type == other.potential_type and self.parameters == other.parameters
                    and self.cutoff == other.cutoff and self.coordinator == other.coordinator)
        except AttributeError:
            return False

    def __ne__(self, other):
        return not self.__eq__(other)

    def __repr__(self):
        return ("Potential('{0}',symbols={1},tags={2},indices={3},parameters={4},cutoff={5},cutoff_margin={6},"
                "coordinator={7})").format(self.potential_type, self.symbols, self.tags, self.indices,
                                           self.parameters, self.cutoff, self.cutoff_margin, self.coordinator)

    def get_number_of_parameters(self):
        return core.number_of_parameters(self.potential_type)

    def get_symbols(self):
        return self.symbols

    def get_tags(self):
        return self.tags

    def get_indices(self):
        return self.indices

    def get_different_symbols(self):
        return _different(self.symbols)

    def get_different_tags(self):
        return _different(self.tags)

    def get_different_indices(self):
        return _different(self.indices)

    def get_parameter_values(self):
        return self.parameters

    def get_parameter_names(self):
        return self.names_of_params

    def get_parameter_value(self, param_name):
        return self.parameters[core.index_of_parameter(self.potential_type, param_name)]

    def get_potential_type(self):
        return self.potential_type

    def get_cutoff(self):
        return self.cutoff

    def get_cutoff_margin(self):
        return self.cutoff_margin

    def get_soft_cutoff(self):
        return self.cutoff - self.cutoff_margin

    def get_number_of_targets(self):
        return self.n_targets

    def accepts_target_list(self, targets):
        return _accepts_target_list(targets, self.n_targets)

    def get_coordinator(self):
        return self.coordinator

    def set_coordinator(self, coordinator):
        self.coordinator = coordinator

    def set_symbols(self, symbols):
        if symbols is None:
            return
        self.symbols = _normalise_targets(symbols, self.n_targets, InvalidPotentialError)

    def set_tags(self, tags):
        if tags is None:
            return
        self.tags = _normalise_targets(tags, self.n_targets, InvalidPotentialError)

    def set_indices(self, indices):
        if indices is None:
            return
        self.indices = _normalise_targets(indices, self.n_targets, InvalidPotentialError)

    def _add(self, attr, values):
        new = _normalise_targets(values, self.n_targets, InvalidPotentialError)
        cur = getattr(self, attr)
        setattr(self, attr, (cur or []) + new)

    def add_symbols(self, symbols):
        self._add("symbols", symbols)

    def add_tags(self, tags):
        self._add("tags", tags)

    def add_indices(self, indices):
        self._add("indices", indices)

    def set_parameters(self, values):
        self.set_parameter_values(values)

    def set_parameter_values(self, values):
        if len(values) != self.get_number_of_parameters():
            raise InvalidPotentialError("The potential '{0}' takes {1} parameters, not {2}.".format(
                self.potential_type, self.get_number_of_parameters(), len(values)))
        self.parameters = list(values)

    def set_parameter_value(self, parameter_name, value):
        index = core.index_of_parameter(self.potential_type, parameter_name)
        if index < 0:
            raise InvalidPotentialError("The potential '{0}' does not have a parameter '{1}'".format(
                self.potential_type, parameter_name))
        self.parameters[index] = value

    def set_cutoff(self, cutoff):
        self.cutoff = cutoff

    def set_cutoff_margin(self, margin):
        if margin < 0.0:
            raise InvalidPotentialError("A negative cutoff margin of {0} was given.".format(margin))
        if margin > self.cutoff:
            raise InvalidPotentialError(
                "A cutoff margin ({0}) longer than the hard cutoff ({1}) was given.".format(margin, self.cutoff))
        self.cutoff_margin = margin

    def set_soft_cutoff(self, cutoff):
        self.set_cutoff_margin(self.cutoff - cutoff)

    def get_potentials(self):
        return [self]

    def is_multiplier(self):
        return [False]

    def describe(self):
        core.description_of_potential(self.potential_type, self.parameters, self.cutoff, self.symbols, self.tags,
                                      self.indices)


class ProductPotential:
    """A potential that is the product of several potentials with the same
    number of targets (pysic/interactions/local.py:7-283).  The first potential
    leads: its targets, cutoff, cutoff margin and coordinator are the
    product's; the others only multiply (``is_multiplier``).  Energies,
    forces and electronegativities follow the product rule
    (Potentials.f90:2512-2700), the leading potential's smooth cutoff applies
    to the whole product."""

    def __init__(self, potentials):
        self.potentials = []
        self.n_targets = None
        self.add_potential(potentials)

    def __eq__(self, other):
        try:
            return self.n_targets == other.n_targets and self.potentials == other.potentials
        except AttributeError:
            return False

    def __ne__(self, other):
        return not self.__eq__(other)

    def __repr__(self):
        return "ProductPotential({0})".format(self.potentials)

    def set_potentials(self, potentials):
        self.potentials = []
        self.n_targets = None
        self.add_potential(potentials)

    def add_potential(self, potential):
        """Adds a potential, a list of potentials or the factors of another product."""
        for pot in (potential if isinstance(potential, list) else [potential]):
            if self.n_targets is None:
                self.n_targets = pot.get_number_of_targets()
            elif self.n_targets != pot.get_number_of_targets():
                raise InvalidPotentialError("You may only multiply potentials with the same number of targets.")
            for p in pot.get_potentials():
                self.potentials.append(copy.deepcopy(p))

    def get_potentials(self):
        return self.potentials

    def is_multiplier(self):
        return [False] + [True] * (len(self.potentials) - 1)

    def get_potential_type(self):
        return self.potentials[0].get_potential_type()

    def get_number_of_targets(self):
        return self.n_targets

    def accepts_target_list(self, targets):
        return self.potentials[0].accepts_target_list(targets)

    def __getattr__(self, name):
        # targets, cutoffs and the coordinator are those of the leading potential
        if name in ("get_symbols", "get_tags", "get_indices", "get_different_symbols", "get_different_tags",
                    "get_different_indices", "get_cutoff", "get_cutoff_margin", "get_soft_cutoff",
                    "get_coordinator", "set_coordinator", "set_symbols", "set_tags", "set_indices",
                    "add_symbols", "add_tags", "add_indices", "set_cutoff", "set_cutoff_margin",
                    "set_soft_cutoff"):
            pots = self.__dict__.get("potentials")
            if not pots:
                raise InvalidPotentialError("an empty product of potentials")
            return getattr(pots[0], name)
        raise AttributeError(name)


class BondOrderParameters:
    """Parameters of one bond-order factor (pysic/interactions/bondorder.py:7-376).

    ``parameters`` is ``[[scaling ...], [local ...]]``; for 'tersoff' that is
    ``[[beta, eta], [a, c, d, h, mu]]`` (Potentials.f90:5715-5728)."""

    def __init__(self, bond_order_type, cutoff=0.0, cutoff_margin=0.0, parameters=None, symbols=None):
        if not core.is_valid_bond_order_factor(bond_order_type):
            raise InvalidParametersError('There is no bond order factor called "{0}"'.format(bond_order_type))
        self.bond_order_type = bond_order_type
        self.cutoff = cutoff
        self.cutoff_margin = 0.0
        self.set_cutoff_margin(cutoff_margin)
        self.n_targets = core.number_of_targets(bond_order_type)
        self.names_of_params = core.names_of_parameters(bond_order_type)
        self.n_params = core.number_of_parameters(bond_order_type)
        self.level = core.level_of_factor(bond_order_type)
        if parameters is None:
            self.parameters = [[0.0] * self.n_params[0], [0.0] * self.n_params[1]]
        else:
            self.set_parameters(parameters)
        self.symbols = None
        self.set_symbols(symbols)

    def __repr__(self):
        return "BondOrderParameters( bond_order_type='{0}',cutoff={1},cutoff_margin={2},parameters={3},symbols={4} )"\
            .format(self.bond_order_type, self.cutoff, self.cutoff_margin, self.parameters, self.symbols)

    def __eq__(self, other):
        try:
            return (self.bond_order_type == other.bond_order_type and self.cutoff == other.cutoff
                    and self.cutoff_margin == other.cutoff_margin and self.parameters == other.parameters
                    and self.symbols == other.symbols)
        except AttributeError:
            return False

    def __ne__(self, other):
        return not self.__eq__(other)

    def accepts_parameters(self, params):
        if len(params) != len(self.n_params):
            return False
        return all(len(params[i]) == self.n_params[i] for i in range(len(self.n_params)))

    def get_number_of_parameters(self):
        return self.n_params

    def includes_scaling(self):
        return self.n_params[0] > 0

    def get_level(self):
        return self.level

    def get_number_of_targets(self):
        return self.n_targets

    def get_parameters_as_list(self):
        return [p for group in self.parameters for p in group]

    def set_symbols(self, symbols):
        if symbols is None:
            return
        self.symbols = _normalise_targets(symbols, self.n_targets, InvalidParametersError)

    def add_symbols(self, symbols):
        new = _normalise_targets(symbols, self.n_targets, InvalidParametersError)
        self.symbols = (self.symbols or []) + new

    def get_symbols(self):
        return self.symbols

    def get_different_symbols(self):
        return _different(self.symbols)

    def get_parameter_values(self):
        return self.parameters

    def get_parameter_names(self):
        return self.names_of_params

    def get_parameter_value(self, param_name):
        idx = core.index_of_parameter(self.bond_order_type, param_name)
        return self.parameters[idx[0]][idx[1]]

    def get_bond_order_type(self):
        return self.bond_order_type

    def get_cutoff(self):
        return self.cutoff

    def get_cutoff_margin(self):
        return self.cutoff_margin

    def get_soft_cutoff(self):
        return self.cutoff - self.cutoff_margin

    def set_parameter_values(self, values):
        self.set_parameters(values)

    def set_parameter_value(self, parameter_name, value):
        idx = core.index_of_parameter(self.bond_order_type, parameter_name)
        if idx is None:
            raise InvalidParametersError("The bond order factor '{0}' does not have a parameter '{1}'".format(
                self.bond_order_type, parameter_name))
        self.parameters[idx[0]][idx[1]] = value

    def set_cutoff(self, cutoff):
        self.cutoff = cutoff

    def set_cutoff_margin(self, margin):
        if margin < 0.0:
            raise InvalidParametersError("A negative cutoff margin of {0} was given.".format(margin))
        if margin > self.cutoff:
            raise InvalidParametersError(
                "A cutoff margin ({0}) longer than the hard cutoff ({1}) was given.".format(margin, self.cutoff))
        self.cutoff_margin = margin

    def set_soft_cutoff(self, cutoff):
        self.set_cutoff_margin(self.cutoff - cutoff)

    def accepts_target_list(self, targets):
        return _accepts_target_list(targets, self.n_targets)

    def set_parameters(self, params):
        """Accepts [[scaling], [local]] or a flat list (bondorder.py:351-376)."""
        params = copy.deepcopy(list(params))
        if len(params) == len(self.n_params) and all(isinstance(p, (list, tuple)) for p in params):
            if self.accepts_parameters(params):
                self.parameters = [list(p) for p in params]
                return
        if len(params) == self.n_params[0] + self.n_params[1] and not any(isinstance(p, (list, tuple))
                                                                          for p in params):
            new = [params[:self.n_params[0]], params[self.n_params[0]:]]
            warn("Using parameters \n{0}\ninstead of \n{1}".format(new, params), 3)
            self.parameters = new
            return
        raise InvalidParametersError('The bond order factor "{0}" requires {1} parameters.'.format(
            self.bond_order_type, self.n_params))


class Coordinator:
    """A group of bond-order factors scaling a potential
    (pysic/interactions/bondorder.py:379-534).

    In the GB300 engine the per-bond factors live on the device; the
    Fortran-core queries (bond-order factors and gradients per atom) are
    served by the calculator the coordinator is used in."""

    def __init__(self, bond_order_parameters=None):
        self.bond_order_params = []
        self.bond_order_factors = None
        if bond_order_parameters is not None:
            self.set_bond_order_parameters(bond_order_parameters)
        self.group_index = -1
        self._calculator = None

    def __eq__(self, other):
        try:
            return self.group_index == other.group_index and self.bond_order_params == other.bond_order_params
        except AttributeError:
            return False

    def __ne__(self, other):
        return not self.__eq__(other)

    def __deepcopy__(self, memo):
        # the calculator the coordinator reports to is shared, not copied
        new = Coordinator.__new__(Coordinator)
        memo[id(self)] = new
        for k, v in self.__dict__.items():
            setattr(new, k, v if k == "_calculator" else copy.deepcopy(v, memo))
        return new

    def __repr__(self):
        return "Coordinator(bond_order_parameters={0})".format(self.bond_order_params)

    def get_bond_order_parameters(self):
        return self.bond_order_params

    def set_bond_order_parameters(self, params):
        self.bond_order_params = list(params) if isinstance(params, list) else [params]

    def add_bond_order_parameters(self, params):
        if isinstance(params, list):
            self.bond_order_params.extend(params)
        else:
            self.bond_order_params.append(params)

    def set_group_index(self, index):
        self.group_index = index

    def get_group_index(self):
        return self.group_index

    def calculate_bond_order_factors(self):
        """Per-atom (level-1) bond-order factors B_i of this group at the current
        positions (bondorder.py:493-506 -> core_get_bond_order_factors,
        Core.f90:759-783), computed on the device.  A group made only of
        pairwise (level-2) factors such as 'tersoff' has none, and the reference
        returns zeros for it; so does this engine."""
        calc = self._calculator
        if calc is None:
            raise InvalidCoordinatorError("The coordinator is not attached to a calculator.")
        calc.set_core()
        self.bond_order_factors = calc.engine.atom_factors(self.group_index, calc._prec())

    def get_bond_order_factors(self):
        return self.bond_order_factors

    def get_bond_order_gradients(self, atom_index):
        """Gradients (n x 3) of every atom's factor of this group with respect to
        moving atom `atom_index` (bondorder.py:508-519), computed on the device."""
        calc = self._attached()
        return calc.engine.atom_factor_gradients(self.group_index, atom_index, False, calc._prec())

    def get_bond_order_gradients_of_factor(self, atom_index):
        """Gradients (n x 3) of atom `atom_index`'s factor of this group with
        respect to moving every atom (bondorder.py:521-534)."""
        calc = self._attached()
        return calc.engine.atom_factor_gradients(self.group_index, atom_index, True, calc._prec())

    def _attached(self):
        calc = self._calculator
        if calc is None:
            raise InvalidCoordinatorError("The coordinator is not attached to a calculator.")
        calc.set_core()
        return calc


class CoulombSummation:
    """Ewald summation parameters (pysic/interactions/coulomb.py:6-176):
    ``[real_cutoff, k_cutoff, sigma, epsilon]`` and optional per-atom charge scalers."""

    summation_modes = ["ewald"]
    summation_parameters = {"ewald": ["real_cutoff", "k_cutoff", "sigma", "epsilon"]}
    summation_parameter_descriptions = {"ewald": ["real space cutoff radius", "reciprocal space cutoff radius",
                                                  "ewald summation split parameter", "vacuum permittivity"]}

    def __init__(self, method="ewald", parameters=None, scaler=None):
        self.set_summation(method)
        self.set_parameters(parameters)
        self.set_scaling_factors(scaler)

    def __eq__(self, other):
        try:
            return self.method == other.method and self.parameters == other.parameters and \
                _same_scaler(self.scaler, other.scaler)
        except AttributeError:
            return False

    def __ne__(self, other):
        return not self == other

    def __repr__(self):
        return "CoulombSummation(method='{0}',parameters={1},scaler={2})".format(self.method, self.parameters,
                                                                                  self.scaler)

    def set_summation(self, method):
        if method not in CoulombSummation.summation_modes:
            raise InvalidSummationError("no such summation mode " + str(method))
        self.method = method
        self.initialize_parameters()

    def initialize_parameters(self):
        self.parameters = {p: 0.0 for p in CoulombSummation.summation_parameters[self.method]}

    def set_parameters(self, parameters):
        self.set_parameter_values(parameters)

    def set_parameter_values(self, parameters):
        if parameters is None:
            return
        names = CoulombSummation.summation_parameters[self.method]
        if len(parameters) != len(names):
            raise InvalidSummationError("The summation mode {0} requires {1} parameters.".format(
                self.method, len(names)))
        for key, value in zip(names, parameters):
            self.parameters[key] = value

    def set_parameter_value(self, parameter_name, value):
        self.parameters[parameter_name] = value

    def set_scaling_factors(self, scaler):
        self.scaler = scaler

    def get_scaling_factors(self):
        return self.scaler

    def get_summation(self):
        return self.method

    def get_parameters(self):
        return self.parameters

    def get_realspace_cutoff(self):
        if self.method == "ewald":
            return self.parameters["real_cutoff"]
        return 0.0


def _same_scaler(a, b):
    if a is None or b is None:
        return a is None and b is None
    return list(a) == list(b)


def estimate_ewald_parameters(real_cutoff=10.0, accuracy="normal"):
    """First guess (real_cutoff, k_cutoff, sigma, epsilon) by the scaling rules
    of pysic/interactions/coulomb.py:179-218; epsilon = 0.00552635 e^2/(eV A)."""
    epsilon = 0.00552635
    rules = {"low": (2.0, 2.0), "normal": (3.0, 3.0), "high": (4.0, 4.0), "real": (3.0, 2.0),
             "reciprocal": (2.0, 3.0)}
    sdiv, kmul = rules[accuracy]
    sigma = real_cutoff / sdiv
    return (real_cutoff, kmul / sigma, sigma, epsilon)


class CompoundPotential(Potential):
    """A potential assembled from elementary Potential objects
    (pysic/interactions/compound.py:8-213): the calculator adds its pieces,
    which define_elements() builds, one by one."""

    def __init__(self, n_targets, n_params, symbols=None, tags=None, indices=None, parameters=None, cutoff=0.0,
                 cutoff_margin=0.0):
        self.n_targets = n_targets
        self.n_params = n_params
        self.symbols = None
        self.tags = None
        self.indices = None
        self.cutoff = cutoff
        self.cutoff_margin = 0.0
        self.coordinator = None
        self.parameters = [0.0] * n_params if parameters is None else list(parameters)
        self.set_cutoff_margin(cutoff_margin)
        self.set_symbols(symbols)
        self.set_tags(tags)
        self.set_indices(indices)
        self.potential_type = None
        self.names_of_params = ["anonymous"] * n_params
        self.descriptions_of_params = ["description missing"] * n_params
        self.description = "This compound potential has no description."
        self.pieces = []

    def __eq__(self, other):
        try:
            if (self.potential_type != other.potential_type or self.symbols != other.symbols
                    or self.tags != other.tags or self.indices != other.indices
                    or self.parameters != other.parameters or self.cutoff != other.cutoff):
                return False
            return len(self.pieces) == len(other.pieces) and all(a == b for a, b in zip(self.pieces, other.pieces))
        except AttributeError:
            return False

    def __ne__(self, other):
        return not self.__eq__(other)

    def __repr__(self):
        return "{0}(symbols={1},tags={2},indices={3},parameters={4},cutoff={5},cutoff_margin={6})".format(
            type(self).__name__, self.symbols, self.tags, self.indices, self.parameters, self.cutoff,
            self.cutoff_margin)

    def get_number_of_parameters(self):
        return self.n_params

    def get_parameter_names(self):
        return self.names_of_params

    def set_potential_type(self, potential_type):
        self.potential_type = potential_type

    def get_elements(self):
        return self.pieces

    def build(self, calculator):
        self.define_elements()
        for piece in self.pieces:
            calculator.add_potential(piece)

    def remove(self, calculator):
        self.define_elements()
        for piece in self.pieces:
            try:
                calculator.remove_potential(piece)
            except ValueError:
                warn("Could not remove a potential {0} from the calculator.".format(piece.get_potential_type()), 2)

    def define_elements(self):
        self.pieces = []

    def describe(self):
        print("potential '{0}'\n{1}-body interaction\n{2}".format(self.potential_type, self.n_targets,
                                                                 self.description))


class SuttonChenPotential(CompoundPotential):
    """U = epsilon [ sum_ij (a/r)^n - c sum_i sqrt(rho_i) ], rho_i = sum_j (a/r)^m
    (pysic/interactions/suttonchen.py:8-176), parameters [epsilon, a, c, n, m].

    The pieces are the reference's: a 'power' pair potential eps (a/r)^n on the
    given targets, and per element a 'constant' potential eps scaled by a
    Coordinator of 'sqrt_scale' (epsilon = -c) over 'power_bond' (a, m) on the
    element pairs that the element leads.  Element targets only."""

    def __init__(self, symbols=None, tags=None, indices=None, parameters=None, cutoff=0.0, cutoff_margin=0.0):
        super(SuttonChenPotential, self).__init__(n_params=5, n_targets=2, symbols=symbols, tags=tags,
                                                  indices=indices, parameters=parameters, cutoff=cutoff,
                                                  cutoff_margin=cutoff_margin)
        self.density_symbols = None
        self.set_potential_type("suttonchen")
        self.names_of_params = ["epsilon", "a", "c", "n", "m"]
        self.descriptions_of_params = ["energy scale constant", "lenght scale or lattice constant",
                                       "density coefficient", "power decay exponent", "density decay exponent"]
        self.description = ("A potential of type\n U = epsilon [ sum_ij (a/r)^n - c sum_i sqrt(rho) ],\nwhere\n"
                            " rho = sum_j (a/r)^m.\nand r is the interatomic distance.")

    def set_density_symbols(self, symbols):
        self.density_symbols = symbols

    def define_elements(self):
        if self.tags or self.indices:
            raise InvalidPotentialError("the Sutton-Chen density terms are built for element targets only")
        eps, a, c, n, m = [float(x) for x in self.parameters]
        pair = Potential("power", symbols=self.symbols, cutoff=self.cutoff, cutoff_margin=self.cutoff_margin)
        pair.set_parameter_value("epsilon", eps)
        pair.set_parameter_value("a", a)
        pair.set_parameter_value("n", n)
        self.pieces = [pair]
        elements, pairs = [], []
        for t in self.symbols or []:
            for e in t:
                if e not in elements:
                    elements.append(e)
            pairs.append(list(t))
            if len(t) == 2 and t[0] != t[1]:
                pairs.append([t[1], t[0]])
        for e in elements:
            if self.density_symbols is not None and e not in self.density_symbols:
                continue
            scaler = BondOrderParameters("sqrt_scale")
            scaler.set_parameter_value("epsilon", -c)
            scaler.set_symbols([[e]])
            density = BondOrderParameters("power_bond", cutoff=self.cutoff, cutoff_margin=self.cutoff_margin)
            density.set_parameter_value("a", a)
            density.set_parameter_value("n", m)
            density.set_symbols([p for p in pairs if p[0] == e])
            piece = Potential("constant", parameters=[eps], symbols=[[e]])
            piece.set_coordinator(Coordinator([scaler, density]))
            self.pieces.append(piece)
