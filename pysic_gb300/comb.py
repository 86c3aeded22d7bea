"""The COMB potential for Si / SiO2 as a compound of elementary terms.

Mirror of ``pysic.interactions.comb.CombPotential``
(pysic/interactions/comb.py:15-1329, the COMB10 parameter set): the same
parameter names and default values, the same component keywords for
``exclude`` / ``include``, and ``define_elements`` builds the same pieces in
the same order, which the calculator adds one by one:

- bond bending: ``bond_bend`` on Si-O-Si and O-Si-O (comb.py:637-663);
- attraction per element pair: charge_exp x charge_abs x exponential under a
  Coordinator of ``tersoff`` factors, one Coordinator per pair (665-895);
- repulsion per element pair: charge_exp x exponential (897-984);
- charge self energies c1 q + c2 q^2 + c3 q^3 + c4 q^4 per element
  (``charge_self``, 986-1036);
- field ("penalty") terms: charge_pair x power (r^-5) per element pair
  (1038-1178);
- Slater-orbital Coulomb corrections: charge_pair x power x exponential
  (x shift_power) per element pair (1180-1317);
- Ewald summation on the calculator (1319-1327): real space only with the
  default exclusions (the reference's screened "cheat"), with k-space when
  ``long_coulomb`` is included.

Every piece runs on the engine's kernels (bond-order kernels for the
Tersoff-scaled products, pair kernel for the other products, triplet kernel
for the bond bending, single-atom kernel for the self energies, Ewald
kernels).  One behaviour of the reference is kept as it is, because a drop-in
must give its numbers: the O-O Coulomb corrections get the Slater cutoff
margin (0.1 A) as their cutoff (the reference calls ``set_cutoff`` twice,
comb.py:1274-1275), so they vanish at every physical O-O distance.
"""
import copy
import math

from .error import warn
from .interactions import (BondOrderParameters, CompoundPotential, Coordinator, CoulombSummation, Potential,
                           ProductPotential, estimate_ewald_parameters)

# component keywords, in the reference's order (comb.py:52-72)
POSSIBLE_EXCLUDES = ("siosi_bend", "osio_bend", "sisi_attractive", "oo_attractive", "sio_attractive",
                     "sisi_bondorder", "oo_bondorder", "sio_bondorder", "sisi_repulsive", "oo_repulsive",
                     "sio_repulsive", "si_self", "o_self", "sisi_penalty", "oo_penalty", "sio_penalty",
                     "sisi_coulomb", "oo_coulomb", "sio_coulomb", "direct_coulomb", "long_coulomb")


def _comb10_defaults():
    """The COMB10 parameter set of the reference (comb.py:81-517), by name.
    The mixed Si-O values are derived from the per-element ones as there."""
    p = {}

    def put(prefix, names, values):
        for n, v in zip(names, values):
            p[(prefix + " " + n) if prefix else n] = float(v)

    put("coulomb", ("cutoff", "sigma", "epsilon"), (12.0, 3.535533906, 0.00552635))
    put("si-o-si bend", ("epsilon", "theta", "cutoff", "cutoff margin"), (2.6, 2.508561734, 3.05, 0.5))
    put("o-si-o bend", ("epsilon", "theta", "cutoff", "cutoff margin"), (0.3122, 1.910611932, 3.05, 0.5))
    element = {
        "si": {"attractive epsilon": 471.18, "rmax": -1.658949, "rmin": 1.651725, "qmax": 4.0, "qmin": -4.0,
               "attractive alpha": 1.7322, "attractive a": 1.0, "attractive b": -9.5367431640625e-07,
               "attractive q": 0.0, "attractive n": 10.0, "attractive zeta": 1.7322, "attractive cutoff": 3.0,
               "attractive cutoff margin": 0.2, "bondorder beta": 1.0999e-6, "bondorder eta": 0.78734,
               "bondorder mu": 3.0, "bondorder a": 1.7322, "bondorder c": 100390.0, "bondorder d": 16.218,
               "bondorder h": -0.59826},
        "o": {"attractive epsilon": 260.8931, "rmax": -0.00112, "rmin": 0.00148, "qmax": 5.5046, "qmin": -1.8349,
              "attractive alpha": 2.68, "attractive a": 1.00098, "attractive b": -2.26e-06, "attractive q": 1.83485,
              "attractive n": 10.0, "attractive zeta": 2.68, "attractive cutoff": 3.0,
              "attractive cutoff margin": 0.4, "bondorder beta": 2.0, "bondorder eta": 1.0, "bondorder mu": 1.0,
              "bondorder a": 2.68, "bondorder c": 6.6, "bondorder d": 1.0, "bondorder h": -0.229},
    }
    for el, table in element.items():
        put(el, table.keys(), table.values())
    put("", ("si-si-o bondorder cutoff", "si-si-o bondorder cutoff margin", "si-si-si bondorder cutoff",
             "si-si-si bondorder cutoff margin", "o-o-si bondorder cutoff", "o-o-si bondorder cutoff margin",
             "o-o-o bondorder cutoff", "o-o-o bondorder cutoff margin"), (3.05, 0.5, 3.0, 0.2, 3.05, 0.5, 3.0, 0.4))
    p["si-o attractive epsilon"] = math.sqrt(p["si attractive epsilon"] * p["o attractive epsilon"])
    p["si-o attractive zeta"] = (p["si attractive zeta"] + p["o attractive zeta"]) * 0.5
    p["si-o attractive cutoff"] = 3.05
    p["si-o attractive cutoff margin"] = 0.5
    p["si-o bondorder a"] = (p["si bondorder a"] + p["o bondorder a"]) * 0.5
    for t in ("o-si-si", "o-si-o", "si-o-si", "si-o-o"):
        p[t + " bondorder cutoff"] = 3.05
        p[t + " bondorder cutoff margin"] = 0.5
    put("si repulsive", ("epsilon", "lambda", "zeta", "cutoff", "cutoff margin"), (1830.8, 2.4799, 2.4799, 3.0, 0.2))
    put("o repulsive", ("epsilon", "lambda", "zeta", "cutoff", "cutoff margin"), (3326.699, 5.36, 5.36, 3.0, 0.4))
    p["si-o repulsive epsilon"] = math.sqrt(p["si repulsive epsilon"] * p["o repulsive epsilon"])
    p["si-o repulsive zeta"] = (p["si repulsive zeta"] + p["o repulsive zeta"]) * 0.5
    p["si-o repulsive cutoff"] = 3.05
    p["si-o repulsive cutoff margin"] = 0.5
    put("si charge", ("c1", "c2", "c3", "c4"), (0.0, 3.625144859, 0.0, 0.087067714))
    put("o charge", ("c1", "c2", "c3", "c4"), (5.63441383, 7.689598017, 4.51426991, 1.330079082))
    put("si field", ("rho1", "rho2"), (-0.499378, 2.999911))
    put("o field", ("rho1", "rho2"), (-3.922011, 0.971086))
    put("field", ("cutoff", "cutoff margin"), (12.0, 0.1))
    put("", ("si slater zeta", "o slater zeta", "slater cutoff margin"), (0.772871, 2.243072, 0.1))
    return p


class CombPotential(CompoundPotential):
    """COMB potential for Si / O (pysic/interactions/comb.py:15-1329).

    Use as in the reference::

        calc = pysic.Pysic()
        pot = CombPotential()
        pot.set_calculator(calc, True)

    The default exclusions (``direct_coulomb``, ``long_coulomb``) put an Ewald
    summation on the calculator, so the potential needs the calculator before
    it is built; ``set_calculator(calc, True)`` also adds the potential."""

    def __init__(self, excludes=None):
        super(CombPotential, self).__init__(n_params=0, n_targets=3)
        self.set_potential_type("comb")
        self.description = "Comb potential."
        self.excludes = ["direct_coulomb", "long_coulomb"] if excludes is None else list(excludes)
        self.calc = None
        self.possible_excludes = list(POSSIBLE_EXCLUDES)
        self.params = _comb10_defaults()
        self.names_of_params = list(self.params.keys())
        self.n_params = len(self.params)

    # ---- parameters and components (comb.py:520-608) ----
    def get_parameter_value(self, param_name):
        return self.params[param_name]

    def set_parameter_value(self, param_name, value):
        self.params[param_name] = value

    def set_calculator(self, calc, reciprocal=False):
        """Attach the calculator (needed for the Ewald summation); with
        ``reciprocal`` also run ``calc.set_potentials(self)``."""
        self.calc = calc
        if reciprocal:
            calc.set_potentials(self)

    def check_exclude(self, ex):
        if ex not in self.possible_excludes:
            warn("unknown COMB component keyword " + str(ex), 2)

    def toggle_exclude(self, ex):
        self.check_exclude(ex)
        if ex in self.excludes:
            self.excludes.remove(ex)
        else:
            self.excludes.append(ex)

    def exclude(self, ex):
        self.check_exclude(ex)
        if ex not in self.excludes:
            self.excludes.append(ex)

    def include(self, ex):
        self.check_exclude(ex)
        if ex in self.excludes:
            self.excludes.remove(ex)

    def list_excludes(self):
        return self.excludes

    def list_possible_excludes(self):
        return self.possible_excludes

    def is_included(self, ex):
        self.check_exclude(ex)
        return ex not in self.excludes

    def is_excluded(self, ex):
        return not self.is_included(ex)

    def include_all(self):
        """Everything but the unscreened and the long-range Coulomb parts."""
        self.excludes = ["direct_coulomb", "long_coulomb"]

    def exclude_all(self):
        self.excludes = copy.deepcopy(self.possible_excludes)

    def set_ewald(self, calc, cheat):
        """Put an Ewald summation on ``calc`` (comb.py:610-629): with ``cheat``
        the real-space part alone (k cutoff 0) with the potential's own sigma,
        otherwise the standard first guess for the Coulomb cutoff."""
        if cheat:
            rc, kc = self.params["coulomb cutoff"], 0.0
            sigma, eps = self.params["coulomb sigma"], self.params["coulomb epsilon"]
        else:
            rc, kc, sigma, eps = estimate_ewald_parameters(self.params["coulomb cutoff"])
        ewald = CoulombSummation()
        for name, value in (("real_cutoff", rc), ("k_cutoff", kc), ("sigma", sigma), ("epsilon", eps)):
            ewald.set_parameter_value(name, value)
        calc.set_coulomb_summation(ewald)

    # ---- the pieces (comb.py:631-1327) ----
    def _included(self, ex):
        return ex not in self.excludes

    def _charge_exp(self, eps, e1, e2, xi1, xi2):
        P = self.params
        return Potential("charge_exp", parameters=[eps, P[e1 + " rmax"], P[e1 + " rmin"], P[e1 + " qmax"],
                                                   P[e1 + " qmin"], P[e2 + " rmax"], P[e2 + " rmin"],
                                                   P[e2 + " qmax"], P[e2 + " qmin"], xi1, xi2])

    def _charge_abs(self, e1, e2):
        P = self.params
        return Potential("charge_abs", parameters=[P[e1 + " attractive a"], P[e1 + " attractive b"],
                                                   P[e1 + " attractive q"], P[e1 + " attractive n"],
                                                   P[e2 + " attractive a"], P[e2 + " attractive b"],
                                                   P[e2 + " attractive q"], P[e2 + " attractive n"]])

    def _tersoff(self, symbols, el, a, cut_key):
        """One Tersoff factor on the triplet ``symbols`` with element ``el``'s
        beta, eta, mu, c, d, h and the given a; cutoff from ``cut_key``."""
        P = self.params
        b = BondOrderParameters("tersoff", symbols=symbols)
        for name in ("beta", "eta", "mu", "c", "d", "h"):
            b.set_parameter_value(name, P[el + " bondorder " + name])
        b.set_parameter_value("a", a)
        b.set_cutoff(P[cut_key + " bondorder cutoff"])
        b.set_cutoff_margin(P[cut_key + " bondorder cutoff margin"])
        return b

    @staticmethod
    def _cut(pot, cutoff, margin):
        pot.set_cutoff(cutoff)
        pot.set_cutoff_margin(margin)
        return pot

    def define_elements(self):
        P = self.params
        inc = self._included
        pieces = []
        # bond bending (comb.py:637-663)
        for key, ex, symbols in (("si-o-si", "siosi_bend", ["Si", "O", "Si"]),
                                 ("o-si-o", "osio_bend", ["O", "Si", "O"])):
            if inc(ex):
                bend = Potential("bond_bend", symbols=symbols,
                                 parameters=[P[key + " bend epsilon"], P[key + " bend theta"], 1, 2])
                pieces.append(self._cut(bend, P[key + " bend cutoff"], P[key + " bend cutoff margin"]))
        # attraction, Tersoff-scaled (comb.py:665-895)
        si_o_a = P["si-o bondorder a"]
        attraction = (
            ("sisi_attractive", "sisi_bondorder", ["Si", "Si"], ("si", "si"), "si attractive",
             [(["Si", "Si", "O"], "si", P["si bondorder a"], "si-si-o"),
              (["Si", "Si", "Si"], "si", P["si bondorder a"], "si-si-si")]),
            ("oo_attractive", "oo_bondorder", ["O", "O"], ("o", "o"), "o attractive",
             [(["O", "O", "Si"], "o", P["o bondorder a"], "o-o-si"),
              (["O", "O", "O"], "o", P["o bondorder a"], "o-o-o")]),
            ("sio_attractive", "sio_bondorder", ["Si", "O"], ("si", "o"), "si-o attractive",
             [(["O", "Si", "Si"], "o", si_o_a, "o-si-si"), (["O", "Si", "O"], "o", si_o_a, "o-si-o"),
              (["Si", "O", "O"], "si", si_o_a, "si-o-o"), (["Si", "O", "Si"], "si", si_o_a, "si-o-si")]),
        )
        for ex, ex_bo, pair, (e1, e2), key, factors in attraction:
            if not inc(ex):
                continue
            prod = ProductPotential([
                self._charge_exp(P[key + " epsilon"], e1, e2, P[e1 + " attractive alpha"],
                                 P[e2 + " attractive alpha"]),
                self._charge_abs(e1, e2),
                Potential("exponential", parameters=[-1.0, P[key + " zeta"]])])
            self._cut(prod, P[key + " cutoff"], P[key + " cutoff margin"])
            prod.set_symbols(pair)
            pieces.append(prod)
            if inc(ex_bo):
                prod.set_coordinator(Coordinator([self._tersoff(s, el, a, c) for s, el, a, c in factors]))
        # repulsion (comb.py:897-984)
        for ex, pair, (e1, e2), key in (("sisi_repulsive", ["Si", "Si"], ("si", "si"), "si repulsive"),
                                        ("oo_repulsive", ["O", "O"], ("o", "o"), "o repulsive"),
                                        ("sio_repulsive", ["Si", "O"], ("si", "o"), "si-o repulsive")):
            if not inc(ex):
                continue
            prod = ProductPotential([
                self._charge_exp(P[key + " epsilon"], e1, e2, P[e1 + " repulsive lambda"],
                                 P[e2 + " repulsive lambda"]),
                Potential("exponential", parameters=[1.0, P[key + " zeta"]])])
            self._cut(prod, P[key + " cutoff"], P[key + " cutoff margin"])
            prod.set_symbols(pair)
            pieces.append(prod)
        # charge self energies (comb.py:986-1036)
        for ex, el, sym in (("si_self", "si", "Si"), ("o_self", "o", "O")):
            if inc(ex):
                for n in range(1, 5):
                    pieces.append(Potential("charge_self", symbols=[sym],
                                            parameters=[P["{0} charge c{1}".format(el, n)], n]))
        # field terms (comb.py:1038-1178): charge_pair (rho, n1, n2) x (1/r)^5
        r5 = Potential("power", parameters=[1.0, 1.0, 5.0])

        def field(el):
            rho1, rho2 = P[el + " field rho1"], P[el + " field rho2"]
            return [(rho1, 0, 1), (rho2, 0, 2), (rho1, 1, 0), (rho2, 2, 0)]

        si_f, o_f = field("si"), field("o")
        for ex, pair, terms in (("sisi_penalty", ["Si", "Si"], si_f), ("oo_penalty", ["O", "O"], o_f),
                                ("sio_penalty", ["Si", "O"], si_f[:2] + o_f[2:])):
            if not inc(ex):
                continue
            for eps, n1, n2 in terms:
                prod = ProductPotential([Potential("charge_pair", parameters=[eps, n1, n2]), r5])
                prod.set_symbols(pair)
                pieces.append(self._cut(prod, P["field cutoff"], P["field cutoff margin"]))
        # Slater-orbital Coulomb corrections (comb.py:1180-1317)
        zs, zo = P["si slater zeta"], P["o slater zeta"]
        qq = Potential("charge_pair", parameters=[1.0, 1.0, 1.0])
        k_e = Potential("power", parameters=[14.3996, 1.0, 1.0])
        si_decay = Potential("exponential", parameters=[-1.0, 2.0 * zs])
        o_decay = Potential("exponential", parameters=[-1.0, 2.0 * zo])
        direct = inc("direct_coulomb")

        def poly(eps, n):
            return Potential("shift_power", parameters=[eps, 0.0, 1.0, n])

        def same_element(z, decay):
            chains = [[qq, k_e]] if direct else []
            chains += [[qq, k_e, decay], [qq, k_e, decay, poly(11.0 / 8.0 * z, 1)],
                       [qq, k_e, decay, poly(3.0 / 4.0 * z * z, 2)], [qq, k_e, decay, poly(1.0 / 6.0 * z * z * z, 3)]]
            return chains

        if inc("sisi_coulomb"):
            for chain in same_element(zs, si_decay):
                prod = ProductPotential(chain)
                prod.set_symbols(["Si", "Si"])
                pieces.append(self._cut(prod, P["coulomb cutoff"], P["slater cutoff margin"]))
        if inc("oo_coulomb"):
            for chain in same_element(zo, o_decay):
                prod = ProductPotential(chain)
                prod.set_symbols(["O", "O"])
                # the reference sets the cutoff twice, the second time to the
                # Slater margin, and leaves the margin at 0 (comb.py:1274-1275)
                prod.set_cutoff(P["coulomb cutoff"])
                prod.set_cutoff(P["slater cutoff margin"])
                pieces.append(prod)
        if inc("sio_coulomb"):
            kappa = (zs * zs + zo * zo) / (zs * zs - zo * zo)
            chains = [[qq, k_e]] if direct else []
            chains += [[qq, k_e, Potential("exponential", parameters=[-(1 - kappa) * (1 - kappa) * (2 + kappa) / 4.0, 2 * zs])],
                       [qq, k_e, Potential("exponential", parameters=[-(1 + kappa) * (1 + kappa) * (2 - kappa) / 4.0, 2 * zo])],
                       [qq, k_e, poly((1 - kappa) * (1 - kappa) * 1.0 / 4.0 * zs, 1), si_decay],
                       [qq, k_e, poly((1 + kappa) * (1 + kappa) * 1.0 / 4.0 * zo, 1), o_decay]]
            for chain in chains:
                prod = ProductPotential(chain)
                prod.set_symbols(["Si", "O"])
                pieces.append(self._cut(prod, P["coulomb cutoff"], P["slater cutoff margin"]))
        self.pieces = pieces
        # Ewald summation in place of the unscreened Coulomb products (comb.py:1319-1327)
        if not direct:
            if self.calc is None:
                raise Exception("A Pysic calculator needed for Ewald. Use set_calculator(calc).")
            self.set_ewald(self.calc, cheat=not inc("long_coulomb"))
