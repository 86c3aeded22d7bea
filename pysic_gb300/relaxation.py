"""Charge relaxation (pysic/charges/relaxation.py:11-550).

'dynamic' runs the reference's damped charge dynamics (relaxation.py:417-450)
entirely on the device through pg_relax_charges: the electronegativity kernels
and the velocity-Verlet-with-friction update are launched back to back
without host round trips, and only the convergence statistics come back.
'potentiostat' (453-481) runs on the device the same way
(pg_relax_charges_potentiostat: undamped, chi minus a fixed external
potential, a fixed number of steps).  With observers attached the device loop
returns to the host at every step where one is due, so that each sees the
atoms' charges of its step as in the reference (510-550); the cut loop takes
the same steps as the uncut one.  'optimize' (483-488) finds the constrained
energy minimum on the device by projected conjugate gradients when the energy
is quadratic in the charges (pg_optimize_charges; it stops on
max |chi - mean(chi)| <= tolerance), else it runs SciPy's SLSQP on the GPU
energy and gradient as the reference does.
"""
import math

import numpy as np

from .error import InvalidRelaxationError, warn


class ChargeRelaxation:
    relaxation_modes = ["dynamic", "potentiostat", "optimize"]
    relaxation_parameters = {
        "dynamic": ["n_steps", "timestep", "inertia", "friction", "tolerance"],
        "potentiostat": ["n_steps", "timestep", "inertia", "potential"],
        "optimize": ["n_steps", "tolerance"],
    }
    relaxation_parameter_descriptions = {
        "dynamic": ["number of time steps of charge dynamics between molecular dynamics",
                    "time step of charge dynamics", "fictional charge mass",
                    "friction coefficient for damped charge dynamics", "convergence tolerance"],
        "potentiostat": ["number of time steps of charge dynamics between molecular dynamics",
                         "time step of charge dynamics", "fictional charge mass", "external potential"],
        "optimize": ["maximum number of optimization steps", "convergence tolerance"],
    }

    def __init__(self, relaxation="dynamic", calculator=None, parameters=None, atoms=None, warm_start=None):
        self.calculator = None
        self.warm_start = warm_start  # a trained mlp.ChargeNetwork, or None
        self.set_relaxation(relaxation)
        self.set_calculator(calculator)
        self.set_parameters(parameters)
        self.set_atoms(atoms)
        self.piped_relaxation = None
        self.charge_rates = None
        self.observers = []
        self.last_steps = 0
        self.last_error = None
        self.last_max_dq = None
        self.last_converged = None
        self.last_warm_start_seconds = 0.0

    def set_warm_start(self, network):
        """Start the 'dynamic' relaxation from the charges a trained
        ChargeNetwork predicts (None: from the current charges, as the
        reference does).  The relaxation itself is unchanged and runs to the
        same tolerance."""
        self.warm_start = network

    def __eq__(self, other):
        try:
            return (self.relaxation == other.relaxation and self.calculator is other.calculator
                    and self.parameters == other.parameters and self.atoms is other.atoms)
        except AttributeError:
            return False

    def __ne__(self, other):
        return not self == other

    def __repr__(self):
        return "ChargeRelaxation('{0}',calculator={1},parameters={2},atoms={3})".format(
            self.relaxation, self.calculator, self.parameters, self.atoms)

    # --- configuration ---------------------------------------------------------
    def set_relaxation_pipe(self, relaxation, pass_info=True):
        if relaxation is self:
            raise InvalidRelaxationError("Trying to create a looped relaxation pipe.")
        if relaxation is not None:
            for rel in relaxation.get_relaxation_pipe():
                if rel is self:
                    raise InvalidRelaxationError("Trying to create a looped relaxation pipe.")
        self.piped_relaxation = relaxation
        if pass_info and relaxation is not None:
            for rel in self.get_relaxation_pipe():
                rel.set_calculator(self.calculator)
                rel.set_atoms(self.atoms)

    def clear_relaxation_pipe(self):
        self.piped_relaxation = None

    def get_relaxation_pipe(self, recursive=True):
        if not recursive:
            return self.piped_relaxation
        pipe = []
        nxt = self.piped_relaxation
        while nxt is not None:
            pipe.append(nxt)
            nxt = nxt.piped_relaxation
        return pipe

    def set_calculator(self, calculator, reciprocal=False):
        if self.calculator is not None and self.calculator is not calculator:
            try:
                self.calculator.set_charge_relaxation(None)
            except AttributeError:
                pass
        self.calculator = calculator
        if reciprocal and calculator is not None:
            calculator.set_charge_relaxation(self)

    def get_calculator(self):
        return self.calculator

    def set_relaxation(self, relaxation):
        if relaxation not in ChargeRelaxation.relaxation_modes:
            raise InvalidRelaxationError("no such relaxation mode " + str(relaxation))
        self.relaxation = relaxation
        self.initialize_parameters()

    def get_relaxation(self):
        return self.relaxation

    def initialize_parameters(self):
        self.parameters = {p: 0.0 for p in ChargeRelaxation.relaxation_parameters[self.relaxation]}

    def set_parameters(self, parameters):
        self.set_parameter_values(parameters)

    def set_parameter_values(self, parameters):
        """Values in the order of ``relaxation_parameters[mode]``.  (The
        reference zips them with a dict's key order, relaxation.py:273, which in
        Python 2 is not the documented order; here the documented order is used.)"""
        if parameters is None:
            return
        names = ChargeRelaxation.relaxation_parameters[self.relaxation]
        if len(parameters) != len(names):
            raise InvalidRelaxationError("The relaxation mode {0} requires {1} parameters.".format(
                self.relaxation, len(names)))
        for k, v in zip(names, parameters):
            self.parameters[k] = v

    def set_parameter_value(self, parameter_name, value):
        self.parameters[parameter_name] = value

    def get_parameters(self):
        return self.parameters

    def set_atoms(self, atoms, pass_to_calculator=False):
        self.atoms = atoms
        if pass_to_calculator:
            self.calculator.set_atoms(atoms)

    def get_atoms(self):
        return self.atoms

    # --- relaxation --------------------------------------------------------------
    def charge_relaxation(self, precision=None):
        """Relax the charges of the calculator's structure and return them."""
        calc = self.calculator
        atoms = calc.get_atoms()
        try:
            charges = np.array(atoms.get_initial_charges(), dtype=np.float64)
        except AttributeError:
            charges = np.array(atoms.get_charges(), dtype=np.float64)
        if self.relaxation == "dynamic":
            p = self.parameters
            if self.charge_rates is None:
                self.charge_rates = np.zeros(len(atoms))
            if self.warm_start is not None:
                import time

                t0 = time.perf_counter()
                charges = self.warm_start.predict_charges(calc, total_charge=float(np.sum(charges)))
                self._set(atoms, charges)
                # the engine already holds the predicted charges
                pushed = getattr(calc, "_pushed", None)
                if pushed is not None:
                    pushed["charges"] = np.array(charges, dtype=np.float64)
                self.charge_rates = np.zeros(len(atoms))
                self.last_warm_start_seconds = time.perf_counter() - t0
            calc.set_core()
            prec = calc._prec() if precision is None else precision
            n_steps = int(p["n_steps"])

            def run(k):
                return calc.engine.relax_charges(prec, k, p["timestep"], p["inertia"], p["friction"],
                                                 p["tolerance"], self.charge_rates)

            r = self._run_segments(calc, atoms, n_steps, run)
            charges = r["charges"]
            self.last_error = r["error"]
            self.last_max_dq = r["max_dq"]
            self.last_converged = r["converged"]
        elif self.relaxation == "potentiostat":
            p = self.parameters
            if self.charge_rates is None:
                self.charge_rates = np.zeros(len(atoms))
            calc.set_core()
            prec = calc._prec() if precision is None else precision

            def run(k):
                r = calc.engine.relax_charges_potentiostat(prec, k, p["timestep"], p["inertia"], p["potential"],
                                                           self.charge_rates)
                r["converged"] = False  # no tolerance: the step count decides
                r["error"] = r["max_dchi"]
                return r

            r = self._run_segments(calc, atoms, int(p["n_steps"]), run)
            charges = r["charges"]
            self.last_error = r["max_dchi"]
        elif self.relaxation == "optimize":
            # on the device when the energy is quadratic in the charges
            calc.set_core()
            prec = calc._prec() if precision is None else precision
            r = calc.engine.optimize_charges(prec, int(self.parameters["n_steps"]), self.parameters["tolerance"])
            if r is not None:
                charges = r["charges"]
                self._set(atoms, charges)
                pushed = getattr(calc, "_pushed", None)
                if pushed is not None:
                    pushed["charges"] = np.array(charges, dtype=np.float64)
                self.last_steps = r["iterations"]
                self.last_error = r["error"]
                self.last_converged = r["converged"]
                return self._finish(charges)
            try:
                from scipy.optimize import fmin_slsqp
            except ImportError:
                raise InvalidRelaxationError("'optimize' needs SciPy")
            total = float(np.sum(charges))

            def energy(q, *args):
                self._set(atoms, q)
                return calc.get_potential_energy(skip_charge_relaxation=True)

            def grad(q, *args):
                self._set(atoms, q)
                return -calc.get_electronegativities()

            charges = fmin_slsqp(energy, charges, fprime=grad, eqcons=[lambda q, *a: np.sum(q) - total],
                                 acc=self.parameters["tolerance"], iter=int(self.parameters["n_steps"]), disp=0)
            self._set(atoms, charges)
        return self._finish(charges)

    def _finish(self, charges):
        """The reference's epilogue (relaxation.py:492-503): the attached
        structure gets the charges, then a piped relaxation runs."""
        if self.atoms is not None:
            try:
                self.atoms.set_initial_charges(charges)
            except AttributeError:
                self.atoms.set_charges(charges)
        if self.piped_relaxation is not None:
            charges = self.piped_relaxation.charge_relaxation()
        return charges

    def _observer_stride(self):
        """Steps between returns to the host: every step at which an observer
        may be due (the gcd of the intervals; 1 for an interval that is not an
        integer, which the reference then calls every step).  None: no
        observers, one device run."""
        if not self.observers:
            return None
        g = 0
        for _, interval, _, _ in self.observers:
            iv = int(interval) if isinstance(interval, (int, np.integer)) and interval > 0 else 1
            g = math.gcd(g, iv)
        return max(g, 1)

    def _run_segments(self, calc, atoms, n_steps, run):
        """The device loop, cut where observers are due.  A segment restarts
        from the charges and rates the previous one left and recomputes their
        electronegativities, the value the reference carries over, so the cut
        run takes the same steps as an uncut one.  Observers see the atoms'
        charges of their step (relaxation.py:510-550)."""
        stride = self._observer_stride()
        total = 0
        while True:
            k = n_steps - total if stride is None else min(stride, n_steps - total)
            r = run(max(k, 0))
            total += r["steps"]
            self.last_steps = total
            self.charge_rates = r["rates"]
            self._set(atoms, r["charges"])
            # the engine's own copy of the charges is now the relaxed one
            pushed = getattr(calc, "_pushed", None)
            if pushed is not None:
                pushed["charges"] = np.array(r["charges"], dtype=np.float64)
            if stride is not None and r["steps"] > 0:
                self.call_observers(total)
            diverged = not np.isfinite(r["error"])
            if stride is None or r["converged"] or diverged or total >= n_steps or k <= 0:
                break
        self.last_steps = total
        r["steps"] = total
        return r

    @staticmethod
    def _set(atoms, q):
        try:
            atoms.set_initial_charges(q)
        except AttributeError:
            atoms.set_charges(q)

    def add_observer(self, function, interval=1, *args, **kwargs):
        if not hasattr(function, "__call__"):
            function = function.write
        self.observers.append((function, interval, args, kwargs))

    def clear_observers(self):
        self.observers = []

    def call_observers(self, step):
        for function, interval, args, kwargs in self.observers:
            try:
                if step % interval == 0:
                    function(*args, **kwargs)
            except Exception as exc:  # observers must not break a relaxation
                warn("observer failed: {0}".format(exc), 3)
