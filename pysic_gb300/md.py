"""Velocity Verlet molecular dynamics with the steps on the device.

The reference runs MD through ASE (doc/run examples.rst): ASE's
VelocityVerlet.step (ase/md/verlet.py) reads the momenta, asks the Pysic
calculator for forces and writes the positions back, every step crossing into
the Fortran core.  ``VelocityVerlet`` here keeps ASE's interface (timestep in
ASE units, ``run(steps)``, ``attach(function, interval)``, ``nsteps``) and its
update, operation for operation, but the steps run on the GPU (pg_md_run):
forces, both kicks and the drift stay in device memory, the neighbour list is
rebuilt on the device when an atom has moved more than skin/2 (the
FastNeighborList / ASE update policy), and the host only launches captured
steps, reads a flag word per chunk and serves observers.  ASE itself is not
needed.

With a ChargeRelaxation attached to the calculator, every force call of the
reference relaxes the charges first (Pysic.get_forces ->
ChargeRelaxation.charge_relaxation).  The steps then alternate host-side kicks
and drifts (the same update, operation for operation) with the calculator's
device relaxation loop and force evaluation.
"""
import math

import numpy as np

from .error import MissingAtomsError


class VelocityVerlet:
    def __init__(self, atoms, timestep, precision=None):
        self.atoms = atoms
        self.dt = float(timestep)
        self.precision = precision
        self.nsteps = 0
        self.observers = []

    def get_time(self):
        return self.nsteps * self.dt

    def attach(self, function, interval=1, *args, **kwargs):
        """Call function(*args, **kwargs) after every `interval` steps (and
        before the first step), as ASE's Dynamics.attach does."""
        if not hasattr(function, "__call__"):
            function = function.write
        self.observers.append((function, int(interval), args, kwargs))

    def call_observers(self):
        for function, interval, args, kwargs in self.observers:
            if interval > 0 and self.nsteps % interval == 0:
                function(*args, **kwargs)

    def _stride(self):
        g = 0
        for _, interval, _, _ in self.observers:
            if interval > 0:
                g = math.gcd(g, interval)
        return g or None

    def _sync_atoms(self, calc, eng):
        """The device state into the atoms and the calculator's copy of them."""
        p, r = eng.md_get_state()
        self.atoms.set_positions(r)
        self.atoms.set_momenta(p)
        s = calc.get_atoms()
        s.set_positions(r)
        s.set_momenta(p)
        pushed = getattr(calc, "_pushed", None)
        if pushed is not None:
            pushed["positions"] = np.array(r)
        calc._invalidate()
        return r

    def _run_relaxing(self, steps):
        """ASE's update around the calculator's relaxation and forces."""
        atoms = self.atoms
        if self.nsteps == 0:
            self.call_observers()
        forces = atoms.get_forces()
        for _ in range(int(steps)):
            p = atoms.get_momenta()
            p += 0.5 * self.dt * forces
            masses = atoms.get_masses()[:, np.newaxis]
            r = atoms.get_positions()
            atoms.set_positions(r + self.dt * p / masses)
            atoms.set_momenta(p)
            forces = atoms.get_forces()
            atoms.set_momenta(atoms.get_momenta() + 0.5 * self.dt * forces)
            self.nsteps += 1
            self.call_observers()
        return True

    def run(self, steps=50):
        calc = self.atoms.get_calculator()
        if calc is None:
            raise MissingAtomsError("the atoms have no Pysic calculator")
        if calc.get_charge_relaxation() is not None:
            return self._run_relaxing(steps)
        calc.set_atoms(self.atoms)
        calc.set_core()  # engine, tables and lists up to date for these atoms
        eng = calc.engine
        nl = calc.get_neighbor_lists()
        prec = calc._prec() if self.precision is None else self.precision
        eng.md_set_state(self.atoms.get_masses(), self.atoms.get_momenta())
        if self.nsteps == 0:
            self.call_observers()
        stride = self._stride()
        left = int(steps)
        rebuilt = False
        while left > 0:
            k = left if stride is None else min(left, stride - self.nsteps % stride)
            # k steps, the lists rebuilt on the device whenever an atom has moved
            # more than skin/2 (pg_md_run)
            done, rebuilds = eng.md_run(prec, k, self.dt, nl.skin)
            left -= done
            self.nsteps += done
            if rebuilds:
                nl.positions = eng.list_positions()
                nl.nupdates += rebuilds
                rebuilt = True
            if stride is not None:
                self._sync_atoms(calc, eng)
                self.call_observers()
        self._sync_atoms(calc, eng)
        if rebuilt:
            nl.refresh_from(eng)
        return True
