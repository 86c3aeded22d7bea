"""A minimal stand-in for ``ase.Atoms``.

The reference calculator is an ASE calculator (pysic/calculator.py:192-1832)
and only uses a small part of the ``Atoms`` interface: positions, cell,
periodicity, chemical symbols, tags, charges, momenta, masses, volume,
reciprocal cell, copying and comparison.  The GB300 calculator duck-types on
those methods, so a real ``ase.Atoms`` works as well; this class exists so
that the package runs where ASE is not installed.  Defaults follow ASE 3.6/3.7
(the versions the reference targets, pysic/calculator.py:566): a unit cubic
cell and no periodicity.
"""
import re

import numpy as np

# atomic masses (u) of the elements the examples and benchmarks use
_MASSES = {
    "X": 1.0, "H": 1.008, "He": 4.0026, "Li": 6.94, "C": 12.011, "N": 14.007, "O": 15.999, "F": 18.998,
    "Ne": 20.180, "Na": 22.990, "Mg": 24.305, "Al": 26.982, "Si": 28.085, "P": 30.974, "S": 32.06,
    "Cl": 35.45, "Ar": 39.948, "K": 39.098, "Ca": 40.078, "Ti": 47.867, "Fe": 55.845, "Cu": 63.546,
    "Zn": 65.38, "Ge": 72.630, "Ag": 107.87, "Au": 196.97, "Hf": 178.49, "Zr": 91.224,
}


def _parse_symbols(symbols):
    if symbols is None:
        return []
    if isinstance(symbols, str):
        out = []
        for sym, cnt in re.findall(r"([A-Z][a-z]?)(\d*)", symbols):
            out.extend([sym] * (int(cnt) if cnt else 1))
        return out
    return [str(s) for s in symbols]


class _AtomView:
    """``atoms[i]`` proxy with writable x, y, z (used by finite differences,
    pysic/calculator.py:1639-1677)."""

    def __init__(self, atoms, index):
        self._a = atoms
        self._i = index

    def _get(self, c):
        return float(self._a._positions[self._i, c])

    def _set(self, c, v):
        self._a._positions[self._i, c] = v

    x = property(lambda s: s._get(0), lambda s, v: s._set(0, v))
    y = property(lambda s: s._get(1), lambda s, v: s._set(1, v))
    z = property(lambda s: s._get(2), lambda s, v: s._set(2, v))

    @property
    def position(self):
        return self._a._positions[self._i].copy()

    @property
    def symbol(self):
        return self._a._symbols[self._i]


class Atoms:
    def __init__(self, symbols=None, positions=None, cell=None, pbc=False, charges=None, tags=None,
                 momenta=None, masses=None):
        self._symbols = _parse_symbols(symbols)
        n = len(self._symbols)
        if positions is None:
            positions = np.zeros((n, 3))
        self._positions = np.array(positions, dtype=np.float64).reshape(n, 3)
        if cell is None:
            cell = np.eye(3)
        cell = np.array(cell, dtype=np.float64)
        if cell.shape == (3,):
            cell = np.diag(cell)
        self._cell = cell.reshape(3, 3)
        if np.isscalar(pbc) or np.ndim(pbc) == 0:
            pbc = [bool(pbc)] * 3
        self._pbc = np.array(pbc, dtype=bool)
        self._charges = np.zeros(n) if charges is None else np.array(charges, dtype=np.float64).reshape(n)
        self._tags = np.zeros(n, dtype=int) if tags is None else np.array(tags, dtype=int).reshape(n)
        self._momenta = np.zeros((n, 3)) if momenta is None else np.array(momenta, dtype=np.float64).reshape(n, 3)
        if masses is None:
            masses = [_MASSES.get(s, 1.0) for s in self._symbols]
        self._masses = np.array(masses, dtype=np.float64).reshape(n)
        self.calc = None

    # --- ASE interface subset -------------------------------------------
    def __len__(self):
        return len(self._symbols)

    def get_number_of_atoms(self):
        return len(self._symbols)

    def get_positions(self):
        return self._positions.copy()

    def set_positions(self, positions):
        self._positions = np.array(positions, dtype=np.float64).reshape(len(self), 3)

    @property
    def positions(self):
        return self._positions

    @positions.setter
    def positions(self, value):
        self.set_positions(value)

    def get_cell(self):
        return self._cell.copy()

    def set_cell(self, cell, scale_atoms=False):
        cell = np.array(cell, dtype=np.float64)
        if cell.shape == (3,):
            cell = np.diag(cell)
        if scale_atoms:
            frac = np.linalg.solve(self._cell.T, self._positions.T).T
            self._positions = frac @ cell
        self._cell = cell

    @property
    def cell(self):
        return self._cell

    def get_pbc(self):
        return self._pbc.copy()

    def set_pbc(self, pbc):
        if np.isscalar(pbc):
            pbc = [bool(pbc)] * 3
        self._pbc = np.array(pbc, dtype=bool)

    @property
    def pbc(self):
        return self._pbc

    def get_chemical_symbols(self):
        return list(self._symbols)

    def get_atomic_numbers(self):
        order = list(_MASSES.keys())
        return np.array([order.index(s) if s in order else 0 for s in self._symbols])

    def get_tags(self):
        return self._tags.copy()

    def set_tags(self, tags):
        self._tags = np.array(tags, dtype=int).reshape(len(self))

    def get_initial_charges(self):
        return self._charges.copy()

    def set_initial_charges(self, charges):
        self._charges = np.array(charges, dtype=np.float64).reshape(len(self))

    get_charges = get_initial_charges
    set_charges = set_initial_charges

    def get_momenta(self):
        return self._momenta.copy()

    def set_momenta(self, momenta):
        self._momenta = np.array(momenta, dtype=np.float64).reshape(len(self), 3)

    def get_masses(self):
        return self._masses.copy()

    def get_volume(self):
        return abs(float(np.linalg.det(self._cell)))

    def get_reciprocal_cell(self):
        """Reciprocal cell without the factor 2 pi, as ASE defines it."""
        return np.linalg.inv(self._cell).T

    def copy(self):
        a = Atoms(self._symbols, self._positions, self._cell, self._pbc, self._charges, self._tags,
                  self._momenta, self._masses)
        return a

    def __getitem__(self, index):
        return _AtomView(self, index)

    def set_calculator(self, calc):
        self.calc = calc

    def get_calculator(self):
        return self.calc

    def get_potential_energy(self):
        return self.calc.get_potential_energy(self)

    def get_forces(self):
        return self.calc.get_forces(self)

    def get_stress(self):
        return self.calc.get_stress(self)

    def __eq__(self, other):
        try:
            return (len(self) == len(other) and self.get_chemical_symbols() == other.get_chemical_symbols()
                    and np.array_equal(self.get_positions(), other.get_positions())
                    and np.array_equal(self.get_cell(), other.get_cell())
                    and np.array_equal(self.get_pbc(), other.get_pbc()))
        except Exception:
            return False

    def __ne__(self, other):
        return not self.__eq__(other)

    def __repr__(self):
        return "Atoms(n={0}, pbc={1})".format(len(self), self._pbc.tolist())
