"""Minimal ``ase`` stand-in, for importing the reference in this container.

Golden-fixture shim only (never imported by the product or the GPU tests).
The reference subclasses ``ase.Atoms`` for its ``Ions`` (``dftpy/ions.py:2``)
and reads ``ase.units`` constants (``dftpy/constants.py:3``).  This module
provides the small part of that surface the OF-DFT path touches: symbols,
Cartesian/scaled positions, the cell, per-atom arrays and initial charges.
"""
import copy as _copy

import numpy as np

from . import units  # noqa: F401
from .cell import Cell

# element symbols indexed by atomic number (0 is a placeholder)
_SYMBOLS = (
    "X H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
    "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb "
    "Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md No Lr Rf "
    "Db Sg Bh Hs Mt Ds Rg Cn Nh Fl Mc Lv Ts Og").split()


class _Symbols(list):
    def __eq__(self, other):
        return list(self) == list(other)


class Atoms:
    def __init__(self, symbols=None, positions=None, numbers=None, tags=None,
                 momenta=None, masses=None, magmoms=None, charges=None,
                 scaled_positions=None, cell=None, pbc=None, celldisp=None,
                 constraint=None, calculator=None, info=None, velocities=None):
        if isinstance(symbols, Atoms):
            other = symbols
            self.cell = other.cell.copy()
            self.arrays = {k: np.array(v, copy=True) for k, v in other.arrays.items()}
            self._symbols = _Symbols(other._symbols)
            self._celldisp = np.array(other._celldisp, dtype=float)
            self.info = dict(other.info)
            return
        self.cell = Cell(np.zeros((3, 3)) if cell is None else cell)
        if isinstance(symbols, str):
            symbols = [symbols]
        if symbols is None and numbers is not None:
            symbols = [_SYMBOLS[int(z)] for z in numbers]
        self._symbols = _Symbols(symbols or [])
        n = len(self._symbols)
        self.arrays = {}
        if positions is not None:
            self.arrays["positions"] = np.array(positions, dtype=float).reshape(n, 3)
        elif scaled_positions is not None:
            self.arrays["positions"] = self.cell.cartesian_positions(
                np.asarray(scaled_positions, float).reshape(n, 3))
        else:
            self.arrays["positions"] = np.zeros((n, 3))
        if charges is not None:
            self.arrays["initial_charges"] = np.array(charges, dtype=float)
        self._celldisp = np.zeros(3) if celldisp is None else np.array(celldisp, float)
        self.info = dict(info or {})

    # --- positions / symbols -------------------------------------------------
    @property
    def positions(self):
        return self.arrays["positions"]

    @positions.setter
    def positions(self, value):
        self.arrays["positions"][:] = value

    def get_positions(self):
        return self.arrays["positions"].copy()

    def set_positions(self, value):
        self.arrays["positions"][:] = value

    @property
    def symbols(self):
        return self._symbols

    @property
    def numbers(self):
        return np.array([_SYMBOLS.index(s) for s in self._symbols], dtype=int)

    def get_chemical_symbols(self):
        return list(self._symbols)

    def get_scaled_positions(self, wrap=True):
        s = self.cell.scaled_positions(self.arrays["positions"])
        if wrap:
            s = s % 1.0
            s[np.isclose(s, 1.0, rtol=0, atol=1e-15)] = 0.0
        return s

    def set_scaled_positions(self, s):
        self.arrays["positions"][:] = self.cell.cartesian_positions(s)

    def get_cell(self):
        return self.cell

    def set_cell(self, cell, scale_atoms=False):
        cell = Cell(cell)
        if scale_atoms:
            s = self.get_scaled_positions(wrap=False)
            self.cell = cell
            self.set_scaled_positions(s)
        else:
            self.cell = cell

    def get_volume(self):
        return self.cell.volume

    # --- per-atom arrays -----------------------------------------------------
    def has(self, name):
        return name in self.arrays

    def set_initial_charges(self, charges=None):
        if charges is None:
            self.arrays.pop("initial_charges", None)
        else:
            self.arrays["initial_charges"] = np.array(charges, dtype=float).reshape(len(self))

    def get_initial_charges(self):
        return self.arrays["initial_charges"].copy()

    def get_global_number_of_atoms(self):
        return len(self)

    def __len__(self):
        return len(self._symbols)

    def copy(self):
        return _copy.deepcopy(self)
