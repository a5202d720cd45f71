"""Ions in atomic units (mirror of the data side of ``dftpy/ions.py``).

Positions and cell are in Bohr.  ``Ions.from_any`` accepts this class, the
reference's ``Ions`` (an ``ase.Atoms`` subclass) or anything with
``positions``, ``symbols`` and ``cell``.
"""
import numpy as np


class Ions:
    def __init__(self, symbols, positions=None, cell=None, scaled_positions=None, charges=None):
        if hasattr(cell, "array"):
            cell = cell.array
        self.cell = np.array(cell, dtype=float).reshape(3, 3)
        self.symbols = [str(s) for s in symbols]
        if positions is None:
            positions = np.asarray(scaled_positions, float) @ self.cell
        self.positions = np.array(positions, dtype=float).reshape(len(self.symbols), 3)
        self._charges = None if charges is None else np.array(charges, dtype=float)

    @classmethod
    def from_any(cls, ions):
        if isinstance(ions, Ions):
            return ions
        cell = ions.cell.array if hasattr(ions.cell, "array") else ions.cell
        ch = None
        try:
            ch = np.array(ions.charges, dtype=float)
        except Exception:
            ch = None
        return cls(list(ions.symbols), positions=np.array(ions.positions), cell=cell, charges=ch)

    @property
    def nat(self):
        return len(self.symbols)

    def __len__(self):
        return self.nat

    @property
    def symbols_uniq(self):
        return np.sort(np.unique(self.symbols))

    def get_scaled_positions(self):
        """Fractional coordinates wrapped into [0, 1)."""
        s = np.linalg.solve(self.cell.T, self.positions.T).T
        return s % 1.0

    def set_charges(self, charges):
        """``Ions.set_charges`` (``ions.py:94-107``): dict per symbol, scalar or array."""
        if isinstance(charges, dict):
            charges = [charges[s] for s in self.symbols]
        elif np.isscalar(charges):
            charges = np.ones(self.nat) * charges
        self._charges = np.array(charges, dtype=float)

    @property
    def charges(self):
        if self._charges is None:
            raise AttributeError("Please call 'set_charges' before use 'charges'.")
        return self._charges

    def get_ncharges(self):
        return float(self.charges.sum())

    @property
    def zval(self):
        z = {}
        for s, q in zip(self.symbols, self.charges):
            z.setdefault(s, float(q))
        return z
