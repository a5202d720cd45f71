"""Minimal unit cell (rows are lattice vectors), for importing the reference.

Golden-fixture shim only.  The reference uses ``ase.cell.Cell`` as a 3x3
matrix holder (``dftpy/grid.py:4,31-33``): ``.array``, ``.volume``,
``.lengths()``, indexing and ``numpy`` conversion.
"""
import numpy as np


class Cell:
    def __init__(self, array):
        if isinstance(array, Cell):
            array = array.array
        a = np.asarray(array, dtype=float)
        if a.shape == (3,):
            a = np.diag(a)
        self.array = np.array(a, dtype=float).reshape(3, 3)

    @classmethod
    def new(cls, cell=None):
        return cls(np.zeros((3, 3)) if cell is None else cell)

    @property
    def volume(self):
        return abs(float(np.linalg.det(self.array)))

    def lengths(self):
        return np.sqrt((self.array ** 2).sum(axis=1))

    def reciprocal(self):
        return np.linalg.inv(self.array).T

    @property
    def T(self):
        return self.array.T

    @property
    def shape(self):
        return self.array.shape

    def __array__(self, dtype=None, copy=None):
        return self.array if dtype is None else self.array.astype(dtype)

    def __getitem__(self, i):
        return self.array[i]

    def __setitem__(self, i, v):
        self.array[i] = v

    def __len__(self):
        return 3

    def __iter__(self):
        return iter(self.array)

    def __eq__(self, other):
        return np.allclose(self.array, np.asarray(other))

    def __mul__(self, x):
        return self.array * x

    __rmul__ = __mul__

    def __truediv__(self, x):
        return self.array / x

    def copy(self):
        return Cell(self.array.copy())

    def scaled_positions(self, positions):
        return np.linalg.solve(self.array.T, np.asarray(positions, float).T).T

    def cartesian_positions(self, scaled_positions):
        return np.asarray(scaled_positions, float) @ self.array
