"""Direct and reciprocal grids (mirror of ``dftpy/grid.py``).

``DirectGrid(lattice, nr, full=True)`` keeps the reference's conventions:
rows of ``lattice`` are the lattice vectors (Bohr), ``dV = |det L| / N``,
the reciprocal lattice is ``2 pi inv(L)^T`` (``grid.py:384-415``), and
``full`` selects between the full complex spectrum (the reference default)
and the half spectrum ``(n0, n1, n2//2+1)``.  Each grid owns one GPU plan per
precision (FFT schedule, twiddle tables, workspaces).
"""
import math

import os
import weakref

import numpy as np

from . import _lib


def _lattice_array(lattice):
    if hasattr(lattice, "array"):
        lattice = lattice.array
    elif hasattr(lattice, "lattice") and not isinstance(lattice, np.ndarray):
        lattice = lattice.lattice
    a = np.array(lattice, dtype=float)
    if a.shape == (3,):
        a = np.diag(a)
    return a.reshape(3, 3)


def spacing2ecut(spacing):
    """``math_utils.spacing2ecut`` (``math_utils.py:331-336``): pi^2 / (2 h^2)."""
    return np.pi ** 2 / (2 * spacing ** 2)


def ecut2spacing(ecut):
    return np.sqrt(np.pi ** 2 / ecut * 0.5)


def best_fft_size(n, max_prime=7):
    """Smallest even ``2^a 3^b 5^c 7^d >= 0.99 n`` (``mpi/mp_serial.py:17-80`` with
    its defaults: primes 2,3,5,7, even sizes, scale 0.99)."""
    target = int(math.ceil(0.99 * n)) - 1
    m = max(2, target + 1)
    while True:
        if m % 2 == 0:
            k = m
            for p in (2, 3, 5, 7):
                if p > max_prime:
                    break
                while k % p == 0:
                    k //= p
            if k == 1:
                return m
        m += 1


def ecut2nr(ecut=None, lattice=None, optfft=True, spacing=None, **kwargs):
    """Grid points per axis for a cutoff or spacing (``math_utils.py:349-365``)."""
    lat = _lattice_array(lattice)
    sp = np.ones(3) * (ecut2spacing(ecut) if spacing is None else spacing)
    nr = np.zeros(3, dtype=np.int32)
    for i in range(3):
        nr[i] = int(np.sqrt(np.dot(lat[i], lat[i])) / sp[i])
        nr[i] += nr[i] % 2
        if optfft:
            nr[i] = best_fft_size(nr[i])
    return nr


class _Cell:
    def __init__(self, array):
        self.array = np.array(array, dtype=float)

    @property
    def volume(self):
        return abs(float(np.linalg.det(self.array)))

    def lengths(self):
        return np.sqrt((self.array ** 2).sum(axis=1))

    def __array__(self, dtype=None, copy=None):
        return self.array if dtype is None else self.array.astype(dtype)

    def __getitem__(self, i):
        return self.array[i]


class BaseGrid:
    def __init__(self, lattice, nr, full=True, direct=True):
        self._cell = _Cell(_lattice_array(lattice))
        self._nrR = np.array(nr, dtype=np.int32).reshape(3)
        if np.any(self._nrR < 1):
            raise ValueError("grid sizes must be positive, got %s" % (self._nrR,))
        self._nnrR = int(np.prod(self._nrR))
        self._full = bool(full)
        self._direct = direct
        self._nrG = self._nrR.copy()
        if not self._full:
            self._nrG[-1] = self._nrG[-1] // 2 + 1
        self._dV = abs(self._cell.volume) / self._nnrR

    @property
    def cell(self):
        return self._cell

    @property
    def lattice(self):
        return self._cell.array

    @property
    def nrR(self):
        return self._nrR

    @property
    def nnrR(self):
        return self._nnrR

    @property
    def nrG(self):
        return self._nrG

    @property
    def nnrG(self):
        return int(np.prod(self._nrG))

    @property
    def full(self):
        return self._full

    @property
    def volume(self):
        return self._cell.volume

    @property
    def dV(self):
        return self._dV

    def __eq__(self, other):
        return (isinstance(other, BaseGrid) and np.allclose(self.lattice, other.lattice)
                and np.array_equal(self.nrR, other.nrR))

    def __hash__(self):
        return id(self)


class DirectGrid(BaseGrid):
    """Real-space grid; ``nr`` from ``ecut``/``spacing`` when not given."""

    def __init__(self, lattice, nr=None, origin=np.zeros(3), full=True, ecut=None, spacing=None, **kwargs):
        if nr is None:
            nr = ecut2nr(ecut=ecut, lattice=lattice, spacing=spacing)
        super().__init__(lattice, nr, full=full, direct=True)
        self.origin = np.asarray(origin, dtype=float)
        self._reciprocal = None
        self._plans = {}

    @property
    def nr(self):
        return self._nrR

    @property
    def nnr(self):
        return self._nnrR

    @property
    def spacings(self):
        return self._cell.lengths() / self._nrR

    def plan(self, dtype):
        """GPU plan for ``torch.float64`` / ``torch.float32`` fields."""
        import torch
        prec = _lib.F64 if dtype == torch.float64 else _lib.F32
        if prec not in self._plans:
            plan = _lib.Plan(self._nrR, self.lattice, precision=prec, full=self._full)
            if prec == _lib.F32 and os.environ.get("GBOFDFT_AUTOTUNE", "1") != "0":
                from . import autotune
                autotune.tune(plan)
            self._plans[prec] = plan
        return self._plans[prec]

    def delta_state(self):
        """Delta-evaluation state of this grid's FP64 and FP32 plans (the FP64
        evaluations of the mixed-precision refinement), or None when the grid
        has no FP32 plane-pipeline specialisation."""
        import torch
        if "delta" not in self._plans:
            try:
                self._plans["delta"] = _lib.Delta(self.plan(torch.float64), self.plan(torch.float32))
            except ValueError:            # no plane-pipeline specialisation
                self._plans["delta"] = None
        return self._plans["delta"]

    def get_reciprocal(self):
        """The reciprocal grid (cached weakly: it refers to this grid, and a
        strong reference both ways would keep the pair -- with its plans and
        device workspaces -- alive until Python's cycle collector runs)."""
        r = self._reciprocal() if self._reciprocal is not None else None
        if r is None:
            r = ReciprocalGrid(self)
            self._reciprocal = weakref.ref(r)
        return r

    def guess_ecut(self):
        """``DirectGrid.guess_ecut`` (``grid.py:477-480``)."""
        sp2 = self._cell.lengths() / (self._nrR - 1)
        return spacing2ecut((0.5 * (self.spacings + sp2)).max())

    @property
    def ecut(self):
        return self.guess_ecut()


class ReciprocalGrid(BaseGrid):
    """Reciprocal grid of a ``DirectGrid``; G-vector arrays live on the GPU."""

    def __init__(self, direct):
        bg = (2.0 * np.pi * np.linalg.inv(direct.lattice)).T
        super().__init__(bg, direct.nrR, full=direct.full, direct=False)
        self._dgrid = direct
        self._dV = direct.dV
        self._g = None

    @property
    def nr(self):
        return self._nrG

    def get_direct(self):
        return self._dgrid

    def _freqs(self):
        import torch
        n = self._nrR
        ax = [torch.fft.fftfreq(int(n[0]), d=1.0 / int(n[0]), dtype=torch.float64, device="cuda"),
              torch.fft.fftfreq(int(n[1]), d=1.0 / int(n[1]), dtype=torch.float64, device="cuda")]
        if self._full:
            ax.append(torch.fft.fftfreq(int(n[2]), d=1.0 / int(n[2]), dtype=torch.float64, device="cuda"))
        else:
            ax.append(torch.arange(int(n[2]) // 2 + 1, dtype=torch.float64, device="cuda"))
        return ax

    @property
    def g(self):
        """Cartesian G vectors ``[3, *nr]`` (``grid.py:584-620``)."""
        if self._g is None:
            import torch
            f = self._freqs()
            S = torch.stack(torch.meshgrid(*f, indexing="ij"))
            bg = torch.tensor(self.lattice, dtype=torch.float64, device="cuda")
            self._g = torch.einsum("j...,jk->k...", S, bg)
        return self._g

    @property
    def gg(self):
        return (self.g * self.g).sum(0)

    @property
    def q(self):
        return self.gg.sqrt()

    @property
    def invgg(self):
        gg = self.gg
        gg[0, 0, 0] = 1.0
        inv = 1.0 / gg
        inv[0, 0, 0] = 0.0
        return inv
