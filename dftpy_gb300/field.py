"""Fields on a grid (mirror of ``dftpy/field.py``), backed by CUDA tensors.

``DirectField`` / ``ReciprocalField`` are ``torch.Tensor`` subclasses that
carry their ``grid``, the way the reference's fields are ndarray subclasses.
Elementwise algebra is ordinary tensor arithmetic on the device; the
transforms go through the gbofdft C ABI:

* ``DirectField.fft()`` multiplies by dV (``field.py:373-390``);
* ``ReciprocalField.ifft()`` divides by dV and returns the real part
  (``field.py:739-764``).

Full grids (``DirectGrid(full=True)``, the reference default) expose the full
complex spectrum; the transform itself always runs as R2C/C2R on the half
spectrum (the real part of a full inverse transform equals the C2R of the
Hermitian-averaged half spectrum).
"""
import numpy as np
import torch

from . import _lib, torch_ops
from .grid import DirectGrid, ReciprocalGrid


def _find_grid(objs):
    for o in objs:
        if isinstance(o, BaseField):
            g = getattr(o, "grid", None)
            if g is not None:
                return g, type(o)
        elif isinstance(o, (list, tuple)):
            r = _find_grid(o)
            if r[0] is not None:
                return r
    return None, None


class BaseField(torch.Tensor):
    """Tensor with a ``grid`` attribute that survives tensor operations."""

    @classmethod
    def __torch_function__(cls, func, types, args=(), kwargs=None):
        kwargs = kwargs or {}
        ret = super().__torch_function__(func, types, args, kwargs)
        grid, _ = _find_grid(list(args) + list(kwargs.values()))
        _attach(ret, grid)
        return ret

    # ---- numpy-like conveniences of the reference fields -------------------
    def copy(self):
        return self.clone()

    def to_numpy(self):
        return self.detach().cpu().numpy()

    def asum(self):
        return float(self.sum())

    def amean(self):
        return float(self.mean())

    def amax(self):
        return float(self.max())

    def amin(self):
        return float(self.min())

    @property
    def rank(self):
        return self.shape[0] if self.dim() == 4 else 1

    @property
    def memo(self):
        return getattr(self, "_memo", "")


def _attach(ret, grid):
    if grid is None:
        return
    if isinstance(ret, BaseField):
        if getattr(ret, "grid", None) is None:
            ret.grid = grid
    elif isinstance(ret, (list, tuple)):
        for r in ret:
            _attach(r, grid)


def _as_tensor(data, shape, dtype, cplx):
    if data is None:
        return torch.zeros(tuple(int(x) for x in shape), dtype=dtype, device="cuda")
    if isinstance(data, torch.Tensor):
        t = data.to(device="cuda", dtype=dtype)
    else:
        t = torch.as_tensor(np.ascontiguousarray(np.asarray(data)), device="cuda").to(dtype)
    shape = tuple(int(x) for x in shape)
    if t.numel() != int(np.prod(shape)):
        # a buffer of the wrong size never reaches the library
        raise ValueError("field data has %d values, the grid needs %s = %d" % (t.numel(), shape, int(np.prod(shape))))
    return t.reshape(shape).contiguous()


class DirectField(BaseField):
    """Real field on a ``DirectGrid``; default dtype float64."""

    @staticmethod
    def __new__(cls, grid, memo="", rank=1, data=None, dtype=None, cplx=False, griddata_3d=None,
                griddata_C=None, griddata_F=None, order="C", **kwargs):
        if hasattr(grid, "get_direct") and not isinstance(grid, DirectGrid):
            grid = grid.get_direct()
        if not isinstance(grid, DirectGrid):
            raise TypeError("the grid argument is not an instance of DirectGrid")
        if data is None:
            data = griddata_3d if griddata_3d is not None else griddata_C
        if data is None and griddata_F is not None:
            data = np.reshape(np.asarray(griddata_F), tuple(grid.nrR) if rank == 1 else (rank, *grid.nrR),
                              order="F")
        if dtype is None:
            dtype = data.dtype if isinstance(data, torch.Tensor) and data.dtype in (torch.float32, torch.float64) \
                else torch.float64
        if cplx:
            raise NotImplementedError("complex direct-space fields are not part of this path")
        shape = tuple(grid.nrR) if rank == 1 else (rank, *grid.nrR)
        t = _as_tensor(data, shape, dtype, False)
        obj = t.as_subclass(cls)
        obj.grid = grid
        obj._memo = memo
        return obj

    @property
    def N(self):
        return self.integral()

    def integral(self):
        """``DirectField.integral`` (``field.py:186-192``)."""
        if self.rank == 1:
            return float(self.as_subclass(torch.Tensor).to(torch.float64).sum()) * self.grid.dV
        return (self.as_subclass(torch.Tensor).to(torch.float64).sum(dim=(1, 2, 3)) * self.grid.dV).cpu().numpy()

    def fft(self):
        """Forward transform times dV (``field.py:373-390``)."""
        g = self.grid
        if self.rank != 1:
            raise NotImplementedError("fft of rank>1 fields")
        plan = g.plan(self.dtype)
        x = self.as_subclass(torch.Tensor).contiguous()
        out = torch.ops.gbofdft.fft_r2c(x, torch_ops.handle(plan))
        if g.full:
            out = _hermitian_extend(out, int(g.nrR[2]))
        return ReciprocalField(g.get_reciprocal(), data=out)


def _partner(X):
    """X[(-i0) % n0, (-i1) % n1, (-i2) % n2] of a full spectrum."""
    return torch.roll(torch.flip(X, dims=(0, 1, 2)), shifts=(1, 1, 1), dims=(0, 1, 2))


def _hermitian_extend(half, n2):
    n0, n1, h = half.shape
    full = torch.empty((n0, n1, n2), dtype=half.dtype, device=half.device)
    full[:, :, :h] = half
    if n2 > h:
        # X(-k) = conj(X(k)): index k2 in [h, n2) mirrors n2 - k2 in (0, n2 - h]
        src = half[:, :, 1:n2 - h + 1]
        mirrored = torch.roll(torch.flip(src, dims=(0, 1)), shifts=(1, 1), dims=(0, 1)).conj()
        full[:, :, h:] = torch.flip(mirrored, dims=(2,))
    return full


class ReciprocalField(BaseField):
    """Complex field on a ``ReciprocalGrid`` (half or full spectrum)."""

    @staticmethod
    def __new__(cls, grid, memo="", rank=1, data=None, dtype=None, griddata_3d=None, **kwargs):
        if hasattr(grid, "get_reciprocal") and not isinstance(grid, ReciprocalGrid):
            grid = grid.get_reciprocal()
        if not isinstance(grid, ReciprocalGrid):
            raise TypeError("the grid argument is not an instance of ReciprocalGrid")
        if data is None:
            data = griddata_3d
        if dtype is None:
            dtype = data.dtype if isinstance(data, torch.Tensor) and data.is_complex() else torch.complex128
        t = _as_tensor(data, tuple(grid.nrG), dtype, True)
        obj = t.as_subclass(cls)
        obj.grid = grid
        obj._memo = memo
        return obj

    def integral(self):
        """``ReciprocalField.integral`` (``field.py:727-731``)."""
        s = complex(self.as_subclass(torch.Tensor).sum())
        return s * self.grid.dV * self.grid.nnrG / (2.0 * np.pi) ** 3

    def ifft(self, check_real=False, force_real=True):
        """Inverse transform divided by dV; real part (``field.py:739-764``)."""
        rg = self.grid
        dg = rg.get_direct()
        X = self.as_subclass(torch.Tensor)
        n2 = int(dg.nrR[2])
        if rg.full:
            X = 0.5 * (X + _partner(X).conj())
            X = X[:, :, : n2 // 2 + 1]
        X = X.contiguous()
        rdt = torch.float64 if X.dtype == torch.complex128 else torch.float32
        plan = dg.plan(rdt)
        out = torch.ops.gbofdft.fft_c2r(X, torch_ops.handle(plan), n2)
        return DirectField(dg, data=out)
