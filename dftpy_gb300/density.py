"""Initial densities (``density/density.py``).

``DensityGenerator.guess_rho`` gives the uniform electron gas when it holds no
atomic tables (``guess_rho_heg``, ``:199-208``) and otherwise superposes
per-species atomic densities given in reciprocal space
(``get_3d_value_recipe``, ``:252-300``): rho(G) = sum_s rho_s(|G|) S_s(G) with
the PME or the exact structure factor, transformed to real space, clamped at
``dtol`` and scaled to the electron count.  The grid-sized work runs on the
GPU (``gbofdft_density_guess``); the host fits the 1-D splines.
"""
import numpy as np
import torch

from . import _lib
from ._tables import pme_bm, spline_notaknot
from .field import DirectField, ReciprocalField
from .ions import Ions


class _RadialTable:
    """Device copy of one species' rho_s(|G|) as ``RadialGrid.to_3d_grid``
    evaluates it (``grid.py:766-779``): the interpolating cubic spline of the
    whole table, 0 outside [q[0], q[-1])."""

    def __init__(self, q, v):
        q = np.asarray(q, dtype=float)
        v = np.asarray(v, dtype=float)
        if q.ndim != 1 or q.size < 4 or q.shape != v.shape or np.any(np.diff(q) <= 0):
            raise ValueError("a radial table needs >= 4 increasing |G| points and as many values")
        x, c = spline_notaknot(q, v)
        self.x = torch.tensor(x, dtype=torch.float64, device="cuda")
        self.c = torch.tensor(c.reshape(-1), dtype=torch.float64, device="cuda")
        self.m = int(x.size)
        self.gmin = float(q[0])
        self.gmax = float(q[-1])

    def ctypes(self):
        t = _lib.VTable()
        t.x = self.x.data_ptr()
        t.c = self.c.data_ptr()
        t.m = self.m
        for i in range(5):
            t.q4[i] = 0.0
        t.dp, t.gmin, t.gmax = 1.0, self.gmin, self.gmax
        return t


_TABLES = {}
_SMALL = {}


def _publish(obj):
    """A device object about to be shared between threads and streams: wait
    for the copies that made it on the creating stream, so a solve on another
    stream never reads it half-written."""
    torch.cuda.current_stream().synchronize()
    return obj


def _cached(key, make):
    """Small structure-independent device arrays (PME moduli of a grid,
    species indices of a symbol list), kept by key."""
    v = _SMALL.get(key)
    if v is None:
        if len(_SMALL) >= 256:
            _SMALL.clear()
        v = _SMALL[key] = _publish(make())
    return v


def _radial_table(q, v):
    """_RadialTable of (q, v), cached by content (the spline fit is host work;
    tables are per species, not per structure)."""
    q = np.ascontiguousarray(q, dtype=float)
    v = np.ascontiguousarray(v, dtype=float)
    key = (q.shape, v.shape, hash(q.tobytes()), hash(v.tobytes()))
    t = _TABLES.get(key)
    if t is None:
        if len(_TABLES) >= 64:
            _TABLES.clear()
        t = _TABLES[key] = _publish(_RadialTable(q, v))
    return t


def get_3d_value_recipe(r, arho, ions, grid, ncharge=None, rho=None, dtol=0.0, direct=True, pme=True, order=10,
                        **kwargs):
    """Superposed atomic values from reciprocal-space tables ``r[key]`` (|G|)
    and ``arho[key]`` (``density/density.py:252-300``).  ``direct=True``
    returns the real-space field clamped at ``dtol`` and scaled to ``ncharge``
    (default: the ions' valence charge); ``direct=False`` the reciprocal field."""
    if hasattr(grid, "get_direct"):
        grid = grid.get_direct()
    ions = Ions.from_any(ions)
    keys = sorted(k for k in r if arho.get(k) is not None)
    if not keys:
        raise ValueError("no atomic tables to superpose")
    missing = set(ions.symbols) - set(keys)
    if missing:
        raise ValueError("no atomic table for %s" % sorted(missing))
    dtype = rho.dtype if rho is not None else torch.float64
    plan = grid.plan(dtype)
    tables = [_radial_table(r[k], arho[k]) for k in keys]
    tabs = (_lib.VTable * len(keys))(*[t.ctypes() for t in tables])
    # positions and species indices: copies on this stream; the PME moduli of
    # the grid shape and the radial tables are cached and shared by every
    # stream, so this stream is recorded on them: should a cache drop one,
    # its memory is not reused before this stream's kernels have read it
    spos = torch.from_numpy(np.ascontiguousarray(ions.get_scaled_positions(), dtype=np.float64)).to("cuda")
    species = torch.tensor([keys.index(s) for s in ions.symbols], dtype=torch.int32, device="cuda")
    bm = _cached(("bm", tuple(int(x) for x in grid.nrR), int(order)),
                 lambda: torch.tensor(pme_bm(grid.nrR, order).view(np.float64), device="cuda")) if pme else None
    cur = torch.cuda.current_stream()
    for t in tables:
        t.x.record_stream(cur)
        t.c.record_stream(cur)
    if bm is not None:
        bm.record_stream(cur)
    nb = _lib.setup_workspace_bytes(plan, ions.nat)
    work = torch.empty(nb // 8 + 64, dtype=torch.float64, device="cuda")
    n0, n1, n2 = (int(x) for x in grid.nrR)
    cdt = torch.complex128 if dtype == torch.float64 else torch.complex64
    rg = torch.empty((n0, n1, n2 // 2 + 1), dtype=cdt, device="cuda")
    out = rho if rho is not None else DirectField(grid, dtype=dtype)
    if direct:
        if ncharge is None:
            ncharge = ions.get_ncharges()
        _lib.check(_lib.load().gbofdft_density_guess(
            plan.handle, len(keys), tabs, ions.nat, _lib.ptr(spos), _lib.ptr(species), int(bool(pme)), int(order),
            _lib.ptr(bm) if bm is not None else None, _lib.aligned_ptr(work, 256), nb, _lib.ptr(rg), _lib.ptr(out),
            float(dtol), float(ncharge), _lib.stream_ptr()), "density_guess")
        return out
    _lib.check(_lib.load().gbofdft_vloc(
        plan.handle, len(keys), tabs, ions.nat, _lib.ptr(spos), _lib.ptr(species), int(bool(pme)), int(order),
        _lib.ptr(bm) if bm is not None else None, _lib.aligned_ptr(work, 256), nb, _lib.ptr(rg), None,
        _lib.stream_ptr()), "density_guess")
    if grid.full:
        from .field import _hermitian_extend
        rg = _hermitian_extend(rg, n2)
    return ReciprocalField(grid.get_reciprocal(), data=rg)


class DensityGenerator:
    """``DensityGenerator`` (``density/density.py:71-250``) for reciprocal-space
    atomic tables: ``r`` / ``arho`` dicts per species, or a ``pseudo`` object
    exposing ``_atomic_density_grid`` / ``_atomic_density`` (``:114-134``)."""

    def __init__(self, files=None, pseudo=None, is_core=False, direct=False, r=None, arho=None, **kwargs):
        if files:
            raise NotImplementedError("atomic density files are not read by this build; pass r / arho tables")
        if direct:
            raise NotImplementedError("the real-space atomic superposition (guess_rho_atom) is not part of this "
                                      "path; use direct=False (the reference's default)")
        self.direct = False
        self.is_core = bool(is_core)
        self._r = dict(r or {})
        self._arho = dict(arho or {})
        if pseudo is not None:
            readpp = getattr(pseudo, "readpp", pseudo)
            gname, vname = (("_core_density_grid", "_core_density") if self.is_core
                            else ("_atomic_density_grid", "_atomic_density"))
            g, v = getattr(readpp, gname, None), getattr(readpp, vname, None)
            if g is not None and v is not None:
                self._r, self._arho = dict(g), dict(v)

    @property
    def r(self):
        return self._r

    @property
    def arho(self):
        return self._arho

    def guess_rho(self, ions, grid=None, ncharge=None, rho=None, dtol=1e-30, nspin=1, **kwargs):
        """``guess_rho`` (``:151-180``); ``nspin`` > 1 stacks equal spin channels."""
        if grid is None:
            if rho is None:
                raise AttributeError("Please give one grid.")
            grid = rho.grid
        if self.is_core and ncharge is None:
            ncharge = 0
        if self.is_core and not any(v is not None for v in self._arho.values()):
            return None
        target = rho if (rho is not None and rho.ndim == 3) else None
        if not self._arho:
            out = self.guess_rho_heg(ions, grid, ncharge, target, dtol=dtol)
        else:
            out = get_3d_value_recipe(self._r, self._arho, ions, grid, ncharge, target, dtol=dtol, **kwargs)
        if self.is_core or nspin == 1:
            if rho is not None and rho.ndim == 4:
                rho[:] = out
                return rho
            return out
        stacked = DirectField(grid, rank=nspin, dtype=out.dtype)
        stacked[:] = out / nspin
        return stacked

    def guess_rho_heg(self, ions, grid, ncharge=None, rho=None, dtol=1e-30, **kwargs):
        """Uniform density ``ncharge / volume`` (``:199-208``)."""
        if ncharge is None:
            ncharge = Ions.from_any(ions).get_ncharges()
        if rho is None:
            rho = DirectField(grid=grid)
        rho[:] = ncharge / grid.volume
        return rho

    def get_3d_value_recipe(self, ions, grid, ncharge=None, rho=None, dtol=1e-30, direct=True, **kwargs):
        return get_3d_value_recipe(self._r, self._arho, ions, grid, ncharge, rho, dtol, direct, **kwargs)
