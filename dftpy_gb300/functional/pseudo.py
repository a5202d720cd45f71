"""Local pseudopotential and ion-ion energy (``functional/pseudo/__init__.py``,
``ewald.py``).

All grid-sized work runs on the GPU (``gbofdft_vloc``, ``gbofdft_ewald``);
the host builds the per-species 1-D spline tables, the PME b(m) factors and
the Ewald scalars (eta, cutoff, lattice images, correction term).
"""
import math
import os

import numpy as np
import torch

from .. import _lib
from .._tables import pme_bm, quartic_coefficients, spline_notaknot
from ..field import DirectField, ReciprocalField
from ..ions import Ions
from .output import AbstractFunctional, FunctionalOutput
from ._eval import Spec, evaluate


class AnalyticPP:
    """Analytic local pseudopotential v(G) = -4 pi Z exp(-(G rc)^2 / 4) / G^2 on
    the reference's |G| table layout (a ``BasePseudo`` with ``direct=False``,
    ``functional/pseudo/abstract_pseudo.py:49-111``)."""

    def __init__(self, Z, rc, npts=10000, gmin=1e-4, gmax=30.0):
        from ..systems import analytic_pp_table
        self._zval = float(Z)
        self.rc = float(rc)
        self.r, self.v = analytic_pp_table(Z, rc, npts, gmin, gmax)
        self.info = {}

    @property
    def zval(self):
        return self._zval

    @property
    def radial_grid(self):
        return self.r

    @property
    def local_potential(self):
        return self.v

    @property
    def direct(self):
        return False

    def __call__(self, *args, **kwargs):
        return self


def _read_pp(obj):
    """(gp, vp, zval) of a PP_list entry: a file path (recpot, psp8/psp6,
    UPF v2; ``ReadPseudo._init_pp``, ``pseudo/__init__.py:726-779``) or a
    ``BasePseudo``-like object; real-space tables are transformed to |G|
    (``_real2recip``) on the host."""
    from ..pseudo_files import read_pp, reciprocal_atomic_density, reciprocal_table
    if isinstance(obj, (str, bytes)) or hasattr(obj, "__fspath__"):
        obj = read_pp(os.fsdecode(obj))
    gp, vp, z = reciprocal_table(obj)
    atom = reciprocal_atomic_density(obj) if hasattr(obj, "atomic_density") else None
    return gp, vp, z, atom


class _VTable:
    """Device copy of one species' v(|G|) spline (``calc_vlines``, ``:350-375``)."""

    def __init__(self, gp, vp):
        x, c = spline_notaknot(gp[1:], vp[1:])
        self.x = torch.tensor(x, dtype=torch.float64, device="cuda")
        self.c = torch.tensor(c.reshape(-1), dtype=torch.float64, device="cuda")
        self.m = int(x.size)
        self.q4 = quartic_coefficients(vp)
        self.dp = float(gp[1] - gp[0])
        self.gmin = float(gp[1])
        self.gmax = float(gp[-1])

    def ctypes(self):
        t = _lib.VTable()
        t.x = self.x.data_ptr()
        t.c = self.c.data_ptr()
        t.m = self.m
        for i in range(5):
            t.q4[i] = self.q4[i]
        t.dp, t.gmin, t.gmax = self.dp, self.gmin, self.gmax
        return t


class LocalPseudo(AbstractFunctional):
    """E = int v_loc rho, V = v_loc (``LocalPseudo.compute``, ``:219-234``)."""

    def __init__(self, grid=None, ions=None, PP_list=None, PME=True, BsplineOrder=10, **kwargs):
        self.type = "PSEUDO"
        self.name = "PSEUDO"
        if PP_list is None:
            raise AttributeError("Must specify PP_list for Pseudopotentials")
        if grid is None:
            raise AttributeError("Must specify grid for Pseudopotentials")
        self.PME = bool(PME)
        self.BsplineOrder = int(BsplineOrder)
        self.grid = grid
        self.PP_list = dict(PP_list)
        self._pp = {k: _read_pp(v) for k, v in self.PP_list.items()}
        self.zval = {k: v[2] for k, v in self._pp.items()}
        # reciprocal-space atomic densities of the species whose files have
        # one (read by DensityGenerator(pseudo=...), density.py:114-134)
        self._atomic_density_grid = {k: v[3][0] for k, v in self._pp.items() if v[3] is not None}
        self._atomic_density = {k: v[3][1] for k, v in self._pp.items() if v[3] is not None}
        self.ions = Ions.from_any(ions)
        for key in self.ions.symbols_uniq:
            if key not in self._pp:
                raise ValueError("There is no pseudopotential for {:4s} atom".format(key))
        self.ions.set_charges(self.zval)
        self._vreal = {}
        self._vG = None
        self.ewald = None

    def _device_inputs(self):
        keys = sorted(self._pp)
        spos = torch.tensor(self.ions.get_scaled_positions(), dtype=torch.float64, device="cuda").contiguous()
        species = torch.tensor([keys.index(s) for s in self.ions.symbols], dtype=torch.int32, device="cuda")
        return keys, spos, species

    def restart(self, grid=None, ions=None, full=False, duplicate=False):
        """Drop the cached v_loc, device inputs and Ewald sum and take new ions
        and/or grid (``restart``, ``pseudo/__init__.py:152-175``): the next use
        recomputes them for the new positions."""
        if ions is not None:
            self.ions = Ions.from_any(ions)
            self.ions.set_charges(self.zval)
        if grid is not None:
            self.grid = grid
        self._vreal = {}
        self._vG = None
        self._dev = None
        self.ewald = None

    def _device_setup(self):
        """Device copies of the positions, species, v(|G|) tables and PME b(m)."""
        if getattr(self, "_dev", None) is None:
            keys, spos, species = self._device_inputs()
            self._tables = [_VTable(*self._pp[k][:2]) for k in keys]
            tabs = (_lib.VTable * len(keys))(*[t.ctypes() for t in self._tables])
            bm = None
            if self.PME:
                bm = torch.tensor(pme_bm(self.grid.nrR, self.BsplineOrder).view(np.float64), device="cuda")
            self._dev = (keys, spos, species, tabs, bm)
        return self._dev

    def local_PP(self):
        """v_loc(G) and v_loc(r) in FP64 (``local_PP``, ``:237-246``)."""
        if getattr(self, "_vG", None) is not None:
            return
        g = self.grid
        plan = g.plan(torch.float64)
        keys, spos, species, tabs, bm = self._device_setup()
        nb = _lib.setup_workspace_bytes(plan, self.ions.nat)
        work = torch.empty(nb // 8 + 64, dtype=torch.float64, device="cuda")
        wptr = _lib.aligned_ptr(work, 256)
        n0, n1, n2 = (int(x) for x in g.nrR)
        vG = torch.empty((n0, n1, n2 // 2 + 1), dtype=torch.complex128, device="cuda")
        vR = torch.empty((n0, n1, n2), dtype=torch.float64, device="cuda")
        _lib.check(_lib.load().gbofdft_vloc(
            plan.handle, len(keys), tabs, self.ions.nat, _lib.ptr(spos), _lib.ptr(species), int(self.PME),
            self.BsplineOrder, _lib.ptr(bm) if bm is not None else None, wptr, nb, _lib.ptr(vG), _lib.ptr(vR),
            _lib.stream_ptr()), "vloc")
        self._vG = vG
        self._vreal[torch.float64] = vR

    def stress(self, rho, energy=None):
        """Local-pseudopotential stress, 3x3 (``stress``, ``:248-258``: ``_StressPME``
        with PME, ``_Stress`` without).  ``energy``: E_PSEUDO at rho (computed
        when not given)."""
        if rho is None:
            raise AttributeError("Must specify rho")
        if not isinstance(rho, DirectField):
            raise TypeError("rho must be DirectField")
        if energy is None:
            energy = self.compute(rho, calcType={"E"}).energy
        keys, spos, species, tabs, bm = self._device_setup()
        plan = self.grid.plan(rho.dtype)
        nat = self.ions.nat
        nb = _lib.stress_workspace_bytes(plan, nat)
        work = torch.empty(nb // 8 + 64, dtype=torch.float64, device="cuda")
        out = torch.empty(9, dtype=torch.float64, device="cuda")
        _lib.check(_lib.load().gbofdft_pp_stress(
            plan.handle, _lib.ptr(rho.as_subclass(torch.Tensor).contiguous()), len(keys), tabs, nat,
            _lib.ptr(spos), _lib.ptr(species), int(self.PME), self.BsplineOrder,
            _lib.ptr(bm) if bm is not None else None, float(energy), _lib.aligned_ptr(work, 256), nb,
            _lib.ptr(out), _lib.stream_ptr()), "pp_stress")
        return out.cpu().numpy().reshape(3, 3)

    def forces(self, rho):
        """Forces of the local pseudopotential on the ions, nat x 3 numpy array
        (``forces``, ``:260-271``: ``_ForcePME`` with PME, ``_Force`` without).
        The transforms run in the density's precision; sums in FP64."""
        if rho is None:
            raise AttributeError("Must specify rho")
        if not isinstance(rho, DirectField):
            raise TypeError("rho must be DirectField")
        if rho.ndim > 3:
            rho = DirectField(self.grid, data=rho.sum(dim=0))
        keys, spos, species, tabs, bm = self._device_setup()
        plan = self.grid.plan(rho.dtype)
        nat = self.ions.nat
        nb = _lib.forces_workspace_bytes(plan, nat)
        work = torch.empty(nb // 8 + 64, dtype=torch.float64, device="cuda")
        F = torch.empty((nat, 3), dtype=torch.float64, device="cuda")
        _lib.check(_lib.load().gbofdft_pp_forces(
            plan.handle, _lib.ptr(rho), len(keys), tabs, nat, _lib.ptr(spos), _lib.ptr(species), int(self.PME),
            self.BsplineOrder, _lib.ptr(bm) if bm is not None else None, _lib.aligned_ptr(work, 256), nb,
            _lib.ptr(F), _lib.stream_ptr()), "pp_forces")
        return F.cpu().numpy()

    def vreal_of(self, dtype):
        self.local_PP()
        if dtype not in self._vreal:
            self._vreal[dtype] = self._vreal[torch.float64].to(dtype)
        return self._vreal[dtype]

    @property
    def vreal(self):
        return DirectField(self.grid, data=self.vreal_of(torch.float64))

    @property
    def v(self):
        self.local_PP()
        n2 = int(self.grid.nrR[2])
        if self.grid.full:
            from ..field import _hermitian_extend
            return ReciprocalField(self.grid.get_reciprocal(), data=_hermitian_extend(self._vG, n2))
        return ReciprocalField(self.grid.get_reciprocal(), data=self._vG)

    def spec(self, rho):
        sp = Spec()
        sp.vloc = self.vreal_of(rho.dtype)
        return sp

    def compute(self, density, calcType={"E", "V"}, **kwargs):
        en, _ = evaluate(density, self.spec(density), {"E"} if "E" in calcType else set())
        out = FunctionalOutput(name="eN", energy=0.0 if en is None else float(en[_lib.E_PSEUDO]))
        if "V" in calcType:
            out.potential = DirectField(self.grid, data=self.vreal_of(density.dtype))
        return out

    def get_ewald(self, PME=None):
        if self.ewald is None:
            self.ewald = ewald(ions=self.ions, grid=self.grid, PME=self.PME if PME is None else PME,
                               BsplineOrder=self.BsplineOrder)
        return self.ewald


def _erfcinv(y):
    """Inverse of erfc for 0 < y < 1 (bisection + Newton on math.erfc)."""
    lo, hi = 0.0, 30.0
    for _ in range(200):
        mid = 0.5 * (lo + hi)
        if math.erfc(mid) > y:
            lo = mid
        else:
            hi = mid
    x = 0.5 * (lo + hi)
    for _ in range(3):
        fx = math.erfc(x) - y
        d = -2.0 / math.sqrt(math.pi) * math.exp(-x * x)
        if d == 0.0:
            break
        x -= fx / d
    return x


class ewald:
    """Ion-ion energy: correction + real-space + reciprocal (PME or exact)
    (``ewald.py:197-508``)."""

    def __init__(self, precision=1.0e-8, ions=None, rho=None, grid=None, verbose=False, BsplineOrder=10, PME=False,
                 **kwargs):
        if ions is None:
            raise AttributeError("Must pass ions to Ewald")
        self.ions = Ions.from_any(ions)
        self.grid = grid if grid is not None else getattr(rho, "grid", None)
        if self.grid is None:
            raise AttributeError("Must pass grid or rho to Ewald")
        self.precision = precision
        self.order = BsplineOrder
        self.PME = PME
        self.eta = self.Get_Best_eta(precision, math.sqrt(2.0 * self.grid.guess_ecut()), self.ions)
        self._energy = None
        self._parts = None

    @staticmethod
    def Get_Best_eta(precision, gmax, ions):
        """``ewald.py:256-279``: largest eta (from 1.6 down in 0.01 steps) whose
        reciprocal-space error bound is below ``precision``."""
        q = ions.charges
        chargeSquare = float(np.sum(q * q))
        eta = 1.6
        while True:
            up = 4.0 * math.pi * ions.nat * chargeSquare * math.sqrt(eta / math.pi) * math.erfc(
                gmax / 2.0 * math.sqrt(1.0 / eta))
            if up < precision:
                return eta
            eta = eta - 0.01

    def Energy_corr(self):
        """``ewald.py:468-484``."""
        q = self.ions.charges
        e = -math.sqrt(self.eta / math.pi) * float(np.sum(q * q))
        e += -4.0 * math.pi * (1.0 / (4.0 * self.eta * self.grid.volume) / 2.0) * float(q.sum()) ** 2
        return e

    def _device_setup(self):
        """rmax, lattice images and device copies of positions, charges, b(m)."""
        if getattr(self, "_dev", None) is None:
            g = self.grid
            rmax = _erfcinv(self.precision / 3.0) / math.sqrt(self.eta)
            L = np.sqrt((g.lattice ** 2).sum(axis=1))
            N = np.ceil(rmax / L).astype(int)
            rng = [np.arange(-N[d], N[d] + 1) for d in range(3)]
            I = np.array(np.meshgrid(*rng, indexing="ij")).reshape(3, -1).T.astype(float)
            images = torch.tensor(I @ g.lattice, dtype=torch.float64, device="cuda").contiguous()
            ions = self.ions
            pos = torch.tensor(ions.positions, dtype=torch.float64, device="cuda").contiguous()
            spos = torch.tensor(ions.get_scaled_positions(), dtype=torch.float64, device="cuda").contiguous()
            q = torch.tensor(ions.charges, dtype=torch.float64, device="cuda").contiguous()
            bm = torch.tensor(pme_bm(g.nrR, self.order).view(np.float64), device="cuda") if self.PME else None
            self._dev = (rmax, images, pos, spos, q, bm)
        return self._dev

    def _gpu_parts(self):
        if self._parts is None:
            plan = self.grid.plan(torch.float64)
            rmax, images, pos, spos, q, bm = self._device_setup()
            nat = self.ions.nat
            nb = _lib.setup_workspace_bytes(plan, nat)
            work = torch.empty(nb // 8 + 64, dtype=torch.float64, device="cuda")
            out = torch.zeros(2, dtype=torch.float64, device="cuda")
            _lib.check(_lib.load().gbofdft_ewald(
                plan.handle, nat, _lib.ptr(pos), _lib.ptr(spos), _lib.ptr(q), float(self.eta), float(rmax),
                _lib.ptr(images), int(images.shape[0]), int(self.PME), int(self.order),
                _lib.ptr(bm) if bm is not None else None, _lib.aligned_ptr(work, 256), nb, _lib.ptr(out),
                _lib.stream_ptr()), "ewald")
            self._parts = [float(x) for x in out.cpu().numpy()]
        return self._parts

    @property
    def stress(self):
        """Ion-ion stress, 3x3 (``stress``, ``ewald.py:523-538``): ``Stress_real``
        plus ``Stress_rec_PME`` or ``Stress_rec``, in FP64."""
        if getattr(self, "_stress", None) is None:
            plan = self.grid.plan(torch.float64)
            rmax, images, pos, spos, q, bm = self._device_setup()
            nat = self.ions.nat
            nb = _lib.stress_workspace_bytes(plan, nat)
            work = torch.empty(nb // 8 + 64, dtype=torch.float64, device="cuda")
            out = torch.empty(9, dtype=torch.float64, device="cuda")
            _lib.check(_lib.load().gbofdft_ewald_stress(
                plan.handle, nat, _lib.ptr(pos), _lib.ptr(spos), _lib.ptr(q), float(self.eta), float(rmax),
                _lib.ptr(images), int(images.shape[0]), int(self.PME), int(self.order),
                _lib.ptr(bm) if bm is not None else None, float(self.ions.get_ncharges()),
                _lib.aligned_ptr(work, 256), nb, _lib.ptr(out), _lib.stream_ptr()), "ewald_stress")
            self._stress = out.cpu().numpy().reshape(3, 3)
        return self._stress

    @property
    def forces(self):
        """Ion-ion forces, nat x 3 numpy array (``forces``, ``ewald.py:510-521``):
        ``Forces_real`` plus ``Forces_rec_PME`` or ``Forces_rec``, in FP64."""
        if getattr(self, "_forces", None) is None:
            plan = self.grid.plan(torch.float64)
            rmax, images, pos, spos, q, bm = self._device_setup()
            nat = self.ions.nat
            nb = _lib.forces_workspace_bytes(plan, nat)
            work = torch.empty(nb // 8 + 64, dtype=torch.float64, device="cuda")
            F = torch.empty((nat, 3), dtype=torch.float64, device="cuda")
            _lib.check(_lib.load().gbofdft_ewald_forces(
                plan.handle, nat, _lib.ptr(pos), _lib.ptr(spos), _lib.ptr(q), float(self.eta), float(rmax),
                _lib.ptr(images), int(images.shape[0]), int(self.PME), int(self.order),
                _lib.ptr(bm) if bm is not None else None, _lib.aligned_ptr(work, 256), nb, _lib.ptr(F),
                _lib.stream_ptr()), "ewald_forces")
            self._forces = F.cpu().numpy()
        return self._forces

    def Energy_real(self):
        return self._gpu_parts()[0]

    def Energy_rec(self):
        return self._gpu_parts()[1]

    Energy_real_fast2 = Energy_real
    Energy_rec_PME = Energy_rec

    @property
    def energy(self):
        if self._energy is None:
            self._energy = self.Energy_corr() + self.Energy_real() + self.Energy_rec()
        return self._energy
