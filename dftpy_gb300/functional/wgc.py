"""WGC nonlocal kinetic term (density-dependent kernel, second order about
the mean density).

No reference counterpart: the reference's KEDF set has no WGC.  The method is
Wang, Govind and Carter, Phys. Rev. B 60, 16350 (1999): the Wang-Teter double
integral with the kernel taken at the two-body Fermi wavevector
xi = [(k_F(r)^gamma + k_F(r')^gamma)/2]^(1/gamma), expanded to second order
in (rho - rho0)/rho0.  Defaults: alpha = (5 + sqrt 5)/6, beta = (5 - sqrt 5)/6,
gamma = 2.7.  The kernel's shape is the solution of the linear-response
equation of ``kernel_table`` (host, once); the kernels on the half spectrum
(K0, K1, Kq, Kx) are interpolated from it on the GPU by
``gbofdft_wgc_kernels`` when the mean density moves by more than 1e-6, as
the Wang-Teter kernel cache does; one evaluation runs in ``gbofdft_eval``
through the ``gbofdft_wgc`` descriptor.
"""
import ctypes
import math

import numpy as np
import torch

from .. import _lib
from .._tables import lindhard

ALPHA = (5.0 + math.sqrt(5.0)) / 6.0
BETA = (5.0 - math.sqrt(5.0)) / 6.0
GAMMA = 2.7


# table points on ln(eta): the inverse Lindhard function has a logarithmic
# singularity in its derivative at eta = 1, where the interpolated Kx is off
# by ~3e-4 with 16001 points and by ~4e-6 with 160001 (0.2 s on the host, once)
ETA_MIN, ETA_MAX, NTAB = 1e-5, 200.0, 160001


def _bounded_solve(lam, g, h):
    """y on the uniform grid t_i (spacing h) with (d/dt - lam) y = g and y
    bounded as t -> +inf (Re lam > 0): y(t) = -int_t^inf exp(lam (t - s)) g(s) ds,
    integrated backwards exactly for g linear between grid points, starting
    from the constant solution -g/lam at the last point."""
    from scipy.signal import lfilter
    e = np.exp(-lam * h)
    E0 = (1.0 - e) / lam
    E1 = (1.0 - e * (1.0 + lam * h)) / lam ** 2
    g = np.asarray(g, dtype=complex)
    # y[i] = e y[i+1] - c[i] from the last point down: a first-order
    # recursive filter over the reversed sequence
    c = g[:-1] * E0 + (g[1:] - g[:-1]) / h * E1
    x = np.empty(g.shape, dtype=complex)
    x[0] = -g[-1] / lam
    x[1:] = -c[::-1]
    return lfilter([1.0], [1.0, -e], x)[::-1]


_TABLES = {}


def kernel_table(alpha=None, beta=None, gamma=None, x=1.0, order=2, eta_min=ETA_MIN, eta_max=ETA_MAX, m=NTAB):
    """``_kernel_table`` cached by its arguments (the table depends on the
    exponents only, not on the structure)."""
    key = (alpha, beta, gamma, float(x), int(order), float(eta_min), float(eta_max), int(m))
    t = _TABLES.get(key)
    if t is None:
        t = _TABLES[key] = _kernel_table(alpha, beta, gamma, x, order, eta_min, eta_max, m)
    return t


def _kernel_table(alpha=None, beta=None, gamma=None, x=1.0, order=2, eta_min=ETA_MIN, eta_max=ETA_MAX, m=NTAB):
    """WGC kernels per unit prefactor on t = ln(eta), eta = |G| / 2k: columns
    K0, K1, Kq, Kx (times C = 5 C_TF / (9 alpha beta rho^(alpha+beta-5/3))).

    K(G; k) = C(k) w(G / 2k) with the shape w chosen so that the expanded
    functional keeps the Lindhard response at the expansion density: the
    second functional derivative of the nonlocal term at a uniform density
    is 2 rho^(alpha+beta-2) [alpha beta K0 + (alpha+beta)/6 K1 + Kx], which
    must equal the Wang-Teter value 2 alpha beta rho^(alpha+beta-2) C L(eta)
    (L the inverse Lindhard function less the TF and vW responses).  With
    D = d/dt, K1 = C (p w - Dw), K2 = C (p(p-1) w - (2p-1) Dw + D^2 w),
    p = 5 - 3 (alpha + beta), Kx = (1-g)/36 K1 + K2/36 that is

      order 2:  D^2 w - (1 + b) D w + a w = (alpha beta / c2) L,
                c1 = (alpha+beta)/6 + (1-g)/36, c2 = 1/36,
                1 + b = (c1 + c2 (2p-1)) / c2,  a = (alpha beta + c1 p + c2 p(p-1)) / c2;
      order 1:  Kx = Kq = 0 and (alpha beta + (alpha+beta) p/6) w - (alpha+beta)/6 Dw = alpha beta L;
      order 0:  w = L (the Wang-Teter kernel).

    Both roots of the characteristic polynomial have positive real parts, so
    the solution bounded at large eta is unique; below eta_min w goes as
    eta^2 (as L does) and above eta_max it is constant."""
    alpha = ALPHA if alpha is None else float(alpha)
    beta = BETA if beta is None else float(beta)
    gamma = GAMMA if gamma is None else float(gamma)
    t = np.linspace(np.log(eta_min), np.log(eta_max), m)
    h = t[1] - t[0]
    L = lindhard(np.exp(t), x, 1.0)
    ab, sab = alpha * beta, alpha + beta
    p = 5.0 - 3.0 * sab
    zeros = np.zeros_like(t)
    if order == 0:
        return float(t[0]), float(h), np.stack([L, zeros, zeros, zeros])
    if order == 1:
        lam = (ab + sab * p / 6.0) / (sab / 6.0)
        w = _bounded_solve(lam, -(ab / (sab / 6.0)) * L, h).real
        wt = lam * w - (ab / (sab / 6.0)) * L          # Dw from the ODE
        K1 = p * w - wt
        return float(t[0]), float(h), np.stack([w, K1, zeros, zeros])
    c2 = 1.0 / 36.0
    c1 = sab / 6.0 + (1.0 - gamma) / 36.0
    s1 = (c1 + c2 * (2.0 * p - 1.0)) / c2                # lam1 + lam2
    pr = (ab + c1 * p + c2 * p * (p - 1.0)) / c2          # lam1 lam2
    disc = np.sqrt(complex(s1 * s1 - 4.0 * pr))
    lam1, lam2 = (s1 + disc) / 2.0, (s1 - disc) / 2.0
    if lam1.real <= 0 or lam2.real <= 0:
        raise ValueError("WGC kernel equation has no bounded solution for these parameters")
    f = (ab / c2) * L
    z = _bounded_solve(lam1, f.astype(complex), h)       # (D - lam1) z = f
    w = _bounded_solve(lam2, z, h)                        # (D - lam2) w = z
    wt = lam2 * w + z
    wtt = lam2 * wt + lam1 * z + f
    w, wt, wtt = w.real, wt.real, wtt.real
    K1 = p * w - wt
    K2 = p * (p - 1.0) * w - (2.0 * p - 1.0) * wt + wtt
    Kq = (gamma - 5.0) / 72.0 * K1 + K2 / 72.0
    Kx = (1.0 - gamma) / 36.0 * K1 + K2 / 36.0
    return float(t[0]), float(h), np.stack([w, K1, Kq, Kx])


_DEVICE_TABLES = {}


class WGCTerm:
    def __init__(self, alpha=ALPHA, beta=BETA, gamma=GAMMA, x=1.0, order=2, rho0=None, **kwargs):
        if int(order) not in (0, 1, 2):
            raise ValueError("WGC order must be 0, 1 or 2")
        self.alpha, self.beta, self.gamma = float(alpha), float(beta), float(gamma)
        self.x, self.order = float(x), int(order)
        self.fixed_rho0 = float(rho0) if rho0 else None
        self._state = {}
        self._table = None

    def table(self):
        """Device copy of the kernel table (one per exponents and device,
        shared by every WGC term)."""
        if self._table is None:
            key = (self.alpha, self.beta, self.gamma, self.x, self.order, torch.cuda.current_device())
            t = _DEVICE_TABLES.get(key)
            if t is None:
                t0, h, cols = kernel_table(self.alpha, self.beta, self.gamma, self.x, self.order)
                dev = torch.tensor(np.ascontiguousarray(cols), dtype=torch.float64, device="cuda")
                # shared by every thread and stream: complete before publishing
                torch.cuda.current_stream().synchronize()
                t = _DEVICE_TABLES[key] = (t0, h, cols.shape[1], dev)
            self._table = t
        return self._table

    def prepare(self, rho):
        """Kernels and workspace for rho's grid and dtype; returns the descriptor."""
        key = (id(rho.grid), rho.dtype)
        st = self._state.get(key)
        rho0 = self.fixed_rho0 or float(rho.as_subclass(torch.Tensor).to(torch.float64).mean())
        if not (math.isfinite(rho0) and rho0 > 0.0):
            raise ValueError("WGC: the mean density must be positive and finite (got %r)" % rho0)
        plan = rho.grid.plan(rho.dtype)
        if st is None:
            nb = ctypes.c_int64()
            _lib.check(_lib.load().gbofdft_wgc_workspace_bytes(plan.handle, ctypes.byref(nb)))
            buf = torch.empty(int(nb.value) // 8 + 64, dtype=torch.float64, device="cuda")
            g = rho.grid
            K = torch.empty((4, int(g.nrR[0]), int(g.nrR[1]), int(g.nrR[2]) // 2 + 1), dtype=rho.dtype, device="cuda")
            d = _lib.Wgc()
            d.alpha, d.beta, d.gamma, d.order = self.alpha, self.beta, self.gamma, self.order
            d.kernels = K.data_ptr()
            d.work = _lib.aligned_ptr(buf, 256)
            d.work_bytes = int(nb.value)
            d.rho0 = 0.0
            st = self._state[key] = {"buf": buf, "K": K, "d": d}
        d = st["d"]
        if abs(d.rho0 - rho0) > 1e-6:
            t0, h, m, tab = self.table()
            _lib.check_alloc(lambda: _lib.load().gbofdft_wgc_kernels(
                plan.handle, rho0, self.alpha, self.beta, _lib.ptr(tab), int(m), t0, h, _lib.ptr(st["K"]),
                _lib.stream_ptr()), "wgc_kernels")
            d.rho0 = rho0
        return d
