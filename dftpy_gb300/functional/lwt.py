"""LWT / LMGP nonlocal kinetic term (``functional/kedf/lwt.py``).

Tables (``LWT``, ``lwt.py:531-561``): the kernel on eta = linspace(0, etamax,
neta) -- the MGP integral (``kernel.py:267-322``, evaluated on the GPU by
``gbofdft_mgp_table``) or the WT kernel table -- and K'(eta)(-eta), both as
cubic splines.  The per-evaluation work runs in ``gbofdft_eval`` through the
``gbofdft_lwt`` descriptor; its automatic k_F bounds persist between calls
like the reference's ``ke_kernel_saved``.
"""
import ctypes

import numpy as np
import torch

from .. import _lib
from .._tables import lindhard, spline_notaknot, spline_values_deriv

C_TF = 0.3 * (3.0 * np.pi ** 2) ** (2.0 / 3.0)


class LWTTerm:
    def __init__(self, kerneltype="MGP", interp="linear", etamax=50.0, neta=50000, maxpoints=1000, ratio=1.15,
                 kdd=3, alpha=5.0 / 6.0, beta=5.0 / 6.0, ldw=None, kfmin=None, kfmax=None, x=1.0, **kwargs):
        if interp not in ("linear", "newton", "hermite"):
            raise AttributeError("interp %r is not part of this path" % (interp,))
        if kwargs.get("lumpfactor") is not None or kwargs.get("symmetrization") is not None:
            raise NotImplementedError("LMGP lump factors / symmetrisation are not part of this path")
        if kwargs.get("nsp") is not None or kwargs.get("delta") is not None:
            raise NotImplementedError("uniform k_F knot spacing (nsp / delta) is not part of this path")
        self.kerneltype = kerneltype
        self.d = _lib.Lwt()
        self.d.interp = 1 if interp == "hermite" else 0
        self.d.kdd = int(kdd)
        self.d.alpha, self.d.beta, self.d.ratio = float(alpha), float(beta), float(ratio)
        self.d.ldw = float(ldw) if ldw is not None else 0.0
        self.d.etamax, self.d.neta = float(etamax), int(neta)
        self.d.kfmin_opt = float(kfmin) if kfmin else 0.0
        self.d.kfmax_opt = float(kfmax) if kfmax else 0.0
        self.d.kfmin_state = 0.0
        self.d.kfmax_state = 0.0
        self.maxpoints, self.x = int(maxpoints), float(x)
        self._tabs = None
        self._work = {}

    def _tables(self):
        if self._tabs is not None:
            return
        etamax, neta = self.d.etamax, self.d.neta
        eta = np.linspace(0, etamax, neta)
        if self.kerneltype == "MGP":
            gp = np.logspace(np.log10(eta[1] / 10), np.log10(eta[-1] + 2), num=neta)
            xg, cg = spline_notaknot(gp, lindhard(gp, 1.0, 1.0))
            dev = dict(gp=torch.tensor(xg, dtype=torch.float64, device="cuda"),
                       c=torch.tensor(cg.reshape(-1), dtype=torch.float64, device="cuda"),
                       eta=torch.tensor(eta, dtype=torch.float64, device="cuda"))
            out = torch.empty(neta, dtype=torch.float64, device="cuda")
            _lib.check(_lib.load().gbofdft_mgp_table(_lib.ptr(dev["gp"]), _lib.ptr(dev["c"]), int(xg.size),
                                                      _lib.ptr(dev["eta"]), int(neta), self.maxpoints,
                                                      _lib.ptr(out), _lib.stream_ptr()), "mgp_table")
            table = out.cpu().numpy()
        elif self.kerneltype == "WT":
            table = lindhard(eta, self.x, 1.0) * (4.0 / 5.0 * C_TF)
        else:
            raise AttributeError("kerneltype %r is not part of this path" % (self.kerneltype,))
        x, c = spline_notaknot(eta, table)
        dtab = spline_values_deriv(x, c) * (-1.0 * eta)
        xd, cd = spline_notaknot(eta, dtab)
        self._kc = torch.tensor(c.reshape(-1), dtype=torch.float64, device="cuda")
        self._dc = torch.tensor(cd.reshape(-1), dtype=torch.float64, device="cuda")
        self.d.ktab_c = self._kc.data_ptr()
        self.d.dtab_c = self._dc.data_ptr()
        self.d.ktab_end = float(table[-1])
        self.d.dtab_end = float(dtab[-1])
        self._table = table
        self._tabs = True

    def prepare(self, rho):
        """Tables and a workspace for rho's grid and dtype; returns that
        (grid, dtype)'s descriptor.  Each descriptor owns its workspace, so an
        FP64 and an FP32 evaluation of the same term can interleave (the
        mixed-precision refinement does); each carries its own automatic k_F
        bounds, seeded from the first descriptor's at creation."""
        self._tables()
        key = (id(rho.grid), rho.dtype)
        if key not in self._work:
            plan = rho.grid.plan(rho.dtype)
            nb = ctypes.c_int64()
            _lib.check(_lib.load().gbofdft_lwt_workspace_bytes(plan.handle, ctypes.byref(nb)))
            buf = torch.empty(int(nb.value) // 8 + 64, dtype=torch.float64, device="cuda")
            d = _lib.Lwt()
            ctypes.pointer(d)[0] = self.d          # copy the options, tables and k_F state
            d.work = _lib.aligned_ptr(buf, 256)
            d.work_bytes = int(nb.value)
            self._work[key] = (buf, d)
        return self._work[key][1]
