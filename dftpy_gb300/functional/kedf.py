"""Kinetic energy density functionals (``functional/kedf/__init__.py``).

Supported names (``KEDFEngines``, ``kedf/__init__.py:27-69``): TF, VW, the
TF+vW family (TFVW, X_TF_Y_VW, XTFYVW), WT-NL and WT (= TF + VW + WT-NL),
LWT/LMGP; and WGC / WGC-NL (density-dependent kernel, no reference counterpart).
"""
import torch

from .. import _lib
from .output import AbstractFunctional, FunctionalOutput
from ._eval import Spec, evaluate

KEDF_PARTS = {
    "LMGP": ("TF", "VW", "LWT"),
    "LMGP-NL": ("LWT",),
    "LWT": ("TF", "VW", "LWT"),
    "LWT-NL": ("LWT",),
    "TF": ("TF",),
    "VW": ("VW",),
    "TFVW": ("TF", "VW"),
    "X_TF_Y_VW": ("TF", "VW"),
    "XTFYVW": ("TF", "VW"),
    "WT-NL": ("WT",),
    "WT": ("TF", "VW", "WT"),
    "WGC-NL": ("WGC",),
    "WGC": ("TF", "VW", "WGC"),
}


class KEDF(AbstractFunctional):
    def __init__(self, name="WT", kedf=None, **kwargs):
        self.type = "KEDF"
        self.name = (kedf or name).upper()
        if self.name not in KEDF_PARTS:
            raise AttributeError("%s KEDF to be implemented" % self.name)
        self.options = dict(kwargs)
        self.options["kedf"] = self.name
        # kernel cache, as the reference's ke_kernel_saved (kedf/__init__.py:96-106)
        self.ke_kernel_saved = {"Kernel": None, "rho0": 0.0, "shape": None, "dtype": None}
        self._kernels_by_dtype = {}
        self.energies = {}
        self._lwt = None
        if "LWT" in KEDF_PARTS[self.name]:
            from .lwt import LWTTerm
            kt = "MGP" if self.name.startswith("LMGP") else "WT"
            opts = {k: v for k, v in self.options.items() if k not in ("kedf", "y", "sigma")}
            self._lwt = LWTTerm(kerneltype=kt, **opts)
        self._wgc = None
        if "WGC" in KEDF_PARTS[self.name]:
            from .wgc import WGCTerm
            opts = {k: v for k, v in self.options.items() if k not in ("kedf", "y", "sigma")}
            self._wgc = WGCTerm(**opts)

    @property
    def parts(self):
        return KEDF_PARTS[self.name]

    def _wt_kernel(self, rho):
        """``get_ke_kernel_wt`` (``kedf/wt.py:58-73``): rebuild only when the mean
        density moves by more than 1e-6 or the grid changes."""
        rho0 = self.options.get("rho0", None)
        if not rho0:
            rho0 = float(rho.as_subclass(torch.Tensor).to(torch.float64).mean())
        s = self._kernels_by_dtype.setdefault(rho.dtype, {"Kernel": None, "rho0": 0.0, "shape": None,
                                                          "dtype": rho.dtype})
        self.ke_kernel_saved = s
        shape = tuple(rho.shape)
        if abs(s["rho0"] - rho0) > 1e-6 or s["shape"] != shape:
            g = rho.grid
            plan = g.plan(rho.dtype)
            k = torch.empty((int(g.nrR[0]), int(g.nrR[1]), int(g.nrR[2]) // 2 + 1), dtype=rho.dtype, device="cuda")
            _lib.check_alloc(lambda: _lib.load().gbofdft_wt_kernel(
                plan.handle, float(rho0), float(self.options.get("x", 1.0)), float(self.alpha),
                float(self.beta), _lib.ptr(k), _lib.stream_ptr()), "wt_kernel")
            s.update(Kernel=k, rho0=rho0, shape=shape)
        return s["Kernel"]

    @property
    def alpha(self):
        return self.options.get("alpha", 5.0 / 6.0)

    @property
    def beta(self):
        return self.options.get("beta", 5.0 / 6.0)

    def spec(self, rho):
        sp = Spec()
        parts = self.parts
        if "TF" in parts:
            sp.tf, sp.tf_x = True, float(self.options.get("x", 1.0))
        if "VW" in parts:
            sp.vw, sp.vw_y = True, float(self.options.get("y", 1.0))
            if self.options.get("sigma") is not None:
                raise NotImplementedError("vW with Gaussian smearing (sigma) is not part of this path")
        if "WT" in parts:
            if abs(self.alpha - self.beta) > 1e-9:
                raise NotImplementedError("WT with alpha != beta is not part of this path")
            sp.wt, sp.wt_alpha, sp.wt_beta = True, float(self.alpha), float(self.beta)
            sp.wt_kernel = self._wt_kernel(rho)
        if "LWT" in parts:
            sp.lwt = self._lwt.prepare(rho)
        if "WGC" in parts:
            sp.wgc = self._wgc.prepare(rho)
        return sp

    def stress(self, density, split=False, **kwargs):
        """Stress of the KEDF parts (``KEDF.stress``, ``kedf/__init__.py:186-229``):
        a dict by part ("TF", "VW", "NL") with ``split``, else their sum."""
        from .stress import functional_stress
        out = functional_stress(density, self.spec(density))
        return out if split else sum(out.values())

    def compute(self, density, calcType={"E", "V"}, split=False, **kwargs):
        en, pot = evaluate(density, self.spec(density), calcType)
        out = FunctionalOutput(name="KEDF")
        if en is not None:
            if split:
                res = {}
                for p, slot in (("TF", _lib.E_TF), ("VW", _lib.E_VW), ("WT", _lib.E_NL), ("LWT", _lib.E_NL),
                                ("WGC", _lib.E_NL)):
                    if p in self.parts:
                        res[p if p != "WT" else "NL"] = FunctionalOutput(name=p, energy=float(en[slot]))
                        self.energies[p] = float(en[slot])
                return res
            out.energy = float(en[_lib.E_TF] + en[_lib.E_VW] + en[_lib.E_NL])
        if "V" in calcType:
            out.potential = pot
        return out
