"""One call of ``gbofdft_eval`` for a set of functional components."""
import ctypes

import torch

from .. import _lib, torch_ops
from ..field import DirectField


class Spec:
    """Which components a ``gbofdft_eval`` call assembles (and their options)."""

    def __init__(self):
        self.tf = False
        self.tf_x = 1.0
        self.vw = False
        self.vw_y = 1.0
        self.wt = False
        self.wt_alpha = 5.0 / 6.0
        self.wt_beta = 5.0 / 6.0
        self.wt_kernel = None
        self.xc = 0
        self.hartree = False
        self.vloc = None
        self.e_ion = 0.0
        self.lwt = None           # LWTTerm descriptor (gbofdft_lwt)
        self.wgc = None           # WGCTerm descriptor (gbofdft_wgc)

    def merge(self, other):
        for k in ("tf", "vw", "wt", "hartree", "lwt", "wgc"):
            if getattr(self, k) and getattr(other, k):
                raise ValueError("functional component %s given twice" % k)
        if self.xc and other.xc:
            raise ValueError("two XC functionals")
        if self.vloc is not None and other.vloc is not None:
            raise ValueError("two local pseudopotentials")
        out = Spec()
        for k, v in self.__dict__.items():
            setattr(out, k, v)
        for k in ("tf", "vw", "wt", "hartree"):
            if getattr(other, k):
                setattr(out, k, True)
        if other.tf:
            out.tf_x = other.tf_x
        if other.vw:
            out.vw_y = other.vw_y
        if other.wt:
            out.wt_alpha, out.wt_beta, out.wt_kernel = other.wt_alpha, other.wt_beta, other.wt_kernel
        if other.xc:
            out.xc = other.xc
        if other.vloc is not None:
            out.vloc = other.vloc
        if other.lwt is not None:
            out.lwt = other.lwt
        if other.wgc is not None:
            out.wgc = other.wgc
        out.e_ion = self.e_ion + other.e_ion
        return out

    def ctypes(self):
        f = _lib.Functional()
        f.tf, f.tf_x = int(self.tf), float(self.tf_x)
        f.vw, f.vw_y = int(self.vw), float(self.vw_y)
        f.wt, f.wt_alpha, f.wt_beta = int(self.wt), float(self.wt_alpha), float(self.wt_beta)
        f.wt_kernel = self.wt_kernel.data_ptr() if self.wt_kernel is not None else None
        f.xc, f.hartree = int(self.xc), int(self.hartree)
        f.vloc = self.vloc.data_ptr() if self.vloc is not None else None
        f.e_ion = float(self.e_ion)
        if self.lwt is not None:
            f.lwt = ctypes.pointer(self.lwt)
        if self.wgc is not None:
            f.wgc = ctypes.pointer(self.wgc)
        return f


def plain(t):
    return t.as_subclass(torch.Tensor) if isinstance(t, torch.Tensor) else t


def evaluate(rho, spec, calcType):
    """Returns (energies numpy[NE] or None, potential DirectField)."""
    if not isinstance(rho, DirectField):
        raise TypeError("rho must be a DirectField")
    if rho.rank != 1:
        raise NotImplementedError("spin-polarised densities are not part of this path")
    grid = rho.grid
    plan = grid.plan(rho.dtype)
    r = plain(rho).contiguous()
    for name, t in (("wt_kernel", spec.wt_kernel), ("vloc", spec.vloc)):
        if t is not None and t.dtype != rho.dtype:
            raise TypeError("%s has dtype %s, density %s" % (name, t.dtype, rho.dtype))
    want_e = "E" in calcType or "D" in calcType
    f = spec.ctypes()
    calc = _lib.CALC_V | (_lib.CALC_E if want_e else 0)
    # torch.ops.gbofdft.eval: the registered operator over gbofdft_eval
    pot, en = torch.ops.gbofdft.eval(r, torch_ops.handle(plan), ctypes.addressof(f), calc)
    energies = en.cpu().numpy() if want_e else None
    return energies, DirectField(grid, data=pot)
