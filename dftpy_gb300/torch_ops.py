"""The library's entry points registered as PyTorch custom operators.

``torch.ops.gbofdft.eval``, ``convolve``, ``fft_r2c``, ``fft_c2r``,
``optimize_tn`` and ``optimize_tn_split`` wrap the C ABI of
``include/gbofdft.h`` (bound by ctypes in ``_lib``).  Each has a fake
(meta) implementation, so the operators trace under ``torch.compile``,
``torch.fx`` and graph capture with the right output shapes and dtypes; the
real implementations run only on CUDA tensors (there is no CPU kernel: a CPU
tensor raises).

The reference's equivalents are Python methods on its field and functional
classes: ``TotalFunctional.compute`` (``functional/total_functional.py:107-146``,
through ``AbstractFunctional.__call__``, ``functional/abstract_functional.py:12-30``),
``DirectField.fft`` / ``ReciprocalField.ifft`` (``field.py:373-390, 739-764``)
and ``Optimization.optimize_rho`` (``optimization/optimization.py:281-520``).
The package's classes keep those names and route their device work through
these operators.

Library objects that are not tensors -- a grid plan, a functional
descriptor (``gbofdft_functional``, which points at the caller's kernel
tables and v_loc), optimiser options and the result record -- travel as
integer handles (their addresses, declared ``int`` in the schemas so that
tracing never makes them symbolic); the caller keeps them alive for the
call.
"""
import ctypes
from typing import Optional

import torch

from . import _lib

_FP = ctypes.POINTER(_lib.Functional)


def _vp(h):
    return ctypes.c_void_p(int(h))


def _cdt(dt):
    return torch.complex128 if dt == torch.float64 else torch.complex64


def _rdt(dt):
    return torch.float64 if dt == torch.complex128 else torch.float32


# --------------------------------------------------------------------------
@torch.library.custom_op("gbofdft::eval", mutates_args=(), device_types="cuda",
                         schema="(Tensor rho, int plan, int functional, int calc) -> (Tensor, Tensor)")
def eval_op(rho: torch.Tensor, plan: int, functional: int, calc: int) -> tuple[torch.Tensor, torch.Tensor]:
    """``gbofdft_eval``: total potential and the 8 energy slots (zeros unless
    ``calc`` has GBOFDFT_CALC_E) of the functional at ``rho``."""
    r = rho.contiguous()
    pot = torch.empty_like(r)
    en = torch.zeros(_lib.NE, dtype=torch.float64, device=r.device)
    want_e = bool(int(calc) & _lib.CALC_E)
    _lib.check(_lib.load().gbofdft_eval(_vp(plan), _lib.ptr(r), ctypes.cast(int(functional), _FP), _lib.ptr(pot),
                                        _lib.ptr(en) if want_e else None, int(calc), _lib.stream_ptr()), "eval")
    return pot, en


@eval_op.register_fake
def _(rho, plan, functional, calc):
    return torch.empty_like(rho), rho.new_empty(_lib.NE, dtype=torch.float64)


# --------------------------------------------------------------------------
@torch.library.custom_op("gbofdft::convolve", mutates_args=(), device_types="cuda",
                         schema="(Tensor x, int plan, int kernel, Tensor? kernel_array, float coef) -> Tensor")
def convolve_op(x: torch.Tensor, plan: int, kernel: int, kernel_array: Optional[torch.Tensor],
                coef: float) -> torch.Tensor:
    """``gbofdft_convolve``: ifft(fft(x) * coef * K(G)), K = 4 pi / G^2, G^2
    or ``kernel_array`` (a real half spectrum)."""
    xc = x.contiguous()
    out = torch.empty_like(xc)
    ka = kernel_array.contiguous() if kernel_array is not None else None
    _lib.check(_lib.load().gbofdft_convolve(_vp(plan), _lib.ptr(xc), _lib.ptr(out), int(kernel), _lib.ptr(ka),
                                            float(coef), _lib.stream_ptr()), "convolve")
    return out


@convolve_op.register_fake
def _(x, plan, kernel, kernel_array, coef):
    return torch.empty_like(x)


# --------------------------------------------------------------------------
@torch.library.custom_op("gbofdft::fft_r2c", mutates_args=(), device_types="cuda",
                         schema="(Tensor x, int plan) -> Tensor")
def fft_r2c_op(x: torch.Tensor, plan: int) -> torch.Tensor:
    """``gbofdft_fft_r2c``: half spectrum [n0][n1][n2/2+1], times dV."""
    xc = x.contiguous()
    n0, n1, n2 = xc.shape
    out = torch.empty((n0, n1, n2 // 2 + 1), dtype=_cdt(xc.dtype), device=xc.device)
    _lib.check(_lib.load().gbofdft_fft_r2c(_vp(plan), _lib.ptr(xc), _lib.ptr(out), _lib.stream_ptr()), "fft")
    return out


@fft_r2c_op.register_fake
def _(x, plan):
    n0, n1, n2 = x.shape
    return x.new_empty((n0, n1, n2 // 2 + 1), dtype=_cdt(x.dtype))


@torch.library.custom_op("gbofdft::fft_c2r", mutates_args=(), device_types="cuda",
                         schema="(Tensor xg, int plan, int n2) -> Tensor")
def fft_c2r_op(xg: torch.Tensor, plan: int, n2: int) -> torch.Tensor:
    """``gbofdft_fft_c2r``: real field [n0][n1][n2] from a half spectrum,
    divided by dV (``xg`` is not modified)."""
    X = xg.contiguous()
    n0, n1, _ = X.shape
    out = torch.empty((n0, n1, int(n2)), dtype=_rdt(X.dtype), device=X.device)
    _lib.check(_lib.load().gbofdft_fft_c2r(_vp(plan), _lib.ptr(X), _lib.ptr(out), _lib.stream_ptr()), "ifft")
    return out


@fft_c2r_op.register_fake
def _(xg, plan, n2):
    n0, n1, _ = xg.shape
    return xg.new_empty((n0, n1, int(n2)), dtype=_rdt(xg.dtype))


# --------------------------------------------------------------------------
@torch.library.custom_op("gbofdft::optimize_tn", mutates_args=("workspace",), device_types="cuda",
                         schema="(Tensor rho, int plan, int functional, int options, Tensor(a!) workspace, "
                                "int workspace_bytes, int result) -> Tensor")
def optimize_tn_op(rho: torch.Tensor, plan: int, functional: int, options: int, workspace: torch.Tensor,
                   workspace_bytes: int, result: int) -> torch.Tensor:
    """``gbofdft_optimize_tn``: the density minimising the functional from
    ``rho`` (a new tensor); scalars go to the ``gbofdft_tn_result`` at
    ``result``.  ``workspace`` holds ``workspace_bytes`` from its first
    256-byte aligned address on."""
    out = rho.contiguous().clone()
    _lib.check(_lib.load().gbofdft_optimize_tn(_vp(plan), ctypes.cast(int(functional), _FP), _lib.ptr(out),
                                               ctypes.cast(int(options), ctypes.POINTER(_lib.TnOptions)),
                                               _lib.aligned_ptr(workspace, 256), int(workspace_bytes),
                                               ctypes.cast(int(result), ctypes.POINTER(_lib.TnResult)),
                                               _lib.stream_ptr()), "optimize_tn")
    return out


@optimize_tn_op.register_fake
def _(rho, plan, functional, options, workspace, workspace_bytes, result):
    return torch.empty_like(rho)


@torch.library.custom_op("gbofdft::optimize_tn_split", mutates_args=("workspace", "hworkspace"),
                         device_types="cuda",
                         schema="(Tensor rho, int plan, int functional, int hplan, int hfunctional, int options, "
                                "Tensor(a!) workspace, int workspace_bytes, Tensor(b!) hworkspace, "
                                "int hworkspace_bytes, int result) -> Tensor")
def optimize_tn_split_op(rho: torch.Tensor, plan: int, functional: int, hplan: int, hfunctional: int, options: int,
                         workspace: torch.Tensor, workspace_bytes: int, hworkspace: torch.Tensor,
                         hworkspace_bytes: int, result: int) -> torch.Tensor:
    """``gbofdft_optimize_tn_split``: FP64 truncated Newton whose inner CG's
    Hessian products use the FP32 plan ``hplan`` and functional
    ``hfunctional``."""
    out = rho.contiguous().clone()
    _lib.check(_lib.load().gbofdft_optimize_tn_split(
        _vp(plan), ctypes.cast(int(functional), _FP), _vp(hplan), ctypes.cast(int(hfunctional), _FP), _lib.ptr(out),
        ctypes.cast(int(options), ctypes.POINTER(_lib.TnOptions)), _lib.aligned_ptr(workspace, 256),
        int(workspace_bytes), _lib.aligned_ptr(hworkspace, 256), int(hworkspace_bytes),
        ctypes.cast(int(result), ctypes.POINTER(_lib.TnResult)), _lib.stream_ptr()), "optimize_tn_split")
    return out


@optimize_tn_split_op.register_fake
def _(rho, plan, functional, hplan, hfunctional, options, workspace, workspace_bytes, hworkspace, hworkspace_bytes,
      result):
    return torch.empty_like(rho)


def handle(obj):
    """Integer handle of a plan (``_lib.Plan``), a ctypes structure, or a raw
    ``ctypes.c_void_p``."""
    if hasattr(obj, "handle"):
        obj = obj.handle
    if isinstance(obj, ctypes.c_void_p):
        return int(obj.value or 0)
    if isinstance(obj, ctypes.Structure):
        return ctypes.addressof(obj)
    return int(obj)


OPS = ("eval", "convolve", "fft_r2c", "fft_c2r", "optimize_tn", "optimize_tn_split")
