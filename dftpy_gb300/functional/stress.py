"""Stress tensors on the device (``TotalFunctional.get_stress``,
``functional/total_functional.py:176-209``).

``functional_stress`` runs ``gbofdft_stress_functional`` for the density
terms of a Spec (TF, vW, WT, LDA, Hartree) from the energies of one
``gbofdft_eval`` at the same density; the local pseudopotential and the Ewald
sum have their own entry points (``LocalPseudo.stress``, ``ewald.stress``).
Tensors are 3x3 numpy arrays in Ha/Bohr^3.
"""
import ctypes

import numpy as np
import torch

from .. import _lib
from ._eval import evaluate, plain

TERMS = ("TF", "VW", "NL", "XC", "HARTREE")


def workspace(plan, nat):
    nb = _lib.stress_workspace_bytes(plan, nat)
    return torch.empty(nb // 8 + 64, dtype=torch.float64, device="cuda"), nb


def functional_stress(rho, spec, energies=None):
    """Dict term -> 3x3 for the terms the Spec enables (keys of TERMS)."""
    if spec.lwt is not None:
        raise NotImplementedError("the LWT/LMGP stress is not part of this path")
    if spec.wgc is not None:
        raise NotImplementedError("the WGC stress is not part of this path")
    if energies is None:
        energies, _ = evaluate(rho, spec, {"E"})
    plan = rho.grid.plan(rho.dtype)
    work, nb = workspace(plan, 0)
    out = torch.zeros(45, dtype=torch.float64, device="cuda")
    en = (ctypes.c_double * _lib.NE)(*[float(x) for x in energies])
    f = spec.ctypes()
    _lib.check(_lib.load().gbofdft_stress_functional(
        plan.handle, _lib.ptr(plain(rho).contiguous()), ctypes.byref(f), en, _lib.aligned_ptr(work, 256), nb,
        _lib.ptr(out), _lib.stream_ptr()), "stress_functional")
    s = out.cpu().numpy().reshape(5, 3, 3)
    on = {"TF": spec.tf, "VW": spec.vw, "NL": spec.wt, "XC": bool(spec.xc), "HARTREE": spec.hartree}
    return {k: s[i].copy() for i, k in enumerate(TERMS) if on[k]}
