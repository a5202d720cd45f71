"""Restore ``scipy.optimize._minpack2.dcsrch`` for the reference's line search.

Golden-fixture shim only.  The reference imports ``minpack2`` at
``dftpy/math_utils.py:6-9`` and drives ``dcsrch`` by reverse communication
(``LineSearchDcsrch2``, ``math_utils.py:76-106``).  scipy 1.18 no longer ships
that extension; it keeps the same Moré–Thuente routine as the private class
``scipy.optimize._dcsrch.DCSRCH``.  ``dcsrch`` here keeps one ``DCSRCH`` per
``isave`` buffer, recreated whenever the caller passes ``task=b"START"``.
"""
import sys
import types

from scipy.optimize._dcsrch import DCSRCH

_STATE = {}


def dcsrch(stp, f, g, ftol, gtol, xtol, task, stpmin, stpmax, isave, dsave):
    key = id(isave)
    if task[:5] == b"START" or key not in _STATE:
        _STATE[key] = DCSRCH(None, None, ftol, gtol, xtol, stpmin, stpmax)
    stp, f, g, task = _STATE[key]._iterate(stp, f, g, task)
    return stp, f, g, task


def install():
    mod = types.ModuleType("scipy.optimize._minpack2")
    mod.dcsrch = dcsrch
    sys.modules["scipy.optimize._minpack2"] = mod
    import scipy.optimize as so
    so._minpack2 = mod
