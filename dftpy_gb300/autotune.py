"""Evaluation-schedule autotuner.

No reference counterpart (the reference's FFT planning is pyFFTW's
``FFTW_MEASURE``, ``math_utils.py:181-222``; its size choice is
``best_fft_size``).  A plan offers several schedules for the potential
evaluation (``gbofdft_plan_schedules``): the column-pass pipeline and, where
the (n0, n1) plane has a specialisation, the plane pipeline with each of its
radix-schedule variants.  All give the same result within FP32 rounding.
``tune(plan)`` times a Wang-Teter + LDA + Hartree + local-PP potential
evaluation with every schedule on a synthetic density (CUDA events on the
current stream, after warm-up), keeps the fastest on the plan and remembers
it per (grid, cell shape class, precision) for the process; with
``GBOFDFT_TUNE_CACHE`` set to a file path the choices persist there.
"""
import ctypes
import json
import os
import threading

import numpy as np
import torch

from . import _lib

_CACHE = {}
_LOCK = threading.Lock()


def _key(plan):
    return "%dx%dx%d/%s/%s" % (plan.nr[0], plan.nr[1], plan.nr[2], plan.precision, int(plan.full))


def _load_file():
    path = os.environ.get("GBOFDFT_TUNE_CACHE")
    if path and os.path.exists(path):
        try:
            with open(path) as f:
                return json.load(f)
        except (OSError, ValueError):
            return {}
    return {}


def _save_file():
    path = os.environ.get("GBOFDFT_TUNE_CACHE")
    if path:
        tmp = path + ".tmp%d" % os.getpid()
        with open(tmp, "w") as f:
            json.dump(_CACHE, f, indent=1, sort_keys=True)
        os.replace(tmp, path)


def schedules(plan):
    n = ctypes.c_int()
    _lib.check(_lib.load().gbofdft_plan_schedules(plan.handle, ctypes.byref(n)))
    return int(n.value)


def get_schedule(plan):
    n = ctypes.c_int()
    _lib.check(_lib.load().gbofdft_plan_get_schedule(plan.handle, ctypes.byref(n)))
    return int(n.value)


def set_schedule(plan, s):
    _lib.check(_lib.load().gbofdft_plan_set_schedule(plan.handle, int(s)), "plan_set_schedule")


def _time_schedules(plan, reps=20):
    L = _lib.load()
    nr = plan.nr
    dt = torch.float64 if plan.precision == _lib.F64 else torch.float32
    g = torch.Generator(device="cpu").manual_seed(7)
    rho = (0.02 + 0.005 * torch.rand(tuple(nr), generator=g, dtype=torch.float64)).to(device="cuda", dtype=dt)
    vloc = (0.1 * torch.rand(tuple(nr), generator=g, dtype=torch.float64)).to(device="cuda", dtype=dt)
    kern = torch.empty((nr[0], nr[1], nr[2] // 2 + 1), dtype=dt, device="cuda")
    s = _lib.stream_ptr()
    _lib.check(L.gbofdft_wt_kernel(plan.handle, float(rho.mean()), 1.0, 5 / 6, 5 / 6, _lib.ptr(kern), s))
    f = _lib.Functional()
    f.tf, f.tf_x, f.vw, f.vw_y, f.xc, f.hartree = 1, 1.0, 1, 1.0, 1, 1
    f.wt, f.wt_alpha, f.wt_beta, f.wt_kernel = 1, 5 / 6, 5 / 6, kern.data_ptr()
    f.vloc = vloc.data_ptr()
    pot = torch.empty_like(rho)
    st = torch.cuda.current_stream()
    times = []
    for sc in range(schedules(plan)):
        set_schedule(plan, sc)
        for _ in range(3):
            _lib.check(L.gbofdft_eval(plan.handle, _lib.ptr(rho), f, _lib.ptr(pot), None, _lib.CALC_V, s))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(st)
        for _ in range(reps):
            L.gbofdft_eval(plan.handle, _lib.ptr(rho), f, _lib.ptr(pot), None, _lib.CALC_V, s)
        e1.record(st)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / reps)
    return times


def tune(plan, force=False):
    """Choose the fastest schedule for ``plan`` (timed once per grid class
    and process) and set it.  Returns (schedule, per-schedule ms or None)."""
    n = schedules(plan)
    if n <= 1:
        return 0, None
    key = _key(plan)
    with _LOCK:
        if not _CACHE:
            _CACHE.update(_load_file())
        hit = _CACHE.get(key)
        if hit is not None and not force and int(hit["schedule"]) < n:
            set_schedule(plan, int(hit["schedule"]))
            return int(hit["schedule"]), None
        times = _time_schedules(plan)
        best = int(np.argmin(times))
        set_schedule(plan, best)
        _CACHE[key] = {"schedule": best, "ms": [round(t, 5) for t in times]}
        _save_file()
        return best, times
