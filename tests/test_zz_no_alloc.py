"""The allocation-free convolution entry point against the regular one.

``gbofdft_convolve_noalloc`` serves callers that cannot allocate device
memory (they run under another framework's allocator, or must avoid the
synchronisation cudaMalloc/cudaFree can cause): it needs no plan and keeps its
scratch in a fixed array inside the library.  This test calls it through the
C ABI twice in a row (the second call reuses the array the first one left
behind) and compares each result with ``gbofdft_convolve`` on the same input:
FP64 within 1e-12 and FP32 within 2e-5 of the output's largest magnitude, the
tolerances of the convolution tests.  It also checks that a grid whose
scratch does not fit is refused with a clear error.  This file sorts last so
a run that stops at the first failure has run every other test first.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CASES = [
    ((32, 32, 32), 1, False, "hartree"),
    ((36, 36, 72), 1, True, "g2"),
    ((64, 64, 64), 0, False, "hartree"),
    ((96, 96, 96), 1, False, "g2"),
]


def _lattice(nr, skew):
    L = np.diag([7.65 * nr[0] / 32, 7.65 * nr[1] / 32, 7.65 * nr[2] / 32])
    if skew:
        L[1, 0] = 0.4 * L[0, 0]
        L[2, 1] = 0.3 * L[1, 1]
    return L


@pytest.mark.parametrize("nr,prec,skew,kernel", CASES)
def test_noalloc_matches_convolve_twice(nr, prec, skew, kernel):
    import torch
    from dftpy_gb300 import _lib
    _lib.require_cuda()
    L = _lib.load()
    lat = _lattice(nr, skew)
    full = skew
    plan = _lib.Plan(nr, lat, precision=prec, full=full)
    dt = torch.float64 if prec == 1 else torch.float32
    k = _lib.KER_HARTREE if kernel == "hartree" else _lib.KER_G2
    nr_c = (ctypes.c_int * 3)(*nr)
    lat_c = (ctypes.c_double * 9)(*[float(x) for x in lat.reshape(9)])
    tol = 1e-12 if prec == 1 else 2e-5
    for call in range(2):
        rng = np.random.default_rng(10 + call)
        x = torch.tensor(rng.random(nr) + 0.1, dtype=dt, device="cuda")
        ref = torch.empty_like(x)
        _lib.check(L.gbofdft_convolve(plan.handle, _lib.ptr(x), _lib.ptr(ref), k, None, 1.0, _lib.stream_ptr()))
        out = torch.full_like(x, float("nan"))
        _lib.check(L.gbofdft_convolve_noalloc(nr_c, lat_c, prec, int(full), _lib.ptr(x), _lib.ptr(out), k, None,
                                              1.0, _lib.stream_ptr()), "convolve_noalloc")
        torch.cuda.synchronize()
        err = float((out - ref).abs().max())
        scale = float(ref.abs().max())
        assert err <= tol * scale, (call, err, scale)


def test_noalloc_rejects_oversized_grid():
    import torch
    from dftpy_gb300 import _lib
    _lib.require_cuda()
    L = _lib.load()
    nr = (256, 256, 256)
    x = torch.zeros(nr, dtype=torch.float64, device="cuda")
    out = torch.empty_like(x)
    rc = L.gbofdft_convolve_noalloc((ctypes.c_int * 3)(*nr), (ctypes.c_double * 9)(20, 0, 0, 0, 20, 0, 0, 0, 20),
                                    1, 0, _lib.ptr(x), _lib.ptr(out), _lib.KER_HARTREE, None, 1.0,
                                    _lib.stream_ptr())
    assert rc == 3
    assert "scratch" in _lib.last_error()
