"""The allocation-free convolution entry point against the regular one and
against the oracle.

``gbofdft_convolve_noalloc`` serves callers that cannot allocate device
memory (they run under another framework's allocator, or must avoid the
synchronisation cudaMalloc/cudaFree can cause): it needs no plan and keeps its
scratch in a fixed array inside the library.  This test calls it through the
C ABI twice in a row (the second call reuses the array the first one left
behind) and compares each result with ``gbofdft_convolve`` on the same input
and with the oracle's ``ifft(fft(x) * coef * K)``: FP64 within 1e-12 and FP32
within 2e-5 of the output's largest magnitude (times log2 of the longest axis
against the oracle), the tolerances of the convolution tests.  Kernels:
Hartree 4 pi / G^2, G^2, none, and a caller's half-spectrum array (a random
one against the regular entry point; a radial function of |G| against the
oracle, whose ``irfftn`` needs a Hermitian-symmetric spectrum).  It also
checks that a grid whose scratch does not fit is refused with a clear error.
This file sorts last so a run that stops at the first failure has run every
other test first.
"""
import ctypes

import numpy as np
import pytest

from oracle import ofdft as O

pytestmark = pytest.mark.gpu

# (grid, precision 1=f64 0=f32, skewed + full grid, kernel)
CASES = [
    ((32, 32, 32), 1, False, "hartree"),
    ((36, 36, 72), 1, True, "g2"),
    ((36, 36, 72), 0, True, "hartree"),
    ((64, 64, 64), 0, False, "hartree"),
    ((64, 64, 64), 0, False, "array_radial"),
    ((32, 32, 32), 1, False, "array_random"),
    ((96, 96, 96), 1, False, "g2"),
    ((96, 96, 96), 1, False, "none"),
]


def _lattice(nr, skew):
    L = np.diag([7.65 * nr[0] / 32, 7.65 * nr[1] / 32, 7.65 * nr[2] / 32])
    if skew:
        L[1, 0] = 0.4 * L[0, 0]
        L[2, 1] = 0.3 * L[1, 1]
    return L


@pytest.mark.parametrize("nr,prec,skew,kernel", CASES)
def test_noalloc_matches_convolve_and_oracle_twice(nr, prec, skew, kernel):
    import torch
    from dftpy_gb300 import _lib
    _lib.require_cuda()
    L = _lib.load()
    lat = _lattice(nr, skew)
    full = skew
    plan = _lib.Plan(nr, lat, precision=prec, full=full)
    dt = torch.float64 if prec == 1 else torch.float32
    k = {"hartree": _lib.KER_HARTREE, "g2": _lib.KER_G2, "none": _lib.KER_NONE}.get(kernel, _lib.KER_ARRAY)
    g = O.Grid(lat, nr, full=full)
    coef = 0.75
    K = None
    if kernel == "hartree":
        Kref = 4 * np.pi * g.invgg
    elif kernel == "g2":
        Kref = g.gg
    elif kernel == "none":
        Kref = np.ones(g.nrG)
    elif kernel == "array_radial":
        Kref = 1.0 / (1.0 + g.gg) + 0.3 * np.exp(-g.gg / 4.0)
        K = torch.tensor(Kref, dtype=dt, device="cuda")
    else:
        Kref = None
        K = torch.tensor(np.random.default_rng(7).random((nr[0], nr[1], nr[2] // 2 + 1)), dtype=dt, device="cuda")
    nr_c = (ctypes.c_int * 3)(*nr)
    lat_c = (ctypes.c_double * 9)(*[float(x) for x in lat.reshape(9)])
    tol = 1e-12 if prec == 1 else 2e-5
    for call in range(2):
        rng = np.random.default_rng(10 + call)
        xh = rng.random(nr) + 0.1
        x = torch.tensor(xh, dtype=dt, device="cuda")
        ref = torch.empty_like(x)
        _lib.check(L.gbofdft_convolve(plan.handle, _lib.ptr(x), _lib.ptr(ref), k, _lib.ptr(K), coef,
                                      _lib.stream_ptr()))
        out = torch.full_like(x, float("nan"))
        _lib.check(L.gbofdft_convolve_noalloc(nr_c, lat_c, prec, int(full), _lib.ptr(x), _lib.ptr(out), k,
                                              _lib.ptr(K), coef, _lib.stream_ptr()), "convolve_noalloc")
        torch.cuda.synchronize()
        err = float((out - ref).abs().max())
        scale = float(ref.abs().max())
        assert err <= tol * scale, (call, err, scale)
        if Kref is not None:
            ora = O.ifft(O.fft(xh, g) * coef * Kref, g)
            err_o = float(np.abs(out.cpu().numpy() - ora).max())
            assert err_o <= tol * np.abs(ora).max() * np.log2(max(nr)), (call, err_o)


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
