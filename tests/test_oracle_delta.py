"""The pointwise changes of the delta evaluation (oracle/delta.py, the
formulas the GPU epilogue evaluates in FP32) against float64 differences of
the functions: relative error below 2e-6 of the largest change for density
changes of 1e-5 to 3e-2 relative, on both sides of r_s = 1."""
import numpy as np
import pytest

from oracle import delta as DL


@pytest.mark.parametrize("lo,hi", [(0.002, 0.2), (0.25, 0.6)])
@pytest.mark.parametrize("eps", [1e-5, 1e-3, 3e-2])
def test_pointwise_changes(lo, hi, eps):
    rng = np.random.default_rng(3)
    rho0 = rng.uniform(lo, hi, 50000)
    rho = rho0 * (1.0 + eps * rng.standard_normal(rho0.size))
    rs0, rs = DL.RSC / np.cbrt(rho0), DL.RSC / np.cbrt(rho)
    same = (rs0 < 1) == (rs < 1)
    got = DL.changes(rho, rho0)
    beta = 5.0 / 6.0
    exact = {"p23": rho ** (2 / 3) - rho0 ** (2 / 3), "p53": rho ** (5 / 3) - rho0 ** (5 / 3),
             "pm12": rho ** -0.5 - rho0 ** -0.5, "p12": rho ** 0.5 - rho0 ** 0.5,
             "pbm1": rho ** (beta - 1) - rho0 ** (beta - 1), "pb": rho ** beta - rho0 ** beta}
    v1, e1 = DL.lda(rho)
    v0, e0 = DL.lda(rho0)
    exact["vxc"] = v1 - v0
    exact["exc"] = e1 * rho - e0 * rho0
    for k, ex in exact.items():
        g = got[k].astype(np.float64)[same]
        x = ex[same]
        assert np.abs(g - x).max() <= 2e-6 * np.abs(x).max(), k
