"""The WGC oracle (no reference counterpart, so these are its own checks):
the potential is the functional derivative of the energy, order 0 is the
Wang-Teter term, a uniform density has no nonlocal energy, and the kernels
keep the Lindhard response at the expansion density (the product's and the
oracle's solutions of the kernel equation agree)."""
import numpy as np
import pytest

from oracle import ofdft as O
from oracle import wgc as W


def _density(nr, seed=0):
    rng = np.random.default_rng(seed)
    x = np.linspace(0, 2 * np.pi, nr[0], endpoint=False)
    y = np.linspace(0, 2 * np.pi, nr[1], endpoint=False)
    base = 1 + 0.3 * np.sin(x)[:, None, None] * np.cos(y)[None, :, None]
    return 0.03 * base + 0.002 * rng.random(nr)


@pytest.mark.parametrize("full", [False, True])
@pytest.mark.parametrize("ab", [(W.ALPHA, W.BETA), (5 / 6, 5 / 6)])
def test_potential_is_energy_derivative(full, ab):
    nr = (20, 18, 24)
    L = np.diag([8.0, 7.0, 9.0])
    L[1, 0] = 0.5
    g = O.Grid(L, nr, full=full)
    rho = _density(nr)
    f = W.WGCNL(alpha=ab[0], beta=ab[1], rho0=float(rho.mean()))
    e, v = f(rho, g)
    rng = np.random.default_rng(1)
    h = rng.standard_normal(nr)
    h -= h.mean()
    h *= 1e-3 * rho.std() / h.std()
    eps = 1e-2
    fd = (f(rho + eps * h, g)[0] - f(rho - eps * h, g)[0]) / (2 * eps)
    an = float((v * h).sum() * g.dV)
    assert abs(fd - an) <= 1e-8 * abs(an)


def test_order0_is_wang_teter_and_uniform_limit():
    nr = (16, 20, 18)
    g = O.Grid(np.diag([7.0, 8.0, 7.5]), nr)
    rho = _density(nr, 3)
    e0, v0 = W.WGCNL(alpha=5 / 6, beta=5 / 6, order=0)(rho, g)
    ew, vw = O.WTNL()(rho, g)
    assert abs(e0 - ew) <= 1e-14 * abs(ew)
    assert np.abs(v0 - vw).max() <= 1e-14 * np.abs(vw).max()
    eu, vu = W.WGCNL()(np.full(nr, 0.025), g)
    assert abs(eu) < 1e-25 and np.abs(vu).max() < 1e-14


@pytest.mark.parametrize("order", [1, 2])
@pytest.mark.parametrize("ab", [(W.ALPHA, W.BETA), (5 / 6, 5 / 6)])
def test_kernel_shape_and_response(order, ab):
    """The kernel shape the product tabulates (exponential integrator) and
    the oracle's (backward RK4 / trapezoid) agree, and the oracle's kernels
    keep the Wang-Teter (Lindhard) response at the expansion density:
    a b K0 + (a+b)/6 K1 + Kx = a b K_WT."""
    from dftpy_gb300.functional.wgc import kernel_table
    a, b = ab
    t, w, wt, wtt = W.kernel_shape(a, b, W.GAMMA, 1.0, order)
    t0, h, cols = kernel_table(a, b, W.GAMMA, 1.0, order)
    tp = t0 + h * np.arange(cols.shape[1])
    m = (t > np.log(1e-3)) & (t < np.log(100.0))
    assert np.abs(np.interp(t, tp, cols[0]) - w)[m].max() <= 1e-5 * np.abs(w[m]).max()
    q = np.linspace(0.0, 10.0, 4001)
    K0, K1, Kq, Kx = W.wgc_kernels(q, 0.03, a, b, W.GAMMA, 1.0, order, shape=(t, w, wt, wtt))
    kwt = O.wt_kernel(q, 0.03, 1.0, a, b)
    resp = a * b * K0 + (a + b) / 6.0 * K1 + Kx
    err = np.abs(resp - a * b * kwt)
    assert err.max() <= 1e-4 * np.abs(a * b * kwt).max()
    assert np.median(err) <= 1e-7 * np.abs(a * b * kwt).max()
    if order == 1:
        assert not Kq.any() and not Kx.any()
