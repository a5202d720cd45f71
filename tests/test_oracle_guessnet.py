"""The network oracle's operations against finite differences and adjoint
identities (no reference counterpart)."""
import numpy as np

from oracle import guessnet as G


def test_conv_adjoints_and_weight_gradient():
    rng = np.random.default_rng(0)
    x = rng.standard_normal((3, 4, 6, 8))
    w = rng.standard_normal((5, 3, 27))
    b = rng.standard_normal(5)
    g = rng.standard_normal((5, 4, 6, 8))
    y = G.conv3d(x, w, b)
    # <g, conv(x)> = <conv^T(g), x> (bias aside)
    lhs = float((g * (y - b[:, None, None, None])).sum())
    rhs = float((G.conv3d_input_grad(g, w) * x).sum())
    assert abs(lhs - rhs) < 1e-10 * abs(lhs)
    gw, gb = G.conv3d_weight_grad(x, g)
    e = 1e-6
    for (o, i, t) in [(0, 0, 0), (4, 2, 13), (2, 1, 26)]:
        wp = w.copy()
        wp[o, i, t] += e
        wm = w.copy()
        wm[o, i, t] -= e
        fd = float((g * (G.conv3d(x, wp, b) - G.conv3d(x, wm, b))).sum()) / (2 * e)
        assert abs(fd - gw[o, i, t]) < 1e-6 * max(1.0, abs(fd))
    np.testing.assert_allclose(gb, g.sum(axis=(1, 2, 3)))


def test_resampling_adjoints():
    rng = np.random.default_rng(1)
    x = rng.standard_normal((2, 4, 6, 8))
    c = rng.standard_normal((2, 2, 3, 4))
    assert abs(float((G.pool2(x) * c).sum()) - float((x * G.pool2_adjoint(c)).sum())) < 1e-12
    assert abs(float((G.up2(c) * x).sum()) - float((c * G.up2_adjoint(x)).sum())) < 1e-12
    assert abs(float((G.uplin(c) * x).sum()) - float((c * G.uplin_adjoint(x)).sum())) < 1e-12
    # linear upsampling keeps constants and linear-in-index ramps (away from the wrap)
    np.testing.assert_allclose(G.uplin(np.full((1, 2, 3, 4), 1.5)), 1.5)
    ramp = np.arange(4.0)[None, None, None, :] * np.ones((1, 2, 2, 4))
    up = G.uplin(ramp)[0, 0, 0]
    np.testing.assert_allclose(up[1:-1], (np.arange(1, 7) - 0.5) / 2.0)
    z = np.linspace(-4, 4, 101)
    fd = (G.silu(z + 1e-6) - G.silu(z - 1e-6)) / 2e-6
    np.testing.assert_allclose(G.silu_grad(z), fd, rtol=1e-6, atol=1e-9)
