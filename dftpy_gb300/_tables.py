"""Small 1-D set-up tables built on the host (sizes ~1e4 at most).

Grid-sized work never happens here; these are the per-species / per-axis
tables the device kernels interpolate from.
"""
import numpy as np


def spline_notaknot(x, y):
    """Cubic spline through (x, y) with not-a-knot ends.

    ``scipy.interpolate.splrep(x, y, k=3, s=0)`` (FITPACK) builds exactly this
    interpolant (interior knots at x[2..m-3]); here it is computed directly.
    Unknowns are the second derivatives M; the not-a-knot conditions (third
    derivative continuous at x[1] and x[m-2]) express M[0] and M[m-1] through
    their neighbours, which leaves a diagonally dominant tridiagonal system
    for M[1..m-2] (Thomas algorithm).  Returns (x, c) with c[i] = (a, b, c, d)
    of a + b u + c u^2 + d u^3 on [x[i], x[i+1]], u = t - x[i].
    """
    x = np.asarray(x, float)
    y = np.asarray(y, float)
    n = x.size
    if n < 4:
        raise ValueError("spline needs >= 4 points")
    h = np.diff(x)
    delta = np.diff(y) / h
    m = n - 2                                   # unknowns M[1..n-2]
    lo = h[:-1].copy()                          # row j: lo M[j] + di M[j+1] + up M[j+2]
    di = 2.0 * (h[:-1] + h[1:])
    up = h[1:].copy()
    r = 6.0 * (delta[1:] - delta[:-1])
    # M0 = ((h0 + h1) M1 - h0 M2) / h1
    di[0] += h[0] * (h[0] + h[1]) / h[1]
    up[0] -= h[0] * h[0] / h[1]
    # M[n-1] = ((h[n-3] + h[n-2]) M[n-2] - h[n-2] M[n-3]) / h[n-3]
    a, b = h[n - 3], h[n - 2]
    di[m - 1] += b * (a + b) / a
    lo[m - 1] -= b * b / a
    cp = np.zeros(m)
    dp = np.zeros(m)
    cp[0] = up[0] / di[0]
    dp[0] = r[0] / di[0]
    for i in range(1, m):
        den = di[i] - lo[i] * cp[i - 1]
        cp[i] = up[i] / den if i < m - 1 else 0.0
        dp[i] = (r[i] - lo[i] * dp[i - 1]) / den
    M = np.zeros(n)
    M[m] = dp[m - 1]
    for i in range(m - 2, -1, -1):
        M[i + 1] = dp[i] - cp[i] * M[i + 2]
    M[0] = ((h[0] + h[1]) * M[1] - h[0] * M[2]) / h[1]
    M[n - 1] = ((a + b) * M[n - 2] - b * M[n - 3]) / a
    ca = y[:-1]
    cb = delta - h * (2.0 * M[:-1] + M[1:]) / 6.0
    cc = M[:-1] / 2.0
    cd = (M[1:] - M[:-1]) / (6.0 * h)
    return x, np.ascontiguousarray(np.stack([ca, cb, cc, cd], axis=1))


def quartic_coefficients(vp):
    """Coefficients of ``quartic_interpolation`` through (v2, v1, v0, v1, v2)
    (``math_utils.py:457-467``): value = q4[0] + dx (q4[1] + dx (...)) / 24."""
    f = [vp[2], vp[1], vp[0], vp[1], vp[2]]
    t0 = f[2]
    t1 = 2.0 * f[0] - 16.0 * f[1] + 16.0 * f[3] - 2.0 * f[4]
    t2 = -f[0] + 16.0 * f[1] - 30.0 * f[2] + 16.0 * f[3] - f[4]
    t3 = -2.0 * f[0] + 4.0 * f[1] - 4.0 * f[3] + 2.0 * f[4]
    t4 = f[0] - 4.0 * f[1] + 6.0 * f[2] - 4.0 * f[3] + f[4]
    return [t0, t1, t2, t3, t4]


def bspline_mn(x, order, size=None):
    """Cardinal B-spline values M_n(x + k), k = 0..order-1, at index 1..order
    (recursion of ``CBspline.calc_Mn``, ``ewald.py:63-80``)."""
    Mn = np.zeros((order if size is None else size) + 1)
    Mn[1] = x
    Mn[2] = 1.0 - x
    for i in range(3, order + 1):
        for j in range(0, i):
            n = i - j
            Mn[n] = ((x + n - 1) * Mn[n] + (j + 1 - x) * Mn[n - 1]) / (i - 1)
    return Mn


def pme_bm(nr, order=10):
    """PME b(m) factors of the three axes concatenated: axis 0 (n0), axis 1
    (n1), axis 2 (n2//2+1) (``CBspline._calc_bm``, ``ewald.py:82-98``)."""
    Mn = bspline_mn(1.0, order)
    out = []
    lens = (nr[0], nr[1], nr[2] // 2 + 1)
    for i in range(3):
        m = np.arange(lens[i])
        q = 2.0 * np.pi * m / nr[i]
        num = np.exp(-1j * (order - 1.0) * q)
        den = np.zeros_like(num)
        for k in range(1, order):
            den += Mn[k] * np.exp(-1j * k * q)
        out.append(num / den)
    return np.concatenate(out).astype(np.complex128)


# inverse Lindhard function, large-eta series coefficients in 1/eta^2
# (kedf/kernel.py:72-136)
_LIND_LARGE = (-0.13714285714285712, -6.39999999999999875e-2, -3.77825602968460128e-2,
               -2.51824061652633074e-2, -1.80879839616166146e-2, -1.36715733124818332e-2,
               -1.07236045520990083e-2, -8.65192783339199453e-3, -7.1372762502456763e-3,
               -5.9945117538835746e-3, -5.10997527675418131e-3, -4.41060829979912465e-3,
               -3.84763737842981233e-3, -3.38745061493813488e-3, -3.00624946457977689e-3)


def lindhard(eta, lbda, mu, tol=1e-10):
    """Inverse Lindhard function on a 1-D table (``kernel.py:14-136``), the
    same branches as the device evaluation of the WT kernel."""
    eta = np.asarray(eta, float)
    out = eta.copy()
    tol2 = tol / 10
    c0 = (eta > tol2) & (np.abs(eta - 1.0) > tol2)
    e = eta[c0]
    out[c0] = 1.0 / (0.5 + 0.25 * (1.0 - e ** 2) * np.log((1.0 + e) / np.abs(1.0 - e)) / e) - 3.0 * mu * e ** 2 - lbda
    c1 = eta < tol
    e = eta[c1]
    out[c1] = 1.0 - lbda + e ** 2 * (1.0 / 3.0 - 3.0 * mu)
    c2 = np.abs(eta - 1.0) < tol
    e = eta[c2]
    out[c2] = 2.0 - lbda - 3.0 * mu + 20.0 * (e - 1.0)
    c3 = eta > 3.65
    e = eta[c3]
    inv = 1.0 / e ** 2
    s = _LIND_LARGE[-1]
    for c in _LIND_LARGE[-2::-1]:
        s = c + inv * s
    out[c3] = 3.0 * (1.0 - mu) * e ** 2 - lbda - 0.6 + inv * s
    return out


def spline_values_deriv(x, c):
    """First derivative of a ``spline_notaknot`` spline at its knots."""
    d = np.empty(x.size)
    d[:-1] = c[:, 1]
    h = x[-1] - x[-2]
    d[-1] = c[-1, 1] + h * (2.0 * c[-1, 2] + 3.0 * h * c[-1, 3])
    return d
