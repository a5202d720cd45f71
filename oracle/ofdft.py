"""numpy FP64 restatement of DFTpy's OF-DFT energy/potential path and TN solver.

TEST INFRASTRUCTURE ONLY: the checker for the GPU product (see package doc).
References are to DFTpy 2.1.1rc0, paths relative to ``src/dftpy``.

Conventions kept from the reference:
  * real fields are C-order ``float64[n0, n1, n2]``; spectra are the half
    spectrum ``complex128[n0, n1, n2//2+1]`` (``grid.py:45-47``);
  * forward FFT multiplies by dV, inverse divides by dV (``field.py:381,750``)
    on top of numpy's ``rfftn``/``irfftn`` (which carries 1/N);
  * reciprocal lattice ``2 pi inv(L)^T`` in rows (``grid.py:384-415``), G from
    ``fftfreq``/``rfftfreq`` (``grid.py:584-620``), 1/G^2 with G=0 set to 0
    (``grid.py:532-541``).
"""
import math

import numpy as np

ZERO = 1e-30                                            # constants.py:86
C_TF = 0.3 * (3.0 * np.pi ** 2) ** (2.0 / 3.0)          # tf.py:34


# ----------------------------------------------------------------------------
# Grid and FFT
# ----------------------------------------------------------------------------
class Grid:
    """Direct grid + reciprocal grid (``grid.py:291,467``).

    ``full=False``: half spectrum ``(n0, n1, n2//2+1)``, ``rfftn``/``irfftn``.
    ``full=True`` (the reference's ``DirectGrid`` default): full complex
    spectrum with ``fftn`` and the real part of ``ifftn`` (``field.py:159-172,
    702-717``); G uses ``fftfreq`` on every axis, so the Nyquist planes carry
    ``-n/2`` (which matters for non-orthogonal cells).
    """

    def __init__(self, lattice, nr, full=False):
        self.lattice = np.array(lattice, dtype=float).reshape(3, 3)
        self.nr = tuple(int(n) for n in nr)
        self.full = bool(full)
        self.nnr = int(np.prod(self.nr))
        self.volume = abs(float(np.linalg.det(self.lattice)))
        self.dV = self.volume / self.nnr
        self.nrG = self.nr if self.full else (self.nr[0], self.nr[1], self.nr[2] // 2 + 1)
        self.bg = (2.0 * np.pi * np.linalg.inv(self.lattice)).T   # grid.py:404-406
        self._g = None
        self._mask = None

    @property
    def g(self):
        """Cartesian G vectors ``float64[3, *nrG]`` (``grid.py:584-620``)."""
        if self._g is None:
            ax = [np.fft.fftfreq(self.nr[0], d=1.0 / self.nr[0]),
                  np.fft.fftfreq(self.nr[1], d=1.0 / self.nr[1]),
                  (np.fft.fftfreq if self.full else np.fft.rfftfreq)(self.nr[2], d=1.0 / self.nr[2])]
            S = np.asarray(np.meshgrid(*ax, indexing="ij"))
            self._g = np.einsum("j...,jk->k...", S, self.bg)
        return self._g

    @property
    def gg(self):
        return np.einsum("lijk,lijk->ijk", self.g, self.g)

    @property
    def q(self):
        return np.sqrt(self.gg)

    @property
    def invgg(self):
        gg = self.gg
        gg[0, 0, 0] = 1.0
        inv = 1.0 / gg
        inv[0, 0, 0] = 0.0
        return inv

    @property
    def mask(self):
        """Half-space mask counting each +/-G pair once (``grid.py:658-695``)."""
        if self._mask is None:
            n = self.nr
            D = [x // 2 for x in n]
            M = [x % 2 for x in n]
            m = np.ones(self.nrG, dtype=bool)
            if self.full:
                m[:, :, D[2] + 1:] = False
            m[0, D[1] + 1:, 0] = False
            m[D[0] + 1:, :, 0] = False
            if M[2] == 0:
                m[0, 0, D[2]] = False
                m[0, D[1] + 1:, D[2]] = False
                m[D[0] + 1:, :, D[2]] = False
                if M[1] == 0:
                    m[0, D[1], D[2]] = False
                if M[0] == 0:
                    m[D[0], 0, D[2]] = False
                    m[D[0], D[1] + 1:, D[2]] = False
            if M[0] == 0:
                m[D[0], D[1] + 1:, 0] = False
                if M[1] == 0:
                    m[D[0], D[1], 0] = False
            if M[1] == 0:
                m[0, D[1], 0] = False
            if all(x == 0 for x in M):
                m[D[0], D[1], D[2]] = False
            self._mask = m
        return self._mask

    def guess_ecut(self):
        """``DirectGrid.guess_ecut`` (``grid.py:477-480``) + ``spacing2ecut``."""
        lengths = np.sqrt((self.lattice ** 2).sum(axis=1))
        sp1 = lengths / np.array(self.nr)
        sp2 = lengths / (np.array(self.nr) - 1)
        spacing = (0.5 * (sp1 + sp2)).max()
        return np.pi ** 2 / (2.0 * spacing ** 2)        # math_utils.py:331


_FFT_WORKERS = 1


def set_fft_workers(n):
    """Threads for the oracle's FFTs (1: numpy pocketfft, the reference's own
    backend here; >1: scipy's pocketfft with worker threads)."""
    global _FFT_WORKERS
    _FFT_WORKERS = max(1, int(n))


def fft(x, grid):
    """``DirectField.fft`` (``field.py:373-390``)."""
    if _FFT_WORKERS > 1:
        import scipy.fft as sf
        f = sf.fftn if grid.full else sf.rfftn
        return f(x, workers=_FFT_WORKERS) * grid.dV
    if grid.full:
        return np.fft.fftn(x) * grid.dV
    return np.fft.rfftn(x) * grid.dV


def ifft(xg, grid):
    """``ReciprocalField.ifft(force_real=True)`` (``field.py:739-764``)."""
    if _FFT_WORKERS > 1:
        import scipy.fft as sf
        if grid.full:
            return sf.ifftn(xg, workers=_FFT_WORKERS).real / grid.dV
        return sf.irfftn(xg, s=grid.nr, axes=(0, 1, 2), workers=_FFT_WORKERS) / grid.dV
    if grid.full:
        return np.fft.ifftn(xg).real / grid.dV
    return np.fft.irfftn(xg, s=grid.nr, axes=(0, 1, 2)) / grid.dV


# ----------------------------------------------------------------------------
# Cubic spline (the interpolant scipy ``splrep(x, y, k=3, s=0)`` produces)
# ----------------------------------------------------------------------------
def spline_notaknot(x, y):
    """Piecewise-cubic coefficients of the not-a-knot interpolating spline.

    ``splrep(..., s=0, k=3)`` places the interior knots at x[2..m-3], which is
    exactly the not-a-knot interpolant; any method producing that unique
    spline evaluates to the same values.  Returns ``(x, c)`` with
    ``c[i] = (a, b, c, d)`` of ``a + b t + c t^2 + d t^3`` on
    ``[x[i], x[i+1]]``, ``t = u - x[i]``.  Solved for the second derivatives
    with a banded (tridiagonal) solve.
    """
    x = np.asarray(x, float)
    y = np.asarray(y, float)
    n = x.size
    h = np.diff(x)
    delta = np.diff(y) / h
    if n < 4:
        raise ValueError("need >= 4 points")
    # unknown: second derivatives M[0..n-1]; rows 1..n-2 continuity,
    # rows 0 / n-1 not-a-knot (third derivative continuous at x1, x[n-2]).
    # The two end rows have a third entry, eliminated with their neighbour
    # row so the system becomes tridiagonal.
    lo = np.zeros(n)      # sub-diagonal  (row i, col i-1)
    di = np.zeros(n)      # diagonal
    up = np.zeros(n)      # super-diagonal (row i, col i+1)
    r = np.zeros(n)
    lo[1:n - 1] = h[:-1]
    di[1:n - 1] = 2.0 * (h[:-1] + h[1:])
    up[1:n - 1] = h[1:]
    r[1:n - 1] = 6.0 * (delta[1:] - delta[:-1])
    f = h[0] / h[1]
    di[0] = h[1] - f * h[0]
    up[0] = -(h[0] + h[1]) - f * 2.0 * (h[0] + h[1])
    r[0] = -f * r[1]
    f = h[n - 2] / h[n - 3]
    di[n - 1] = h[n - 3] - f * h[n - 2]
    lo[n - 1] = -(h[n - 3] + h[n - 2]) - f * 2.0 * (h[n - 3] + h[n - 2])
    r[n - 1] = -f * r[n - 2]
    from scipy.linalg import solve_banded
    ab = np.zeros((3, n))
    ab[0, 1:] = up[:-1]
    ab[1, :] = di
    ab[2, :-1] = lo[1:]
    M = solve_banded((1, 1), ab, r)
    a = y[:-1]
    b = delta - h * (2.0 * M[:-1] + M[1:]) / 6.0
    c = M[:-1] / 2.0
    d = (M[1:] - M[:-1]) / (6.0 * h)
    return x, np.stack([a, b, c, d], axis=1)


def spline_eval(sp, u):
    """Evaluate a ``spline_notaknot`` spline (extrapolates the end pieces)."""
    x, c = sp
    u = np.asarray(u, float)
    i = np.clip(np.searchsorted(x, u, side="right") - 1, 0, x.size - 2)
    t = u - x[i]
    cc = c[i]
    return cc[..., 0] + t * (cc[..., 1] + t * (cc[..., 2] + t * cc[..., 3]))


def spline_eval_deriv(sp, u):
    x, c = sp
    u = np.asarray(u, float)
    i = np.clip(np.searchsorted(x, u, side="right") - 1, 0, x.size - 2)
    t = u - x[i]
    cc = c[i]
    return cc[..., 1] + t * (2.0 * cc[..., 2] + t * 3.0 * cc[..., 3])


def quartic_interpolation(f, dx):
    """``math_utils.py:457-467``."""
    t0 = f[2]
    t1 = 2.0 * f[0] - 16.0 * f[1] + 16.0 * f[3] - 2.0 * f[4]
    t2 = -f[0] + 16.0 * f[1] - 30.0 * f[2] + 16.0 * f[3] - f[4]
    t3 = -2.0 * f[0] + 4.0 * f[1] - 4.0 * f[3] + 2.0 * f[4]
    t4 = f[0] - 4.0 * f[1] + 6.0 * f[2] - 4.0 * f[3] + f[4]
    return t0 + dx * (t1 + dx * (t2 + dx * (t3 + dx * t4))) / 24.0


# ----------------------------------------------------------------------------
# Kinetic energy functionals
# ----------------------------------------------------------------------------
def tf(rho, grid, x=1.0, calc_e=True):
    """Thomas-Fermi (``kedf/tf.py:13-35,66-80``)."""
    e = None
    if calc_e:
        r5 = rho * rho                                  # PowerInt(rho, 5, 3),
        for _ in range(3):                              # math_utils.py:225-240
            r5 = r5 * rho
        e = float((np.cbrt(r5) * C_TF).sum() * grid.dV * x)
    pot = (3.0 / 10.0) * (5.0 / 3.0) * (3.0 * np.pi ** 2) ** (2.0 / 3.0) * np.cbrt(rho * rho) * x
    return e, pot


def vw(rho, grid, y=1.0, calc_e=True):
    """von Weizsaecker (``kedf/vw.py:29-53,84-94,115-131``)."""
    rhom = rho.copy()
    rhom[~(rho > 0)] = ZERO
    sq = np.sqrt(rhom)
    a = ifft(fft(sq, grid) * grid.gg, grid) * 0.5
    sq[np.abs(sq) < ZERO] = ZERO
    pot = a / sq
    e = None
    if calc_e:
        m = rho > 0
        e = float(np.einsum("i,i->", rho[m], pot[m]) * grid.dV * y)
    return e, pot * y


def lindhard(eta, lbda, mu, tol=1e-10):
    """Inverse Lindhard function (``kedf/kernel.py:14-136``)."""
    eta = np.asarray(eta, float)
    tol2 = tol / 10
    out = eta.copy()
    c0 = (eta > tol2) & (np.abs(eta - 1.0) > tol2)
    c1 = eta < tol
    c2 = np.abs(eta - 1.0) < tol
    c3 = eta > 3.65
    e = eta[c0]
    out[c0] = 1.0 / (0.5 + 0.25 * (1.0 - e ** 2) * np.log((1.0 + e) / np.abs(1.0 - e)) / e) \
        - 3.0 * mu * e ** 2 - lbda
    e = eta[c1]
    out[c1] = 1.0 - lbda + e ** 2 * (1.0 / 3.0 - 3.0 * mu)
    e = eta[c2]
    out[c2] = 2.0 - lbda - 3.0 * mu + 20.0 * (e - 1.0)
    e = eta[c3]
    out[c3] = lindhard_large(e, lbda, mu)
    return out


# large-eta series coefficients of the inverse Lindhard function in 1/eta^2
# (``kernel.py:72-136``)
LINDHARD_LARGE = (-0.13714285714285712, -6.39999999999999875e-2, -3.77825602968460128e-2,
                  -2.51824061652633074e-2, -1.80879839616166146e-2, -1.36715733124818332e-2,
                  -1.07236045520990083e-2, -8.65192783339199453e-3, -7.1372762502456763e-3,
                  -5.9945117538835746e-3, -5.10997527675418131e-3, -4.41060829979912465e-3,
                  -3.84763737842981233e-3, -3.38745061493813488e-3, -3.00624946457977689e-3)


def lindhard_large(eta, lbda, mu):
    inv = 1.0 / eta ** 2
    s = LINDHARD_LARGE[-1]
    for c in LINDHARD_LARGE[-2::-1]:
        s = c + inv * s
    return 3.0 * (1.0 - mu) * eta ** 2 - lbda - 0.6 + inv * s


def wt_kernel(q, rho0, x=1.0, alpha=5.0 / 6.0, beta=5.0 / 6.0):
    """``WTKernel`` (``kernel.py:325-334``): y is always 1 (whole vW removed)."""
    tkf = 2.0 * (3.0 * rho0 * np.pi ** 2) ** (1.0 / 3.0)
    factor = 5.0 / (9.0 * alpha * beta * rho0 ** (alpha + beta - 5.0 / 3.0)) * C_TF
    return lindhard(q / tkf, x, 1.0) * factor


class WTNL:
    """Wang-Teter nonlocal term (``kedf/wt.py:12-28,58-73,109-132``).

    Keeps the reference's kernel cache: the kernel is rebuilt only when the
    mean density moves by more than 1e-6 (``wt.py:63``).
    """

    def __init__(self, x=1.0, alpha=5.0 / 6.0, beta=5.0 / 6.0):
        self.x, self.alpha, self.beta = x, alpha, beta
        self.rho0 = 0.0
        self.shape = None
        self.kernel = None

    def get_kernel(self, rho, grid):
        rho0 = float(rho.mean())
        if abs(self.rho0 - rho0) > 1e-6 or rho.shape != self.shape:
            self.kernel = wt_kernel(grid.q, rho0, self.x, self.alpha, self.beta)
            self.rho0 = rho0
            self.shape = rho.shape
        return self.kernel

    def __call__(self, rho, grid, calc_e=True):
        K = self.get_kernel(rho, grid)
        a = self.alpha
        rc = np.where(rho < ZERO, ZERO, rho)
        rb = rc ** self.beta
        if abs(self.beta - a) < 1e-9:
            pot = 2.0 * a * (rb / rc) * ifft(fft(rb, grid) * K, grid)
        else:
            pot = a * rc ** (a - 1.0) * ifft(fft(rb, grid) * K, grid)
            pot += self.beta * rc ** (self.beta - 1.0) * ifft(fft(rc ** a, grid) * K, grid)
        e = None
        if calc_e:
            e = float((pot * rho / (2.0 * a)).sum() * grid.dV)
        return e, pot


# ----------------------------------------------------------------------------
# XC, Hartree
# ----------------------------------------------------------------------------
PZ = dict(a=0.0311, b=-0.048, c=0.0020, d=-0.0116, gamma=-0.1423, beta1=1.0529, beta2=0.3334)


def lda(rho, grid, calc_e=True):
    """Perdew-Zunger LDA, unpolarised (``xc/semilocal_xc.py:253-290``)."""
    a, b, c, d = PZ["a"], PZ["b"], PZ["c"], PZ["d"]
    g, b1, b2 = PZ["gamma"], PZ["beta1"], PZ["beta2"]
    rc = np.cbrt(rho)
    rc[rc < ZERO] = ZERO
    Rs = np.cbrt(3.0 / (4.0 * np.pi)) / rc
    r1 = Rs < 1
    r2 = ~r1
    sq = np.sqrt(Rs[r2])
    e = None
    if calc_e:
        ex = -3.0 / 4.0 * np.cbrt(3.0 / np.pi) * rc
        ex[r1] += a * np.log(Rs[r1]) + b + c * Rs[r1] * np.log(Rs[r1]) + d * Rs[r1]
        ex[r2] += g / (1.0 + b1 * sq + b2 * Rs[r2])
        e = float(np.einsum("ijk,ijk->", ex, rho) * grid.dV)
    pot = np.cbrt(-3.0 / np.pi) * rc
    pot[r1] += np.log(Rs[r1]) * (a + 2.0 / 3 * c * Rs[r1]) + b - 1.0 / 3 * a + 1.0 / 3 * (2 * d - c) * Rs[r1]
    pot[r2] += (g + (7.0 / 6.0 * g * b1) * sq + (4.0 / 3.0 * g * b2 * Rs[r2])) / (1.0 + b1 * sq + b2 * Rs[r2]) ** 2
    return e, pot


def hartree(rho, grid, calc_e=True):
    """``functional/hartree.py:24-45``."""
    v = ifft(fft(rho, grid) * grid.invgg * 4.0 * np.pi, grid)
    e = float(np.einsum("ijk,ijk->", v, rho) * grid.dV / 2.0) if calc_e else None
    return e, v


# ----------------------------------------------------------------------------
# Local pseudopotential: v(|G|) table, PME / exact structure factor
# ----------------------------------------------------------------------------
def vline(q, gp, vp):
    """``LocalPseudo.calc_vlines`` (``pseudo/__init__.py:350-375``).

    Cubic spline of vp[1:] on gp[1:] for q < gp[-1] (0 beyond), quartic patch
    through (vp2, vp1, vp0, vp1, vp2) for q < gp[1].
    """
    sp = spline_notaknot(gp[1:], vp[1:])
    out = np.zeros_like(q)
    m = q < gp[-1]
    out[m] = spline_eval(sp, q[m])
    m = q < gp[1]
    dp = gp[1] - gp[0]
    out[m] = quartic_interpolation([vp[2], vp[1], vp[0], vp[1], vp[2]], q[m] / dp)
    return out


def bspline_mn(x, order=10, size=None):
    """``CBspline.calc_Mn`` (``ewald.py:63-80``); index 0 unused.

    The reference sizes the array by the spline's own order even when asked
    for a lower order (``size``), leaving the tail at zero.
    """
    Mn = np.zeros((order if size is None else size) + 1)
    Mn[1] = x
    Mn[2] = 1.0 - x
    for i in range(3, order + 1):
        for j in range(0, i):
            n = i - j
            Mn[n] = ((x + n - 1) * Mn[n] + (j + 1 - x) * Mn[n - 1]) / (i - 1)
    return Mn


def bspline_barray(grid, order=10):
    """``CBspline._calc_bm`` / ``Barray`` (``ewald.py:48-61,82-98``)."""
    Mn = bspline_mn(1.0, order)
    bm = []
    for i in range(3):
        m = np.arange(grid.nrG[i])
        qv = 2.0 * np.pi * m / grid.nr[i]
        num = np.exp(-1j * (order - 1.0) * qv)
        den = np.zeros_like(num)
        for k in range(1, order):
            den += Mn[k] * np.exp(-1j * k * qv)
        bm.append(num / den)
    return np.einsum("i,j,k->ijk", bm[0], bm[1], bm[2])


def pme_qarray(grid, scaled_positions, weights, order=10):
    """``CBspline.get_PME_Qarray`` (``ewald.py:172-195``), summed over atoms."""
    Q = np.zeros(grid.nr)
    nr = np.array(grid.nr)
    ia = np.arange(order)
    for s, w in zip(scaled_positions, weights):
        Up = s * nr
        fl = np.floor(Up)
        M = [bspline_mn(Up[d] - fl[d], order)[1:] for d in range(3)]
        l = [np.mod(1 + int(fl[d]) - ia, nr[d]) for d in range(3)]
        Q[np.ix_(l[0], l[1], l[2])] += w * np.einsum("i,j,k->ijk", M[0], M[1], M[2])
    return Q


def local_pp_recip(grid, positions, symbols, tables, pme=True, order=10):
    """v_loc(G) (``pseudo/__init__.py:377-404``). ``tables[sym] = (gp, vp)``."""
    q = grid.q
    v = np.zeros(grid.nrG, dtype=np.complex128)
    lat = grid.lattice
    spos = np.linalg.solve(lat.T, np.asarray(positions).T).T % 1.0
    for key in sorted(set(symbols)):
        vl = vline(q, *tables[key])
        idx = [i for i, s in enumerate(symbols) if s == key]
        if pme:
            Q = pme_qarray(grid, spos[idx], np.ones(len(idx)), order)
            v = v + vl * fft(Q, grid)
        else:
            g = grid.g
            for i in idx:
                v += vl * np.exp(-1j * np.einsum("lijk,l->ijk", g, positions[i]))
    if pme:
        v = v * bspline_barray(grid, order) * grid.nnr / grid.volume
    return v


def radial_to_3d(q, table):
    """``RadialGrid.to_3d_grid`` (``grid.py:766-779``): interpolating cubic
    spline of the (|G|, value) table, 0 outside [q[0], q[-1])."""
    gp, vp = (np.asarray(t, float) for t in table)
    sp = spline_notaknot(gp, vp)
    out = np.zeros_like(q)
    m = (q < gp[-1]) & (q >= gp[0])
    out[m] = spline_eval(sp, q[m])
    return out


def density_guess_recipe(grid, positions, symbols, tables, ncharge, pme=True, order=10, dtol=1e-30):
    """``get_3d_value_recipe`` with ``direct=True`` (``density/density.py:252-300``):
    superposed reciprocal-space atomic tables, inverse transform, clamp at
    ``dtol``, scale to ``ncharge``."""
    q = grid.q
    rg = np.zeros(grid.nrG, dtype=np.complex128)
    spos = np.linalg.solve(grid.lattice.T, np.asarray(positions).T).T % 1.0
    for key in sorted(set(symbols)):
        line = radial_to_3d(q, tables[key])
        idx = [i for i, s in enumerate(symbols) if s == key]
        if pme:
            Q = pme_qarray(grid, spos[idx], np.ones(len(idx)), order)
            rg = rg + line * fft(Q, grid)
        else:
            g = grid.g
            for i in idx:
                rg += line * np.exp(-1j * np.einsum("lijk,l->ijk", g, positions[i]))
    if pme:
        rg = rg * bspline_barray(grid, order) * grid.nnr / grid.volume
    rho = ifft(rg, grid)
    rho[rho < dtol] = dtol
    nc = rho.sum() * grid.dV
    if ncharge > 1e-6:
        rho = rho * (ncharge / nc)
    return rho


def local_pp(grid, positions, symbols, tables, pme=True, order=10):
    """Real-space v_loc (``LocalPseudo.local_PP``, ``pseudo/__init__.py:237-246``)."""
    return ifft(local_pp_recip(grid, positions, symbols, tables, pme, order), grid)


def pp_forces_pme(rho, grid, positions, symbols, tables, order=10):
    """``LocalPseudo._ForcePME`` (``pseudo/__init__.py:475-523``)."""
    rhoG = fft(rho, grid)
    B = np.conj(bspline_barray(grid, order))
    denG = rhoG * B
    nr = np.array(grid.nr)
    cell_inv = (grid.bg / (2.0 * np.pi)).T       # reciprocal lattice^T / 2pi
    spos = np.linalg.solve(grid.lattice.T, np.asarray(positions).T).T % 1.0
    F = np.zeros((len(symbols), 3))
    q = grid.q
    ia = np.arange(order)
    for key in sorted(set(symbols)):
        dg = denG * vline(q, *tables[key])
        dg[0, 0, 0] = 0.0
        rhoPB = ifft(dg, grid)
        for i, s in enumerate(symbols):
            if s != key:
                continue
            Up = spos[i] * nr
            fl = np.floor(Up)
            M = [bspline_mn(Up[d] - fl[d], order) for d in range(3)]
            M2 = [bspline_mn(Up[d] - fl[d], order - 1, order) for d in range(3)]
            dM = [M2[d][1:] - M2[d][:-1] for d in range(3)]
            Mv = [M[d][1:] for d in range(3)]
            QD = np.stack([
                nr[0] * np.einsum("i,j,k->ijk", dM[0], Mv[1], Mv[2]),
                nr[1] * np.einsum("i,j,k->ijk", Mv[0], dM[1], Mv[2]),
                nr[2] * np.einsum("i,j,k->ijk", Mv[0], Mv[1], dM[2])]).reshape(3, -1)
            l = [np.mod(1 + int(fl[d]) - ia, nr[d]) for d in range(3)]
            vals = rhoPB[np.ix_(l[0], l[1], l[2])].ravel()
            F[i] = -np.sum((QD.T @ cell_inv) * vals[:, None], axis=0)
    return F


def pp_forces_exact(rho, grid, positions, symbols, tables):
    """``LocalPseudo._Force`` (``pseudo/__init__.py:457-473``): exact structure
    factor over the half-space mask, ``2/Omega sum G vline Im(rhoG e^{+iG.R})``."""
    rhoG = fft(rho, grid)
    g = grid.g
    mask = grid.mask
    q = grid.q
    F = np.zeros((len(symbols), 3))
    vls = {key: vline(q, *tables[key]) for key in set(symbols)}
    for i, s in enumerate(symbols):
        istrf = np.exp(1j * np.einsum("lijk,l->ijk", g, positions[i]))
        den = vls[s][mask] * (rhoG[mask] * istrf[mask]).imag
        for j in range(3):
            F[i, j] = np.einsum("i,i->", g[j][mask], den)
    return F * 2.0 / grid.volume


# ----------------------------------------------------------------------------
# Ewald (ion-ion), PME or exact reciprocal part
# ----------------------------------------------------------------------------
def ewald_eta(grid, charges, precision=1e-8):
    """``ewald.Get_Best_eta`` (``ewald.py:256-279``); gmax from ``g2max = 2 ecut``."""
    from scipy.special import erfc
    gmax = math.sqrt(2.0 * grid.guess_ecut())
    chargeSquare = float(np.sum(charges * charges))
    nat = len(charges)
    eta = 1.6
    while True:
        up = 4.0 * np.pi * nat * chargeSquare * np.sqrt(eta / np.pi) * erfc(gmax / 2.0 * np.sqrt(1.0 / eta))
        if up < precision:
            return eta
        eta = eta - 0.01


def _images(grid, rmax):
    L = np.sqrt((grid.lattice ** 2).sum(axis=1))
    N = np.ceil(rmax / L).astype(int)
    rng = [np.arange(-N[d], N[d] + 1) for d in range(3)]
    I = np.array(np.meshgrid(*rng, indexing="ij")).reshape(3, -1).T.astype(float)
    return I @ grid.lattice


def ewald_energy(grid, positions, charges, pme=True, precision=1e-8, order=10):
    """``ewald.energy`` (``ewald.py:486-508``): corr + real + rec."""
    from scipy.special import erfc, erfcinv
    pos = np.asarray(positions, float)
    charges = np.asarray(charges, float)
    eta = ewald_eta(grid, charges, precision)
    # Energy_corr (ewald.py:468-484)
    e_corr = -np.sqrt(eta / np.pi) * np.sum(charges ** 2)
    e_corr += -4.0 * np.pi * (1.0 / (4.0 * eta * grid.volume) / 2.0) * charges.sum() ** 2
    # Energy_real (ewald.py:281-317): pairs and images with 1e-3 < d < rmax
    rmax = erfcinv(precision / 3.0) / np.sqrt(eta)
    R = _images(grid, rmax)
    se = np.sqrt(eta)
    e_real = 0.0
    for i in range(len(charges)):
        d = pos[i][None, None, :] - (pos[None, :, :] - R[:, None, :])
        dist = np.sqrt((d * d).sum(axis=-1))
        m = (dist < rmax) & (dist > 0.001)
        qq = np.broadcast_to(charges[None, :], dist.shape)
        e_real += charges[i] * np.sum(qq[m] * erfc(se * dist[m]) / dist[m])
    e_real /= 2.0
    # Energy_rec (ewald.py:449-466) / Energy_rec_PME (ewald.py:786-808)
    gg = grid.gg
    invgg = grid.invgg
    mask = grid.mask
    if pme:
        spos = np.linalg.solve(grid.lattice.T, pos.T).T % 1.0
        Q = pme_qarray(grid, spos, charges, order)
        strf = fft(Q, grid) * bspline_barray(grid, order)
        s2 = (np.conj(strf) * strf).real
        e_rec = np.sum(s2[mask] * np.exp(-gg[mask] / (4.0 * eta)) * invgg[mask])
        e_rec = 4.0 * np.pi * e_rec / grid.volume / grid.dV ** 2
    else:
        g = grid.g
        strf = np.zeros(grid.nrG, dtype=complex)
        for i in range(len(charges)):
            strf += np.exp(-1j * np.einsum("lijk,l->ijk", g, pos[i])) * charges[i]
        s2 = (np.conj(strf) * strf).real
        e_rec = 4.0 * np.pi * np.sum(s2[mask] * np.exp(-gg[mask] / (4.0 * eta)) * invgg[mask]) / grid.volume
    return dict(energy=float(e_corr + e_real + e_rec), corr=float(e_corr), real=float(e_real),
                rec=float(e_rec), eta=eta)


def ewald_forces(grid, positions, charges, pme=True, precision=1e-8, order=10):
    """``ewald.forces`` (``ewald.py:510-521``): ``Forces_real`` + rec (PME or exact)."""
    from scipy.special import erfc, erfcinv
    pos = np.asarray(positions, float)
    charges = np.asarray(charges, float)
    eta = ewald_eta(grid, charges, precision)
    rmax = erfcinv(precision / 3.0) / np.sqrt(eta)
    R = _images(grid, rmax)
    se = np.sqrt(eta)
    nat = len(charges)
    F = np.zeros((nat, 3))
    for i in range(nat):                                   # ewald.py:541-575
        d = pos[i][None, None, :] - (pos[None, :, :] - R[:, None, :])
        dist = np.sqrt((d * d).sum(axis=-1))
        m = (dist < rmax) & (dist > 0.001)
        x = dist[m] * se
        qq = np.broadcast_to(charges[None, :], dist.shape)[m]
        w = erfc(x) / x ** 3 + 2.0 / np.sqrt(np.pi) * np.exp(-x ** 2) / x ** 2
        F[i] = charges[i] * np.einsum("ij,i->j", d[m] * qq[:, None], w)
    F *= se ** 3
    gg = grid.gg
    invgg = grid.invgg
    if pme:                                                # ewald.py:810-857
        spos = np.linalg.solve(grid.lattice.T, pos.T).T % 1.0
        Q = pme_qarray(grid, spos, charges, order)
        B = bspline_barray(grid, order)
        strf = fft(Q, grid) * (B * np.conj(B))
        strf = ifft(strf * np.exp(-gg / (4.0 * eta)) * invgg, grid)
        nr = np.array(grid.nr)
        cell_inv = np.linalg.inv(grid.lattice)
        ia = np.arange(order)
        for i in range(nat):
            Up = spos[i] * nr
            fl = np.floor(Up)
            M = [bspline_mn(Up[d] - fl[d], order) for d in range(3)]
            M2 = [bspline_mn(Up[d] - fl[d], order - 1, order) for d in range(3)]
            dM = [M2[d][1:] - M2[d][:-1] for d in range(3)]
            Mv = [M[d][1:] for d in range(3)]
            QD = np.stack([
                nr[0] * np.einsum("i,j,k->ijk", dM[0], Mv[1], Mv[2]),
                nr[1] * np.einsum("i,j,k->ijk", Mv[0], dM[1], Mv[2]),
                nr[2] * np.einsum("i,j,k->ijk", Mv[0], Mv[1], dM[2])]).reshape(3, -1)
            l = [np.mod(1 + int(fl[d]) - ia, nr[d]) for d in range(3)]
            vals = strf[np.ix_(l[0], l[1], l[2])].ravel()
            F[i] -= charges[i] * np.sum((QD.T @ cell_inv) * vals[:, None], axis=0) * 4.0 * np.pi / grid.dV
    else:                                                  # ewald.py:578-604
        g = grid.g
        mask = grid.mask
        strf = np.zeros(grid.nrG, dtype=complex)
        sfs = []
        for i in range(nat):
            s = np.exp(-1j * np.einsum("lijk,l->ijk", g, pos[i])) * charges[i]
            sfs.append(s)
            strf += s
        w = np.exp(-gg[mask] / (4.0 * eta)) * invgg[mask]
        for i in range(nat):
            s = sfs[i]
            F[i] += np.einsum("ij,j->i", g[:, mask], (s.real[mask] * strf.imag[mask]
                                                       - s.imag[mask] * strf.real[mask]) * w) \
                * 8.0 * np.pi / grid.volume
    return F


# ----------------------------------------------------------------------------
# Stress (3 x 3, Ha/Bohr^3)
# ----------------------------------------------------------------------------
def _invq(grid):
    q = grid.q.copy()
    z = q == 0
    q[z] = 1.0
    out = 1.0 / q
    out[z] = 0.0
    return out


def _sym(s):
    for i in range(3):
        for j in range(i):
            s[i, j] = s[j, i]
    return s


def lindhard_derivative(eta, mu):
    """``LindhardDerivative`` (``kedf/kernel.py:197-211``)."""
    eta = np.asarray(eta, float)
    out = np.zeros_like(eta)
    atol = 1.0e-10
    c0 = (eta > atol) & (np.abs(eta - 1.0) > atol)
    c1 = eta < atol
    c2 = np.abs(eta - 1.0) < atol
    e = eta[c0]
    t = np.log(np.abs((1.0 + e) / (1.0 - e)))
    out[c0] = (0.5 / e - 0.25 * (e ** 2 + 1.0) / e ** 2 * t) / (0.5 + 0.25 * (1 - e ** 2) / e * t) ** 2 \
        + 6.0 * e * mu
    out[c1] = -2.0 * eta[c1] * (1.0 / 3.0 - 3.0 * mu)
    out[c2] = -48
    return out * eta


def stress_tf(energy, grid):
    """``ThomasFermiStress`` (``kedf/tf.py:52-62``)."""
    return np.eye(3) * (-2.0 / 3.0 * energy / grid.volume)


def stress_vw(rho, grid, y=1.0):
    """``vonWeizsackerStress`` (``kedf/vw.py:97-112``)."""
    g = grid.g
    rhoG = fft(rho, grid)
    d = [ifft(1j * g[i] * rhoG, grid) for i in range(3)]
    s = np.zeros((3, 3))
    for i in range(3):
        for j in range(i, 3):
            s[i, j] = -0.25 / grid.volume * grid.dV * np.einsum("ijk->", d[i] * d[j] / rho) * y
    return _sym(s)


def stress_wt(rho, grid, energy, y=1.0, alpha=5.0 / 6.0, beta=5.0 / 6.0):
    """``WTStress`` (``kedf/wt.py:75-105``)."""
    rho0 = rho.mean()
    g, invgg, q, mask = grid.g, grid.invgg, grid.q, grid.mask
    tkf = float(2.0 * (3.0 * rho0 * np.pi ** 2) ** (1.0 / 3.0))
    A = fft(rho ** alpha, grid) / grid.volume
    B = np.conj(fft(rho ** beta, grid)) / grid.volume
    dd = lindhard_derivative(q / tkf, y) * A * B
    s = np.zeros((3, 3))
    for i in range(3):
        for j in range(i, 3):
            fac = 1.0 / 3.0 if i == j else 0.0
            s[i, j] = np.sum((g[i][mask] * g[j][mask] * invgg[mask] - fac) * dd[mask]).real
    s = _sym(s) * (np.pi ** 2 / (alpha * beta * rho0 ** (alpha + beta - 2) * tkf / 2.0))
    return s - np.eye(3) * (2.0 / 3.0 * energy / grid.volume)


def stress_lda(rho, grid, energy, pot):
    """``LDAStress`` (``xc/semilocal_xc.py:308-322``)."""
    return np.eye(3) * ((energy - np.einsum("ijk,ijk->", pot, rho) * grid.dV) / grid.volume)


def stress_hartree(rho, grid, energy):
    """``HartreeFunctionalStress`` (``hartree.py:68-90``)."""
    g, invgg, mask = grid.g, grid.invgg, grid.mask
    rhoG = fft(rho, grid)
    r2 = (rhoG * np.conj(rhoG) * invgg * invgg).real
    s = np.zeros((3, 3))
    for i in range(3):
        for j in range(i, 3):
            s[i, j] = np.sum(g[i][mask] * g[j][mask] * r2[mask]) * 8.0 * np.pi / grid.volume ** 2
    return _sym(s) - np.eye(3) * energy / grid.volume


def _vline_deriv(q, table):
    """``_PP_Derivative_One`` (``pseudo/__init__.py:406-412``): d/dq of the
    spline of vp[1:] on gp[1:] (its first piece extrapolated below gp[1]),
    0 from gp[-1] on."""
    gp, vp = (np.asarray(t, float) for t in table)
    sp = spline_notaknot(gp[1:], vp[1:])
    out = np.zeros_like(q)
    m = q < gp.max()
    out[m] = spline_eval_deriv(sp, q[m])
    return out


def stress_pp_pme(rho, grid, positions, symbols, tables, energy, order=10):
    """``LocalPseudo._StressPME`` (``pseudo/__init__.py:525-562``)."""
    g, mask, q = grid.g, grid.mask, grid.q
    invq = _invq(grid)
    rhoGB = np.conj(fft(rho, grid)) * bspline_barray(grid, order)
    spos = np.linalg.solve(grid.lattice.T, np.asarray(positions).T).T % 1.0
    s = np.zeros((3, 3))
    for key in sorted(set(symbols)):
        idx = [i for i, x in enumerate(symbols) if x == key]
        Q = pme_qarray(grid, spos[idx], np.ones(len(idx)), order)
        v = rhoGB * _vline_deriv(q, tables[key]) * fft(Q, grid)
        for i in range(3):
            for j in range(i, 3):
                s[i, j] -= np.sum(g[i][mask] * g[j][mask] * v[mask] * invq[mask]).real / grid.volume ** 2
    s *= 2.0 * grid.nnr
    s = _sym(s) - np.eye(3) * energy
    return s / grid.volume


def stress_pp_exact(rho, grid, positions, symbols, tables, energy):
    """``LocalPseudo._Stress`` (``pseudo/__init__.py:431-455``)."""
    g, mask, q = grid.g, grid.mask, grid.q
    invq = _invq(grid)
    v = np.zeros(grid.nrG, dtype=np.complex128)
    for key in sorted(set(symbols)):
        dv = _vline_deriv(q, tables[key])
        for i, x in enumerate(symbols):
            if x == key:
                v += dv * np.conj(np.exp(-1j * np.einsum("lijk,l->ijk", g, positions[i])))
    rv = fft(rho, grid) * v * invq
    s = np.zeros((3, 3))
    for i in range(3):
        for j in range(i, 3):
            s[i, j] = -np.sum(g[i][mask] * g[j][mask] * rv[mask]).real / grid.volume * 2.0
    s = _sym(s) - np.eye(3) * energy
    return s / grid.volume


def ewald_stress(grid, positions, charges, pme=True, precision=1e-8, order=10):
    """``ewald.stress`` (``ewald.py:523-538``): ``Stress_real`` (``:609-662``) +
    ``Stress_rec_PME`` (``:915-963``) or ``Stress_rec`` (``:719-760``)."""
    from scipy.special import erfc, erfcinv
    pos = np.asarray(positions, float)
    charges = np.asarray(charges, float)
    eta = ewald_eta(grid, charges, precision)
    rmax = erfcinv(precision / 3.0) / np.sqrt(eta)
    R = _images(grid, rmax)
    se = np.sqrt(eta)
    st = np.zeros(6)
    for ia in range(len(charges)):
        d = pos[ia][None, None, :] - (pos[None, :, :] - R[:, None, :])
        dist = np.sqrt((d * d).sum(axis=-1))
        m = (dist < rmax) & (dist > 0.001)
        rij, rr = d[m], dist[m]
        qq = np.broadcast_to(charges[None, :], dist.shape)[m]
        w = qq * (2 * se / np.sqrt(np.pi) * np.exp(-eta * rr ** 2) + erfc(se * rr) / rr)
        k = 0
        for i in range(3):
            for j in range(i, 3):
                st[k] += charges[ia] * np.sum(w * rij[:, i] * rij[:, j] / rr ** 2)
                k += 1
    st *= -0.5 / grid.volume
    s = np.zeros((3, 3))
    k = 0
    for i in range(3):
        for j in range(i, 3):
            s[i, j] = st[k]
            k += 1
    g, gg, invgg, mask = grid.g, grid.gg, grid.invgg, grid.mask
    if pme:
        spos = np.linalg.solve(grid.lattice.T, pos.T).T % 1.0
        strf = fft(pme_qarray(grid, spos, charges, order), grid) * bspline_barray(grid, order)
        scale = 2.0 * 2.0 * np.pi / grid.volume ** 2 / grid.dV ** 2
    else:
        strf = np.zeros(grid.nrG, dtype=complex)
        for i in range(len(charges)):
            strf += np.exp(-1j * np.einsum("lijk,l->ijk", g, pos[i])) * charges[i]
        scale = 4.0 * np.pi / grid.volume ** 2
    s2 = (np.conj(strf) * strf).real
    w = s2[mask] * np.exp(-gg[mask] / (4.0 * eta)) * invgg[mask]
    k = 0
    for i in range(3):
        for j in range(i, 3):
            f = g[i][mask] * g[j][mask] * 2.0 * invgg[mask] * (1 + gg[mask] / (4.0 * eta))
            if i == j:
                f = f - 1.0
            s[i, j] += np.sum(w * f) * scale
            k += 1
    s_g0 = charges.sum() ** 2 * 4.0 * np.pi * (1.0 / (4.0 * eta * grid.volume ** 2) / 2.0)
    s += np.eye(3) * s_g0
    return _sym(s)


# ----------------------------------------------------------------------------
# Total functional
# ----------------------------------------------------------------------------
class OFDFT:
    """KEDF (TF/vW/WT) + LDA + Hartree + local PP + Ewald (``total_functional.py:115-146``).

    ``kedf``: "TFVW" or "WT" (``kedf/__init__.py:27-69`` name table).
    """

    def __init__(self, lattice, nr, positions, symbols, kedf="WT", pme=True, tables=None,
                 x=1.0, y=1.0, alpha=5.0 / 6.0, beta=5.0 / 6.0):
        from dftpy_gb300 import systems
        self.grid = Grid(lattice, nr)
        self.positions = np.asarray(positions, float)
        self.symbols = list(symbols)
        self.kedf = kedf.upper()
        self.x, self.y = x, y
        if tables is None:
            tables = {s: systems.analytic_pp_table(*systems.SPECIES[s]) for s in set(self.symbols)}
        self.tables = tables
        self.charges = np.array([systems.SPECIES[s][0] for s in self.symbols])
        self.pme = pme
        self.vloc = local_pp(self.grid, self.positions, self.symbols, tables, pme=pme)
        self.ewald = ewald_energy(self.grid, self.positions, self.charges, pme=pme)
        self.wt = WTNL(x=x, alpha=alpha, beta=beta) if self.kedf == "WT" else None
        self.n_eval = {"EV": 0, "V": 0}

    def components(self, rho, calc_e=True):
        g = self.grid
        out = {}
        out["TF"] = tf(rho, g, self.x, calc_e)
        out["VW"] = vw(rho, g, self.y, calc_e)
        if self.wt is not None:
            out["WT"] = self.wt(rho, g, calc_e)
        out["XC"] = lda(rho, g, calc_e)
        out["HARTREE"] = hartree(rho, g, calc_e)
        e_pp = float(np.einsum("ijk,ijk->", self.vloc, rho) * g.dV) if calc_e else None
        out["PSEUDO"] = (e_pp, self.vloc)
        return out

    def __call__(self, rho, calc_e=True):
        """Returns (energy or None, potential)."""
        self.n_eval["EV" if calc_e else "V"] += 1
        comps = self.components(rho, calc_e)
        pot = np.zeros_like(rho)
        for k in comps:
            pot += comps[k][1]
        if not calc_e:
            return None, pot
        e = sum(comps[k][0] for k in comps) + self.ewald["energy"]
        return float(e), pot

    def stress(self, rho, split=False):
        """``TotalFunctional.get_stress`` (``total_functional.py:176-209``)."""
        g = self.grid
        comps = self.components(rho, True)
        out = {"KEDF-TF": stress_tf(comps["TF"][0], g), "KEDF-VW": stress_vw(rho, g, self.y)}
        if self.wt is not None:
            out["KEDF-NL"] = stress_wt(rho, g, comps["WT"][0], 1.0, self.wt.alpha, self.wt.beta)
        out["XC"] = stress_lda(rho, g, comps["XC"][0], comps["XC"][1])
        out["HARTREE"] = stress_hartree(rho, g, comps["HARTREE"][0])
        f = stress_pp_pme if self.pme else stress_pp_exact
        out["PSEUDO"] = f(rho, g, self.positions, self.symbols, self.tables, comps["PSEUDO"][0])
        out["II"] = ewald_stress(g, self.positions, self.charges, pme=self.pme)
        out["TOTAL"] = sum(out.values())
        return out if split else out["TOTAL"]

    def forces(self, rho):
        """``TotalFunctional.get_forces`` (``total_functional.py:148-174``), PME."""
        f = pp_forces_pme(rho, self.grid, self.positions, self.symbols, self.tables) if self.pme else None
        return f + ewald_forces(self.grid, self.positions, self.charges, pme=self.pme)


# ----------------------------------------------------------------------------
# More-Thuente line search (MINPACK-2 dcsrch/dcstep algorithm)
# ----------------------------------------------------------------------------
class DCSRCH:
    """Reverse-communication line search of Moré & Thuente, ACM TOMS 20 (1994).

    Same state machine the reference drives through ``minpack2.dcsrch``
    (``math_utils.py:76-106``): call ``step(stp, f, g)`` with task "START"
    first; it returns ``(stp, task)`` with task "FG" (evaluate at stp),
    "CONVERGENCE", "WARNING..." or "ERROR...".
    """
    XTRAPL, XTRAPU, P5, P66 = 1.1, 4.0, 0.5, 0.66

    def __init__(self, ftol, gtol, xtol, stpmin, stpmax):
        self.ftol, self.gtol, self.xtol = ftol, gtol, xtol
        self.stpmin, self.stpmax = stpmin, stpmax

    def step(self, stp, f, g, task):
        if task[:5] == "START":
            if stp < self.stpmin:
                return stp, "ERROR: STP .LT. STPMIN"
            if stp > self.stpmax:
                return stp, "ERROR: STP .GT. STPMAX"
            if g >= 0.0:
                return stp, "ERROR: INITIAL G .GE. ZERO"
            if self.ftol < 0.0:
                return stp, "ERROR: FTOL .LT. ZERO"
            if self.gtol < 0.0:
                return stp, "ERROR: GTOL .LT. ZERO"
            if self.xtol < 0.0:
                return stp, "ERROR: XTOL .LT. ZERO"
            if self.stpmin < 0.0:
                return stp, "ERROR: STPMIN .LT. ZERO"
            if self.stpmax < self.stpmin:
                return stp, "ERROR: STPMAX .LT. STPMIN"
            self.brackt = False
            self.stage = 1
            self.finit = f
            self.ginit = g
            self.gtest = self.ftol * g
            self.width = self.stpmax - self.stpmin
            self.width1 = self.width / self.P5
            self.stx, self.fx, self.gx = 0.0, f, g
            self.sty, self.fy, self.gy = 0.0, f, g
            self.stmin = 0.0
            self.stmax = stp + self.XTRAPU * stp
            return stp, "FG"
        ftest = self.finit + stp * self.gtest
        if self.stage == 1 and f <= ftest and g >= 0.0:
            self.stage = 2
        task = ""
        if self.brackt and (stp <= self.stmin or stp >= self.stmax):
            task = "WARNING: ROUNDING ERRORS PREVENT PROGRESS"
        if self.brackt and self.stmax - self.stmin <= self.xtol * self.stmax:
            task = "WARNING: XTOL TEST SATISFIED"
        if stp == self.stpmax and f <= ftest and g <= self.gtest:
            task = "WARNING: STP = STPMAX"
        if stp == self.stpmin and (f > ftest or g >= self.gtest):
            task = "WARNING: STP = STPMIN"
        if f <= ftest and abs(g) <= self.gtol * (-self.ginit):
            task = "CONVERGENCE"
        if task.startswith("WARN") or task.startswith("CONV"):
            return stp, task
        if self.stage == 1 and f <= self.fx and f > ftest:
            gt = self.gtest
            fm, fxm, fym = f - stp * gt, self.fx - self.stx * gt, self.fy - self.sty * gt
            gm, gxm, gym = g - gt, self.gx - gt, self.gy - gt
            (self.stx, fxm, gxm, self.sty, fym, gym, stp, self.brackt) = dcstep(
                self.stx, fxm, gxm, self.sty, fym, gym, stp, fm, gm, self.brackt, self.stmin, self.stmax)
            self.fx, self.fy = fxm + self.stx * gt, fym + self.sty * gt
            self.gx, self.gy = gxm + gt, gym + gt
        else:
            (self.stx, self.fx, self.gx, self.sty, self.fy, self.gy, stp, self.brackt) = dcstep(
                self.stx, self.fx, self.gx, self.sty, self.fy, self.gy, stp, f, g, self.brackt,
                self.stmin, self.stmax)
        if self.brackt:
            if abs(self.sty - self.stx) >= self.P66 * self.width1:
                stp = self.stx + self.P5 * (self.sty - self.stx)
            self.width1 = self.width
            self.width = abs(self.sty - self.stx)
            self.stmin = min(self.stx, self.sty)
            self.stmax = max(self.stx, self.sty)
        else:
            self.stmin = stp + self.XTRAPL * (stp - self.stx)
            self.stmax = stp + self.XTRAPU * (stp - self.stx)
        stp = max(stp, self.stpmin)
        stp = min(stp, self.stpmax)
        if (self.brackt and (stp <= self.stmin or stp >= self.stmax)) or \
                (self.brackt and self.stmax - self.stmin <= self.xtol * self.stmax):
            stp = self.stx
        return stp, "FG"


def dcstep(stx, fx, dx, sty, fy, dy, stp, fp, dp, brackt, stpmin, stpmax):
    """Safeguarded cubic/quadratic step of Moré & Thuente (MINPACK-2 dcstep)."""
    sgnd = dp * (dx / abs(dx))
    if fp > fx:
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * math.sqrt((theta / s) ** 2 - (dx / s) * (dp / s))
        if stp < stx:
            gamma = -gamma
        p = (gamma - dx) + theta
        q = ((gamma - dx) + gamma) + dp
        r = p / q
        stpc = stx + r * (stp - stx)
        stpq = stx + ((dx / ((fx - fp) / (stp - stx) + dx)) / 2.0) * (stp - stx)
        if abs(stpc - stx) <= abs(stpq - stx):
            stpf = stpc
        else:
            stpf = stpc + (stpq - stpc) / 2.0
        brackt = True
    elif sgnd < 0.0:
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * math.sqrt((theta / s) ** 2 - (dx / s) * (dp / s))
        if stp > stx:
            gamma = -gamma
        p = (gamma - dp) + theta
        q = ((gamma - dp) + gamma) + dx
        r = p / q
        stpc = stp + r * (stx - stp)
        stpq = stp + (dp / (dp - dx)) * (stx - stp)
        if abs(stpc - stp) > abs(stpq - stp):
            stpf = stpc
        else:
            stpf = stpq
        brackt = True
    elif abs(dp) < abs(dx):
        theta = 3.0 * (fx - fp) / (stp - stx) + dx + dp
        s = max(abs(theta), abs(dx), abs(dp))
        gamma = s * math.sqrt(max(0.0, (theta / s) ** 2 - (dx / s) * (dp / s)))
        if stp > stx:
            gamma = -gamma
        p = (gamma - dp) + theta
        q = (gamma + (dx - dp)) + gamma
        r = p / q
        if r < 0.0 and gamma != 0.0:
            stpc = stp + r * (stx - stp)
        elif stp > stx:
            stpc = stpmax
        else:
            stpc = stpmin
        stpq = stp + (dp / (dp - dx)) * (stx - stp)
        if brackt:
            if abs(stpc - stp) < abs(stpq - stp):
                stpf = stpc
            else:
                stpf = stpq
            if stp > stx:
                stpf = min(stp + 0.66 * (sty - stp), stpf)
            else:
                stpf = max(stp + 0.66 * (sty - stp), stpf)
        else:
            if abs(stpc - stp) > abs(stpq - stp):
                stpf = stpc
            else:
                stpf = stpq
            stpf = min(stpmax, stpf)
            stpf = max(stpmin, stpf)
    else:
        if brackt:
            theta = 3.0 * (fp - fy) / (sty - stp) + dy + dp
            s = max(abs(theta), abs(dy), abs(dp))
            gamma = s * math.sqrt((theta / s) ** 2 - (dy / s) * (dp / s))
            if stp > sty:
                gamma = -gamma
            p = (gamma - dp) + theta
            q = ((gamma - dp) + gamma) + dy
            r = p / q
            stpc = stp + r * (sty - stp)
            stpf = stpc
        elif stp > stx:
            stpf = stpmax
        else:
            stpf = stpmin
    if fp > fx:
        sty, fy, dy = stp, fp, dp
    else:
        if sgnd < 0.0:
            sty, fy, dy = stx, fx, dx
        stx, fx, dx = stp, fp, dp
    return stx, fx, dx, sty, fy, dy, stpf, brackt


def line_search(func, alpha0, f0, g0, c1=1e-4, c2=0.2, amax=np.pi, amin=0.0, xtol=1e-12, maxiter=30):
    """``LineSearchDcsrch2`` (``math_utils.py:76-106``).

    ``func(alpha) -> (value, grad, payload)``.  Returns ``(alpha or None,
    task, iterations, last payload, trial list)``.
    """
    ls = DCSRCH(c1, c2, xtol, amin, amax)
    task = "START"
    alpha, f, g = alpha0, f0, g0
    payload = None
    trials = []
    i = 0
    for i in range(maxiter):
        alpha, task = ls.step(alpha, f, g, task)
        if task[:2] == "FG":
            trials.append(alpha)
            f, g, payload = func(alpha)
        else:
            break
    else:
        alpha = None
    if task[:5] == "ERROR" or task[:4] == "WARN":
        alpha = None
    return alpha, task, i, payload, trials


# ----------------------------------------------------------------------------
# Truncated-Newton density optimisation
# ----------------------------------------------------------------------------
def optimize_tn(evaluator, rho0, grid, econv=1e-5, maxfun=50, maxiter=200, maxls=30,
                c1=1e-4, c2=0.2, xtol=1e-12, ncheck=2):
    """``Optimization.optimize_rho`` with method "TN" (``optimization.py:281-520``).

    ``evaluator(rho, calc_e) -> (energy | None, potential)``.
    Returns dict(rho, phi, energy, mu, converged, history, n_iter).
    """
    dV = grid.dV
    rho = rho0.copy()
    phi = rho.copy()
    m = rho > 0
    phi[m] = np.sqrt(rho[m])
    phi[~m] = 1e-300
    phi *= np.sqrt(np.sum(rho) / np.sum(phi * phi))
    rho = phi * phi
    energy, pot = evaluator(rho, True)
    mu = _integral(pot * rho, dV) / _integral(rho, dV)        # optimization.py:537-539
    residual = (pot - mu) * phi
    history = [energy]
    theta = 0.1
    converged = 1
    it = 0
    for it in range(1, maxiter):
        p = _tn_direction(evaluator, residual, phi, mu, maxfun, dV)
        p, theta0 = _orthonormalize(p, phi, dV)
        if np.einsum("ijk,ijk,ijk->", pot, phi, p) * 2.0 > 0:   # optimization.py:371-380
            p, theta0 = _orthonormalize(-residual, phi, dV)
        theta = min(theta0, theta)

        def vd(t, phi=phi, p=p):
            newphi = phi * np.cos(t) + p * np.sin(t)
            e, v = evaluator(newphi * newphi, True)
            p2 = p * np.cos(t) - phi * np.sin(t)
            return e, 2.0 * np.einsum("ijk,ijk,ijk->", v, newphi, p2) * dV, (newphi, e, v)

        g0 = 2.0 * np.einsum("ijk,ijk,ijk->", pot, phi, p) * dV
        theta, task, nls, payload, _ = line_search(vd, theta, energy, g0, c1=c1, c2=c2,
                                                   amax=np.pi, amin=0.0, xtol=xtol, maxiter=maxls)
        if theta is None:
            converged = 1
            break
        phi, energy, pot = payload
        rho = phi * phi
        mu = _integral(pot * rho, dV) / _integral(rho, dV)
        residual = (pot - mu) * phi
        history.append(energy)
        if len(history) - 1 >= ncheck and all(abs(history[-2 - i] - history[-1]) <= econv
                                               for i in range(ncheck)):
            converged = 0
            break
    else:
        converged = 2
    return dict(rho=phi * phi, phi=phi, energy=energy, mu=mu, converged=converged,
                history=history, n_iter=it)


def _integral(x, dV):
    """``DirectField.integral`` (``field.py:186-192``)."""
    return np.einsum("ijk->", x) * dV


def _orthonormalize(p, phi, dV):
    """``OrthogonalNormalization`` (``optimization.py:204-225``)."""
    Ne = _integral(phi * phi, dV)
    p = p - (_integral(p * phi, dV) / Ne) * phi
    pNorm = _integral(p * p, dV)
    theta = np.sqrt(pNorm / Ne)
    return p * np.sqrt(Ne / pNorm), theta


def _tn_direction(evaluator, res0, phi, mu, maxfun, dV):
    """``get_direction_TN`` (``optimization.py:91-147``)."""
    direction = np.zeros_like(res0)
    epsi = 1.0e-9
    res = -res0.copy()
    p = res.copy()
    r0Norm = np.einsum("ijk,ijk->", res, res)
    rConv = r0Norm * 0.1
    best = direction
    rlists = [1e10]
    for it in range(maxfun):
        phi1 = phi + epsi * p
        _, v = evaluator(phi1 * phi1, False)
        Ap = ((v - mu) * phi1 - res0) / epsi
        pAp = np.einsum("ijk,ijk->", p, Ap)
        if pAp < 0.0:
            if it == 0:
                direction = r0Norm / pAp * p
            break
        alpha = r0Norm / pAp
        direction = direction + alpha * p
        res = res - alpha * Ap
        r1Norm = np.einsum("ijk,ijk->", res, res)
        if r1Norm < min(rlists):
            best = direction.copy()
        rlists.append(r1Norm)
        if r1Norm < rConv:
            break
        elif r1Norm > 1000 * min(rlists[:-1]):
            direction = best
            break
        elif it > 10 and abs(r0Norm - r1Norm) < 0.1 * r0Norm:
            direction = best
            break
        beta = r1Norm / r0Norm
        r0Norm = r1Norm
        p = res + beta * p
    return direction


# ----------------------------------------------------------------------------
# LWT / LMGP: density-dependent kernel by interpolation over k_F knots
# ----------------------------------------------------------------------------
def spline_eval_clamped(sp, u):
    """splev(..., ext=3): values beyond the knot range take the end values."""
    x, c = sp
    u = np.asarray(u, float)
    lo, hi = x[0], x[-1]
    out = spline_eval(sp, np.clip(u, lo, hi))
    return out


def mgp_kernel_table(eta, maxpoints=1000):
    """``MGPKernelTable`` (``kedf/kernel.py:267-322``) for a 1-D eta grid, no
    symmetrisation: sum over t = i/maxpoints of G(eta / t^(1/3)) / t^(1/6),
    G = spline of the inverse Lindhard function (TF and vW removed) on a
    log grid."""
    dt = 1.0 / maxpoints
    coe = 4.0 / 5.0 * C_TF * 5.0 / 6.0 * dt
    gp = np.logspace(np.log10(eta[1] / 10), np.log10(eta[-1] + 2), num=eta.size)
    sp = spline_notaknot(gp, lindhard(gp, 1.0, 1.0))
    kernel = np.zeros_like(eta)
    for i in range(1, maxpoints + 1):
        t = i * dt
        kernel += spline_eval_clamped(sp, eta / np.cbrt(t)) / t ** (1.0 / 6.0)
    return kernel * coe


def lwt_tables(kerneltype="MGP", etamax=50.0, neta=50000, maxpoints=1000, x=1.0, y=1.0):
    """Kernel and kernel-derivative splines (``LWT``, ``kedf/lwt.py:531-561``, order 3)."""
    eta = np.linspace(0, etamax, neta)
    if kerneltype == "MGP":
        table = mgp_kernel_table(eta, maxpoints)
    elif kerneltype == "WT":
        table = lindhard(eta, x, 1.0) * (4.0 / 5.0 * C_TF)     # WTKernelTable, kernel.py:337-345
    else:
        raise ValueError(kerneltype)
    sp = spline_notaknot(eta, table)
    dtab = spline_eval_deriv(sp, eta) * (-1.0 * eta)
    spd = spline_notaknot(eta, dtab)
    return dict(eta=eta, table=table, sp=sp, spd=spd, etamax=etamax)


def lwt_kernel_kf(q, kf, sp, etamax):
    """``LWTKernelKf`` (``kernel.py:379-405``) with a spline table."""
    eta = q / kf
    K = np.where(eta < etamax, spline_eval(sp, np.minimum(eta, etamax)), spline_eval(sp, etamax))
    if q.flat[0] < ZERO:
        K.flat[0] = 0.0
    return K


def guess_kf_bound(kf, saved, kfmin=None, kfmax=None, kftol=1e-3):
    """``guess_kf_bound`` (``lwt.py:36-79``); ``saved`` carries kfmin/kfmax across calls."""
    kfmin_prev = saved.get("kfmin")
    kfmax_prev = saved.get("kfmax")
    if kfmin is not None and kfmax is not None:
        return [kfmin, kfmax]
    kf_l = kf.min()
    kf_r = kf.max()
    if kfmin_prev is None:
        kfmin_prev = 10
        if kfmin is None:
            kfmin = kf_l
    if kfmax_prev is None:
        kfmax_prev = 1.0
        if kfmax is None:
            kfmax = kf_r
    if kfmin is None or kfmin > kfmin_prev:
        kfmin = kfmin_prev
    if kfmax is None or kfmax < kfmax_prev:
        kfmax = kfmax_prev
    if kfmin > kf_l:
        kfl = [1E-5, 1E-4, 5E-3, 1E-3, 5E-3, 1E-2, 5E-2, 0.1, 0.5, 1.0]
        ratio = kf_l / kfmin
        for i in range(len(kfl) - 1, 0, -1):
            if ratio > kfl[i]:
                kfmin *= kfl[i]
                break
    if kfmin < kftol:
        kfmin = kftol
    if kfmax < kf_r:
        dk = kf_r - kfmax
        kfmax += (np.round(dk / 0.5) + 1) * 0.5
    saved["kfmin"] = kfmin
    saved["kfmax"] = kfmax
    return [kfmin, kfmax]


def kf_knots(kfmin, kfmax, ratio=1.15):
    """Geometric k_F knots (``lwt.py:171-187``, nsp and delta unset)."""
    nsp = int(np.ceil(np.log(kfmax / kfmin) / np.log(ratio))) + 1
    kflists = kfmin * ratio ** np.arange(nsp)
    kflists[0] -= 1e-16
    kflists[-1] += 1e-16
    return kflists


class LWTNL:
    """``LWTPotentialEnergy`` (``kedf/lwt.py:82-341``) with the reference's
    defaults of the direct API: kdd 3, ratio 1.15, alpha = beta = 5/6, no
    lump factor, ldw 1/6.  ``interp``: "linear" or "hermite"."""

    def __init__(self, kerneltype="MGP", interp="linear", etamax=50.0, neta=50000, maxpoints=1000, ratio=1.15,
                 kdd=3, alpha=5.0 / 6.0, beta=5.0 / 6.0, ldw=None):
        self.kerneltype, self.interp = kerneltype, interp
        self.etamax, self.neta, self.maxpoints = etamax, neta, maxpoints
        self.ratio, self.kdd, self.alpha, self.beta, self.ldw = ratio, kdd, alpha, beta, ldw
        self.tables = None
        self.saved = {"kfmin": None, "kfmax": None}
        self.last_knots = None

    def __call__(self, rho, grid, calc_e=True, calc_v=True):
        if self.tables is None:
            self.tables = lwt_tables(self.kerneltype, self.etamax, self.neta, self.maxpoints)
        tab = self.tables
        q = grid.q
        alpha, beta = self.alpha, self.beta
        kf = 2.0 * np.cbrt(3.0 * np.pi ** 2 * rho)
        if abs(kf.max() - kf.min()) < 1e-8:
            return 0.0, np.zeros_like(rho)
        kfmin, kfmax = guess_kf_bound(kf, self.saved)
        kdd = self.kdd if calc_v else 1
        kf = np.where(kf > kfmax, kfmax, kf)
        kfl = kf_knots(kfmin, kfmax, self.ratio)
        self.last_knots = kfl
        nsp = kfl.size
        rc = rho.copy()
        rc[~(rho > 0)] = 1e-30
        rA = rc ** alpha
        rA1 = rA / rc
        rB, rB1 = (rA, rA1) if abs(alpha - beta) < 1e-8 else (rc ** beta, rc ** beta / rc)
        rBG = fft(rB, grid)
        mcalc = kdd > 1 or self.interp == "hermite"
        pot1 = np.zeros_like(rho)
        pot3 = np.zeros_like(rho)
        pot2G = None
        for i in range(nsp - 1):
            if i == 0:
                K0 = lwt_kernel_kf(q, kfl[0], tab["sp"], self.etamax)
                p0 = ifft(K0 * rBG, grid)
                if mcalc:
                    D0 = lwt_kernel_kf(q, kfl[0], tab["spd"], self.etamax) / kfl[0]
                    m0 = ifft(D0 * rBG, grid)
            else:
                p0, K0 = p1, K1
                if mcalc:
                    m0, D0 = m1, D1
            K1 = lwt_kernel_kf(q, kfl[i + 1], tab["sp"], self.etamax)
            p1 = ifft(K1 * rBG, grid)
            if mcalc:
                D1 = lwt_kernel_kf(q, kfl[i + 1], tab["spd"], self.etamax) / kfl[i + 1]
                m1 = ifft(D1 * rBG, grid)
            mask = (kf > kfl[i]) & (kf < kfl[i + 1] + 1e-18)
            if i == 0:
                small = kf < kfl[0] + 1e-18
                t = (kf - kfl[0]) / kfl[0]
                pot1[small] = p0[small] * t[small]
                if kdd > 1:
                    rhoU = rA * small
                    if pot2G is None:
                        pot2G = K0 * fft(rhoU * t, grid)
                    if kdd == 3:
                        pot3[mask] = m0[mask] * t[mask]
            rhoU = rA * mask
            Dkf = kfl[i + 1] - kfl[i]
            t = (kf - kfl[i]) / Dkf
            if self.interp == "linear":
                t0 = 1 - t
                pot1[mask] = p0[mask] * t0[mask] + p1[mask] * t[mask]
                if kdd > 1:
                    g = K0 * fft(rhoU * t0, grid) + K1 * fft(rhoU * t, grid)
                    pot2G = g if pot2G is None else pot2G + g
                    if kdd == 3:
                        pot3[mask] = m0[mask] * t0[mask] + m1[mask] * t[mask]
            else:
                t2 = t * t
                t3 = t2 * t
                h00 = 2.0 * t3 - 3.0 * t2 + 1.0
                h10 = t3 - 2.0 * t2 + t
                h01 = 1.0 - h00
                h11 = t3 - t2
                pot1[mask] = h00[mask] * p0[mask] + h01[mask] * p1[mask] + Dkf * (h10[mask] * m0[mask]
                                                                                    + h11[mask] * m1[mask])
                if kdd > 1:
                    g = (K0 * fft(rhoU * h00, grid) + K1 * fft(rhoU * h01, grid)
                         + Dkf * (D0 * fft(rhoU * h10, grid) + D1 * fft(rhoU * h11, grid)))
                    pot2G = g if pot2G is None else pot2G + g
                    if kdd == 3:
                        tm, t2m, t3m = t[mask], t2[mask], t3[mask]
                        h00D = 6.0 * t2m - 6 * tm
                        h10D = 3.0 * t2m - 4 * tm + 1.0
                        h01D = -h00D
                        h11D = 3.0 * t2m - 2 * tm
                        pot3[mask] = (h00D * p0[mask] + h01D * p1[mask]) / Dkf + h10D * m0[mask] + h11D * m1[mask]
        pot2 = ifft(pot2G, grid) if (calc_v and pot2G is not None) else pot1.copy()
        ldw = 1.0 / 6.0 if self.ldw is None else self.ldw
        factor = np.ones_like(rho)
        rhov = rho.max()
        m = rho < 1e-6
        ld = max(0.1, ldw)
        factor[m] = np.abs(rho[m]) ** ld / (rhov ** ld)
        factor[rho < 0] = 0.0
        pot1 = pot1 * factor
        e = float((rA * pot1).sum() * grid.dV) if calc_e else None
        if not calc_v:
            return e, None
        pot2 = pot2 * factor
        pot3 = pot3 * factor
        pot = pot1 * alpha * rA1 + pot2 * beta * rB1 + pot3 * (kf / 3.0) * rA1
        return e, pot
