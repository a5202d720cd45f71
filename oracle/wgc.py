"""numpy FP64 restatement of the WGC nonlocal kinetic term.

TEST INFRASTRUCTURE ONLY: the checker for the GPU product.

The reference has no WGC functional; this follows the published method
(Wang, Govind and Carter, Phys. Rev. B 60, 16350 (1999)): a Wang-Teter-type
double integral whose kernel depends on the two-body Fermi wavevector

    E_NL = int int rho^a(r) w(xi(r, r'), r - r') rho^b(r') dr dr',
    xi(r, r') = [ (k_F(r)^g + k_F(r')^g) / 2 ]^(1/g),   k_F = (3 pi^2 rho)^(1/3),

expanded to second order in u = (rho - rho*) / rho* about the mean density
rho* (a = (5 + sqrt 5)/6, b = (5 - sqrt 5)/6, g = 2.7 by default).  With
delta = xi / k* - 1, the expansion of xi to second order in (u, u') is

    delta = s/6 + (g - 5)/72 (u^2 + u'^2) + (1 - g)/36 u u',   s = u + u',

and K(xi) = K0 + K1 delta + K2 delta^2 / 2 with K1 = k dK/dk, K2 = k^2 d^2K/dk^2
at k*, so (delta^2 = s^2 / 36 at second order)

    K(xi) = K0 + K1 (u + u')/6 + Kq (u^2 + u'^2) + Kx u u',
    Kq = (g - 5)/72 K1 + K2/72,   Kx = (1 - g)/36 K1 + K2/36.

K(G; k) = C(k) w(G / 2k) with C = 5 C_TF / (9 a b rho^(a+b-5/3)) (the
Wang-Teter prefactor, C ~ k^p, p = 5 - 3 (a + b)); with D = d/dln(eta),
K1 = C (p w - Dw), K2 = C (p (p-1) w - (2p-1) Dw + D^2 w).  The shape w is
fixed by requiring the expanded functional to keep the Lindhard response at
rho*: its second functional derivative at a uniform density is
2 rho*^(a+b-2) [a b K0 + (a+b)/6 K1 + Kx], and that must equal the
Wang-Teter value 2 a b rho*^(a+b-2) C L (L the inverse Lindhard function less
the TF and vW responses).  This is an Euler-type equation in eta,
    D^2 w - S Dw + P w = (a b / c2) L,  c1 = (a+b)/6 + (1-g)/36, c2 = 1/36,
    S = (c1 + c2 (2p-1)) / c2,  P = (a b + c1 p + c2 p (p-1)) / c2,
whose solution bounded at large eta is unique (``kernel_shape``).  Order 1
drops Kq and Kx (first-order equation), order 0 is the Wang-Teter kernel.

Energy and potential (A = rho^a, B = rho^b, convolutions with the kernels):
    X0 = K0*B + K1*(uB)/6 + Kq*(u^2 B),  X1 = K1*B/6 + Kx*(uB),  X2 = Kq*B,
    Y0..Y2 the same with A,
    E  = int A (X0 + u X1 + u^2 X2),
    V  = A'(X0 + u X1 + u^2 X2) + (A/rho*)(X1 + 2u X2)
       + B'(Y0 + u Y1 + u^2 Y2) + (B/rho*)(Y1 + 2u Y2).
``order`` 0 keeps K0 only (the Wang-Teter term with exponents a, b), 1 adds
the first-order terms.
"""
import numpy as np

from .ofdft import C_TF, ZERO, fft, ifft, lindhard

ALPHA = (5.0 + np.sqrt(5.0)) / 6.0
BETA = (5.0 - np.sqrt(5.0)) / 6.0
GAMMA = 2.7


# RK4 points on ln(eta); the forcing's derivative is singular at eta = 1,
# which limits the accuracy there to ~7e-7 in Kx at this resolution
ETA_MIN, ETA_MAX, NT = 1e-5, 200.0, 400001


def kernel_shape(alpha=ALPHA, beta=BETA, gamma=GAMMA, x=1.0, order=2):
    """The kernel shape w(t), Dw, D^2 w on t = ln(eta) (D = d/dt) from the
    linear-response condition, integrated backwards from the large-eta
    limit (order 2: classical RK4 on (w, Dw); order 1: trapezoidal rule): an
    independent method from the product's exponential integrator.  Returns
    t, w, Dw, D2w."""
    t = np.linspace(np.log(ETA_MIN), np.log(ETA_MAX), NT)
    h = t[1] - t[0]
    L = lindhard(np.exp(t), x, 1.0)
    ab, sab = alpha * beta, alpha + beta
    p = 5.0 - 3.0 * sab
    if order == 0:
        return t, L, None, None
    if order == 1:
        lam = (ab + sab * p / 6.0) / (sab / 6.0)
        R = ab / (sab / 6.0)
        w = np.empty_like(t)
        w[-1] = R * L[-1] / lam
        for i in range(NT - 2, -1, -1):
            w[i] = (w[i + 1] * (1.0 / h - lam / 2.0) + R * (L[i] + L[i + 1]) / 2.0) / (1.0 / h + lam / 2.0)
        wt = lam * w - R * L
        return t, w, wt, None
    c2 = 1.0 / 36.0
    c1 = sab / 6.0 + (1.0 - gamma) / 36.0
    S = (c1 + c2 * (2.0 * p - 1.0)) / c2
    P = (ab + c1 * p + c2 * p * (p - 1.0)) / c2
    fc = ab / c2

    def f_at(tt):
        return fc * lindhard(np.exp(np.atleast_1d(tt)), x, 1.0)

    # both homogeneous solutions grow with t, so the bounded solution is the
    # terminal-value one: start at the large-eta limit (w = f/P, Dw = 0) and
    # integrate the system (w, Dw) backwards with classical RK4
    f_nodes = f_at(t)
    f_mid = f_at(t[:-1] + 0.5 * h)
    w = np.empty_like(t)
    wt = np.empty_like(t)
    w[-1], wt[-1] = f_nodes[-1] / P, 0.0

    def rhs(y0, y1, fv):
        return y1, fv + S * y1 - P * y0
    for i in range(NT - 1, 0, -1):
        y0, y1 = w[i], wt[i]
        k1 = rhs(y0, y1, f_nodes[i])
        k2 = rhs(y0 - 0.5 * h * k1[0], y1 - 0.5 * h * k1[1], f_mid[i - 1])
        k3 = rhs(y0 - 0.5 * h * k2[0], y1 - 0.5 * h * k2[1], f_mid[i - 1])
        k4 = rhs(y0 - h * k3[0], y1 - h * k3[1], f_nodes[i - 1])
        w[i - 1] = y0 - h / 6.0 * (k1[0] + 2 * k2[0] + 2 * k3[0] + k4[0])
        wt[i - 1] = y1 - h / 6.0 * (k1[1] + 2 * k2[1] + 2 * k3[1] + k4[1])
    wtt = f_nodes + S * wt - P * w
    return t, w, wt, wtt


def wgc_kernels(q, rho0, alpha=ALPHA, beta=BETA, gamma=GAMMA, x=1.0, order=2, shape=None):
    """(K0, K1, Kq, Kx) on |G| = q for the expansion density rho0."""
    kf = (3.0 * np.pi ** 2 * rho0) ** (1.0 / 3.0)
    C = 5.0 / (9.0 * alpha * beta * rho0 ** (alpha + beta - 5.0 / 3.0)) * C_TF
    eta = q / (2.0 * kf)
    if order == 0:
        K0 = C * lindhard(eta, x, 1.0)
        K0.flat[0] = 0.0
        z = np.zeros_like(K0)
        return K0, z, z.copy(), z.copy()
    t, w, wt, wtt = shape if shape is not None else kernel_shape(alpha, beta, gamma, x, order)
    p = 5.0 - 3.0 * (alpha + beta)
    te = np.log(np.where(eta > 0, eta, 1.0))

    def at(col):
        v = np.interp(te, t, col)
        small = eta < np.exp(t[0])
        v[small] = col[0] * (eta[small] / np.exp(t[0])) ** 2
        v[eta <= 0] = 0.0
        return v
    W, Wt = at(w), at(wt)
    K0 = C * W
    K1 = C * (p * W - Wt)
    if order == 1:
        z = np.zeros_like(K0)
        return K0, K1, z, z.copy()
    Wtt = at(wtt)
    K2 = C * (p * (p - 1.0) * W - (2.0 * p - 1.0) * Wt + Wtt)
    Kq = (gamma - 5.0) / 72.0 * K1 + K2 / 72.0
    Kx = (1.0 - gamma) / 36.0 * K1 + K2 / 36.0
    return K0, K1, Kq, Kx


class WGCNL:
    """WGC nonlocal term; the kernels are rebuilt when the mean density moves
    by more than 1e-6 (as the Wang-Teter kernel cache does)."""

    def __init__(self, alpha=ALPHA, beta=BETA, gamma=GAMMA, x=1.0, order=2, rho0=None):
        self.alpha, self.beta, self.gamma, self.x, self.order = alpha, beta, gamma, x, order
        self.fixed_rho0 = rho0
        self.rho0 = 0.0
        self.shape = None
        self.K = None

    def kernels(self, rho, grid):
        rho0 = self.fixed_rho0 or float(rho.mean())
        if abs(self.rho0 - rho0) > 1e-6 or rho.shape != self.shape:
            if self.order > 0 and getattr(self, "_shape", None) is None:
                self._shape = kernel_shape(self.alpha, self.beta, self.gamma, self.x, self.order)
            self.K = wgc_kernels(grid.q, rho0, self.alpha, self.beta, self.gamma, self.x, self.order,
                                 shape=getattr(self, "_shape", None))
            self.rho0, self.shape = rho0, rho.shape
        return self.K

    def __call__(self, rho, grid, calc_e=True):
        K0, K1, Kq, Kx = self.kernels(rho, grid)
        r0 = self.rho0
        a, b = self.alpha, self.beta
        rc = np.where(rho < ZERO, ZERO, rho)
        u = (rc - r0) / r0
        A, B = rc ** a, rc ** b
        Ad, Bd = a * A / rc, b * B / rc

        def parts(F):
            f0, f1, f2 = fft(F, grid), fft(u * F, grid), fft(u * u * F, grid)
            X0 = ifft(K0 * f0 + K1 / 6.0 * f1 + Kq * f2, grid)
            X1 = ifft(K1 / 6.0 * f0 + Kx * f1, grid)
            X2 = ifft(Kq * f0, grid)
            return X0, X1, X2

        X0, X1, X2 = parts(B)
        Y0, Y1, Y2 = (X0, X1, X2) if abs(a - b) < 1e-12 else parts(A)
        sx = X0 + u * X1 + u * u * X2
        pot = Ad * sx + A / r0 * (X1 + 2.0 * u * X2) + Bd * (Y0 + u * Y1 + u * u * Y2) + B / r0 * (Y1 + 2.0 * u * Y2)
        e = float((A * sx).sum() * grid.dV) if calc_e else None
        return e, pot
