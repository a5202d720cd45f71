"""numpy restatement of the pointwise changes of the delta evaluation.

TEST INFRASTRUCTURE ONLY: the checker of the method the GPU product uses for
the FP64 evaluations of its mixed-precision refinement (no reference
counterpart).  With t = (rho - rho0) / rho0 and L = log1p(t), the change of a
power law is

    rho^p - rho0^p = rho0^p expm1(p L),

products change by d(uv) = du v + u0 dv, and the PZ81 correlation (Perdew and
Zunger, Phys. Rev. B 23, 5048 (1981); the reference's LDA,
xc/semilocal_xc.py:253-305) changes, for r_s >= 1 with s = sqrt(r_s),
N(s) = g + a1 s + a2 s^2, D(s) = 1 + b1 s + b2 s^2 (a1 = 7/6 g b1,
a2 = 4/3 g b2), by

    v_c - v_c0 = ds (A' D0^2 - N0 E (2 D0 + ds E)) / (D^2 D0^2),
    e_c - e_c0 = -g ds E / (D D0),
    E = b1 + b2 (s + s0), A' = a1 + a2 (s + s0),

and for r_s < 1 through d ln r_s = -L / 3.  Every formula is evaluated in
float32 here, as the kernel does, and compared with float64 differences of
the functions themselves.
"""
import numpy as np

f32 = np.float32
CX = 0.98474502184269654115          # (3/pi)^(1/3)
RSC = 0.62035049089940001667         # (3/(4 pi))^(1/3)
A, B, C, D = 0.0311, -0.048, 0.0020, -0.0116
G, B1, B2 = -0.1423, 1.0529, 0.3334


def lda(rho):
    """PZ81 LDA potential and energy per particle (float64)."""
    rc = np.cbrt(rho)
    rs = RSC / rc
    lo = rs < 1
    lr = np.log(np.where(lo, rs, 1.0))
    sq = np.sqrt(rs)
    inv = 1.0 / (1.0 + B1 * sq + B2 * rs)
    vc = np.where(lo, lr * (A + 2.0 / 3.0 * C * rs) + B - A / 3.0 + (2.0 * D - C) / 3.0 * rs,
                  (G + 7.0 / 6.0 * G * B1 * sq + 4.0 / 3.0 * G * B2 * rs) * inv * inv)
    ec = np.where(lo, A * lr + B + C * rs * lr + D * rs, G * inv)
    return -CX * rc + vc, -0.75 * CX * rc + ec


def pdelta(bp, L, p):
    return (f32(bp) * np.expm1(f32(p) * L)).astype(f32)


def changes(rho, rho0, beta=5.0 / 6.0):
    """float32 changes (rho vs rho0, both > 0, same r_s side of 1) of
    rho^(2/3), rho^(5/3), rho^(-1/2), rho^(1/2), rho^(beta-1), rho^beta,
    and of the LDA potential and energy density eps rho."""
    dr = (rho - rho0).astype(f32)
    r0 = rho0.astype(f32)
    L = np.log1p(dr / r0).astype(f32)
    z3 = (1.0 / np.cbrt(r0)).astype(f32)
    z2 = (1.0 / np.sqrt(r0)).astype(f32)
    c13 = r0 * z3 * z3
    out = {
        "p23": pdelta(r0 * z3, L, 2.0 / 3.0),
        "p53": pdelta(r0 * r0 * z3, L, 5.0 / 3.0),
        "pm12": pdelta(z2, L, -0.5),
        "p12": pdelta(r0 * z2, L, 0.5),
        "pbm1": pdelta(np.power(r0, f32(beta - 1.0)), L, beta - 1.0),
        "pb": pdelta(np.power(r0, f32(beta)), L, beta),
    }
    dvx = f32(-CX) * pdelta(c13, L, 1.0 / 3.0)
    dex = f32(-0.75 * CX) * pdelta(r0 * c13, L, 4.0 / 3.0)
    rs0 = f32(RSC) * z3
    drs = pdelta(rs0, L, -1.0 / 3.0)
    s0 = np.sqrt(rs0).astype(f32)
    ds = pdelta(s0, L, -1.0 / 6.0)
    s = s0 + ds
    a1, a2 = f32(7.0 / 6.0 * G * B1), f32(4.0 / 3.0 * G * B2)
    n0 = f32(G) + a1 * s0 + a2 * s0 * s0
    d0 = f32(1.0) + f32(B1) * s0 + f32(B2) * s0 * s0
    e = f32(B1) + f32(B2) * (s + s0)
    ap = a1 + a2 * (s + s0)
    dd = d0 + ds * e
    dvc_hi = ds * (ap * d0 * d0 - n0 * e * (f32(2.0) * d0 + ds * e)) / (dd * dd * d0 * d0)
    dec_hi = f32(-G) * ds * e / (dd * d0)
    ec0_hi = f32(G) / d0
    dln = L * f32(-1.0 / 3.0)
    ln0 = np.log(rs0).astype(f32)
    drsln = (rs0 + drs) * dln + drs * ln0
    dvc_lo = f32(A) * dln + f32(2.0 / 3.0 * C) * drsln + f32((2.0 * D - C) / 3.0) * drs
    dec_lo = f32(A) * dln + f32(C) * drsln + f32(D) * drs
    ec0_lo = f32(A) * ln0 + f32(B) + f32(C) * rs0 * ln0 + f32(D) * rs0
    lo = rs0 < 1
    dvc = np.where(lo, dvc_lo, dvc_hi)
    dec = np.where(lo, dec_lo, dec_hi)
    ec0 = np.where(lo, ec0_lo, ec0_hi)
    out["vxc"] = dvx + dvc
    out["exc"] = dex + dec * (r0 + dr) + ec0 * dr
    return out
