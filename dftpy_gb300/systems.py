"""Seeded synthetic structures for the OF-DFT workloads (numpy only).

Every workload is an fcc aluminium (optionally Al/Mg alloy) supercell with
Gaussian positional jitter drawn from ``numpy.random.default_rng(seed)``.  The
same builders feed the oracle, the fixtures, the tests and the benchmark, so
all of them see bit-identical inputs.

The analytic local pseudopotential is tabulated on the same |G| grid layout
the reference builds in ``ReadPseudo._real2recip`` (``dftpy/functional/pseudo/
__init__.py:664-675``): ``logspace(log10(1e-4), log10(30), 10000)`` with the
first point replaced by G=0.  ``v(G) = -4 pi Z exp(-(G rc)^2/4) / G^2`` and the
G=0 entry holds the finite non-Coulomb limit ``pi Z rc^2`` (the reference
subtracts ``4 pi Z / G^2`` from every point except G=0).
"""
from dataclasses import dataclass, field

import numpy as np

FCC_BASIS = np.array([[0.0, 0.0, 0.0], [0.5, 0.5, 0.0], [0.5, 0.0, 0.5], [0.0, 0.5, 0.5]])

#: (Z, rc) of the analytic local pseudopotentials.
SPECIES = {"Al": (3.0, 1.0), "Mg": (2.0, 1.2)}


def analytic_pp_table(Z, rc, npts=10000, gmin=1e-4, gmax=30.0):
    """|G| grid and v(G) of the analytic pseudopotential (see module doc)."""
    gp = np.logspace(np.log10(gmin), np.log10(gmax), num=npts)
    gp[0] = 0.0
    vp = np.empty_like(gp)
    g = gp[1:]
    vp[1:] = -4.0 * np.pi * Z * np.exp(-(g * rc) ** 2 / 4.0) / g ** 2
    vp[0] = np.pi * Z * rc ** 2
    return gp, vp


ATOMIC_SIGMA = {"Al": 0.9, "Mg": 1.1}   # Gaussian valence-density widths (Bohr)


def atomic_density_table(Z, sigma, npts=1000, qmax=10.0):
    """|G| grid and the Fourier transform Z exp(-(G sigma)^2 / 2) of a normalised
    Gaussian valence density of Z electrons (a reciprocal-space atomic density
    table for ``DensityGenerator(r=..., arho=...)``)."""
    q = np.linspace(0.0, qmax, npts)
    return q, Z * np.exp(-0.5 * (q * sigma) ** 2)


@dataclass
class Structure:
    """A periodic cell with atoms (Bohr) and its real-space grid."""
    lattice: np.ndarray          # (3, 3), rows are lattice vectors, Bohr
    positions: np.ndarray        # (nat, 3) Cartesian, Bohr
    symbols: list                # nat chemical symbols
    nr: tuple                    # grid points per axis
    name: str = ""
    meta: dict = field(default_factory=dict)

    @property
    def nat(self):
        return len(self.symbols)

    @property
    def volume(self):
        return abs(float(np.linalg.det(self.lattice)))

    @property
    def charges(self):
        return np.array([SPECIES[s][0] for s in self.symbols])

    @property
    def nelec(self):
        return float(self.charges.sum())

    def scaled_positions(self):
        s = np.linalg.solve(self.lattice.T, self.positions.T).T
        return s % 1.0


def fcc_supercell(reps, a=7.65, sigma=0.0, seed=0, nr=None, mg_fraction=0.0,
                  name=""):
    """fcc supercell ``reps`` conventional cells per axis, jittered positions.

    Draw order from ``default_rng(seed)``: first the Mg substitution mask
    (only when ``mg_fraction > 0``: one uniform per site), then the jitter
    ``normal(0, sigma, (nat, 3))`` in Bohr.
    """
    reps = tuple(int(r) for r in reps)
    rng = np.random.default_rng(seed)
    cells = np.array([[i, j, k] for i in range(reps[0]) for j in range(reps[1])
                      for k in range(reps[2])], dtype=float)
    frac = (cells[:, None, :] + FCC_BASIS[None, :, :]).reshape(-1, 3) / np.array(reps, float)
    lattice = np.diag([a * reps[0], a * reps[1], a * reps[2]]).astype(float)
    nat = frac.shape[0]
    symbols = ["Al"] * nat
    if mg_fraction > 0.0:
        u = rng.random(nat)
        symbols = ["Mg" if x < mg_fraction else "Al" for x in u]
    pos = frac @ lattice
    if sigma > 0.0:
        pos = pos + rng.normal(0.0, sigma, size=(nat, 3))
    if nr is None:
        nr = (32 * reps[0], 32 * reps[1], 32 * reps[2])
    return Structure(lattice=lattice, positions=pos, symbols=symbols, nr=tuple(nr), name=name,
                     meta={"reps": reps, "a": a, "sigma": sigma, "seed": seed,
                           "mg_fraction": mg_fraction})


def config_al4(seed=0):
    """Bulk fcc Al, 4 atoms, a=7.65 bohr, 32^3 grid, jitter 0.05 bohr."""
    return fcc_supercell((1, 1, 1), sigma=0.05, seed=seed, nr=(32, 32, 32), name="al4_32")


def config_al256(seed=0):
    """Bulk fcc Al 4x4x4 supercell, 256 atoms, 128^3 grid, jitter 0.1 bohr."""
    return fcc_supercell((4, 4, 4), sigma=0.1, seed=seed, nr=(128, 128, 128), name="al256_128")


def config_al4000(seed=0):
    """Bulk fcc Al 10x10x10 supercell, 4000 atoms, 360^3 grid, jitter 0.1 bohr."""
    return fcc_supercell((10, 10, 10), sigma=0.1, seed=seed, nr=(360, 360, 360), name="al4000_360")


def good_fft_size(n):
    """Smallest 2^a 3^b 5^c 7^d >= n that is even."""
    m = max(2, int(n))
    while True:
        if m % 2 == 0:
            k = m
            for p in (2, 3, 5, 7):
                while k % p == 0:
                    k //= p
            if k == 1:
                return m
        m += 1


def config_alloy(seed, spacing=0.24, nmin=96, nmax=160):
    """Al/Mg random substitution alloy snapshot (108-500 atoms).

    Cell shape (cubic or orthorhombic, 3..6 conventional cells per axis) and
    the Mg fraction U(0, 0.3) are drawn from ``default_rng(10_000 + seed)``;
    the structure itself then uses ``default_rng(seed)``.  Grid points per
    axis follow the spacing (``L/spacing`` rounded to an even 2,3,5,7-smooth
    size), clamped to [nmin, nmax].
    """
    meta = np.random.default_rng(10_000 + seed)
    shapes = [(3, 3, 3), (4, 4, 4), (5, 5, 5), (3, 4, 5), (4, 4, 6), (3, 3, 4), (4, 5, 5), (3, 4, 4)]
    reps = shapes[int(meta.integers(len(shapes)))]
    f = float(meta.random() * 0.3)
    a = 7.65
    nr = tuple(min(nmax, max(nmin, good_fft_size(int(a * r / spacing)))) for r in reps)
    return fcc_supercell(reps, a=a, sigma=0.15, seed=seed, nr=nr, mg_fraction=f,
                         name="alloy_%d" % seed)
