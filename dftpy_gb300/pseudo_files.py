"""Pseudopotential files (``functional/pseudo/recpot.py``, ``psp.py``, ``upf.py``)
and their reciprocal-space tables (``ReadPseudo._init_pp`` / ``_real2recip``,
``functional/pseudo/__init__.py:660-675, 726-779``).

Host-side set-up only: a file becomes a 1-D table v(|G|) on the G grid the
reference uses (recpot: its own uniform grid; real-space formats:
``logspace(log10(1e-4), log10(30), 10000)`` with G[0] = 0), which
``LocalPseudo`` evaluates on the device.

``read_pp(path)`` returns an object with ``zval``, ``radial_grid``,
``local_potential``, ``direct`` and, where the file has them, the atomic and
core densities -- the ``BasePseudo`` interface (``abstract_pseudo.py:49-111``).
"""
import os
import re
import xml.etree.ElementTree as ET

import numpy as np

# Hartree (eV) and Bohr (A) from the CODATA 2014 constants, derived as ase's
# units module does (the reference converts recpot files with them)
_C, _MU0 = 299792458.0, 4.0e-7 * np.pi
_EPS0 = 1.0 / _MU0 / _C ** 2
_HBAR = 6.626070040e-34 / (2.0 * np.pi)
_E, _ME = 1.6021766208e-19, 9.10938356e-31
BOHR_ANG = 4.0e10 * np.pi * _EPS0 * _HBAR ** 2 / _ME / _E ** 2
HARTREE_EV = _ME * _E ** 3 / 16.0 / np.pi ** 2 / _EPS0 ** 2 / _HBAR ** 2


class PseudoTable:
    """``BasePseudo``: the data a reader produced."""

    def __init__(self, r, v, zval, direct, info=None, atomic_density=None, atomic_density_grid=None,
                 core_density=None, core_density_grid=None, fname=None):
        self.r = np.asarray(r, dtype=np.float64)
        self.v = np.asarray(v, dtype=np.float64)
        self._zval = float(zval)
        self._direct = bool(direct)
        self.info = info or {}
        self._atomic_density = atomic_density
        self._atomic_density_grid = atomic_density_grid
        self._core_density = core_density
        self._core_density_grid = core_density_grid
        self.fname = fname

    @property
    def zval(self):
        return self._zval

    @property
    def radial_grid(self):
        return self.r

    @property
    def local_potential(self):
        return self.v

    @property
    def direct(self):
        return self._direct

    @property
    def atomic_density(self):
        return self._atomic_density

    @property
    def atomic_density_grid(self):
        return self.r if self._atomic_density_grid is None else self._atomic_density_grid

    @property
    def core_density(self):
        return self._core_density

    @property
    def core_density_grid(self):
        return self.r if self._core_density_grid is None else self._core_density_grid

    def __call__(self, *args, **kwargs):
        return self


def read_recpot(fname):
    """CASTEP-style reciprocal-space table (``RECPOT.read``, ``recpot.py:11-39``):
    values in eV A^3 on a uniform |G| grid up to gmax (1/A)."""
    with open(fname) as f:
        lines = f.readlines()
    comment, ibegin, iend = "", 0, None
    for i, line in enumerate(lines):
        if "END COMMENT" in line:
            ibegin = i + 3
        elif ibegin > 1 and (line.strip() == "1000" or len(line.strip()) == 1):
            iend = i
            break
        elif ibegin < 1:
            comment += line
    if iend is None:
        raise ValueError("recpot file %s: no end marker" % fname)
    gmax = float(lines[ibegin - 1].strip()) * BOHR_ANG
    v = np.array(" ".join(l.strip() for l in lines[ibegin:iend]).split()).astype(np.float64)
    v = v / HARTREE_EV / BOHR_ANG ** 3
    r = np.linspace(0, gmax, num=len(v))
    zval = round((v[0] - v[1]) * (r[1] ** 2) / (4.0 * np.pi))
    return PseudoTable(r, v, zval, direct=False, info={"comment": comment}, fname=fname)


def write_recpot(fname, gp, vp, header="dftpy_gb300"):
    """Write a uniform |G| table (Bohr^-1, Ha Bohr^3) as a recpot file
    (``RECPOT.write``, ``recpot.py:41-62``)."""
    gp = np.asarray(gp, float)
    v = np.asarray(vp, float) * HARTREE_EV * BOHR_ANG ** 3
    with open(fname, "w") as fw:
        fw.write("START COMMENT\n" + header + "\nEND COMMENT\n")
        fw.write("3     5\n")
        fw.write(str(gp[-1] / BOHR_ANG) + "\n")
        nl = v.size // 3
        for row in v[:nl * 3].reshape(-1, 3):
            fw.write("     {0[0]:22.15E}     {0[1]:22.15E}     {0[2]:22.15E}\n".format(row))
        for x in v[nl * 3:]:
            fw.write("{0:22.15E}".format(x))
        if v.size > nl * 3:
            fw.write("\n")
        fw.write("1000\n")


def read_psp(fname):
    """ABINIT psp8 / psp6 local part (``PSP.read``, ``psp.py:16-120``)."""
    with open(fname) as f:
        lines = [(l.replace("D", "E") if i > 5 else l) for i, l in enumerate(f)]
    v1 = lines[1].split()
    zval = float(v1[1])
    v2 = lines[2].split()
    pspcod, lmax, lloc, mmax = int(v2[0]), int(v2[2]), int(v2[3]), int(v2[4])
    fchrg = float(lines[3].split()[1])
    info = {"atomicnum": int(float(v1[0])), "zval": zval, "pspcod": pspcod, "pspxc": int(v2[1]), "lmax": lmax,
            "lloc": lloc, "mmax": mmax, "fchrg": fchrg}
    core, core_grid = None, None
    if pspcod == 8:
        data = np.asarray([l.split()[1:3] for l in lines[7:7 + mmax]], dtype=np.float64)
        r, v = data[:, 0], data[:, 1]
        if fchrg > 0.0:
            ib = 6 + (mmax + 1) * lloc + mmax
            cd = np.asarray([l.split()[1:3] for l in lines[ib:ib + mmax]], dtype=np.float64)
            core_grid, core = cd[:, 0], cd[:, 1] / (4.0 * np.pi)
    elif pspcod == 6:
        if lmax > 0:
            raise ValueError("psp6 %s: only local pseudopotentials are supported" % fname)
        data = np.asarray([l.split()[1:4] for l in lines[19:19 + mmax]], dtype=np.float64)
        r, v = data[:, 0], data[:, 2]
        if fchrg > 0.0:
            cd = np.asarray([l.split()[0:2] for l in lines[19 + mmax:19 + 2 * mmax]], dtype=np.float64)
            core_grid, core = cd[:, 0], cd[:, 1] / (4.0 * np.pi)
    else:
        raise ValueError("psp %s: only psp8 / psp6 files are supported (pspcod %d)" % (fname, pspcod))
    return PseudoTable(r, v, zval, direct=True, info=info, core_density=core, core_density_grid=core_grid,
                       fname=fname)


_WS = re.compile(r"\s+")


def _array(text):
    if text is None:
        return None
    parts = [x for x in _WS.split(text.strip()) if x]
    return np.array(parts, dtype=np.float64) if parts else None


def read_upf(fname):
    """Quantum ESPRESSO UPF v2 (``UPFDICT.read``, ``upf.py:134-152``): local
    potential in Ry on PP_MESH/PP_R, valence charge PP_RHOATOM (4 pi r^2 rho),
    core charge PP_NLCC."""
    with open(fname) as f:
        text = f.read()
    try:
        root = ET.fromstring(text.strip())
    except ET.ParseError as e:
        raise ValueError("UPF %s: only the XML (v2) layout is supported (%s)" % (fname, e))
    header = root.find("PP_HEADER")
    if header is None or root.find("PP_LOCAL") is None or root.find("PP_MESH/PP_R") is None:
        raise ValueError("UPF %s: PP_HEADER, PP_MESH/PP_R and PP_LOCAL are required" % fname)
    r = _array(root.find("PP_MESH/PP_R").text)
    v = _array(root.find("PP_LOCAL").text) * 0.5
    zval = float(header.attrib["z_valence"])
    core = _array(root.find("PP_NLCC").text) if root.find("PP_NLCC") is not None else None
    rho = None
    if root.find("PP_RHOATOM") is not None:
        rho = _array(root.find("PP_RHOATOM").text)[:r.size]
        if r[0] > 1e-10:
            rho[:] /= 4 * np.pi * r[:] ** 2
        else:
            rho[1:] /= 4 * np.pi * r[1:] ** 2
    return PseudoTable(r, v, zval, direct=True, info={"PP_HEADER": dict(header.attrib)}, atomic_density=rho,
                       core_density=core, fname=fname)


READERS = {"recpot": read_recpot, "psp": read_psp, "psp8": read_psp, "psp6": read_psp, "lps": read_psp, "fhi": read_psp,
           "cpi": read_psp, "upf": read_upf}


def read_pp(fname):
    suffix = os.path.splitext(str(fname))[1][1:].lower()
    if suffix not in READERS:
        raise AttributeError("Pseudopotential '%s' is not supported (formats: %s)" % (fname, sorted(READERS)))
    return READERS[suffix](fname)


def default_gp(max_points=10000, gmax=30.0, gmin=1e-4):
    gp = np.logspace(np.log10(gmin), np.log10(gmax), num=max_points)
    gp[0] = 0.0
    return gp


def radial_ft(r, vr, gp, direct=True):
    """``RadialGrid.ft`` with ``vr=True`` (``grid.py:781-813``): Simpson
    integral of j0(g r) vr r, times 4 pi (real to reciprocal)."""
    from scipy.integrate import simpson
    from scipy.special import spherical_jn
    out = np.empty_like(gp)
    y0 = vr * r
    for k, g in enumerate(gp):
        out[k] = simpson(spherical_jn(0, g * r) * y0, x=r)
    return out * (4.0 * np.pi if direct else 0.5 / np.pi ** 2)


def real2recip(r, v, zval=0.0, gp=None, rcut=None):
    """``ReadPseudo._real2recip`` (``pseudo/__init__.py:660-675``): the
    transform of v r + Z (short-ranged), minus the Coulomb tail 4 pi Z / G^2."""
    if gp is None:
        gp = default_gp()
    r = np.asarray(r, float)
    v = np.asarray(v, float)
    mk = r < rcut + 1e-6 if rcut else slice(None)
    vr = v * r + zval
    vp = radial_ft(r[mk], vr[mk], gp)
    vp[1:] -= 4.0 * np.pi * zval / (gp[1:] ** 2)
    return gp, vp


def reciprocal_table(pp):
    """(gp, vp, zval) of a file's local potential as ``ReadPseudo._init_pp``
    produces them (real-space formats transformed)."""
    if pp.direct:
        gp, vp = real2recip(pp.radial_grid, pp.local_potential, pp.zval)
    else:
        gp, vp = np.asarray(pp.radial_grid, float), np.asarray(pp.local_potential, float)
    return gp, vp, float(pp.zval)


def reciprocal_atomic_density(pp):
    """(gp, rho(|G|)) of a file's atomic valence density, or None
    (``_init_pp``: the real-space density is transformed with Z = 0)."""
    if pp.atomic_density is None:
        return None
    if pp.direct:
        return real2recip(pp.atomic_density_grid, pp.atomic_density, 0.0)
    return np.asarray(pp.atomic_density_grid, float), np.asarray(pp.atomic_density, float)
