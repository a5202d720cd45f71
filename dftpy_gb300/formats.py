"""Density and potential files: Quantum ESPRESSO ``pp`` (``formats/qepp.py``),
XCrySDen ``xsf`` (``formats/xsf.py``) and DFTpy ``snpy`` (``formats/snpy.py``),
behind the dispatcher of ``formats/io.py`` (``read``, ``read_all``,
``read_density``, ``read_potential``, ``write``, ``write_density``, ...).

Host-side I/O.  Each format has an array layer (``*_arrays`` / ``*_bytes``,
numpy only, usable without a GPU) and the field layer (``read`` / ``write``)
that turns the array into a ``DirectField`` on the device or takes one back.

Units and conventions follow the reference:

* ``pp``: lengths in Bohr (``celldm(1)`` times the file's unit-cell rows),
  data in Fortran order, potentials in Rydberg (halved on reading, doubled on
  writing); ``ibrav`` 0, 1 and 2; ``read`` gives a full-spectrum grid.
* ``xsf``: lengths in Angstrom, densities per A^3, potentials in eV; the
  data grid carries the periodic image on each axis (dropped on reading,
  added on writing); several ``DATAGRID`` blocks become a rank-n field.
* ``snpy``: consecutive ``.npy`` records -- a description (the record keys),
  then cell (Bohr), atomic numbers, positions (Bohr), the C-order data and an
  optional information record.
"""
import io as _pyio
import os

import numpy as np

from .ions import Ions
from .pseudo_files import BOHR_ANG, HARTREE_EV

__all__ = ["read", "read_all", "read_data", "read_density", "read_potential", "write", "write_all", "write_density",
           "write_potential", "guess_format", "IOFormats", "CHEMICAL_SYMBOLS"]

CHEMICAL_SYMBOLS = (
    "X H He Li Be B C N O F Ne Na Mg Al Si P S Cl Ar K Ca Sc Ti V Cr Mn Fe Co Ni Cu Zn Ga Ge As Se Br Kr "
    "Rb Sr Y Zr Nb Mo Tc Ru Rh Pd Ag Cd In Sn Sb Te I Xe Cs Ba La Ce Pr Nd Pm Sm Eu Gd Tb Dy Ho Er Tm Yb "
    "Lu Hf Ta W Re Os Ir Pt Au Hg Tl Pb Bi Po At Rn Fr Ra Ac Th Pa U Np Pu Am Cm Bk Cf Es Fm Md No Lr Rf "
    "Db Sg Bh Hs Mt Ds Rg Cn Nh Fl Mc Lv Ts Og").split()
_ATOMIC_NUMBER = {s: z for z, s in enumerate(CHEMICAL_SYMBOLS)}


def _tok(x):
    """One item the way the reference's writers print it (``str`` of a
    Python or numpy scalar) followed by four blanks."""
    return str(x) + "    "


def _toks(values):
    return "".join(_tok(v) for v in values)


class Volumetric:
    """A grid-sized array and the lattice spanning it (numpy, host)."""

    def __init__(self, lattice, values, full=False):
        self.lattice = np.asarray(lattice, dtype=float).reshape(3, 3)
        self.values = np.asarray(values)
        self.full = bool(full)

    @property
    def nr(self):
        return np.array(self.values.shape[-3:], dtype=int)

    @property
    def rank(self):
        return self.values.shape[0] if self.values.ndim == 4 else 1


def _host_values(data):
    """Grid values of a ``DirectField``, a tensor or an ndarray as float64
    numpy, C order, shape (n0, n1, n2) or (rank, n0, n1, n2)."""
    if hasattr(data, "detach"):
        import torch
        data = data.detach().to("cpu").as_subclass(torch.Tensor).numpy()
    return np.asarray(data, dtype=np.float64)


def _lattice_of(data, ions=None):
    grid = getattr(data, "grid", None)
    if grid is not None:
        return np.asarray(grid.lattice, dtype=float)
    if ions is not None:
        return np.asarray(Ions.from_any(ions).cell, dtype=float)
    raise ValueError("the data carries no grid and no ions were given")


# ---------------------------------------------------------------------------
# Quantum ESPRESSO pp (``formats/qepp.py``)
# ---------------------------------------------------------------------------

def qepp_lattice(ibrav, celldm):
    """Lattice rows for ``ibrav`` 1 and 2 as the reader builds them
    (``PP.celldm2at``, ``qepp.py:113-126``): for ibrav 2 the rows are the
    transpose of Quantum ESPRESSO's fcc vectors, kept so that files read here
    give the reference's cell."""
    a = float(celldm[0])
    if ibrav == 1:
        return a * np.identity(3)
    if ibrav == 2:
        cols = 0.5 * a * np.array([[-1.0, 0.0, 1.0], [0.0, 1.0, 1.0], [-1.0, 1.0, 0.0]])
        return cols.T.copy()
    raise NotImplementedError("pp files: only ibrav = 0, 1 and 2 are supported (got %d)" % ibrav)


def read_qepp_arrays(path, kind="all", data_type="density"):
    """Parse a pp file (``PP.read``, ``qepp.py:18-111``).  Returns
    ``(ions, Volumetric, info)`` for ``kind='all'``, the ions or the
    volumetric data alone for ``'ions'`` / ``'data'``."""
    with open(path) as f:
        f.readline()  # title
        head = f.readline().split()
        nrx = np.array([int(x) for x in head[0:3]])
        nat, ntyp = int(head[6]), int(head[7])
        parts = f.readline().split()
        ibrav = int(parts[0])
        celldm = np.asarray(parts[1:], dtype=float)
        if ibrav == 0:
            lattice = np.array([[float(x) for x in f.readline().split()] for _ in range(3)]) * celldm[0]
        else:
            lattice = qepp_lattice(ibrav, celldm)
        gcutm, dual, ecut, plot_num = (float(x) for x in f.readline().split())
        info = {"ibrav": ibrav, "celldm": celldm, "gcutm": gcutm, "dual": dual, "ecut": ecut,
                "plot_num": int(plot_num)}
        names, zval = [], {}
        for _ in range(ntyp):
            p = f.readline().split()
            names.append(p[1])
            zval[p[1]] = float(p[2])
        symbols, pos = [], []
        for _ in range(nat):
            p = f.readline().split()
            pos.append([float(x) for x in p[1:4]])
            symbols.append(names[int(p[4]) - 1])
        pos = np.asarray(pos, dtype=float).reshape(nat, 3)
        if ibrav == 0:
            ions = Ions(symbols, positions=pos * celldm[0], cell=lattice)
        else:
            ions = Ions(symbols, scaled_positions=pos, cell=lattice)
        ions.set_charges(zval)
        if kind == "ions":
            return ions
        flat = np.array(f.read().split(), dtype=np.float64)
    n = int(np.prod(nrx))
    if flat.size < n:
        raise ValueError("pp file %s: %d grid values for a %s grid" % (path, flat.size, tuple(nrx)))
    values = np.reshape(flat[:n], tuple(nrx), order="F")
    if data_type == "potential":
        values = values * 0.5
    vol = Volumetric(lattice, np.ascontiguousarray(values), full=True)
    if kind == "data":
        return vol
    return ions, vol, info


def qepp_text(ions, values, lattice=None, data_type="density", header=None, information=None):
    """The text of a pp file (``PP.write``, ``qepp.py:128-195``): the same
    header lines, five ``%22.15e`` values per line in Fortran order."""
    ions = Ions.from_any(ions)
    values = np.asarray(values, dtype=np.float64)
    if values.ndim != 3:
        raise ValueError("pp files hold one 3-D field")
    info = {"gcutm": 1.0, "dual": 4.0, "ecut": 1.0}
    if information:
        info.update(information)
    nr = values.shape
    ibrav = info.get("ibrav", 0)
    celldm = info.get("celldm", None)
    if celldm is None:
        celldm = np.zeros(6)
        celldm[0] = np.linalg.norm(np.asarray(ions.cell), axis=1)[0]
    out = _pyio.StringIO()
    out.write(header or "DFTpy")
    out.write("\n  " + _toks(nr) + _toks(nr) + _toks([ions.nat, len(ions.symbols_uniq)]))
    out.write("\n  " + _tok(ibrav) + _toks(celldm))
    if ibrav == 0:
        for row in np.asarray(ions.cell):
            out.write("\n  " + _toks(row / celldm[0]))
    plot_num = info.get("plot_num", 1 if data_type == "potential" else 0)
    out.write("\n  " + _tok(info["gcutm"]) + _tok(info["dual"]) + _tok(info["ecut"]) + _tok(plot_num))
    uniq = list(ions.symbols_uniq)
    zv = ions.zval if ions._charges is not None else dict.fromkeys(uniq, 0)
    for ity, s in enumerate(uniq):
        out.write("\n  " + _toks([ity + 1, s, zv.get(s, 0.0)]))
    tau = ions.positions / celldm[0]
    for iat in range(ions.nat):
        out.write("\n  " + _tok(iat + 1) + _toks(tau[iat]) + _tok(uniq.index(ions.symbols[iat]) + 1))
    out.write("\n")
    flat = values.ravel(order="F")
    if data_type == "potential":
        flat = flat * 2.0
    nfull = flat.size // 5
    body = flat[:nfull * 5].reshape(nfull, 5)
    lines = [" ".join("%22.15e" % v for v in row) for row in body]
    out.write("\n".join(lines))
    if nfull:
        out.write("\n")
    out.write(" ".join("%22.15e" % v for v in flat[nfull * 5:]))
    return out.getvalue()


# ---------------------------------------------------------------------------
# XCrySDen xsf (``formats/xsf.py``)
# ---------------------------------------------------------------------------

def _xsf_lines(text):
    for line in text.splitlines():
        s = line.strip()
        if s and not s.startswith("#"):
            yield s


def _datagrid_frame(vlat, npbc):
    """Complete the spanning vectors of a 2-D / 1-D data grid to a frame
    (``read_xsf``, ``xsf.py:70-83``)."""
    vlat = np.array(vlat, dtype=float)
    if npbc == 1:
        for i in range(3):
            if abs(vlat[0][i]) > 1e-4:
                j = i - 1
                vlat[1][j] = vlat[0][i]
                vlat[1][i] = -vlat[0][j]
                vlat[1] = vlat[1] / np.sqrt(np.dot(vlat[1], vlat[1]))
                break
    if npbc in (1, 2):
        vlat[2] = np.cross(vlat[0], vlat[1])
        vlat[2] = vlat[2] / np.sqrt(np.dot(vlat[2], vlat[2]))
    return vlat


def read_xsf_arrays(path, kind="all", pbc=True, units="angstrom", data_type="density"):
    """Parse a crystal xsf file (``read_xsf``, ``xsf.py:15-129``).  Returns
    ``(ions, Volumetric, None)`` for ``kind='all'``."""
    with open(path) as f:
        lines = _xsf_lines(f.read())
    angstrom = units.lower() == "angstrom"
    if next(lines).upper() != "CRYSTAL":
        raise AttributeError("Only support crystal xsf.")
    line = next(lines).upper()
    cell = np.zeros((3, 3))
    if line.startswith("PRIMVEC"):
        cell = np.array([[float(x) for x in next(lines).split()] for _ in range(3)])
        line = next(lines).upper()
    if line.startswith("CONVVEC"):
        for _ in range(3):
            next(lines)
        line = next(lines).upper()
    symbols, pos = [], []
    if line.startswith("PRIMCOORD"):
        nat = int(next(lines).split()[0])
        for _ in range(nat):
            p = next(lines).split()
            symbols.append(CHEMICAL_SYMBOLS[int(p[0])] if p[0].isdigit() else p[0])
            pos.append([float(x) for x in p[1:4]])
        line = next(lines, "").upper()
    pos = np.asarray(pos, dtype=float).reshape(len(symbols), 3)
    lunit = BOHR_ANG if angstrom else 1.0
    ions = Ions(symbols, positions=pos / lunit, cell=cell / lunit)
    if kind == "ions":
        return ions
    blocks, data_lat = [], None
    for line in lines:
        up = line.upper()
        if up.startswith("BEGIN_DATAGRID"):
            nrx = np.ones(3, dtype=int)
            npbc = 3 if up.startswith("BEGIN_DATAGRID_3D") else 2 if up.startswith("BEGIN_DATAGRID_2D") else 1
            dims = [int(x) for x in next(lines).split()]
            nrx[:npbc] = dims[:npbc]
            next(lines)  # origin
            vlat = np.zeros((3, 3))
            for i in range(npbc):
                vlat[i] = [float(x) for x in next(lines).split()]
            vlat = _datagrid_frame(vlat, npbc)
            data_lat = vlat / lunit
            vals = []
            for dl in lines:
                if dl[0] == "E":
                    break
                vals.extend(float(x) for x in dl.split())
            vals = np.asarray(vals, dtype=np.float64)[: int(np.prod(nrx))]
            blocks.append(np.reshape(vals, tuple(nrx), order="F"))
        elif up.startswith("END_BLOCK_DATAGRID"):
            break
    if not blocks:
        raise AttributeError("!!!ERROR : XSF file have some problem")
    shape0 = blocks[0].shape
    out = []
    for b in blocks:
        if b.shape != shape0:
            raise AttributeError("All DATAGRID should have same shape.")
        if pbc:
            b = b[tuple(slice(0, n - 1 if n > 1 else n) for n in b.shape)]
        if angstrom:
            b = b * BOHR_ANG ** 3
        if data_type == "potential":
            b = b / HARTREE_EV
        out.append(np.ascontiguousarray(b))
    values = out[0] if len(out) == 1 else np.asarray(out)
    vol = Volumetric(data_lat, values, full=False)
    if kind == "data":
        return vol
    return ions, vol, None


def xsf_text(ions, values, lattice, data_type="density", units="angstrom", title="DFTpy", origin=None):
    """The text of an xsf file (``XSF.write``, ``xsf.py:138-246``): cell and
    positions, then one ``DATAGRID_3D`` per spin channel with the periodic
    image on each axis, Fortran order, five values per line."""
    ions = Ions.from_any(ions)
    angstrom = units.lower() == "angstrom"
    lconv = BOHR_ANG if angstrom else 1.0
    values = np.asarray(values, dtype=np.float64)
    chans = [values] if values.ndim == 3 else list(values)
    out = _pyio.StringIO()
    out.write(_toks(("# ", title)))
    out.write("\n  " + _tok("CRYSTAL \n"))
    out.write("\n  " + _tok("PRIMVEC"))
    for row in np.asarray(ions.cell) * lconv:
        out.write("\n  " + _toks(row))
    out.write("\n  " + _tok("PRIMCOORD"))
    out.write("\n  " + _toks((ions.nat, 1)))
    for s, p in zip(ions.symbols, ions.positions * lconv):
        out.write("\n  " + _tok(s) + _toks(p))
    nd = 3
    out.write("\n  " + _tok("BEGIN_BLOCK_DATAGRID_{}D".format(nd)))
    out.write("\n  " + _tok("{}d_datagrid_{}".format(nd, data_type)))
    origin = np.zeros(3) if origin is None else np.asarray(origin, float)
    for i, ch in enumerate(chans):
        padded = np.pad(ch, ((0, 1), (0, 1), (0, 1)), mode="wrap").ravel(order="F")
        if angstrom:
            padded = padded / BOHR_ANG ** 3
        if data_type == "potential":
            padded = padded * HARTREE_EV
        out.write("\n  " + _tok("BEGIN_DATAGRID_{}D#{}".format(nd, i)))
        out.write("\n  " + _toks(np.asarray(ch.shape) + 1))
        out.write("\n  " + _toks(origin * BOHR_ANG))
        for row in np.asarray(lattice, dtype=float):
            out.write("\n  " + _toks(row * lconv if angstrom else row))
        nfull = padded.size // 5
        for k in range(nfull):
            out.write("\n  " + _toks(padded[5 * k:5 * k + 5]))
        if nfull * 5 < padded.size:
            out.write("\n  " + _toks(padded[5 * nfull:]))
        out.write("\n  " + _tok("END_DATAGRID_{}D".format(nd)))
    out.write("\n  " + _tok("END_BLOCK_DATAGRID_{}D".format(nd)))
    return out.getvalue()


# ---------------------------------------------------------------------------
# snpy (``formats/snpy.py``)
# ---------------------------------------------------------------------------

SNPY_CELL, SNPY_NUMBERS, SNPY_POSITIONS, SNPY_DATA, SNPY_INFO = 1, 2, 3, 4, 5


def snpy_bytes(ions, values=None, information=None, kind="all", desc=None):
    """The bytes of an snpy file (``snpy.write``, ``snpy.py:27-60``)."""
    ions = Ions.from_any(ions)
    if desc is None:
        desc = np.arange(1, 4) if kind == "ions" else np.arange(1, 6) if information is not None else np.arange(1, 5)
    buf = _pyio.BytesIO()
    np.save(buf, np.asarray(desc))
    for key in desc:
        if key == SNPY_CELL:
            np.save(buf, np.asarray(ions.cell, dtype=float))
        elif key == SNPY_NUMBERS:
            np.save(buf, np.array([_ATOMIC_NUMBER[s] for s in ions.symbols], dtype=np.int64))
        elif key == SNPY_POSITIONS:
            np.save(buf, np.asarray(ions.positions, dtype=float))
        elif key == SNPY_DATA:
            np.save(buf, np.ascontiguousarray(values))
        elif key == SNPY_INFO:
            np.save(buf, np.asanyarray(information), allow_pickle=True)
    return buf.getvalue()


def read_snpy_arrays(path, kind="all", desc=None, allow_pickle=False):
    """Parse an snpy file (``snpy.read``, ``snpy.py:62-140``, one process).
    The information record is a pickled object; it is read only with
    ``allow_pickle=True``."""
    ions = info = vol = None
    lattice = numbers = None
    with open(path, "rb") as f:
        if desc is None:
            desc = np.load(f)
        for key in desc:
            if key == SNPY_CELL:
                lattice = np.load(f)
            elif key == SNPY_NUMBERS:
                numbers = np.load(f)
            elif key == SNPY_POSITIONS:
                pos = np.load(f)
                ions = Ions([CHEMICAL_SYMBOLS[int(z)] for z in numbers], positions=pos, cell=lattice)
                if kind == "ions":
                    break
            elif key == SNPY_INFO:
                info = np.load(f, allow_pickle=allow_pickle)
            elif key == SNPY_DATA:
                vol = Volumetric(lattice, np.load(f), full=False)
    if kind == "ions":
        return ions
    if kind == "data":
        return vol
    return ions, vol, info


# ---------------------------------------------------------------------------
# dispatcher (``formats/io.py``)
# ---------------------------------------------------------------------------

IOFormats = {"snpy": "snpy", "xsf": "xsf", "qepp": "qepp", "pp": "qepp"}


def guess_format(infile):
    """``guess_format`` (``io.py:36-47``): the file name, else its suffix."""
    base = os.path.basename(str(infile)).lower()
    ext = os.path.splitext(str(infile))[1].lower()
    fmt = IOFormats.get(base)
    if fmt is None and len(ext) > 1:
        fmt = IOFormats.get(ext[1:])
    if fmt is None:
        fmt = ext[1:] if len(ext) > 1 else base
    return fmt


def _driver(infile, format):
    fmt = IOFormats.get(format, format) if format else guess_format(infile)
    if fmt not in ("snpy", "xsf", "qepp"):
        raise AttributeError("%s format not support yet" % fmt)
    return fmt


def read_arrays(infile, format=None, kind="all", data_type="density", **kwargs):
    """Host-side read: ions, ``Volumetric`` and information as numpy."""
    fmt = _driver(infile, format)
    if fmt == "qepp":
        return read_qepp_arrays(infile, kind=kind, data_type=data_type)
    if fmt == "xsf":
        return read_xsf_arrays(infile, kind=kind, data_type=data_type, **kwargs)
    return read_snpy_arrays(infile, kind=kind, **kwargs)


def _to_field(vol, full=None, grid=None, dtype=None):
    import torch

    from .field import DirectField
    from .grid import DirectGrid
    if grid is None:
        grid = DirectGrid(lattice=vol.lattice, nr=vol.nr, full=vol.full if full is None else full)
    elif not np.all(np.asarray(grid.nrR) == vol.nr):
        raise AttributeError("The shape {} is not match with grid {}".format(tuple(vol.nr), tuple(grid.nrR)))
    return DirectField(grid=grid, rank=vol.rank, data=vol.values, dtype=dtype or torch.float64)


def read(infile, format=None, kind="ions", full=None, grid=None, dtype=None, data_type="density", **kwargs):
    """``io.read`` (``io.py:70-135``): ``kind`` 'ions', 'data' (a
    ``DirectField`` on the device) or 'all' (ions, field, information).
    ``full`` overrides the format's default spectrum layout (pp: full,
    xsf / snpy: half)."""
    got = read_arrays(infile, format=format, kind=kind, data_type=data_type, **kwargs)
    if kind == "ions":
        return got
    if kind == "data":
        return _to_field(got, full, grid, dtype)
    ions, vol, info = got
    return ions, _to_field(vol, full, grid, dtype), info


def read_data(infile, format=None, **kwargs):
    return read(infile, format=format, kind="data", **kwargs)


def read_all(infile, format=None, **kwargs):
    return read(infile, format=format, kind="all", **kwargs)


def read_density(infile, format=None, **kwargs):
    kwargs.pop("data_type", None)
    return read(infile, format=format, kind="data", data_type="density", **kwargs)


def read_potential(infile, format=None, **kwargs):
    kwargs.pop("data_type", None)
    return read(infile, format=format, kind="data", data_type="potential", **kwargs)


def write(outfile, ions=None, data=None, information=None, format=None, data_type="density", **kwargs):
    """``io.write`` (``io.py:137-170``) for one process: pp, xsf or snpy by
    suffix or ``format``.  ``data`` is a ``DirectField`` (or an array, with
    the lattice taken from ``ions``)."""
    if isinstance(data, Ions) and (ions is None or hasattr(ions, "grid")):
        ions, data = data, ions
    fmt = _driver(outfile, format)
    if fmt == "snpy":
        values = None if data is None else _host_values(data)
        kind = "ions" if data is None else "all"
        with open(outfile, "wb") as f:
            f.write(snpy_bytes(ions, values, information, kind=kind, desc=kwargs.get("desc")))
        return
    values = _host_values(data)
    if fmt == "qepp":
        text = qepp_text(ions, values, data_type=data_type, header=kwargs.get("header"), information=information)
    else:
        grid = getattr(data, "grid", None)
        text = xsf_text(ions, values, _lattice_of(data, ions), data_type=data_type,
                        units=kwargs.get("units", "angstrom"), title=kwargs.get("title", "DFTpy"),
                        origin=getattr(grid, "origin", None))
    with open(outfile, "w") as f:
        f.write(text)


def write_all(outfile, ions=None, data=None, information=None, format=None, **kwargs):
    return write(outfile, ions=ions, data=data, information=information, format=format, **kwargs)


def write_density(outfile, data=None, ions=None, format=None, **kwargs):
    kwargs.pop("data_type", None)
    return write(outfile, ions=ions, data=data, format=format, data_type="density", **kwargs)


def write_potential(outfile, data=None, ions=None, format=None, **kwargs):
    kwargs.pop("data_type", None)
    return write(outfile, ions=ions, data=data, format=format, data_type="potential", **kwargs)
