"""Density files (pp, xsf, snpy) against the reference's readers and writers.

``tests/golden/formats/`` holds files the reference's writers made for a small
seeded field (``make_golden.py gen_formats``); ``formats.npz`` holds that
field and what the reference's readers returned for those files and for its
own example files.  The writers here must reproduce the files byte for byte
and the readers the arrays exactly.  The example files are read where the
reference's data directory exists; elsewhere those tests skip."""
import os
import pathlib

import numpy as np
import pytest

from dftpy_gb300 import formats as F
from dftpy_gb300.ions import Ions

HERE = pathlib.Path(__file__).resolve().parent
FIX = HERE / "golden" / "formats"
DATA = os.environ.get("DFTPY_REFERENCE_DATA", "/root/reference/examples/DATA")


def _small(d):
    ions = Ions(list(d["small_symbols"]), positions=d["small_pos"], cell=d["small_cell"])
    ions.set_charges({"Ga": 3.0, "As": 5.0})
    return ions, d["small_rho"]


@pytest.mark.parametrize("fname,data_type", [("small_density.pp", "density"), ("small_potential.pp", "potential")])
def test_qepp_writer_bytes(golden, fname, data_type):
    ions, rho = _small(golden("formats"))
    assert F.qepp_text(ions, rho, data_type=data_type) == (FIX / fname).read_text()


@pytest.mark.parametrize("fname,data_type,spin", [("small_density.xsf", "density", False),
                                                  ("small_potential.xsf", "potential", False),
                                                  ("small_spin.xsf", "density", True)])
def test_xsf_writer_bytes(golden, fname, data_type, spin):
    d = golden("formats")
    ions, rho = _small(d)
    values = np.stack([rho, 2.0 * rho]) if spin else rho
    assert F.xsf_text(ions, values, d["small_cell"], data_type=data_type) == (FIX / fname).read_text()


def test_snpy_writer_bytes(golden):
    ions, rho = _small(golden("formats"))
    assert F.snpy_bytes(ions, rho) == (FIX / "small.snpy").read_bytes()


@pytest.mark.parametrize("fname", ["small_density.pp", "small_potential.pp", "small_density.xsf",
                                   "small_potential.xsf", "small_spin.xsf", "small.snpy"])
def test_readers_match_reference(golden, fname):
    d = golden("formats")
    tag = fname.replace(".", "_")
    dt = "potential" if "potential" in fname else "density"
    ions, vol, info = F.read_arrays(str(FIX / fname), data_type=dt)
    np.testing.assert_array_equal(vol.values, d[tag + "_read"])
    np.testing.assert_array_equal(vol.lattice, d[tag + "_read_lattice"])
    np.testing.assert_array_equal(ions.positions, d[tag + "_read_pos"])
    np.testing.assert_array_equal(ions.cell, d[tag + "_read_cell"])
    assert list(ions.symbols) == list(d["small_symbols"])
    assert vol.full == fname.endswith(".pp")


def test_snpy_ions_only_and_information(tmp_path, golden):
    ions, rho = _small(golden("formats"))
    p = tmp_path / "x.snpy"
    p.write_bytes(F.snpy_bytes(ions, rho, information={"energy": -1.5}))
    i2, vol, info = F.read_snpy_arrays(str(p), allow_pickle=True)
    np.testing.assert_array_equal(vol.values, rho)
    assert info.item() == {"energy": -1.5}
    with pytest.raises(ValueError):
        F.read_snpy_arrays(str(p))
    p.write_bytes(F.snpy_bytes(ions, kind="ions"))
    i3 = F.read_snpy_arrays(str(p), kind="ions")
    np.testing.assert_array_equal(i3.positions, ions.positions)


@pytest.mark.parametrize("fname", ["Al_fde_rho.pp", "GaAs_random.xsf", "al_random.xsf", "ti.xsf"])
def test_reference_example_files(golden, fname):
    path = os.path.join(DATA, fname)
    if not os.path.exists(path):
        pytest.skip("reference example data not present")
    d = golden("formats")
    tag = fname.replace(".", "_")
    for dt, key in (("density", tag), ("potential", tag + "_pot")):
        ions, vol, info = F.read_arrays(path, data_type=dt)
        v = vol.values
        assert tuple(v.shape) == tuple(d[key + "_shape"])
        np.testing.assert_array_equal(v.ravel()[d[key + "_idx"]], d[key + "_samples"])
        assert float(v.sum()) == pytest.approx(float(d[key + "_sum"]), rel=1e-14)
        assert float((v * v).sum()) == pytest.approx(float(d[key + "_sumsq"]), rel=1e-14)
    np.testing.assert_array_equal(vol.lattice, d[tag + "_lattice"])
    assert vol.full == bool(d[tag + "_full"])
    np.testing.assert_array_equal(ions.cell, d[tag + "_cell"])
    np.testing.assert_array_equal(ions.positions, d[tag + "_pos"])
    assert list(ions.symbols) == list(d[tag + "_symbols"])
    if info is not None:
        for k, val in info.items():
            np.testing.assert_array_equal(np.asarray(val), d[tag + "_info_" + k])


def test_qepp_round_trip_and_remainder_line(tmp_path):
    rng = np.random.default_rng(5)
    cell = np.diag([5.0, 6.0, 7.0])
    ions = Ions(["Al", "Mg"], positions=rng.random((2, 3)) @ cell, cell=cell)
    ions.set_charges({"Al": 3.0, "Mg": 2.0})
    rho = rng.random((3, 4, 3))  # 36 values: a remainder line of one value
    p = tmp_path / "r.pp"
    p.write_text(F.qepp_text(ions, rho))
    i2, vol, info = F.read_qepp_arrays(str(p))
    np.testing.assert_allclose(vol.values, rho, rtol=1e-15, atol=0)
    np.testing.assert_allclose(i2.positions, ions.positions, rtol=1e-15, atol=1e-15)
    assert i2.zval == {"Al": 3.0, "Mg": 2.0} and info["ibrav"] == 0


def test_qepp_fcc_lattice():
    a = 7.6
    lat = F.qepp_lattice(2, [a, 0, 0, 0, 0, 0])
    assert abs(abs(np.linalg.det(lat)) - a ** 3 / 4) < 1e-12
    with pytest.raises(NotImplementedError):
        F.qepp_lattice(4, [a, 0, 0, 0, 0, 0])


def test_guess_format_and_unknown():
    assert F.guess_format("a/b/rho.pp") == "qepp"
    assert F.guess_format("x.XSF") == "xsf"
    assert F.guess_format("d.snpy") == "snpy"
    with pytest.raises(AttributeError):
        F.read_arrays("nothing.cube")


@pytest.mark.gpu
def test_field_read_write_round_trip(tmp_path, golden):
    import torch
    d = golden("formats")
    ions, vol_ref, _ = F.read_arrays(str(FIX / "small_density.pp"))
    i2, rho, info = F.read_all(str(FIX / "small_density.pp"))
    assert rho.is_cuda and rho.grid.full and tuple(rho.grid.nrR) == (6, 5, 4)
    np.testing.assert_array_equal(rho.to_numpy(), d["small_density_pp_read"])
    for suffix in ("pp", "xsf", "snpy"):
        out = tmp_path / ("w." + suffix)
        F.write(str(out), ions=i2, data=rho)
        back = F.read_density(str(out))
        np.testing.assert_allclose(back.to_numpy(), rho.to_numpy(), rtol=1e-14, atol=1e-14)
        assert back.grid.full == (suffix == "pp")
    half = F.read_density(str(FIX / "small.snpy"), full=True, dtype=torch.float32)
    assert half.grid.full and half.dtype == torch.float32
