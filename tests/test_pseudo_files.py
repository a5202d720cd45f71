"""Pseudopotential file readers and the real-to-reciprocal transform against
the tables the reference's ReadPseudo built from its own example files
(recpot, psp8, UPF v2).  The example files are read where the reference's
data directory exists; elsewhere these tests skip."""
import os

import numpy as np
import pytest

from dftpy_gb300 import pseudo_files as P

DATA = os.environ.get("DFTPY_REFERENCE_DATA", "/root/reference/examples/DATA")
FILES = ["al.lda.recpot", "Al_lda.oe01.recpot", "al.lda.psp", "al.lda.upf", "Mg_OEPP_PZ.UPF"]


@pytest.mark.parametrize("fname", FILES)
def test_reciprocal_table_matches_reference(golden, fname):
    path = os.path.join(DATA, fname)
    if not os.path.exists(path):
        pytest.skip("reference example data not present")
    d = golden("pseudo_files")
    tag = fname.replace(".", "_")
    pp = P.read_pp(path)
    gp, vp, z = P.reciprocal_table(pp)
    assert z == float(d[tag + "_zval"]) and gp.size == int(d[tag + "_n"])
    idx = d[tag + "_idx"]
    np.testing.assert_allclose(gp[idx], d[tag + "_gp"], rtol=1e-14, atol=0)
    np.testing.assert_allclose(vp[idx], d[tag + "_vp"], rtol=1e-12, atol=1e-12 * np.abs(d[tag + "_vp"]).max())
    if tag + "_rho" in d.files:
        gr, rr = P.reciprocal_atomic_density(pp)
        np.testing.assert_allclose(rr[idx], d[tag + "_rho"], rtol=1e-12, atol=1e-12 * np.abs(d[tag + "_rho"]).max())


def test_unknown_format_raises(tmp_path):
    f = tmp_path / "x.unknown"
    f.write_text("1\n")
    with pytest.raises(AttributeError):
        P.read_pp(str(f))
