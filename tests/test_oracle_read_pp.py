"""The reference's pseudopotential-file test (``test_read_pp.py``): the local
pseudopotential energy of its test density ``Al_fde_rho.pp`` with the tables
read from its example recpot, psp8 and UPF files equals 1.3497046 (the
value the reference asserts).  The tables come from this package's readers
(``pseudo_files``), the energy from the oracle's v_loc (PME, the
reference's LocalPseudo default).  The example files are read where the
reference's data directory exists; elsewhere these tests skip."""
import os

import numpy as np
import pytest

from dftpy_gb300 import pseudo_files as P
from oracle import ofdft as O

DATA = os.environ.get("DFTPY_REFERENCE_DATA", "/root/reference/examples/DATA")


@pytest.mark.parametrize("fname", ["al.lda.recpot", "al.lda.psp", "al.lda.upf"])
def test_pp_energy_of_reference_density(golden, fname):
    path = os.path.join(DATA, fname)
    if not os.path.exists(path):
        pytest.skip("reference example data not present")
    d = golden("fde")
    nr = tuple(int(x) for x in d["nr"])
    g = O.Grid(d["lattice"], nr, full=True)
    gp, vp, _ = P.reciprocal_table(P.read_pp(path))
    v = O.local_pp(g, d["positions"], ["Al", "Al"], {"Al": (gp, vp)}, pme=True)
    e = float((v * d["rho"]).sum() * g.dV)
    assert abs(e - 1.3497046) < 1e-4, e
