"""The TN preconditioner's convolutions through the plane pipeline
(``GBOFDFT_PLANE_PRECOND=1``, read when a plan is created) give the same
mixed-precision solve as the column passes: the same energy within 1e-9
eV/atom and evaluation counts within one TN iteration's worth."""
import os

import pytest

pytestmark = pytest.mark.gpu

HA_EV = 27.211386024367243


def _solve(env):
    import torch
    from dftpy_gb300 import _lib, batch, systems
    _lib.require_cuda()
    old = os.environ.get("GBOFDFT_PLANE_PRECOND")
    os.environ["GBOFDFT_PLANE_PRECOND"] = env
    try:
        st = systems.fcc_supercell((2, 2, 2), sigma=0.15, seed=5, nr=(64, 64, 64), mg_fraction=0.2, name="pc")
        total, rho_u = batch.build_evaluator(st, kedf="WGC")
        total.PSEUDO.grid.plan(torch.float32)   # created under the setting
        res = batch.optimize_batch([(total, rho_u)], workers=1,
                                   options={"precision": "mixed", "econv_per_atom": 1e-8})[0]
    finally:
        if old is None:
            os.environ.pop("GBOFDFT_PLANE_PRECOND", None)
        else:
            os.environ["GBOFDFT_PLANE_PRECOND"] = old
    n = sum(s["n_eval_ev"] + s["n_eval_v"] + s.get("n_eval_hess", 0) for s in res.stats["stages"])
    return res, st, n


def test_plane_preconditioner_matches_column_passes():
    r_col, st, n_col = _solve("0")
    r_pl, _, n_pl = _solve("1")
    assert r_col.converged == 0 and r_pl.converged == 0
    assert abs(r_col.energy - r_pl.energy) * HA_EV / st.nat <= 1e-9, (r_col.energy, r_pl.energy)
    assert abs(n_col - n_pl) <= 6, (n_col, n_pl)
