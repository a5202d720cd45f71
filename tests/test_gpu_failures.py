"""Failure paths made on the host (no GPU fault): invalid inputs come back as
C-ABI status codes and Python exceptions, and the device stays usable.

* a density with a NaN, or with no electrons -> GBOFDFT_ERR_NUMERIC from
  gbofdft_optimize_tn (FloatingPointError in Python);
* a workspace smaller than gbofdft_tn_workspace_bytes -> GBOFDFT_ERR_ARG;
* a field buffer of the wrong size -> ValueError before any library call;
* negative density values are the reference's business, not an error: the
  evaluation equals the oracle's (TF/vW/LDA clamp as the reference does).
After each failure a normal evaluation still matches the oracle."""
import ctypes

import numpy as np
import pytest

from dftpy_gb300 import systems
from oracle import ofdft as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    from dftpy_gb300 import _lib
    from dftpy_gb300 import functional as F
    from dftpy_gb300.field import DirectField
    from dftpy_gb300.grid import DirectGrid
    from dftpy_gb300.ions import Ions
    from dftpy_gb300.optimization import Optimization
    _lib.require_cuda()
    st = systems.config_al4(0)
    grid = DirectGrid(st.lattice, st.nr, full=False)
    ions = Ions(st.symbols, positions=st.positions, cell=st.lattice)
    ps = F.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": F.AnalyticPP(3.0, 1.0)}, PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="TFVW"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    ev = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")
    return dict(torch=torch, lib=_lib, st=st, grid=grid, total=total, DF=DirectField, Opt=Optimization, ev=ev)


def _still_works(env):
    rng = np.random.default_rng(5)
    st = env["st"]
    rho = np.full(st.nr, st.nelec / st.volume) * (1.0 + 0.05 * rng.standard_normal(st.nr))
    out = env["total"](env["DF"](env["grid"], data=rho))
    e_ref, v_ref = env["ev"](rho)
    assert abs(out.energy - e_ref) < 1e-10 * abs(e_ref)
    assert float(np.abs(out.potential.to_numpy() - v_ref).max()) < 1e-10 * np.abs(v_ref).max()


@pytest.mark.parametrize("bad", ["nan", "inf", "zero", "negative"])
def test_tn_rejects_invalid_density(env, bad):
    st = env["st"]
    rho = np.full(st.nr, st.nelec / st.volume)
    if bad == "nan":
        rho[3, 4, 5] = np.nan
    elif bad == "inf":
        rho[0, 0, 0] = np.inf
    elif bad == "zero":
        rho[:] = 0.0
    else:
        rho[:] = -1e-3
    opt = env["Opt"](EnergyEvaluator=env["total"], optimization_method="TN", optimization_options={"econv": 1e-7})
    with pytest.raises(FloatingPointError, match="non-finite values or no electrons"):
        opt.optimize_rho(guess_rho=env["DF"](env["grid"], data=rho))
    _still_works(env)


def test_tn_rejects_small_workspace(env):
    torch, lib = env["torch"], env["lib"]
    grid, st = env["grid"], env["st"]
    plan = grid.plan(torch.float64)
    nb = ctypes.c_int64()
    lib.check(lib.load().gbofdft_tn_workspace_bytes(plan.handle, ctypes.byref(nb)))
    ws = torch.empty(int(nb.value) // 8 + 64, dtype=torch.float64, device="cuda")
    rho = torch.full(st.nr, st.nelec / st.volume, dtype=torch.float64, device="cuda")
    f = env["total"].spec(env["DF"](grid, data=rho)).ctypes()
    opts = lib.TnOptions()
    lib.check(lib.load().gbofdft_tn_options_default(ctypes.byref(opts)))
    res = lib.TnResult()
    rc = lib.load().gbofdft_optimize_tn(plan.handle, ctypes.byref(f), lib.ptr(rho), ctypes.byref(opts),
                                        lib.aligned_ptr(ws, 256), int(nb.value) - 8, ctypes.byref(res),
                                        lib.stream_ptr())
    assert rc == 1 and "workspace" in lib.last_error()
    _still_works(env)


def test_wrong_sized_field_is_refused(env):
    st = env["st"]
    with pytest.raises(ValueError, match="grid needs"):
        env["DF"](env["grid"], data=np.zeros(int(np.prod(st.nr)) - 1))
    _still_works(env)


def test_negative_values_follow_the_reference(env):
    st = env["st"]
    rng = np.random.default_rng(9)
    rho = np.full(st.nr, st.nelec / st.volume) * (1.0 + 0.05 * rng.standard_normal(st.nr))
    rho[:2] = -1e-4
    out = env["total"](env["DF"](env["grid"], data=rho))
    e_ref, v_ref = env["ev"](rho)
    assert abs(out.energy - e_ref) < 1e-10 * abs(e_ref)
    assert float(np.abs(out.potential.to_numpy() - v_ref).max()) < 1e-9 * np.abs(v_ref).max()
