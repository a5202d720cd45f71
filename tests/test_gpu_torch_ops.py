"""The registered operators (``torch.ops.gbofdft.*``) on the GPU: they match
the oracle, ``torch.library.opcheck`` passes on each (schema, fake tensors,
autograd registration, AOT dispatch), and the public classes run through
them.

Tolerances: FP64 energies 1e-10 relative, potentials and transforms 1e-10 of
the field's max magnitude."""
import ctypes

import numpy as np
import pytest

from dftpy_gb300 import systems
from oracle import ofdft as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    import torch
    from dftpy_gb300 import _lib, torch_ops
    from dftpy_gb300 import functional as F
    from dftpy_gb300.field import DirectField
    from dftpy_gb300.grid import DirectGrid
    from dftpy_gb300.ions import Ions
    _lib.require_cuda()
    st = systems.config_al4(0)
    grid = DirectGrid(st.lattice, st.nr, full=False)
    ions = Ions(st.symbols, positions=st.positions, cell=st.lattice)
    ps = F.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": F.AnalyticPP(3.0, 1.0)}, PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="TFVW"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rng = np.random.default_rng(1)
    rho = np.full(st.nr, st.nelec / st.volume) * (1.0 + 0.05 * rng.standard_normal(st.nr))
    return dict(torch=torch, lib=_lib, ops=torch_ops, st=st, grid=grid, total=total, rho=rho,
                DirectField=DirectField)


def test_eval_operator_matches_oracle(env):
    torch = env["torch"]
    st, grid, total = env["st"], env["grid"], env["total"]
    r = torch.tensor(env["rho"], device="cuda")
    spec = total.spec(env["DirectField"](grid, data=r))
    f = spec.ctypes()
    pot, en = torch.ops.gbofdft.eval(r, env["ops"].handle(grid.plan(torch.float64)), ctypes.addressof(f),
                                     env["lib"].CALC_E | env["lib"].CALC_V)
    ev = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")
    e_ref, v_ref = ev(env["rho"])
    assert abs(float(en[env["lib"].E_TOTAL]) - e_ref) < 1e-10 * abs(e_ref)
    assert float(np.abs(pot.cpu().numpy() - v_ref).max()) < 1e-10 * np.abs(v_ref).max()
    # V only: the energy slots stay zero
    pot2, en2 = torch.ops.gbofdft.eval(r, env["ops"].handle(grid.plan(torch.float64)), ctypes.addressof(f),
                                       env["lib"].CALC_V)
    assert torch.equal(pot2, pot) and float(en2.abs().max()) == 0.0


def test_fft_and_convolve_operators_match_oracle(env):
    torch = env["torch"]
    st, grid = env["st"], env["grid"]
    h = env["ops"].handle(grid.plan(torch.float64))
    x = torch.tensor(env["rho"], device="cuda")
    g = O.Grid(st.lattice, st.nr)
    X = torch.ops.gbofdft.fft_r2c(x, h)
    Xr = O.fft(env["rho"], g)
    assert float(np.abs(X.cpu().numpy() - Xr).max()) < 1e-10 * np.abs(Xr).max()
    y = torch.ops.gbofdft.fft_c2r(X, h, st.nr[2])
    assert float((y - x).abs().max()) < 1e-12 * float(x.abs().max())
    vh = torch.ops.gbofdft.convolve(x, h, env["lib"].KER_HARTREE, None, 1.0)
    inv = g.invgg.copy()
    vref = O.ifft(Xr * 4.0 * np.pi * inv, g)
    assert float(np.abs(vh.cpu().numpy() - vref).max()) < 1e-10 * np.abs(vref).max()


def test_opcheck_every_operator(env):
    torch = env["torch"]
    lib, ops = env["lib"], env["ops"]
    st, grid, total = env["st"], env["grid"], env["total"]
    x = torch.tensor(env["rho"], device="cuda")
    h = ops.handle(grid.plan(torch.float64))
    f = total.spec(env["DirectField"](grid, data=x)).ctypes()
    X = torch.ops.gbofdft.fft_r2c(x, h)
    K = torch.rand(X.shape, dtype=torch.float64, device="cuda")
    torch.library.opcheck(torch.ops.gbofdft.eval.default, (x, h, ctypes.addressof(f), lib.CALC_E | lib.CALC_V))
    torch.library.opcheck(torch.ops.gbofdft.fft_r2c.default, (x, h))
    torch.library.opcheck(torch.ops.gbofdft.fft_c2r.default, (X, h, st.nr[2]))
    torch.library.opcheck(torch.ops.gbofdft.convolve.default, (x, h, lib.KER_ARRAY, K, 0.5))
    # the optimiser: a short TN solve per call (deterministic, so every
    # replay of opcheck gives the same density)
    opts = lib.TnOptions()
    lib.check(lib.load().gbofdft_tn_options_default(ctypes.byref(opts)))
    opts.econv, opts.maxiter, opts.maxfun = 1e-6, 4, 10
    nb = ctypes.c_int64()
    lib.check(lib.load().gbofdft_tn_workspace_bytes(grid.plan(torch.float64).handle, ctypes.byref(nb)))
    ws = torch.empty(int(nb.value) // 8 + 64, dtype=torch.float64, device="cuda")
    res = lib.TnResult()
    rho0 = torch.full(st.nr, st.nelec / st.volume, dtype=torch.float64, device="cuda")
    torch.library.opcheck(torch.ops.gbofdft.optimize_tn.default,
                          (rho0, h, ctypes.addressof(f), ctypes.addressof(opts), ws, int(nb.value),
                           ctypes.addressof(res)))
    assert res.n_iter >= 1


def test_public_api_runs_through_the_operators(env):
    """TotalFunctional.compute, DirectField.fft/ifft and Optimization call
    the registered operators (counted with a dispatch-mode hook)."""
    torch = env["torch"]
    from torch.utils._python_dispatch import TorchDispatchMode
    from dftpy_gb300.optimization import Optimization

    seen = []

    class Spy(TorchDispatchMode):
        def __torch_dispatch__(self, func, types, args=(), kwargs=None):
            if str(func).startswith("gbofdft."):
                seen.append(str(func).split(".")[1])
            return func(*args, **(kwargs or {}))

    grid, total = env["grid"], env["total"]
    rho = env["DirectField"](grid, data=env["rho"])
    with Spy():
        total(rho)
        rho.fft().ifft()
        rho0 = env["DirectField"](grid)
        rho0[:] = env["st"].nelec / env["st"].volume
        Optimization(EnergyEvaluator=total, optimization_method="TN",
                     optimization_options={"econv": 1e-6, "maxiter": 3}).optimize_rho(guess_rho=rho0)
    assert {"eval", "fft_r2c", "fft_c2r", "optimize_tn"} <= set(seen), seen
