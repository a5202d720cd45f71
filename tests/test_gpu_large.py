"""The 4000-atom LMGP workload at its full size (360^3) against the oracle.

1. At a fixed density -- the superposed Gaussian atomic densities of
   ``get_3d_value_recipe`` (PME) -- every energy term, the total potential at
   4096 fixed grid points and the PP + Ewald forces on all 4000 atoms equal
   the oracle's (``tests/golden/al4000_oracle.npz``, made by
   ``make_oracle_large.py``).  FP64: energies within 1e-9 relative per term,
   potentials within 1e-9 of max|V|, forces within 1e-8 Ha/Bohr; FP32:
   energies within 2e-5 relative per term, total energy 2e-6 relative.
2. At the density the mixed-precision solve reaches from the learned guess,
   the oracle evaluates energy, potential and forces itself: the GPU's
   energy equals the oracle's functional there (1e-9 relative), the GPU's
   forces equal the oracle's (1e-5 Ha/Bohr), and the oracle's residual
   ||(V - mu) phi|| is at most 2e-3 of the guess's (the solved density is a
   minimum of the oracle's functional, not only of the GPU's).  The LMGP
   term keeps its k_F interpolation range from call to call and only widens
   it (``guess_kf_bound``, ``kedf/lwt.py:36-79``), so its value at a density
   depends on the densities it has seen: the oracle starts from the range
   the GPU term holds after the solve.
"""
import os

import numpy as np
import pytest

from dftpy_gb300 import systems
from oracle import ofdft as O

pytestmark = [pytest.mark.gpu, pytest.mark.slow]

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def large():
    import torch
    from dftpy_gb300 import _lib
    from dftpy_gb300 import functional as F
    from dftpy_gb300.density import DensityGenerator
    from dftpy_gb300.field import DirectField
    from dftpy_gb300.grid import DirectGrid
    from dftpy_gb300.ions import Ions
    _lib.require_cuda()
    st = systems.config_al4000(0)
    grid = DirectGrid(st.lattice, st.nr, full=False)
    ions = Ions(st.symbols, positions=st.positions, cell=st.lattice)
    ps = F.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": F.AnalyticPP(*systems.SPECIES["Al"])}, PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="LMGP"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    r, a = systems.atomic_density_table(3.0, systems.ATOMIC_SIGMA["Al"])
    rho = DensityGenerator(r={"Al": r}, arho={"Al": a}).guess_rho(ions, grid=grid)
    return dict(torch=torch, st=st, grid=grid, total=total, rho=rho, DF=DirectField)


def _split_energies(total, rho):
    from dftpy_gb300 import _lib
    total(rho, calcType={"E", "V"})
    en = total.last_energies
    return {"TF": en[_lib.E_TF], "VW": en[_lib.E_VW], "NL": en[_lib.E_NL], "XC": en[_lib.E_XC],
            "HARTREE": en[_lib.E_HARTREE], "PSEUDO": en[_lib.E_PSEUDO]}


def test_fixed_density_matches_oracle(large, golden):
    torch = large["torch"]
    d = golden("al4000_oracle")
    total, rho = large["total"], large["rho"]
    idx = d["sample_idx"]
    r = rho.as_subclass(torch.Tensor).reshape(-1)[torch.tensor(idx, device="cuda")].cpu().numpy()
    assert np.abs(r - d["rho_s"]).max() <= 1e-12 * np.abs(d["rho_s"]).max()
    for dt, etol, vtol in ((torch.float64, 1e-9, 1e-9), (torch.float32, 2e-5, 2e-4)):
        x = rho.to(dt)
        out = total(x, calcType={"E", "V"})
        parts = _split_energies(total, x)
        for k, v in parts.items():
            ref = float(d["E_" + k])
            assert abs(v - ref) <= etol * abs(ref), (dt, k, v, ref)
        e_ref = float(d["E_total"])
        assert abs(out.energy - e_ref) <= (etol if dt == torch.float64 else 2e-6) * abs(e_ref), (dt, out.energy)
        v = out.potential.as_subclass(torch.Tensor).reshape(-1)[torch.tensor(idx, device="cuda")].double()
        assert np.abs(v.cpu().numpy() - d["V_s"]).max() <= vtol * float(d["V_absmax"]), dt
    f = total.get_forces(rho)
    fref = d["forces_pp"] + d["forces_ii"]
    assert np.abs(f - fref).max() <= 1e-8, np.abs(f - fref).max()


def test_mixed_solution_is_the_oracle_minimum(large):
    """The mixed-precision solve of the 4000-atom cell (learned guess, econv
    1e-8 Ha/atom), then the oracle at the solved density."""
    torch = large["torch"]
    from dftpy_gb300 import guess as G
    from dftpy_gb300.optimization import Optimization
    st, grid, total = large["st"], large["grid"], large["total"]
    lg = G.LearnedGuess(G.GuessNet.load(os.path.join(ROOT, "dftpy_gb300", "data", "guessnet_al_wt.npz")))
    g0 = lg.guess(total, grid)
    opt = Optimization(EnergyEvaluator=total, optimization_method="TN",
                       optimization_options={"econv": 1e-8 * st.nat, "maxfun": 50, "maxiter": 100,
                                             "precision": "mixed"})
    rho_m = opt.optimize_rho(guess_rho=g0)
    # 0: converged; 1: the refinement's last line search found no decrease.
    # The LMGP term widens its k_F range during the solve, so the functional
    # moves between iterations and a final line search can stop at the FP64
    # rounding level (the plain FP64 TN stops the same way on this cell); the
    # oracle's residual at the returned density below is what decides.
    assert opt.converged in (0, 1), opt.converged
    f_gpu = total.get_forces(rho_m)
    e_gpu = float(total(rho_m, calcType={"E"}).energy)
    d = total.KineticEnergyFunctional._lwt.prepare(rho_m)
    kf_state = {"kfmin": float(d.kfmin_state), "kfmax": float(d.kfmax_state)}
    # the oracle at the solved density (FFTs on every host core)
    O.set_fft_workers(os.cpu_count() or 1)
    try:
        ev = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")

        def oracle(rn, saved):
            lw = O.LWTNL("MGP", "linear")
            lw.saved = dict(saved)
            e, v = ev(rn, True)
            e2, v2 = lw(rn, ev.grid, calc_e=True, calc_v=True)
            return e + e2, v + v2

        def residual(rn, saved):
            e, v = oracle(rn, saved)
            dV = ev.grid.dV
            mu = float((v * rn).sum() / rn.sum())
            res = (v - mu) * np.sqrt(np.maximum(rn, 0.0))
            return e, float(np.sqrt((res * res).sum() * dV))

        rm = rho_m.to_numpy()
        e_o, res_m = residual(rm, kf_state)
        _, res_g = residual(g0.to_numpy(), {"kfmin": None, "kfmax": None})
        f_o = ev.forces(rm)
    finally:
        O.set_fft_workers(1)
    assert abs(e_gpu - e_o) <= 1e-9 * abs(e_o), (e_gpu, e_o)
    assert np.abs(f_gpu - f_o).max() <= 1e-5, np.abs(f_gpu - f_o).max()
    print("residual: guess %.3e solved %.3e" % (res_g, res_m))
    # the TN stops on the energy change (econv = 4e-5 Ha over the 4000 atoms),
    # not on the residual: there the oracle's residual is ~1e-3 of the
    # guess's (measured 1.07e-3)
    assert res_m <= 2e-3 * res_g, (res_m, res_g)
