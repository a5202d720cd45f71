"""The public API (reference-shaped classes) on the GPU against the oracle and
the reference-generated fixtures.

Tolerances (FP64): energies 1e-10 Ha relative to the component, potentials
1e-10 of max|V|; full TN solves: energy within 1e-6 Ha/atom and forces
context-free (density) within the reference's own run-to-run spread.
"""
import numpy as np
import pytest

from dftpy_gb300 import systems
from oracle import ofdft as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def api():
    import torch
    from dftpy_gb300 import _lib
    _lib.require_cuda()
    from dftpy_gb300 import field, functional, grid, ions, optimization
    return dict(torch=torch, field=field, functional=functional, grid=grid, ions=ions, opt=optimization)


def _ions(api, st):
    return api["ions"].Ions(st.symbols, positions=st.positions, cell=st.lattice)


def _pp(api, symbols):
    F = api["functional"]
    return {s: F.AnalyticPP(*systems.SPECIES[s]) for s in set(symbols)}


@pytest.mark.parametrize("pme", [True, False])
@pytest.mark.parametrize("case", ["al4", "fde"])
def test_local_pseudo_and_ewald(api, golden, case, pme):
    if case == "al4":
        st = systems.config_al4(0)
        lat, nr, pos, sym, full = st.lattice, st.nr, st.positions, st.symbols, False
    else:
        d = golden("fde")
        lat, nr, pos, sym, full = d["lattice"], tuple(int(x) for x in d["nr"]), d["positions"], ["Al", "Al"], True
    grid = api["grid"].DirectGrid(lat, nr, full=full)
    ions = api["ions"].Ions(sym, positions=pos, cell=lat)
    ps = api["functional"].LocalPseudo(grid=grid, ions=ions, PP_list=_pp(api, sym), PME=pme)
    g = O.Grid(lat, nr, full=full)
    tab = {s: systems.analytic_pp_table(*systems.SPECIES[s]) for s in set(sym)}
    vref = O.local_pp(g, pos, sym, tab, pme=pme)
    v = ps.vreal.to_numpy()
    assert np.abs(v - vref).max() <= 1e-10 * np.abs(vref).max()
    ew = ps.get_ewald()
    ref = O.ewald_energy(g, pos, np.array([systems.SPECIES[s][0] for s in sym]), pme=pme)
    assert abs(ew.eta - ref["eta"]) < 1e-12
    assert abs(ew.Energy_real() - ref["real"]) < 1e-9
    assert abs(ew.Energy_rec() - ref["rec"]) < 1e-9 * max(1.0, abs(ref["rec"]))
    assert abs(ew.energy - ref["energy"]) < 1e-9 * max(1.0, abs(ref["energy"]))
    if case == "fde" and pme:
        # the reference's own asserted values (test_ewald.py:46-49)
        assert abs(ref["corr"] - -13.003839613564997) < 1e-5
        assert abs(ref["rec"] - 7.606943756474895) < 1e-5


@pytest.mark.parametrize("pme", [True, False])
@pytest.mark.parametrize("case", ["al4", "fde"])
def test_forces_match_oracle_and_fixture(api, golden, case, pme):
    """PP and Ewald forces (FP64) against the oracle (1e-10 Ha/Bohr) and the
    forces the reference computed for the same density."""
    if case == "al4":
        d = golden("al4")
        st = systems.config_al4(0)
        lat, nr, pos, sym, full = st.lattice, st.nr, st.positions, st.symbols, False
    else:
        d = golden("fde")
        lat, nr, pos, sym, full = d["lattice"], tuple(int(x) for x in d["nr"]), d["positions"], ["Al", "Al"], True
    rho_np = np.ascontiguousarray(d["rho"])
    grid = api["grid"].DirectGrid(lat, nr, full=full)
    ions = api["ions"].Ions(sym, positions=pos, cell=lat)
    ps = api["functional"].LocalPseudo(grid=grid, ions=ions, PP_list=_pp(api, sym), PME=pme)
    rho = api["field"].DirectField(grid, data=rho_np)
    g = O.Grid(lat, nr, full=full)
    tab = {s: systems.analytic_pp_table(*systems.SPECIES[s]) for s in set(sym)}
    f_pp = ps.forces(rho)
    ref_pp = (O.pp_forces_pme if pme else O.pp_forces_exact)(rho_np, g, pos, sym, tab)
    np.testing.assert_allclose(f_pp, ref_pp, rtol=0, atol=1e-10)
    f_ii = ps.get_ewald().forces
    q = np.array([systems.SPECIES[s][0] for s in sym])
    np.testing.assert_allclose(f_ii, O.ewald_forces(g, pos, q, pme=pme), rtol=0, atol=1e-9)
    if case == "fde":
        np.testing.assert_allclose(f_pp, d["F_PP_PME" if pme else "F_PP_EXACT"], rtol=0, atol=1e-10)
        np.testing.assert_allclose(f_ii, d["EW_forces_pme" if pme else "EW_forces"], rtol=0, atol=1e-9)
    elif pme:
        np.testing.assert_allclose(f_pp, d["forces_pp"], rtol=0, atol=1e-10)
        np.testing.assert_allclose(f_ii, d["forces_ii"], rtol=0, atol=1e-9)


def test_forces_fp32_density(api, golden):
    """PME PP forces from an FP32 density agree with the FP64 ones to FP32
    transform accuracy (far inside the 1e-5 Ha/Bohr force gate)."""
    torch = api["torch"]
    d = golden("al4")
    st = systems.config_al4(0)
    grid = api["grid"].DirectGrid(st.lattice, st.nr, full=False)
    ps = api["functional"].LocalPseudo(grid=grid, ions=_ions(api, st), PP_list=_pp(api, st.symbols), PME=True)
    rho = api["field"].DirectField(grid, data=np.ascontiguousarray(d["rho"]))
    f64 = ps.forces(rho)
    f32 = ps.forces(rho.to(torch.float32))
    assert np.abs(f32 - f64).max() < 1e-6


def test_total_functional_fused_vs_members(api, golden):
    """Fused single-launch evaluation equals the sum of the members' outputs."""
    torch = api["torch"]
    F = api["functional"]
    a = golden("al4")
    st = systems.config_al4(0)
    grid = api["grid"].DirectGrid(st.lattice, st.nr, full=False)
    ions = _ions(api, st)
    ps = F.LocalPseudo(grid=grid, ions=ions, PP_list=_pp(api, st.symbols), PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="TFVW"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rho = api["field"].DirectField(grid, data=a["rho"])
    out = total(rho)
    parts = total.get_energy_potential(rho, split=True)
    assert abs(out.energy - parts["TOTAL"].energy) < 1e-10 * abs(out.energy)
    assert float((out.potential - parts["TOTAL"].potential).abs().max()) < 1e-10
    ev = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")
    e_ref, v_ref = ev(a["rho"])
    assert abs(out.energy - e_ref) < 1e-10 * abs(e_ref)
    assert abs(out.energy - float(a["E_final"])) < 1e-8
    assert np.abs(out.potential.to_numpy() - v_ref).max() < 1e-10 * np.abs(v_ref).max()
    # FunctionalOutput algebra (test_functional.py:18-21)
    assert abs((out + out).energy - 2 * out.energy) < 1e-12 * abs(out.energy)
    assert abs((out * 2).energy - 2 * out.energy) < 1e-12 * abs(out.energy)
    assert abs((out / 2).energy - out.energy / 2) < 1e-12 * abs(out.energy)


def test_field_fft_roundtrip_full_grid(api, golden):
    torch = api["torch"]
    d = golden("fde")
    grid = api["grid"].DirectGrid(d["lattice"], tuple(int(x) for x in d["nr"]), full=True)
    rho = api["field"].DirectField(grid, data=np.ascontiguousarray(d["rho"]))
    rg = rho.fft()
    assert tuple(rg.shape) == tuple(int(x) for x in d["nr"])
    ref = np.fft.fftn(d["rho"]) * grid.dV
    assert np.abs(rg.to_numpy() - ref).max() < 1e-12 * np.abs(ref).max()
    back = rg.ifft()
    assert np.abs(back.to_numpy() - d["rho"]).max() < 1e-12 * np.abs(d["rho"]).max()
    assert abs(rho.integral() - float(d["rho"].sum() * grid.dV)) < 1e-10


def _solve(api, st, kedf, econv, precision="fp64", **extra):
    torch = api["torch"]
    F = api["functional"]
    grid = api["grid"].DirectGrid(st.lattice, st.nr, full=False)
    ions = _ions(api, st)
    ps = F.LocalPseudo(grid=grid, ions=ions, PP_list=_pp(api, st.symbols), PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name=kedf),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rho0 = api["field"].DirectField(grid)
    rho0[:] = st.nelec / st.volume
    opts = {"econv": econv, "maxfun": 50, "maxiter": 100, "precision": precision}
    opts.update(extra)
    opt = api["opt"].Optimization(EnergyEvaluator=total, optimization_method="TN", optimization_options=opts)
    rho = opt.optimize_rho(guess_rho=rho0)
    return opt, rho, total


def test_tn_al4_matches_reference_solve(api, golden):
    a = golden("al4")
    st = systems.config_al4(0)
    opt, rho, total = _solve(api, st, "TFVW", 1e-7)
    assert opt.converged == 0
    E = total.Energy(rho)
    assert abs(E - float(a["E_final"])) < 1e-6 * st.nat
    assert abs(E - float(a["E_final"])) < 1e-8
    s = opt.stats["stages"][-1]
    # same control flow as the reference: evaluation counts within a couple
    assert abs(s["n_eval_ev"] - int(a["n_ev"])) <= 2 and abs(s["n_eval_v"] - int(a["n_v"])) <= 6
    assert np.abs(rho.to_numpy() - a["rho"]).max() < 1e-5
    F = total.get_forces(rho)
    assert np.abs(F - a["forces"]).max() < 1e-5
    parts = total.get_forces(rho, split=True)
    np.testing.assert_allclose(parts["TOTAL"], parts["PSEUDO"] + parts["II"], rtol=0, atol=1e-14)


def test_tn_al256_wt_matches_reference_solve(api, golden):
    """Config 2 at full size: 256 Al, 128^3, WT; the reference solve took 81 s."""
    a = golden("al256")
    st = systems.config_al256(0)
    opt, rho, total = _solve(api, st, "WT", 1e-7)
    assert opt.converged == 0
    E = total.Energy(rho)
    assert abs(E - float(a["E_final"])) < 1e-6 * st.nat
    r = rho.to_numpy().ravel()[a["sample_idx"]]
    assert np.abs(r - a["rho_s"]).max() < 1e-4
    # forces of the converged density within 1e-5 Ha/Bohr of the reference's
    assert np.abs(total.get_forces(rho) - a["forces"]).max() < 1e-5


@pytest.mark.parametrize("refine", ["split", "fp64"])
def test_tn_al4_mixed_precision(api, golden, refine):
    a = golden("al4")
    st = systems.config_al4(0)
    opt, rho, total = _solve(api, st, "TFVW", 1e-7, precision="mixed", refine=refine)
    last = opt.stats["stages"][-1]
    assert (last["n_eval_hess"] > 0) == (refine == "split")
    E = total.Energy(rho.to(api["torch"].float64))
    # 1e-5 eV/atom of the FP64 reference solve
    assert abs(E - float(a["E_final"])) < 1e-5 / 27.211386 * st.nat
    assert np.abs(total.get_forces(rho) - a["forces"]).max() < 1e-5


def test_tn_al256_mixed_split_refine(api, golden):
    """256 Al, 128^3, WT: FP32 TN then FP64 refinement with FP32 Hessian
    products; energy within 1e-5 eV/atom and forces within 1e-5 Ha/Bohr of the
    reference's FP64 solve."""
    a = golden("al256")
    t = golden("al256_tight")      # the reference's solve converged to econv 1e-10
    st = systems.config_al256(0)
    opt, rho, total = _solve(api, st, "WT", 1e-7, precision="mixed")
    E = total.Energy(rho)
    assert abs(E - float(a["E_final"])) < 1e-5 / 27.211386 * st.nat
    F = total.get_forces(rho)
    assert np.abs(F - a["forces"]).max() < 1e-5
    assert np.abs(F - t["forces"]).max() < 1e-5
    # the refinement after its first evaluation runs delta evaluations
    assert opt.stats["stages"][-1]["n_eval_delta"] > 0


def test_tn_al256_mixed_delta_refine_matches_full_refine(api):
    """The delta-evaluated refinement against the same refinement with every
    FP64 evaluation in full: energies within 1e-9 eV/atom, forces within
    1e-6 Ha/Bohr, densities within 1e-5 of max rho."""
    st = systems.config_al256(0)
    opt_d, rho_d, total = _solve(api, st, "WT", 1e-7, precision="mixed")
    opt_f, rho_f, _ = _solve(api, st, "WT", 1e-7, precision="mixed", refine_delta=False)
    assert opt_f.stats["stages"][-1]["n_eval_delta"] == 0
    assert opt_d.stats["stages"][-1]["n_eval_delta"] > 0
    assert abs(opt_d.energy - opt_f.energy) < 1e-9 / 27.211386 * st.nat
    a, b = rho_d.to_numpy(), rho_f.to_numpy()
    assert np.abs(a - b).max() < 1e-5 * np.abs(b).max()
    assert np.abs(total.get_forces(rho_d) - total.get_forces(rho_f)).max() < 1e-6


@pytest.mark.parametrize("interp", ["linear", "hermite"])
@pytest.mark.parametrize("prec", [1, 0])
def test_lmgp_reference_fixture(api, golden, interp, prec):
    """KEDF LMGP (TF + vW + LMGP-NL) on the reference's test density (full grid,
    non-orthogonal cell) against the reference-generated energy and potential
    (test_functional.py:29-34 asserts 2.9145872498710492 for linear)."""
    torch = api["torch"]
    F = api["functional"]
    d = golden("fde")
    grid = api["grid"].DirectGrid(d["lattice"], tuple(int(x) for x in d["nr"]), full=True)
    dt = torch.float64 if prec == 1 else torch.float32
    rho = api["field"].DirectField(grid, data=np.ascontiguousarray(d["rho"]), dtype=dt)
    ke = F.Functional(type="KEDF", name="LMGP", interp=interp)
    out = ke(rho)
    E = float(d["E_LMGP_" + interp])
    vs = d["Vs_LMGP_" + interp]
    etol, vtol = (1e-10, 1e-9) if prec == 1 else (2e-5, 2e-3)
    assert abs(out.energy - E) <= etol * abs(E), (out.energy, E)
    v = out.potential.to_numpy().ravel()[d["sample_idx"]]
    assert np.abs(v - vs).max() <= vtol * np.abs(vs).max()
    if interp == "linear" and prec == 1:
        assert abs(out.energy - 2.9145872498710492) < 1e-10
        assert ke._lwt.prepare(rho).nknots == 15


def test_tn_al4_lmgp_matches_oracle(api):
    """TN with LMGP + LDA + Hartree + PP (config-5 functional, config-1 size)
    against the oracle's TN solve: energy within 1e-6 Ha/atom."""
    torch = api["torch"]
    F = api["functional"]
    st = systems.config_al4(0)
    grid = api["grid"].DirectGrid(st.lattice, st.nr, full=False)
    ps = F.LocalPseudo(grid=grid, ions=_ions(api, st), PP_list=_pp(api, st.symbols), PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="LMGP"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rho0 = api["field"].DirectField(grid)
    rho0[:] = st.nelec / st.volume
    opt = api["opt"].Optimization(EnergyEvaluator=total, optimization_method="TN",
                                  optimization_options={"econv": 1e-7, "maxfun": 50, "maxiter": 100})
    rho = opt.optimize_rho(guess_rho=rho0)
    # oracle: same functional, same TN
    ev = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")
    lw = O.LWTNL("MGP", "linear")

    def evaluator(r, calc_e):
        e, v = ev(r, calc_e)
        e2, v2 = lw(r, ev.grid, calc_e=calc_e, calc_v=True)
        return (None if e is None else e + e2), v + v2
    ref = O.optimize_tn(evaluator, np.full(st.nr, st.nelec / st.volume), ev.grid, econv=1e-7, maxfun=50,
                        maxiter=100)
    # the reference algorithm stops this solve on a line-search failure after
    # a few iterations (status 1); the device solve must end the same way at
    # the same energy
    assert opt.converged == ref["converged"], (opt.converged, ref["converged"])
    assert abs(opt.energy - ref["energy"]) < 1e-6 * st.nat, (opt.energy, ref["energy"])


@pytest.mark.parametrize("pme", [True, False])
@pytest.mark.parametrize("case", ["al4", "fde"])
def test_density_guess_matches_reference(api, golden, case, pme):
    """Superposed atomic densities on the GPU against the reference's
    get_3d_value_recipe output (FP64: 1e-12 of max rho) and the oracle; the
    FP32 plan to 1e-6 relative; the electron count exactly restored."""
    torch = api["torch"]
    from dftpy_gb300.density import DensityGenerator
    d = golden("guess")
    if case == "al4":
        st = systems.config_al4(0)
        lat, nr, pos, sym, full = st.lattice, st.nr, st.positions, list(st.symbols), False
    else:
        f = golden("fde")
        lat, nr, pos, sym, full = f["lattice"], tuple(int(x) for x in f["nr"]), f["positions"], ["Al", "Al"], True
    grid = api["grid"].DirectGrid(lat, nr, full=full)
    ions = api["ions"].Ions(sym, positions=pos, cell=lat)
    ions.set_charges({s: systems.SPECIES[s][0] for s in set(sym)})
    r, arho = {}, {}
    for s in set(sym):
        r[s], arho[s] = systems.atomic_density_table(systems.SPECIES[s][0], systems.ATOMIC_SIGMA[s])
    gen = DensityGenerator(r=r, arho=arho)
    rho = gen.guess_rho(ions, grid=grid, pme=pme)
    x = rho.to_numpy()
    tag = case + ("_pme" if pme else "_exact")
    ref = d[tag + "_s"]
    assert np.abs(x.ravel()[d[case + "_idx"]] - ref).max() <= 1e-12 * np.abs(ref).max()
    nel = sum(systems.SPECIES[s][0] for s in sym)
    assert abs(rho.integral() - nel) < 1e-10
    g = O.Grid(lat, nr, full=full)
    tab = {s: (r[s], arho[s]) for s in set(sym)}
    o = O.density_guess_recipe(g, pos, sym, tab, nel, pme=pme)
    assert np.abs(x - o).max() <= 1e-12 * np.abs(o).max()
    rho32 = DensityGenerator(r=r, arho=arho).guess_rho(
        ions, grid=grid, rho=api["field"].DirectField(grid, dtype=torch.float32), pme=pme)
    assert rho32.dtype == torch.float32
    assert np.abs(rho32.to_numpy().astype(np.float64) - o).max() <= 1e-6 * np.abs(o).max()


def test_tn_from_atomic_guess(api, golden):
    """A TN solve started from the superposed atomic density reaches the
    reference's energy."""
    from dftpy_gb300.density import DensityGenerator
    a = golden("al4")
    st = systems.config_al4(0)
    F = api["functional"]
    grid = api["grid"].DirectGrid(st.lattice, st.nr, full=False)
    ions = _ions(api, st)
    ps = F.LocalPseudo(grid=grid, ions=ions, PP_list=_pp(api, st.symbols), PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="TFVW"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    r, arho = {}, {}
    for s in set(st.symbols):
        r[s], arho[s] = systems.atomic_density_table(systems.SPECIES[s][0], systems.ATOMIC_SIGMA[s])
    rho0 = DensityGenerator(r=r, arho=arho).guess_rho(ps.ions, grid=grid)
    opt = api["opt"].Optimization(EnergyEvaluator=total, optimization_method="TN",
                                  optimization_options={"econv": 1e-7, "maxfun": 50, "maxiter": 100})
    rho = opt.optimize_rho(guess_rho=rho0)
    assert opt.converged == 0
    assert abs(total.Energy(rho) - float(a["E_final"])) < 1e-6 * st.nat


def test_config5_lmgp_translation_invariance(api):
    """4000 Al, 360^3, LMGP + LDA + Hartree + PP (PME) at full size, through a
    size-independent property: moving every atom by one grid step along a
    lattice vector and rolling the density by one point gives the same energy
    (1e-11 relative) and the rolled potential (1e-10 of max|V|); the FP32
    evaluation agrees with the FP64 one to 1e-6 relative."""
    torch = api["torch"]
    F = api["functional"]
    from dftpy_gb300.density import DensityGenerator
    st = systems.config_al4000(0)
    grid = api["grid"].DirectGrid(st.lattice, st.nr, full=False)
    r, a = {"Al": None}, {"Al": None}
    r["Al"], a["Al"] = systems.atomic_density_table(3.0, systems.ATOMIC_SIGMA["Al"])

    def energy_potential(positions, rho=None, shift=0, dtype=torch.float64):
        ions = api["ions"].Ions(st.symbols, positions=positions, cell=st.lattice)
        ps = F.LocalPseudo(grid=grid, ions=ions, PP_list=_pp(api, st.symbols), PME=True)
        total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="LMGP"),
                                  XCFunctional=F.Functional(type="XC", name="LDA"),
                                  HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
        if rho is None:
            rho = DensityGenerator(r=r, arho=a).guess_rho(ps.ions, grid=grid)
        x = torch.roll(rho.as_subclass(torch.Tensor), shifts=shift, dims=0).to(dtype).contiguous()
        out = total(api["field"].DirectField(grid, data=x), calcType={"E", "V"})
        return rho, float(out.energy), out.potential.as_subclass(torch.Tensor)

    step = st.lattice[0] / st.nr[0]
    rho, e0, v0 = energy_potential(st.positions)
    _, e1, v1 = energy_potential(st.positions + step, rho=rho, shift=1)
    assert abs(e1 - e0) <= 1e-11 * abs(e0), (e0, e1)
    vmax = float(v0.abs().max())
    assert float((torch.roll(v0, shifts=1, dims=0) - v1).abs().max()) <= 1e-10 * vmax
    _, e32, _ = energy_potential(st.positions, rho=rho, dtype=torch.float32)
    assert abs(e32 - e0) <= 1e-6 * abs(e0), (e0, e32)


@pytest.mark.parametrize("pme", [True, False])
def test_stress_fde_matches_reference(api, golden, pme):
    """Every stress term (WT + LDA + Hartree + PP + Ewald) on the reference's
    skewed test density (full grid), FP64: within 1e-11 Ha/Bohr^3 of the
    reference's tensors (values ~1e-3)."""
    F = api["functional"]
    d = golden("fde")
    S = golden("stress")
    grid = api["grid"].DirectGrid(d["lattice"], tuple(int(x) for x in d["nr"]), full=True)
    ions = api["ions"].Ions(["Al", "Al"], positions=d["positions"], cell=d["lattice"])
    ps = F.LocalPseudo(grid=grid, ions=ions, PP_list=_pp(api, ["Al"]), PME=pme)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="WT"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rho = api["field"].DirectField(grid, data=np.ascontiguousarray(d["rho"]))
    out = total.get_stress(rho, split=True)
    tag = "fde_%s_" % ("pme" if pme else "exact")
    for k in ("KEDF-TF", "KEDF-VW", "KEDF-NL", "XC", "HARTREE", "PSEUDO", "II", "TOTAL"):
        np.testing.assert_allclose(out[k], S[tag + k], rtol=0, atol=1e-11, err_msg=k)


def test_stress_al4_total_and_fp32(api, golden):
    """4-Al converged density (TFVW): the total stress against the reference
    (1e-11); the FP32 path to 1e-7 Ha/Bohr^3."""
    torch = api["torch"]
    F = api["functional"]
    a = golden("al4")
    S = golden("stress")
    st = systems.config_al4(0)
    grid = api["grid"].DirectGrid(st.lattice, st.nr, full=False)
    ps = F.LocalPseudo(grid=grid, ions=_ions(api, st), PP_list=_pp(api, st.symbols), PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="TFVW"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rho = api["field"].DirectField(grid, data=np.ascontiguousarray(a["rho"]))
    out = total.get_stress(rho, split=True)
    for k in ("KEDF-TF", "KEDF-VW", "XC", "HARTREE", "PSEUDO", "II", "TOTAL"):
        np.testing.assert_allclose(out[k], S["al4_" + k], rtol=0, atol=1e-11, err_msg=k)
    s32 = total.get_stress(rho.to(torch.float32))
    assert np.abs(s32 - S["al4_TOTAL"]).max() < 1e-7


def test_local_pseudo_from_recpot_file(api, tmp_path):
    """A pseudopotential given as a recpot file path: the device v_loc equals
    the oracle's for the table the file holds (FP64, 1e-10 of max|v|)."""
    from dftpy_gb300 import pseudo_files as P
    st = systems.config_al4(0)
    gp = np.linspace(0.0, 30.0, 6001)
    vp = np.empty_like(gp)
    vp[1:] = -4.0 * np.pi * 3.0 * np.exp(-(gp[1:] * 1.0) ** 2 / 4.0) / gp[1:] ** 2
    vp[0] = np.pi * 3.0
    path = str(tmp_path / "al.recpot")
    P.write_recpot(path, gp, vp)
    pp = P.read_pp(path)
    assert pp.zval == 3.0
    grid = api["grid"].DirectGrid(st.lattice, st.nr, full=False)
    ps = api["functional"].LocalPseudo(grid=grid, ions=_ions(api, st), PP_list={"Al": path}, PME=True)
    g = O.Grid(st.lattice, st.nr)
    ref = O.local_pp(g, st.positions, st.symbols, {"Al": (pp.radial_grid, pp.local_potential)}, pme=True)
    v = ps.vreal.to_numpy()
    assert np.abs(v - ref).max() <= 1e-10 * np.abs(ref).max()


class _Atoms:
    """The few ``ase.Atoms`` members the calculator reads (Angstrom)."""

    def __init__(self, symbols, positions, cell):
        self.symbols = list(symbols)
        self.positions = np.array(positions, float)
        self.cell = np.array(cell, float)

    def get_positions(self):
        return self.positions.copy()

    def get_chemical_symbols(self):
        return list(self.symbols)


def test_ase_calculator_forces_are_energy_gradient(api):
    """DFTpyCalculator (evaluator path) on 4 Al: forces equal the central
    difference of the optimised energy (eV/A), and the second ionic step,
    starting from the first step's density, takes fewer evaluations than the
    first one from the uniform density."""
    from dftpy_gb300.api4ase import DFTpyCalculator
    from dftpy_gb300.pseudo_files import BOHR_ANG
    F = api["functional"]
    st = systems.config_al4(0)
    grid = api["grid"].DirectGrid(st.lattice, st.nr, full=False)
    ps = F.LocalPseudo(grid=grid, ions=_ions(api, st), PP_list=_pp(api, st.symbols), PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="TFVW"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rho0 = api["field"].DirectField(grid)
    rho0[:] = st.nelec / st.volume
    opt = api["opt"].Optimization(EnergyEvaluator=total, optimization_method="TN",
                                  optimization_options={"econv": 1e-10, "maxfun": 50, "maxiter": 200})
    calc = DFTpyCalculator(evaluator=total, optimizer=opt, rho=rho0)
    atoms = _Atoms(st.symbols, st.positions * BOHR_ANG, st.lattice * BOHR_ANG)
    calc.get_potential_energy(atoms)
    n_first = sum(s["n_eval_ev"] + s["n_eval_v"] for s in opt.stats["stages"])
    f = calc.get_forces(atoms)
    assert f.shape == (4, 3)
    h = 0.004
    e = []
    for sgn in (1, -1):
        a = _Atoms(st.symbols, st.positions * BOHR_ANG, st.lattice * BOHR_ANG)
        a.positions[0, 0] += sgn * h
        e.append(calc.get_potential_energy(a))
        if sgn == 1:
            n_second = sum(s["n_eval_ev"] + s["n_eval_v"] for s in opt.stats["stages"])
    fd = -(e[0] - e[1]) / (2 * h)
    assert abs(fd - f[0, 0]) < 2e-3 + 1e-2 * abs(f[0, 0]), (fd, f[0, 0])
    assert n_second < n_first
    s = calc.get_stress(atoms)
    assert s.shape == (6,)


@pytest.mark.parametrize("full", [False, True])
@pytest.mark.parametrize("case", ["up", "up_even", "down", "down_even"])
def test_grid_map_matches_reference(api, golden, case, full):
    """Spectral interpolation between grids against the reference's
    grid_map_data / field2distrib (half and full spectra, both directions)."""
    from dftpy_gb300.utils import field2distrib, grid_map_data
    d = golden("gridmap")
    tag = case + ("_full" if full else "_half")
    x, ref = d[tag + "_in"], d[tag + "_out"]
    g1 = api["grid"].DirectGrid(d["cell"], x.shape, full=full)
    f1 = api["field"].DirectField(g1, data=x)
    y = grid_map_data(f1, nr=np.array(ref.shape))
    assert tuple(y.shape) == ref.shape and y.grid.full == full
    np.testing.assert_allclose(y.to_numpy(), ref, rtol=0, atol=1e-13 * np.abs(ref).max())
    o2 = api["field"].DirectField(api["grid"].DirectGrid(d["cell"], ref.shape, full=full))
    field2distrib(f1, o2, tol=0.8)
    np.testing.assert_allclose(o2.to_numpy(), d[tag + "_distrib"], rtol=0, atol=1e-13 * np.abs(ref).max())


def test_multistep_al4_reaches_fine_grid_minimum(api, golden):
    """Coarse (16^3) then fine (32^3) TN solve ends at the reference's 32^3
    minimum: same energy and density as the direct fine-grid solve."""
    a = golden("al4")
    st = systems.config_al4(0)
    F = api["functional"]
    grid = api["grid"].DirectGrid(st.lattice, (16, 16, 16), full=False)
    ps = F.LocalPseudo(grid=grid, ions=_ions(api, st), PP_list=_pp(api, st.symbols), PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="TFVW"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rho0 = api["field"].DirectField(grid)
    rho0[:] = st.nelec / st.volume
    opt = api["opt"].Optimization(EnergyEvaluator=total, optimization_method="TN",
                                  optimization_options={"econv": 1e-7, "maxfun": 50, "maxiter": 100})
    rho = opt.optimize_rho_multistep(rho0, multistep=2, nr_final=tuple(st.nr))
    assert tuple(rho.grid.nrR) == tuple(st.nr) and ps.grid is rho.grid
    assert opt.converged == 0
    assert abs(rho.integral() - st.nelec) < 1e-9
    E = total.Energy(rho)
    assert abs(E - float(a["E_final"])) < 1e-7
    assert np.abs(rho.to_numpy() - a["rho"]).max() < 1e-4


def test_batch_matches_individual_solves(api):
    """Several Al/Mg structures of different cells and grids optimised
    concurrently (one stream and host thread each) give exactly the energies
    of the same solves run one after another, and those energies equal the
    oracle's functional at the solved densities."""
    from dftpy_gb300 import batch
    sts = [systems.fcc_supercell(r, sigma=0.15, seed=s, nr=n, mg_fraction=0.25, name="b%d" % s)
           for s, (r, n) in enumerate([((1, 1, 1), (32, 32, 32)), ((1, 1, 2), (32, 32, 64)),
                                       ((1, 2, 2), (32, 64, 64)), ((1, 1, 1), (36, 36, 36))])]
    opts = {"econv": 1e-8, "precision": "fp64"}  # total, Ha
    par = batch.optimize_batch(sts, workers=4, options=opts, kedf="TFVW")
    seq = batch.optimize_batch(sts, workers=1, options=opts, kedf="TFVW")
    assert [r.name for r in par] == [st.name for st in sts]
    for st, a, b in zip(sts, par, seq):
        assert a.converged == 0 and b.converged == 0
        assert a.energy == b.energy
        np.testing.assert_array_equal(a.rho.to_numpy(), b.rho.to_numpy())
        ev = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")
        e_ref, _ = ev(a.rho.to_numpy())
        assert abs(a.energy - e_ref) < 1e-9 * abs(e_ref)


def test_wgc_solve_alloy(api):
    """TN with the WGC KEDF (second-order density-dependent kernel) on an
    Al/Mg cell: converges, the energy equals the oracle's functional at the
    solved density, and the mixed-precision solve agrees with FP64 within
    1e-5 eV/atom."""
    from dftpy_gb300 import batch
    from oracle import wgc as W
    st = systems.fcc_supercell((1, 1, 2), sigma=0.15, seed=4, nr=(32, 32, 64), mg_fraction=0.25, name="wgc")
    res = {}
    for prec in ("fp64", "mixed"):
        r = batch.optimize_batch([st], workers=1, options={"precision": prec, "econv": 1e-8}, kedf="WGC")[0]
        assert r.converged == 0, prec
        res[prec] = r
    rho = res["fp64"].rho.to_numpy()
    g = O.Grid(st.lattice, st.nr)
    ev = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")
    e_base, _ = ev(rho)
    e_nl, _ = W.WGCNL()(rho, g)
    # the oracle solves the kernel equation by another method (agreement ~1e-6)
    assert abs(res["fp64"].energy - (e_base + e_nl)) < 2e-5 * abs(e_nl)
    assert abs(res["mixed"].energy - res["fp64"].energy) / st.nat * 27.211386 < 1e-5


class _TablePP:
    """A reciprocal-space pseudopotential table (the ``BasePseudo`` members
    LocalPseudo reads)."""

    def __init__(self, gp, vp, z):
        self.radial_grid, self.local_potential, self.zval = np.asarray(gp), np.asarray(vp), float(z)
        self.direct = False


def test_tn_gaas_recpot_matches_reference_test(api, golden):
    """The reference's own TN test (``test_density_opt.py:15-46``): GaAs_random
    (5 Ga + 5 As) with the tables its ReadPseudo builds from the recpot files,
    PME, WT + LDA + Hartree on the ecut2nr(spacing=0.4) grid, from the uniform
    density.  The reference asserts isclose(E, -43.3046); its own converged
    energy (econv 1e-6 Ha/atom) is the fixture.  Here econv 1e-8 Ha/atom:
    within 1e-6 Ha/atom of the reference's energy."""
    d = golden("gaas")
    torch = api["torch"]
    F = api["functional"]
    nr = tuple(int(x) for x in d["nr"])
    grid = api["grid"].DirectGrid(d["lattice"], nr, full=False)
    symbols = [str(s) for s in d["symbols"]]
    ions = api["ions"].Ions(symbols, positions=d["positions"], cell=d["lattice"])
    pp = {k: _TablePP(d[k + "_gp"], d[k + "_vp"], d[k + "_zval"]) for k in ("Ga", "As")}
    ps = F.LocalPseudo(grid=grid, ions=ions, PP_list=pp, PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="WT"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rho0 = api["field"].DirectField(grid)
    rho0[:] = float(d["nelec"]) / grid.volume
    opt = api["opt"].Optimization(EnergyEvaluator=total, optimization_method="TN",
                                  optimization_options={"econv": 1e-8 * len(symbols), "maxfun": 50,
                                                        "maxiter": 100})
    rho = opt.optimize_rho(guess_rho=rho0)
    E = total.Energy(rho)
    assert np.isclose(E, -43.3046)
    assert abs(E - float(d["E_final"])) < 1e-6 * len(symbols), (E, float(d["E_final"]))


def test_tn_wgc_mixed_delta_refine_matches_full_refine(api):
    """WGC: the refinement with delta evaluations (the WGC term included)
    against the same refinement with every FP64 evaluation in full: energies
    within 1e-9 eV/atom, forces within 1e-6 Ha/Bohr."""
    from dftpy_gb300 import batch
    st = systems.config_alloy(2)
    res = {}
    for delta in (True, False):
        r = batch.optimize_batch([st], workers=1, kedf="WGC",
                                 options={"precision": "mixed", "econv_per_atom": 1e-8, "refine_delta": delta})[0]
        assert r.converged == 0
        res[delta] = r
    assert res[True].stats["stages"][-1]["n_eval_delta"] > 0
    assert res[False].stats["stages"][-1]["n_eval_delta"] == 0
    assert abs(res[True].energy - res[False].energy) < 1e-9 / 27.211386 * st.nat


@pytest.mark.parametrize("name,method,extra", [("cghs", "CG-HS", {}), ("cgpr", "CG-PR", {}),
                                               ("lbfgs", "LBFGS", {"h0": 1.0})])
def test_first_order_methods_match_reference(api, golden, name, method, extra):
    """The reference's first-order optimisers (CG-HS is its default method) on
    the 4-atom cell against the reference's own runs: the same starting
    energy (1e-9 Ha), convergence status, evaluation count within 10 % (the
    long CG-PR run's trajectory drifts with round-off), final energy within
    1e-6 Ha/atom and forces within 1e-5 Ha/Bohr."""
    d = golden("first_order")
    st = systems.config_al4(0)
    F = api["functional"]
    grid = api["grid"].DirectGrid(st.lattice, st.nr, full=False)
    ps = F.LocalPseudo(grid=grid, ions=_ions(api, st), PP_list=_pp(api, st.symbols), PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="TFVW"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rho0 = api["field"].DirectField(grid)
    rho0[:] = st.nelec / st.volume
    opts = {"econv": 1e-7, "maxiter": 200}
    opts.update(extra)
    kw = {} if method == "CG-HS" else {"optimization_method": method}
    opt = api["opt"].Optimization(EnergyEvaluator=total, optimization_options=opts, **kw)
    rho = opt.optimize_rho(guess_rho=rho0)
    h_ref = d[name + "_E_history"]
    assert opt.converged == int(d[name + "_converged"])
    n_ref = int(d[name + "_n_ev"])
    assert abs(opt.stats["stages"][0]["n_eval_ev"] - n_ref) <= max(2, 0.1 * n_ref)
    assert abs(opt.history[0] - h_ref[0]) < 1e-9
    E = total.Energy(rho)
    assert abs(E - float(d[name + "_E_final"])) < 1e-6 * st.nat
    assert np.abs(total.get_forces(rho) - d[name + "_forces"]).max() < 1e-5
