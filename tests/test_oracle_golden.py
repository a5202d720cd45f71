"""The CPU oracle against fixtures produced by running the reference DFTpy.

Pins the oracle before it is trusted as the checker of the GPU path:
component energies and potentials on the reference's own test density
(``examples/test/test_functional.py:24-34`` values included), Ewald terms
(``test_ewald.py:33-54``), the line-search trial sequences and a full TN solve.
"""
import numpy as np
import pytest

from dftpy_gb300 import systems
from oracle import ofdft as O


def _checks(v):
    v = np.asarray(v).ravel()
    return np.array([v.sum(), (v * v).sum(), np.abs(v).max(), v.min(), v.max()])


@pytest.fixture(scope="module")
def fde(golden):
    d = golden("fde")
    g = O.Grid(d["lattice"], d["nr"], full=True)   # the .pp reader builds a full grid
    return d, g


def _cmp(d, name, e, v, etol=1e-12, vtol=1e-12):
    assert abs(e - float(d["E_" + name])) <= etol * max(1.0, abs(float(d["E_" + name])))
    vs = d["Vs_" + name]
    assert np.abs(np.asarray(v).ravel()[d["sample_idx"]] - vs).max() <= vtol * np.abs(vs).max()
    ref = d["Vc_" + name]
    np.testing.assert_allclose(_checks(v), ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())


def test_reference_test_values(fde):
    d, _ = fde
    # the reference's own asserted values
    assert np.isclose(float(d["E_KEDF_WT"]), 2.916818700014412)
    assert np.isclose(float(d["EW_corr"]), -13.003839613564997, atol=1e-5)
    assert np.isclose(float(d["EW_rec"]), 7.606943756474895, atol=1e-5)
    assert np.isclose(float(d["EW_rec_pme"]), 7.606943756474895, atol=1e-5)
    assert np.isclose(float(d["E_LMGP_linear"]), 2.9145872498710492, atol=1e-3)


def test_kedf_components(fde):
    d, g = fde
    rho = d["rho"]
    e1, v1 = O.tf(rho, g)
    e2, v2 = O.vw(rho, g)
    e3, v3 = O.WTNL()(rho, g)
    _cmp(d, "TF", e1, v1)
    _cmp(d, "VW", e2, v2)
    _cmp(d, "WTNL", e3, v3)
    _cmp(d, "KEDF_WT", e1 + e2 + e3, v1 + v2 + v3)
    assert abs(e1 + e2 + e3 - 2.916818700014412) < 1e-12


def test_lda_hartree(fde):
    d, g = fde
    _cmp(d, "LDA", *O.lda(d["rho"], g))
    _cmp(d, "HARTREE", *O.hartree(d["rho"], g))


@pytest.mark.parametrize("pme", [True, False])
def test_local_pseudo(fde, pme):
    d, g = fde
    rho = d["rho"]
    tab = {"Al": systems.analytic_pp_table(*systems.SPECIES["Al"])}
    sym = ["Al"] * len(d["positions"])
    v = O.local_pp(g, d["positions"], sym, tab, pme=pme)
    tag = "PME" if pme else "EXACT"
    _cmp(d, "PP_" + tag, float(np.einsum("ijk,ijk->", v, rho) * g.dV), v)
    if pme:
        f = O.pp_forces_pme(rho, g, d["positions"], sym, tab)
        np.testing.assert_allclose(f, d["F_PP_PME"], atol=1e-12)
    else:
        f = O.pp_forces_exact(rho, g, d["positions"], sym, tab)
        np.testing.assert_allclose(f, d["F_PP_EXACT"], atol=1e-12)


@pytest.mark.parametrize("pme", [True, False])
def test_ewald(fde, pme):
    d, g = fde
    ew = O.ewald_energy(g, d["positions"], d["charges"], pme=pme)
    assert abs(ew["eta"] - float(d["EW_eta"])) < 1e-12
    assert abs(ew["corr"] - float(d["EW_corr"])) < 1e-10
    assert abs(ew["real"] - float(d["EW_real"])) < 1e-10
    ref = d["EW_rec_pme"] if pme else d["EW_rec"]
    assert abs(ew["rec"] - float(ref)) < 1e-10
    F = O.ewald_forces(g, d["positions"], d["charges"], pme=pme)
    np.testing.assert_allclose(F, d["EW_forces_pme"] if pme else d["EW_forces"], atol=1e-10)


def test_fft_convention(fde):
    d, g = fde
    np.testing.assert_allclose(O.fft(d["rho"], g).ravel()[d["FFT_idx"]], d["FFT_s"], rtol=0, atol=1e-12)


def test_spline_matches_fitpack():
    from scipy.interpolate import splev, splrep
    gp, vp = systems.analytic_pp_table(3.0, 1.0)
    sp = O.spline_notaknot(gp[1:], vp[1:])
    q = np.random.default_rng(0).uniform(gp[1], gp[-1], 20000)
    ref = splev(q, splrep(gp[1:], vp[1:]))
    assert np.max(np.abs(O.spline_eval(sp, q) - ref) / np.abs(ref)) < 1e-12


LS_CASES = {
    "quad": lambda a: ((a - 0.7) ** 2, 2.0 * (a - 0.7)),
    "cos": lambda a: (-np.cos(a - 0.3) + 0.01 * a ** 4, np.sin(a - 0.3) + 0.04 * a ** 3),
    "steep": lambda a: (np.exp(-3.0 * a) + 3.0 * a * a, -3.0 * np.exp(-3.0 * a) + 6.0 * a),
    "flat": lambda a: (-a / (1.0 + 40.0 * a * a), -(1.0 - 40.0 * a * a) / (1.0 + 40.0 * a * a) ** 2),
    "mt1": lambda a: (-a / (a * a + 2.0), (a * a - 2.0) / (a * a + 2.0) ** 2),
}


@pytest.mark.parametrize("name", sorted(LS_CASES))
@pytest.mark.parametrize("a0", [0.1, 1e-3, 1.5])
def test_line_search_sequences(golden, name, a0):
    d = golden("dcsrch")
    fn = LS_CASES[name]
    f0, g0 = fn(0.0)
    th, task, _, _, trials = O.line_search(lambda a: (*fn(a), None), a0, f0, g0)
    key = "%s_%g" % (name, a0)
    np.testing.assert_array_equal(np.array(trials), d[key + "_trials"])
    assert task == str(d[key + "_task"])


def test_tn_solve_al4(golden):
    a = golden("al4")
    st = systems.config_al4(0)
    ev = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")
    np.testing.assert_allclose(ev.vloc.ravel()[a["sample_idx"]], a["vloc_s"], atol=1e-12)
    assert abs(ev.ewald["energy"] - float(a["E_ewald"])) < 1e-10
    rho0 = np.full(st.nr, st.nelec / st.volume)
    r = O.optimize_tn(ev, rho0, ev.grid, econv=1e-7, maxfun=50, maxiter=100)
    assert r["converged"] == 0
    assert ev.n_eval["EV"] == int(a["n_ev"]) and ev.n_eval["V"] == int(a["n_v"])
    E, _ = ev(r["rho"])
    assert abs(E - float(a["E_final"])) < 1e-9
    assert np.abs(r["rho"] - a["rho"]).max() < 1e-5
    F = ev.forces(r["rho"])
    np.testing.assert_allclose(F, a["forces"], atol=1e-5)


@pytest.mark.parametrize("pme", [True, False])
@pytest.mark.parametrize("case", ["al4", "fde"])
def test_density_guess_recipe(golden, case, pme):
    """Superposed atomic densities (get_3d_value_recipe) against the reference."""
    d = golden("guess")
    if case == "al4":
        st = systems.config_al4(0)
        lat, nr, pos, sym, full = st.lattice, st.nr, st.positions, list(st.symbols), False
    else:
        f = golden("fde")
        lat, nr, pos, sym, full = f["lattice"], tuple(int(x) for x in f["nr"]), f["positions"], ["Al", "Al"], True
    g = O.Grid(lat, nr, full=full)
    tab = {s: systems.atomic_density_table(systems.SPECIES[s][0], systems.ATOMIC_SIGMA[s]) for s in set(sym)}
    nel = sum(systems.SPECIES[s][0] for s in sym)
    rho = O.density_guess_recipe(g, pos, sym, tab, nel, pme=pme)
    tag = case + ("_pme" if pme else "_exact")
    np.testing.assert_allclose(rho.ravel()[d[case + "_idx"]], d[tag + "_s"], rtol=0, atol=1e-12)
    np.testing.assert_allclose([rho.sum(), (rho * rho).sum()], d[tag + "_c"][:2], rtol=1e-12)


@pytest.mark.parametrize("pme", [True, False])
def test_stress_components_fde(golden, pme):
    """Every stress term on the reference's skewed test density (full grid)."""
    d = golden("fde")
    S = golden("stress")
    g = O.Grid(d["lattice"], tuple(int(x) for x in d["nr"]), full=True)
    rho = d["rho"]
    sym = ["Al"] * len(d["positions"])
    tab = {"Al": systems.analytic_pp_table(*systems.SPECIES["Al"])}
    tag = "fde_%s_" % ("pme" if pme else "exact")
    e_tf, _ = O.tf(rho, g)
    np.testing.assert_allclose(O.stress_tf(e_tf, g), S[tag + "KEDF-TF"], rtol=0, atol=1e-14)
    np.testing.assert_allclose(O.stress_vw(rho, g), S[tag + "KEDF-VW"], rtol=0, atol=1e-14)
    e_wt, _ = O.WTNL()(rho, g)
    np.testing.assert_allclose(O.stress_wt(rho, g, e_wt), S[tag + "KEDF-NL"], rtol=0, atol=1e-14)
    e_xc, v_xc = O.lda(rho, g)
    np.testing.assert_allclose(O.stress_lda(rho, g, e_xc, v_xc), S[tag + "XC"], rtol=0, atol=1e-14)
    e_h, _ = O.hartree(rho, g)
    np.testing.assert_allclose(O.stress_hartree(rho, g, e_h), S[tag + "HARTREE"], rtol=0, atol=1e-14)
    v = O.local_pp(g, d["positions"], sym, tab, pme=pme)
    e_pp = float(np.einsum("ijk,ijk->", v, rho) * g.dV)
    f = O.stress_pp_pme if pme else O.stress_pp_exact
    np.testing.assert_allclose(f(rho, g, d["positions"], sym, tab, e_pp), S[tag + "PSEUDO"], rtol=0, atol=1e-13)
    np.testing.assert_allclose(O.ewald_stress(g, d["positions"], d["charges"], pme=pme), S[tag + "II"],
                               rtol=0, atol=1e-12)


def test_stress_total_al4(golden):
    a = golden("al4")
    S = golden("stress")
    st = systems.config_al4(0)
    ev = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")
    out = ev.stress(a["rho"], split=True)
    for k in ("KEDF-TF", "KEDF-VW", "XC", "HARTREE", "PSEUDO", "II", "TOTAL"):
        np.testing.assert_allclose(out[k], S["al4_" + k], rtol=0, atol=1e-12, err_msg=k)
