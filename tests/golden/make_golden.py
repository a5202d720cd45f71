"""Generate the golden fixtures by running the reference DFTpy here.

Run from the repository root:  ``python tests/golden/make_golden.py [name ...]``

It imports the reference from its source tree through the two shims in
``_shims/`` (see ``refenv.py``) and writes small ``.npz`` files next to this
script.  The GPU tests and the CPU oracle tests read only those ``.npz``
files; the reference tree is not needed to run them.

Fixtures
--------
fde.npz      the reference's own test density ``Al_fde_rho.pp`` (2 Al,
             36x36x72) with each functional's energy, potential samples and
             potential checksums, Ewald terms and forces (reference tests
             ``test_functional.py:24-34``, ``test_ewald.py:33-54``).
al4.npz      32^3, 4 Al: full TN optimisation (TFVW+LDA+Hartree+analytic PP,
             PME), converged density, energies, forces, evaluation counts.
al256.npz    128^3, 256 Al, WT: full TN optimisation; scalars and a density
             sample (the full field is 16 MB).
guess.npz    superposed atomic densities (``get_3d_value_recipe``, PME and
             exact) from Gaussian reciprocal-space tables on the 4-Al grid and
             on the skewed ``Al_fde_rho.pp`` grid (full=True).
al256_tight.npz  the same 256-atom solve at econv 1e-10 Ha (converged
             energy and forces).
stress.npz   stress tensors of every term (WT+LDA+Hartree+PP+Ewald, PME and
             exact) on the skewed test density, and the 4-Al total.
pseudo_files.npz  reciprocal tables of the reference's example pseudopotential
             files as its ReadPseudo builds them (needs the ``xmltodict``
             stand-in in ``_shims`` for UPF).
dcsrch.npz   trial-step sequences of the reference's Moré–Thuente line search
             (``LineSearchDcsrch2``) on analytic 1-D functions.
first_order.npz  the reference's CG-HS, CG-PR and LBFGS solves of the
             4-atom cell (energies, evaluation counts, forces).
gaas.npz     the reference's own TN test (GaAs_random, recpot pseudopotentials,
             WT + LDA + Hartree, PME): structure, full reciprocal PP tables,
             converged energy and forces.
"""
import os
import sys
import time
import pathlib

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
sys.path.insert(0, str(HERE))
sys.path.insert(0, str(ROOT))

import refenv  # noqa: E402

refenv.load()

from dftpy.field import DirectField  # noqa: E402
from dftpy.formats import io  # noqa: E402
from dftpy.functional import Functional, TotalFunctional  # noqa: E402
from dftpy.functional.pseudo import LocalPseudo  # noqa: E402
from dftpy.functional.pseudo.abstract_pseudo import BasePseudo  # noqa: E402
from dftpy.grid import DirectGrid  # noqa: E402
from dftpy.ions import Ions  # noqa: E402
from dftpy.ewald import ewald  # noqa: E402
from dftpy.optimization import Optimization  # noqa: E402
from dftpy.time_data import TimeData  # noqa: E402
from dftpy.math_utils import LineSearchDcsrch2  # noqa: E402

from dftpy_gb300 import systems  # noqa: E402

NSAMPLE = 2000


class AnalyticPP(BasePseudo):
    """BasePseudo holding the analytic v(G) table (``direct=False``)."""

    def __init__(self, Z, rc):
        super().__init__(fname=None, direct=False)
        self._zval = float(Z)
        self.r, self.v = systems.analytic_pp_table(Z, rc)


def pp_list(symbols):
    return {s: AnalyticPP(*systems.SPECIES[s]) for s in sorted(set(symbols))}


def sample_index(n, seed=123):
    return np.sort(np.random.default_rng(seed).choice(n, size=min(NSAMPLE, n), replace=False))


def checksums(v):
    v = np.asarray(v, dtype=np.float64).ravel()
    return np.array([v.sum(), (v * v).sum(), np.abs(v).max(), v.min(), v.max()])


def ref_ions(st):
    return Ions(symbols=list(st.symbols), positions=st.positions.copy(), cell=st.lattice.copy(), units="au")


class CountingEvaluator:
    """Wrap a TotalFunctional and count its evaluations by kind."""

    def __init__(self, func):
        self.func = func
        self.n_ev = 0
        self.n_v = 0
        self.energies = []

    def __call__(self, rho, calcType={"E", "V"}, **kw):
        out = self.func(rho, calcType=calcType, **kw)
        if "E" in calcType:
            self.n_ev += 1
            self.energies.append(float(out.energy))
        else:
            self.n_v += 1
        return out


def component_outputs(rho, funcs):
    res = {}
    for name, f in funcs.items():
        out = f(rho, calcType={"E", "V"})
        res[name] = (float(out.energy), np.asarray(out.potential))
    return res


def gen_fde():
    ions, rho, _ = io.read_all(refenv.REF_DATA / "Al_fde_rho.pp")
    grid = rho.grid
    idx = sample_index(rho.size)
    out = {"rho": np.asarray(rho), "lattice": grid.lattice.copy(), "nr": np.array(grid.nrR),
           "positions": ions.positions.copy(), "charges": ions.charges.copy(), "sample_idx": idx}
    funcs = {
        "TF": Functional(type="KEDF", name="TF"),
        "VW": Functional(type="KEDF", name="VW"),
        "WTNL": Functional(type="KEDF", name="WT-NL"),
        "KEDF_WT": Functional(type="KEDF", name="WT"),
        "KEDF_TFVW": Functional(type="KEDF", name="TFVW"),
        "LDA": Functional(type="XC", name="LDA"),
        "HARTREE": Functional(type="HARTREE"),
    }
    t0 = time.time()
    for name, (e, v) in component_outputs(rho, funcs).items():
        out["E_" + name] = e
        out["Vs_" + name] = v.ravel()[idx]
        out["Vc_" + name] = checksums(v)
    # LMGP (reference test_functional.py:29-34): first call builds the MGP table
    for interp in ("linear", "hermite"):
        f = Functional(type="KEDF", name="LMGP", interp=interp)
        o = f(rho, calcType={"E", "V"})
        out["E_LMGP_" + interp] = float(o.energy)
        out["Vs_LMGP_" + interp] = np.asarray(o.potential).ravel()[idx]
        out["Vc_LMGP_" + interp] = checksums(o.potential)
    # analytic local PP on these ions (PME and exact structure factor)
    al = {"Al": AnalyticPP(*systems.SPECIES["Al"])}
    for pme in (True, False):
        tag = "PME" if pme else "EXACT"
        ps = LocalPseudo(grid=grid, ions=ions, PP_list=al, PME=pme)
        o = ps(rho)
        out["E_PP_" + tag] = float(o.energy)
        out["Vs_PP_" + tag] = np.asarray(o.potential).ravel()[idx]
        out["Vc_PP_" + tag] = checksums(o.potential)
        out["F_PP_" + tag] = ps.forces(rho)
    # Ewald (reference test_ewald.py:33-54 values are re-asserted by the tests)
    ew = ewald(rho=rho, ions=ions, verbose=False)
    ewp = ewald(rho=rho, ions=ions, verbose=False, PME=True)
    out["EW_corr"] = ew.Energy_corr()
    out["EW_real"] = ew.Energy_real()
    out["EW_rec"] = ew.Energy_rec()
    out["EW_real_pme"] = ewp.Energy_real_fast2()
    out["EW_rec_pme"] = ewp.Energy_rec_PME()
    out["EW_energy"] = ew.energy
    out["EW_energy_pme"] = ewp.energy
    out["EW_forces"] = ew.forces
    out["EW_forces_pme"] = ewp.forces
    out["EW_eta"] = ew.eta
    # FFT convention: rho.fft() (x dV), sampled on the half spectrum
    rg = np.asarray(rho.fft())
    gidx = sample_index(rg.size, seed=7)
    out["FFT_idx"] = gidx
    out["FFT_s"] = rg.ravel()[gidx]
    print("fde: %.1f s" % (time.time() - t0))
    np.savez_compressed(HERE / "fde.npz", **out)


def build_total(st, kedf, pme=True, **kedf_kw):
    grid = DirectGrid(lattice=st.lattice.copy(), nr=st.nr, full=False)
    ions = ref_ions(st)
    pseudo = LocalPseudo(grid=grid, ions=ions, PP_list=pp_list(st.symbols), PME=pme)
    funcs = dict(KineticEnergyFunctional=Functional(type="KEDF", name=kedf, **kedf_kw),
                 XCFunctional=Functional(type="XC", name="LDA"),
                 HARTREE=Functional(type="HARTREE"), PSEUDO=pseudo)
    return grid, ions, pseudo, TotalFunctional(**funcs), funcs


def run_tn(st, kedf, econv, full_rho=True, **kedf_kw):
    grid, ions, pseudo, total, funcs = build_total(st, kedf, **kedf_kw)
    rho0 = DirectField(grid=grid)
    rho0[:] = ions.get_ncharges() / ions.cell.volume
    t0 = time.time()
    pseudo.local_PP()
    e_ii = total.ewald.energy
    t_setup = time.time() - t0
    ev = CountingEvaluator(total)
    opt = Optimization(EnergyEvaluator=ev, optimization_method="TN",
                       optimization_options={"econv": econv, "maxfun": 50, "maxiter": 100})
    TimeData.reset()
    t0 = time.time()
    rho = opt.optimize_rho(guess_rho=rho0)
    t_opt = time.time() - t0
    n_fft = TimeData.number.get("FFT", 0)
    n_ifft = TimeData.number.get("InvFFT", 0)
    e_final = float(total.Energy(rho))
    out = {"lattice": st.lattice, "positions": st.positions, "nr": np.array(st.nr),
           "symbols": np.array(st.symbols), "econv": econv, "E_final": e_final,
           "E_history": np.array(ev.energies), "n_ev": ev.n_ev, "n_v": ev.n_v,
           "converged": opt.converged, "n_fft": n_fft, "n_ifft": n_ifft,
           "t_opt": t_opt, "t_setup": t_setup, "E_ewald": float(e_ii),
           "mu": float(opt.mu)}
    idx = sample_index(rho.size)
    out["sample_idx"] = idx
    out["rho_s"] = np.asarray(rho).ravel()[idx]
    out["rho_c"] = checksums(rho)
    if full_rho:
        out["rho"] = np.asarray(rho)
    comps = {"KEDF": funcs["KineticEnergyFunctional"], "XC": funcs["XCFunctional"],
             "HARTREE": funcs["HARTREE"], "PSEUDO": funcs["PSEUDO"]}
    for name, (e, v) in component_outputs(rho, comps).items():
        out["E_" + name] = e
        out["Vs_" + name] = v.ravel()[idx]
        out["Vc_" + name] = checksums(v)
    out["vloc_s"] = np.asarray(pseudo.vreal).ravel()[idx]
    out["vloc_c"] = checksums(pseudo.vreal)
    out["forces"] = total.get_forces(rho, ions=ions)
    out["forces_pp"] = pseudo.forces(rho)
    out["forces_ii"] = total.ewald.forces
    # one evaluation at the uniform start density, for per-evaluation checks
    o = total(rho0, calcType={"E", "V"})
    out["E_uniform"] = float(o.energy)
    out["V_uniform_s"] = np.asarray(o.potential).ravel()[idx]
    print("%s: E=%.10f  evals E+V %d, V %d, FFT %d+%d, %.1f s" % (
        st.name, e_final, ev.n_ev, ev.n_v, n_fft, n_ifft, t_opt))
    return out


def gen_al4():
    st = systems.config_al4(seed=0)
    out = run_tn(st, "TFVW", econv=1e-7)
    np.savez_compressed(HERE / "al4.npz", **out)


def gen_al256():
    st = systems.config_al256(seed=0)
    out = run_tn(st, "WT", econv=1e-7, full_rho=False)
    np.savez_compressed(HERE / "al256.npz", **out)


def gen_guess():
    """get_3d_value_recipe (density/density.py:252-300) on two grids."""
    from dftpy.density.density import get_3d_value_recipe
    out = {}
    fde = np.load(HERE / "fde.npz")
    st = systems.config_al4(seed=0)
    cases = {"al4": (st.lattice.copy(), st.nr, st.positions.copy(), list(st.symbols), False),
             "fde": (fde["lattice"], tuple(int(x) for x in fde["nr"]), fde["positions"], ["Al", "Al"], True)}
    for name, (lat, nr, pos, sym, full) in cases.items():
        grid = DirectGrid(lattice=lat.copy(), nr=nr, full=full)
        ions = Ions(symbols=sym, positions=pos.copy(), cell=lat.copy(), units="au")
        ions.set_charges({s: systems.SPECIES[s][0] for s in set(sym)})
        r, arho = {}, {}
        for s_ in set(sym):
            r[s_], arho[s_] = systems.atomic_density_table(systems.SPECIES[s_][0], systems.ATOMIC_SIGMA[s_])
        idx = sample_index(int(np.prod(nr)))
        out[name + "_idx"] = idx
        for pme in (True, False):
            rho = get_3d_value_recipe(r, arho, ions, grid, ncharge=None, rho=None, dtol=1e-30, direct=True,
                                      pme=pme, order=10)
            tag = name + ("_pme" if pme else "_exact")
            out[tag + "_s"] = np.asarray(rho).ravel()[idx]
            out[tag + "_c"] = checksums(rho)
    np.savez_compressed(HERE / "guess.npz", **out)


def gen_al256_tight():
    """The 256-atom solve converged as far as FP64 goes (econv 1e-10 Ha):
    its energy and forces are the converged values the accuracy gates use
    (the econv 1e-7 solve still moves forces by ~1e-5 Ha/Bohr)."""
    st = systems.config_al256(seed=0)
    out = run_tn(st, "WT", econv=1e-10, full_rho=False)
    keep = ("E_final", "E_history", "n_ev", "n_v", "converged", "econv", "forces", "forces_pp", "forces_ii",
            "sample_idx", "rho_s", "rho_c", "t_opt")
    np.savez_compressed(HERE / "al256_tight.npz", **{k: out[k] for k in keep})


def gen_stress():
    """Stress tensors of every term (reference ``TotalFunctional.get_stress``,
    ``total_functional.py:176-209``) on the reference's test density (skewed
    cell, full grid) and on the converged 4-Al density."""
    out = {}
    ions, rho, _ = io.read_all(refenv.REF_DATA / "Al_fde_rho.pp")
    grid = rho.grid
    al = {"Al": AnalyticPP(*systems.SPECIES["Al"])}
    for pme in (True, False):
        tag = "pme" if pme else "exact"
        ps = LocalPseudo(grid=grid, ions=ions, PP_list=al, PME=pme)
        total = TotalFunctional(KineticEnergyFunctional=Functional(type="KEDF", name="WT"),
                                XCFunctional=Functional(type="XC", name="LDA"),
                                HARTREE=Functional(type="HARTREE"), PSEUDO=ps)
        total(rho, calcType={"E", "V"})    # energies of this density (Hartree caches its own per class)
        st = total.get_stress(rho, split=True)
        for k, v in st.items():
            out["fde_%s_%s" % (tag, k)] = np.asarray(v)
    a = np.load(HERE / "al4.npz")
    st4 = systems.config_al4(seed=0)
    grid, ions, pseudo, total, funcs = build_total(st4, "TFVW")
    rho4 = DirectField(grid=grid, data=a["rho"])
    total(rho4, calcType={"E", "V"})
    for k, v in total.get_stress(rho4, split=True).items():
        out["al4_" + k] = np.asarray(v)
    np.savez_compressed(HERE / "stress.npz", **out)
    print({k: float(np.abs(v).max()) for k, v in out.items()})


def gen_pseudo_files():
    """Reciprocal-space tables the reference's ReadPseudo builds from its own
    example pseudopotential files (recpot, psp8, UPF v2; ``_init_pp``,
    ``pseudo/__init__.py:726-779``), sampled."""
    from dftpy.functional.pseudo import ReadPseudo
    out = {}
    for f in ("al.lda.recpot", "Al_lda.oe01.recpot", "al.lda.psp", "al.lda.upf", "Mg_OEPP_PZ.UPF"):
        key = "Al" if f.lower().startswith("al") else "Mg"
        rp = ReadPseudo({key: str(refenv.REF_DATA / f)})
        tag = f.replace(".", "_")
        gp, vp = rp._gp[key], rp._vp[key]
        out[tag + "_zval"] = float(rp._zval[key])
        out[tag + "_n"] = gp.size
        idx = np.unique(np.linspace(0, gp.size - 1, 400).astype(int))
        out[tag + "_idx"] = idx
        out[tag + "_gp"] = gp[idx]
        out[tag + "_vp"] = vp[idx]
        if rp._atomic_density.get(key) is not None:
            out[tag + "_rho_gp"] = rp._atomic_density_grid[key][idx]
            out[tag + "_rho"] = rp._atomic_density[key][idx]
    np.savez_compressed(HERE / "pseudo_files.npz", **out)


def gen_formats():
    """Density files: what the reference's readers return for its example
    files (``formats/qepp.py``, ``xsf.py``; checksums and samples), and the
    files its writers make (qepp, xsf, snpy) for a small seeded field, kept
    byte for byte under ``formats/`` with the arrays they were made from."""
    from dftpy.field import DirectField
    from dftpy.formats import io, qepp, snpy, xsf
    from dftpy.grid import DirectGrid
    from dftpy.ions import Ions
    from numpy.lib import format as npyf
    if not hasattr(npyf, "_check_version"):
        # the reference's npy module calls this private numpy helper (gone in
        # numpy 2.x); it only validates the format version
        def _check_version(version):
            if version not in [(1, 0), (2, 0), (3, 0), None]:
                raise ValueError("we only support format version (1,0), (2,0), and (3,0), not %s" % (version,))
        npyf._check_version = _check_version
    out = {}
    for f in ("Al_fde_rho.pp", "GaAs_random.xsf", "al_random.xsf", "ti.xsf"):
        tag = f.replace(".", "_")
        for dt in ("density", "potential"):
            ions, field, info = io.read_all(str(refenv.REF_DATA / f), data_type=dt)
            v = np.asarray(field)
            key = tag + ("" if dt == "density" else "_pot")
            out[key + "_shape"] = np.array(v.shape)
            out[key + "_sum"] = float(v.sum())
            out[key + "_sumsq"] = float((v * v).sum())
            idx = sample_index(v.size, seed=7)[:300]
            out[key + "_idx"] = idx
            out[key + "_samples"] = v.ravel()[idx]
        out[tag + "_lattice"] = np.asarray(field.grid.lattice)
        out[tag + "_full"] = bool(field.grid.full)
        out[tag + "_cell"] = np.asarray(ions.cell)
        out[tag + "_pos"] = np.asarray(ions.positions)
        out[tag + "_symbols"] = np.array(list(ions.get_chemical_symbols()))
        if info is not None:
            for k, val in info.items():
                out[tag + "_info_" + k] = np.asarray(val)
    # writers on a small seeded field
    rng = np.random.default_rng(2024)
    cell = np.array([[7.1, 0.0, 0.0], [0.3, 6.6, 0.0], [0.2, -0.4, 8.3]])
    pos = rng.random((3, 3)) @ cell
    nr = np.array([6, 5, 4])
    grid = DirectGrid(lattice=cell, nr=nr, full=False)
    rho = DirectField(grid=grid, griddata_3d=0.01 + rng.random(tuple(nr)))
    ions = Ions(symbols=["Ga", "As", "Ga"], positions=pos, cell=cell)
    ions.set_charges({"Ga": 3.0, "As": 5.0})
    d = HERE / "formats"
    d.mkdir(exist_ok=True)
    qepp.write_qepp(str(d / "small_density.pp"), ions=ions, data=rho)
    qepp.write_qepp(str(d / "small_potential.pp"), ions=ions, data=rho, data_type="potential")
    xsf.write_xsf(str(d / "small_density.xsf"), ions=ions, data=rho)
    xsf.write_xsf(str(d / "small_potential.xsf"), ions=ions, data=rho, data_type="potential")
    rho2 = DirectField(grid=grid, rank=2, griddata_3d=np.stack([np.asarray(rho), 2.0 * np.asarray(rho)]))
    xsf.write_xsf(str(d / "small_spin.xsf"), ions=ions, data=rho2)
    snpy.write(str(d / "small.snpy"), ions=ions, data=rho)
    out["small_cell"] = cell
    out["small_pos"] = pos
    out["small_rho"] = np.asarray(rho)
    out["small_symbols"] = np.array(ions.get_chemical_symbols())
    for f in ("small_density.pp", "small_potential.pp", "small_density.xsf", "small_potential.xsf", "small_spin.xsf",
              "small.snpy"):
        dt = "potential" if "potential" in f else "density"
        i2, fld, _ = io.read_all(str(d / f), data_type=dt)
        tag = f.replace(".", "_")
        out[tag + "_read"] = np.asarray(fld)
        out[tag + "_read_lattice"] = np.asarray(fld.grid.lattice)
        out[tag + "_read_pos"] = np.asarray(i2.positions)
        out[tag + "_read_cell"] = np.asarray(i2.cell)
    np.savez_compressed(HERE / "formats.npz", **out)


def gen_gridmap():
    """Spectral interpolation between grids (``grid_map_data``,
    ``field2distrib``, ``utils/utils.py:80-129, 218-287``) for half and full
    spectra, coarse to fine and fine to coarse, odd and even sizes."""
    from dftpy.field import DirectField
    from dftpy.grid import DirectGrid
    from dftpy.utils.utils import field2distrib, grid_map_data
    rng = np.random.default_rng(77)
    cell = np.array([[6.2, 0.0, 0.0], [0.4, 5.9, 0.0], [-0.3, 0.2, 7.1]])
    out = {"cell": cell}
    cases = [("up", (8, 6, 5), (12, 10, 9)), ("up_even", (8, 6, 6), (16, 12, 12)), ("down", (12, 10, 9), (8, 6, 5)),
             ("down_even", (16, 12, 12), (10, 8, 6))]
    for full in (False, True):
        for name, nr1, nr2 in cases:
            tag = name + ("_full" if full else "_half")
            g1 = DirectGrid(lattice=cell, nr=nr1, full=full)
            x = rng.random(nr1) + 0.5
            f1 = DirectField(grid=g1, griddata_3d=x)
            y = grid_map_data(f1, nr=np.array(nr2))
            out[tag + "_in"] = x
            out[tag + "_out"] = np.asarray(y)
            g2 = DirectGrid(lattice=cell, nr=nr2, full=full)
            o2 = DirectField(grid=g2)
            field2distrib(f1, o2, root=0, tol=0.8)
            out[tag + "_distrib"] = np.asarray(o2)
    np.savez_compressed(HERE / "gridmap.npz", **out)


def gen_dcsrch():
    """Trial-step sequences of the reference line search on 1-D test functions."""
    cases = {
        # (phi(a), phi'(a)) pairs, a in [0, pi]
        "quad": lambda a: ((a - 0.7) ** 2, 2.0 * (a - 0.7)),
        "cos": lambda a: (-np.cos(a - 0.3) + 0.01 * a ** 4, np.sin(a - 0.3) + 0.04 * a ** 3),
        "steep": lambda a: (np.exp(-3.0 * a) + 3.0 * a * a, -3.0 * np.exp(-3.0 * a) + 6.0 * a),
        "flat": lambda a: (-a / (1.0 + 40.0 * a * a), -(1.0 - 40.0 * a * a) / (1.0 + 40.0 * a * a) ** 2),
        "mt1": lambda a: (-a / (a * a + 2.0), (a * a - 2.0) / (a * a + 2.0) ** 2),
    }
    out = {}
    for name, fn in cases.items():
        for a0 in (0.1, 1e-3, 1.5):
            trials = []

            def f(a, fn=fn, trials=trials):
                trials.append(float(a))
                v, g = fn(a)
                return [float(v), float(g)]
            f0 = fn(0.0)
            theta, _, _, task, nls, _ = LineSearchDcsrch2(
                f, alpha0=a0, func0=[float(f0[0]), float(f0[1])], c1=1e-4, c2=0.2,
                amax=np.pi, amin=0.0, xtol=1e-12, maxiter=30)
            key = "%s_%g" % (name, a0)
            out[key + "_trials"] = np.array(trials)
            out[key + "_theta"] = np.nan if theta is None else float(theta)
            out[key + "_task"] = task.decode() if isinstance(task, bytes) else str(task)
    np.savez_compressed(HERE / "dcsrch.npz", **out)
    print("dcsrch: %d cases" % len(cases))


def gen_gaas():
    """The reference's own TN test (``test_density_opt.py:15-46``): GaAs_random
    (5 Ga + 5 As), recpot pseudopotentials through ReadPseudo, PME, WT + LDA +
    Hartree, grid from ecut2nr(spacing=0.4), econv 1e-6 * nat; the structure,
    the full reciprocal tables the reference builds, the converged energy and
    forces."""
    from dftpy.functional.pseudo import ReadPseudo
    from dftpy.math_utils import ecut2nr
    ions = io.read(refenv.REF_DATA / "GaAs_random.vasp", names=["Al"])
    files = {"Ga": refenv.REF_DATA / "Ga_lda.oe04.recpot", "As": refenv.REF_DATA / "As_lda.oe04.recpot"}
    nr = ecut2nr(lattice=ions.cell, spacing=0.4)
    grid = DirectGrid(lattice=ions.cell, nr=nr, full=False)
    rho_ini = DirectField(grid=grid)
    pseudo = LocalPseudo(grid=grid, ions=ions, PP_list=files, PME=True)
    total = TotalFunctional(KineticEnergyFunctional=Functional(type="KEDF", name="WT", optional_kwargs={}),
                            XCFunctional=Functional(type="XC", name="LDA"),
                            HARTREE=Functional(type="HARTREE"), PSEUDO=pseudo)
    rho_ini[:] = ions.get_ncharges() / ions.cell.volume
    opt = Optimization(EnergyEvaluator=total, optimization_method="TN",
                       optimization_options={"econv": 1e-6 * ions.nat, "maxfun": 50, "maxiter": 100})
    t0 = time.time()
    rho = opt.optimize_rho(guess_rho=rho_ini)
    e_final = float(total.Energy(rho=rho, ions=ions, usePME=True))
    out = {"lattice": np.array(ions.cell.array if hasattr(ions.cell, "array") else ions.cell, dtype=float),
           "positions": np.array(ions.positions, dtype=float), "symbols": np.array(list(ions.symbols)),
           "nr": np.array(nr), "E_final": e_final, "forces": total.get_forces(rho, ions=ions),
           "nelec": float(ions.get_ncharges())}
    rp = ReadPseudo({k: str(v) for k, v in files.items()})
    for k in files:
        out[k + "_gp"] = np.asarray(rp._gp[k], dtype=float)
        out[k + "_vp"] = np.asarray(rp._vp[k], dtype=float)
        out[k + "_zval"] = float(rp._zval[k])
    np.savez_compressed(HERE / "gaas.npz", **out)
    print("gaas: nr %s E=%.10f (reference test asserts -43.3046), %.1f s" % (list(nr), e_final, time.time() - t0))


def gen_first_order():
    """The reference's first-order optimisers on the 4-atom cell (TFVW + LDA +
    Hartree + analytic PP, PME, econv 1e-7 Ha, uniform start): CG-HS (its
    default method), CG-PR and LBFGS (h0 = 1, which LBFGS requires)."""
    st = systems.config_al4(seed=0)
    out = {}
    for name, method, extra in (("cghs", "CG-HS", {}), ("cgpr", "CG-PR", {}), ("lbfgs", "LBFGS", {"h0": 1.0})):
        grid, ions, pseudo, total, funcs = build_total(st, "TFVW")
        rho0 = DirectField(grid=grid)
        rho0[:] = ions.get_ncharges() / ions.cell.volume
        ev = CountingEvaluator(total)
        opts = {"econv": 1e-7, "maxiter": 200}
        opts.update(extra)
        opt = Optimization(EnergyEvaluator=ev, optimization_method=method, optimization_options=opts)
        t0 = time.time()
        rho = opt.optimize_rho(guess_rho=rho0)
        out[name + "_E_final"] = float(total.Energy(rho))
        out[name + "_converged"] = int(opt.converged)
        out[name + "_n_ev"] = ev.n_ev
        out[name + "_E_history"] = np.array(ev.energies)
        out[name + "_forces"] = total.get_forces(rho, ions=ions)
        print("%s: E=%.10f converged %d, %d evaluations, %.1f s" % (method, out[name + "_E_final"],
                                                                   opt.converged, ev.n_ev, time.time() - t0))
    np.savez_compressed(HERE / "first_order.npz", **out)


GENERATORS = {"first_order": gen_first_order, "gaas": gen_gaas, "fde": gen_fde, "al4": gen_al4, "al256": gen_al256, "dcsrch": gen_dcsrch, "guess": gen_guess, "al256_tight": gen_al256_tight, "stress": gen_stress, "pseudo_files": gen_pseudo_files, "formats": gen_formats, "gridmap": gen_gridmap}

if __name__ == "__main__":
    names = sys.argv[1:] or list(GENERATORS)
    for n in names:
        GENERATORS[n]()
