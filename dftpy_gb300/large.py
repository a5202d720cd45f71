"""The large workload: 4000 Al atoms (10x10x10 fcc supercell, jitter 0.1
Bohr), 360^3 grid, LMGP nonlocal KEDF (+ TF + vW) + LDA + Hartree + local PP
(PME).  ``python -m dftpy_gb300.large`` runs the learned guess and the
mixed-precision TN (FP32 stage, FP64 refinement); unless ``--no-fp64`` the
FP64 reference is the plain FP64 TN continued from the mixed result (the
plain TN from the guess stops on a line-search failure well above the
minimum at this size, so it is not a reference; ``--fp64-from-guess`` times
it anyway).  One JSON line: wall times, evaluation counts, the energy the
FP64 continuation still finds per atom, the largest force change, and the
CUDA-event time and algorithmic bandwidth of one FP32 and one FP64
evaluation.

Algorithmic bytes per evaluation: s N (R + W + 2 F) with R = 2 (rho, v_loc),
W = 1 (V) and F the transforms the reference performs for LMGP: forward and
inverse for vW and Hartree (4), the forward transform of rho^beta (1) and two
inverse transforms per k_F knot (the kernel and its derivative).
"""
import argparse
import json
import os
import time


def build(seed=0):
    from . import functional as F
    from . import systems
    from .field import DirectField
    from .grid import DirectGrid
    from .ions import Ions
    st = systems.config_al4000(seed)
    grid = DirectGrid(st.lattice, st.nr, full=False)
    ions = Ions(st.symbols, positions=st.positions, cell=st.lattice)
    ps = F.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": F.AnalyticPP(*systems.SPECIES["Al"])}, PME=True)
    ke = F.Functional(type="KEDF", name="LMGP")
    total = F.TotalFunctional(KineticEnergyFunctional=ke, XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rho_u = DirectField(grid)
    rho_u[:] = st.nelec / st.volume
    return st, grid, total, ke, rho_u


def solve(total, rho0, precision, econv):
    from .optimization import Optimization
    opt = Optimization(EnergyEvaluator=total, optimization_method="TN",
                       optimization_options={"econv": econv, "maxfun": 50, "maxiter": 100, "precision": precision})
    rho = opt.optimize_rho(guess_rho=rho0)
    return opt, rho


def eval_time(total, rho, reps=3):
    import torch
    for _ in range(2):
        total(rho, calcType={"E", "V"})
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        total(rho, calcType={"E", "V"})
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps * 1e-3


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--no-fp64", action="store_true", help="skip the FP64 reference")
    p.add_argument("--fp64-from-guess", action="store_true", help="also time the plain FP64 TN from the guess")
    p.add_argument("--guess", default="learned", choices=["learned", "uniform"])
    p.add_argument("--econv-per-atom", type=float, default=1e-8)
    a = p.parse_args()
    import numpy as np
    import torch
    from . import guess as G
    t0 = time.perf_counter()
    st, grid, total, ke, rho_u = build()
    total.PSEUDO.local_PP()
    total.ewald.energy
    torch.cuda.synchronize()
    t_setup = time.perf_counter() - t0
    econv = a.econv_per_atom * st.nat
    out = {"workload": "al4000_360_lmgp", "natoms": st.nat, "grid": list(st.nr), "econv_ha": econv,
           "setup_s": t_setup, "guess": a.guess}
    here = os.path.dirname(os.path.abspath(__file__))
    lg = G.LearnedGuess(G.GuessNet.load(os.path.join(here, "data", "guessnet_al_wt.npz"))) if a.guess == "learned" \
        else None

    def start():
        return lg.guess(total, grid) if lg is not None else rho_u

    # a warm-up solve (plans, kernel tables, the MGP table), then the timed one
    solve(total, start(), "mixed", econv)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    g = start()
    torch.cuda.synchronize()
    t_guess = time.perf_counter() - t1
    opt_m, rho_m = solve(total, g, "mixed", econv)
    torch.cuda.synchronize()
    t_mixed = time.perf_counter() - t1
    out["mixed"] = {"wall_s": t_mixed, "guess_s": t_guess, "energy": float(opt_m.energy),
                    "converged": int(opt_m.converged),
                    "stages": [(s["precision"], s["n_eval_ev"], s["n_eval_v"], s.get("n_eval_hess", 0), s["n_iter"])
                               for s in opt_m.stats["stages"]]}
    nk = int(ke._lwt.prepare(rho_m).nknots) if hasattr(ke, "_lwt") else 0
    F = 4 + 1 + 2 * nk
    n = int(np.prod(st.nr))
    for name, dt in (("fp32", torch.float32), ("fp64", torch.float64)):
        r = rho_m.to(dt)
        t = eval_time(total, r)
        b = (4 if dt == torch.float32 else 8) * n * (2 + 1 + 2 * F)
        out["eval_" + name] = {"t_s": t, "algorithmic_bytes": b, "gbs": b / t / 1e9, "knots": nk, "F": F}
    if not a.no_fp64:
        t2 = time.perf_counter()
        opt_r, rho_r = solve(total, rho_m.to(torch.float64), "fp64", econv)
        torch.cuda.synchronize()
        fm = total.get_forces(rho_m)
        fr = total.get_forces(rho_r)
        out["fp64_continued"] = {"wall_s": time.perf_counter() - t2, "energy": float(opt_r.energy),
                                 "converged": int(opt_r.converged),
                                 "stages": [(s["precision"], s["n_eval_ev"], s["n_eval_v"], s["n_iter"])
                                            for s in opt_r.stats["stages"]]}
        out["mixed_vs_fp64"] = {"dE_ev_per_atom": (opt_m.energy - opt_r.energy) / st.nat * 27.211386024367243,
                                "max_dF_ha_per_bohr": float(np.abs(fm - fr).max())}
    if a.fp64_from_guess:
        t3 = time.perf_counter()
        opt_p, _ = solve(total, g, "fp64", econv)
        torch.cuda.synchronize()
        out["fp64_from_guess"] = {"wall_s": time.perf_counter() - t3 + t_guess, "energy": float(opt_p.energy),
                                  "converged": int(opt_p.converged),
                                  "stages": [(s["precision"], s["n_eval_ev"], s["n_eval_v"], s["n_iter"])
                                             for s in opt_p.stats["stages"]]}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
