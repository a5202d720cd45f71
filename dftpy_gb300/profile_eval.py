"""Repeat the functional evaluation of the 256-atom / 128^3 WT workload (or
of one Al/Mg alloy snapshot of the batched WGC workload, ``--workload alloy
--seed S``, or of the 4000-atom 360^3 LMGP cell, ``--workload al4000``).

``python -m dftpy_gb300.profile_eval --precision fp32 --calc V --reps 3``
sets the structure up, runs warm-up evaluations, then ``reps`` evaluations
inside an NVTX range named ``eval`` (so a profiler can select exactly those
launches with ``--nvtx --nvtx-include eval/``) and prints the CUDA-event
time per evaluation.  ``--solve mixed`` runs whole TN solves instead (NVTX
range ``solve``), on this thread and stream.
"""
import argparse
import os
import sys


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--precision", default="fp32", choices=["fp32", "fp64"])
    p.add_argument("--calc", default="V", choices=["V", "EV"])
    p.add_argument("--reps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--workload", default="al256", choices=["al256", "al4", "alloy", "al4000"])
    p.add_argument("--seed", type=int, default=0, help="alloy snapshot seed")
    p.add_argument("--solve", default=None, choices=["mixed", "fp64", "fp32"],
                   help="instead of single evaluations, run whole TN solves (NVTX range 'solve')")
    a = p.parse_args()
    import torch
    from . import _lib, systems
    from . import functional as F
    from .field import DirectField
    from .grid import DirectGrid
    from .ions import Ions
    if a.workload == "alloy":
        from .batch import build_evaluator
        st = systems.config_alloy(a.seed)
        total, _ = build_evaluator(st, kedf="WGC")
        grid = total.PSEUDO.grid
        econv = 1e-8 * st.nat
    elif a.workload == "al4000":
        from .large import build
        st, grid, total, _, _ = build()
        econv = 1e-8 * st.nat
    else:
        st = systems.config_al256(0) if a.workload == "al256" else systems.config_al4(0)
        grid = DirectGrid(st.lattice, st.nr, full=False)
        ions = Ions(st.symbols, positions=st.positions, cell=st.lattice)
        ps = F.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": F.AnalyticPP(3.0, 1.0)}, PME=True)
        total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="WT"),
                                  XCFunctional=F.Functional(type="XC", name="LDA"),
                                  HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
        econv = 1e-7
    if a.solve:
        from .optimization import Optimization
        rho0 = DirectField(grid)
        rho0[:] = st.nelec / st.volume

        def run():
            o = Optimization(EnergyEvaluator=total, optimization_method="TN",
                             optimization_options={"econv": econv, "maxfun": 50, "maxiter": 100,
                                                   "precision": a.solve})
            o.optimize_rho(guess_rho=rho0)
            return o
        for _ in range(a.warmup):
            run()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        torch.cuda.nvtx.range_push("solve")
        e0.record()
        for _ in range(a.reps):
            o = run()
        e1.record()
        torch.cuda.nvtx.range_pop()
        torch.cuda.synchronize()
        print("solve %s %s: %.2f ms per solve, E=%.10f, stages %s" % (
            a.workload, a.solve, e0.elapsed_time(e1) / a.reps, o.energy,
            [(s["precision"], s["n_eval_ev"], s["n_eval_v"]) for s in o.stats["stages"]]))
        return 0
    dt = torch.float32 if a.precision == "fp32" else torch.float64
    g = torch.Generator(device="cuda").manual_seed(0)
    base = st.nelec / st.volume
    x = (base * (1.0 + 0.05 * torch.randn(tuple(st.nr), generator=g, device="cuda", dtype=torch.float64))).to(dt)
    if a.workload == "al4000":
        # the superposed atomic densities: the k_F range (and the LMGP knot
        # count) of a real solve, not of a near-uniform noise field
        from .density import DensityGenerator
        r_, a_ = systems.atomic_density_table(3.0, systems.ATOMIC_SIGMA["Al"])
        x = DensityGenerator(r={"Al": r_}, arho={"Al": a_}).guess_rho(total.PSEUDO.ions, grid=grid).as_subclass(
            torch.Tensor).to(dt)
    rho = DirectField(grid, data=x)
    f = total.spec(rho).ctypes()
    plan = grid.plan(dt)
    xr = rho.as_subclass(torch.Tensor).contiguous()
    pot = torch.empty_like(xr)
    en = torch.empty(_lib.NE, dtype=torch.float64, device="cuda")
    calc = _lib.CALC_V | (_lib.CALC_E if a.calc == "EV" else 0)
    L = _lib.load()
    s = _lib.stream_ptr()
    for _ in range(a.warmup):
        _lib.check(L.gbofdft_eval(plan.handle, _lib.ptr(xr), f, _lib.ptr(pot), _lib.ptr(en), calc, s))
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("eval")
    e0.record()
    for _ in range(a.reps):
        _lib.check(L.gbofdft_eval(plan.handle, _lib.ptr(xr), f, _lib.ptr(pot), _lib.ptr(en), calc, s))
    e1.record()
    torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    kd = getattr(getattr(total, "KineticEnergyFunctional", None), "_lwt", None)
    knots = "" if kd is None else ", %d k_F knots" % kd.prepare(rho).nknots
    print("eval %s %s %s: %.1f us per evaluation%s" % (a.workload, a.precision, a.calc,
                                                       e0.elapsed_time(e1) * 1000.0 / a.reps, knots))
    return 0


if __name__ == "__main__":
    sys.exit(main())
