#!/usr/bin/env python3
"""Benchmark: wall-seconds to a converged OF-DFT energy.

Workload (the single-GPU configuration the metric is quoted on): bulk fcc Al
4x4x4 supercell, 256 atoms, 128^3 grid, KEDF WT (alpha = beta = 5/6) + LDA +
Hartree + analytic local pseudopotential (PME), truncated-Newton direct
minimisation, econv 1e-7 Ha.  One "step" is one full solve.  ``value`` is
the learned + mixed-precision solve: the starting density from the trained
guess network (tensor-core inference on the step's own atomic-density and
v_loc features, inside the timed region), then FP32 TN and the FP64
refinement, with the evaluator's set-up (PP, kernel tables, plans) already
on the device.  The FP64 ("plain") solve from the uniform density -- the
reference's method -- and the mixed solve from the uniform density are timed
beside it.  Each solve's energy is checked against the FP64 reference within
1e-5 eV/atom.

Under torchrun with N ranks every rank solves its own seeded snapshot (weak
scaling, no data-path collective); rank 0 prints one JSON line.
``--impl reference`` times the reference algorithm's CPU implementation (the
numpy oracle) on the host cores instead.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HA_EV = 27.211386024367243
TOL_EV_PER_ATOM = 1e-5


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gbofdft", choices=["gbofdft", "reference"])
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "fp32"])
    p.add_argument("--no-plain", action="store_true", help="skip timing the FP64 plain path")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    p.add_argument("--guess", default="learned", choices=["learned", "uniform"],
                   help="starting density of the timed solves (learned: the trained network's guess)")
    return p.parse_args()


def rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def rank_seed(rank):
    """Each rank solves its own snapshot (weak scaling): seed = rank."""
    return int(rank)


def max_over_ranks(x, world, device="cuda"):
    """Step time of the whole job: the maximum over ranks (one all-reduce,
    outside the timed region; the only collective of the benchmark)."""
    if world <= 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples of the SM clock and throttle reasons during a region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.f = None

    def start(self):
        try:
            self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for k, v in zip(names, r[5:9]):
                    if "Active" in v and "Not" not in v:
                        reasons.add(k)
            except Exception:
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profile_traffic():
    """Per-evaluation DRAM bytes from the committed ncu summary, if present."""
    try:
        with open(os.path.join(ROOT, "profiles", "eval_fp32_al256_traffic.json")) as f:
            return json.load(f)
    except Exception:
        return None


# ---------------------------------------------------------------------------
def build_system(seed):
    import torch
    from dftpy_gb300 import functional as F
    from dftpy_gb300 import systems
    from dftpy_gb300.field import DirectField
    from dftpy_gb300.grid import DirectGrid
    from dftpy_gb300.ions import Ions
    st = systems.config_al256(seed)
    grid = DirectGrid(st.lattice, st.nr, full=False)
    ions = Ions(st.symbols, positions=st.positions, cell=st.lattice)
    ps = F.LocalPseudo(grid=grid, ions=ions, PP_list={"Al": F.AnalyticPP(*systems.SPECIES["Al"])}, PME=True)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name="WT"),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    ps.local_PP()
    total.ewald.energy
    rho0 = DirectField(grid)
    rho0[:] = st.nelec / st.volume
    for dt in (torch.float32, torch.float64):
        total.spec(rho0.to(dt))       # WT kernel tables, v_loc casts
    torch.cuda.synchronize()
    return st, grid, total, rho0


GUESS_WEIGHTS = os.path.join(ROOT, "dftpy_gb300", "data", "guessnet_al_wt.npz")


def learned_guess():
    """The trained guess network for this workload (weights loaded once, like
    the plans; the guess itself is computed inside every timed step)."""
    from dftpy_gb300 import guess as G
    return G.LearnedGuess(G.GuessNet.load(GUESS_WEIGHTS))


def solve(total, rho0, precision, time_evals=False, guesser=None):
    from dftpy_gb300.optimization import Optimization
    if guesser is not None:
        rho0 = guesser.guess(total, rho0.grid)
    opt = Optimization(EnergyEvaluator=total, optimization_method="TN",
                       optimization_options={"econv": 1e-7, "maxfun": 50, "maxiter": 100, "precision": precision,
                                             "time_evals": time_evals})
    rho = opt.optimize_rho(guess_rho=rho0)
    return opt, rho


def timed_solves(total, rho0, precision, steps, warmup, flush, world, guesser=None):
    import torch
    from dftpy_gb300 import _lib
    for _ in range(warmup):
        solve(total, rho0, precision, guesser=guesser)
    torch.cuda.synchronize()
    times, energies, evals, glue = [], [], [], []
    t_ev, n_ev = 0.0, 0
    l0 = _lib.launch_count()
    for _ in range(steps):
        flush.zero_()                      # 512 MB write: evicts L2 between steps
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        torch.cuda.synchronize()
        s = torch.cuda.current_stream()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(s)
        opt, rho = solve(total, rho0, precision, time_evals=True, guesser=guesser)
        e1.record(s)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1000.0)
        for st in opt.stats["stages"]:
            t_ev += st.get("t_eval_timed", 0.0)
            n_ev += st.get("n_eval_timed", 0)
        energies.append(opt.energy)
        glue.append(opt.stats.get("t_glue", 0.0))
        evals.append([{"precision": st["precision"], "n_eval_ev": st["n_eval_ev"], "n_eval_v": st["n_eval_v"],
                       "n_eval_hess_f32": st.get("n_eval_hess", 0),
                       "converged": st["converged"], "n_iter": st["n_iter"], "n_sync": st["n_sync"],
                       "t_sync_s": round(st["t_sync"], 4), "t_host_s": round(st["t_total"], 4),
                       "last_dE": [round(e - st["history"][-1], 12) for e in st["history"][-5:]]}
                      for st in opt.stats["stages"]])
    launches = _lib.launch_count() - l0
    evals[-1].append({"python_glue_s": round(glue[-1], 4)})
    return times, energies, evals, launches, (t_ev, n_ev)


def eval_roofline(total, rho0, reps=50):
    """CUDA-event time of one FP32 potential-only evaluation (the operation
    ~90% of the mixed solve's evaluations are) on the launching stream."""
    import torch
    from dftpy_gb300 import _lib
    r = rho0.to(torch.float32)
    spec = total.spec(r)
    f = spec.ctypes()
    plan = r.grid.plan(torch.float32)
    x = r.as_subclass(torch.Tensor).contiguous()
    pot = torch.empty_like(x)
    L = _lib.load()
    s = _lib.stream_ptr()
    for _ in range(5):
        _lib.check(L.gbofdft_eval(plan.handle, _lib.ptr(x), f, _lib.ptr(pot), None, _lib.CALC_V, s))
    torch.cuda.synchronize()
    st = torch.cuda.current_stream()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        L.gbofdft_eval(plan.handle, _lib.ptr(x), f, _lib.ptr(pot), None, _lib.CALC_V, s)
    e1.record(st)
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1000.0 / reps
    n = int(r.numel())
    # algorithmic bytes per evaluation (WT + LDA + H + PP): s N (R + W + 2F),
    # R = 2 (rho, v_loc), W = 1 (V), F = 6 transforms the reference performs
    b_eval = 4 * n * (2 + 1 + 2 * 6)
    return t, b_eval


def e2e_solves(st, total, precision, steps, warmup, guesser=None):
    """Public API with host buffers, host<->device copies inside the timed
    region: the starting density from pinned host memory (uniform guess) or
    the host positions the learned guess's features are built from (learned),
    out the host density and energy."""
    import numpy as np
    import torch
    from dftpy_gb300.field import DirectField
    grid = total.PSEUDO.grid
    host = torch.full(tuple(st.nr), st.nelec / st.volume, dtype=torch.float64).pin_memory()
    out_host = torch.empty(tuple(st.nr), dtype=torch.float64).pin_memory()
    times = []
    for i in range(warmup + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if guesser is None:
            rho0 = DirectField(grid, data=host.to("cuda", non_blocking=True))
        else:
            rho0 = DirectField(grid)            # only its grid is used: the guess copies the positions in
        opt, rho = solve(total, rho0, precision, guesser=guesser)
        out_host.copy_(rho.as_subclass(torch.Tensor).to(torch.float64), non_blocking=True)
        torch.cuda.synchronize()
        e = float(opt.energy)
        dt = time.perf_counter() - t0
        if i >= warmup:
            times.append(dt)
    nbytes = int(np.prod(st.nr)) * 8
    h2d = nbytes if guesser is None else st.nat * 3 * 8
    return statistics.mean(times), h2d, nbytes + 8, e


def cpu_baseline(st, golden_evals, workers):
    """The numpy oracle of the reference algorithm on the host: a bounded
    sample (E+V evaluations at 128^3), extrapolated to a full solve's
    evaluation count."""
    import numpy as np
    from oracle import ofdft as O
    O.set_fft_workers(workers)
    t0 = time.perf_counter()
    ev = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="WT")
    t_setup = time.perf_counter() - t0
    rho = np.full(st.nr, st.nelec / st.volume)
    rho = rho * (1.0 + 0.01 * np.random.default_rng(0).standard_normal(st.nr))
    nsample = 4
    t0 = time.perf_counter()
    for i in range(nsample):
        ev(rho, calc_e=(i == 0))
    t_eval = (time.perf_counter() - t0) / nsample
    O.set_fft_workers(1)
    return t_eval * golden_evals, t_eval, t_setup, nsample


def golden_evals():
    import numpy as np
    try:
        a = np.load(os.path.join(ROOT, "tests", "golden", "al256.npz"))
        return int(a["n_ev"]) + int(a["n_v"]), float(a["E_final"])
    except Exception:
        return 146, None


# ---------------------------------------------------------------------------
def run_reference(args):
    """--impl reference: the reference algorithm's CPU implementation (numpy
    oracle) on the host cores, same workload and metric."""
    rank, world, _ = rank_info()
    if rank != 0:
        return 0
    from dftpy_gb300 import systems
    st = systems.config_al256(0)
    n_evals, _ = golden_evals()
    workers = os.cpu_count() or 1
    times = []
    for i in range(args.warmup + args.steps):
        v, t_eval, t_setup, ns = cpu_baseline(st, n_evals, workers)
        if i >= args.warmup:
            times.append(v)
    value = statistics.mean(times)
    line = {
        "impl": "reference", "metric": "wall-s to converged OFDFT energy (<=1e-5 eV/atom vs FP64)",
        "value": value, "unit": "s", "n_gpus": 0, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": value * 1000.0, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64", "data": "synthetic (seeded jittered fcc Al)",
        "config": {"workload": "al256_128_wt", "natoms": 256, "grid": [128, 128, 128],
                   "functional": "WT+LDA+Hartree+analyticPP(PME)", "method": "TN econv 1e-7"},
        "cpu_baseline": {"value": value, "unit": "s", "cores": workers, "kind": "port",
                         "sample": "%d oracle E+V evaluations at 128^3 per step (numpy, FFTs on %d threads), "
                                   "extrapolated to the reference solve's %d evaluations" % (ns, workers, n_evals)},
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import torch
    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__
    __graft_entry__.build()
    st, grid, total, rho0 = build_system(rank_seed(rank))
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    n_evals_ref, e_golden = golden_evals()
    # FP64 reference energy for this snapshot (plain GPU path; rank 0 also
    # matches the reference-generated fixture)
    guesser = learned_guess() if args.guess == "learned" else None
    clocks = ClockSampler(local)
    clocks.start()
    times, energies, evals, launches, live = timed_solves(total, rho0, args.precision, args.steps, args.warmup,
                                                          flush, world, guesser=guesser)
    clk = clocks.stop()
    plain = None
    if not args.no_plain:
        pt, pe, pev, _, _ = timed_solves(total, rho0, "fp64", max(1, min(args.steps, 2)), 1, flush, world)
        plain = {"value": statistics.mean(pt), "energy": pe[-1], "evals": pev[-1], "guess": "uniform"}
    uniform = None
    if guesser is not None:
        ut, ue, uev, _, _ = timed_solves(total, rho0, args.precision, max(1, min(args.steps, 2)), 1, flush, world)
        uniform = {"value": statistics.mean(ut), "energy": ue[-1], "evals": uev[-1]}
    e_ref = plain["energy"] if plain else None
    if rank == 0 and e_golden is not None:
        e_ref = e_golden
    err = None if e_ref is None else max(abs(e - e_ref) for e in energies) * HA_EV / st.nat
    t_step = max_over_ranks(statistics.mean(times), world)
    t_iso, b_eval = eval_roofline(total, rho0)
    # the FP32 potential evaluations inside the timed solves (CUDA events on
    # the solve's stream around each one); the isolated loop is reported beside
    t_eval = live[0] / live[1] if live[1] else t_iso
    peak, peak_kind = measured_peaks()
    achieved = b_eval / t_eval / 1e9
    traffic = profile_traffic()
    e2e_v, h2d, d2h, _ = e2e_solves(st, total, args.precision, 1 if args.steps < 2 else 2, 1, guesser=guesser)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        v, t_ev, t_setup, ns = cpu_baseline(st, n_evals_ref, 1)
        cpu = {"value": v, "unit": "s", "cores": 1, "kind": "port",
               "sample": "%d numpy-oracle E+V evaluations at 128^3 (%.2f s each, 1 thread), extrapolated to "
                         "the reference solve's %d evaluations" % (ns, t_ev, n_evals_ref)}
    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()
        return 0
    line = {
        "metric": "wall-s to converged OFDFT energy (<=1e-5 eV/atom vs FP64), learned+mixed vs plain",
        "value": t_step, "unit": "s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": t_step * 1000.0, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": {"mixed": "f32+f64", "fp64": "f64", "fp32": "f32"}[args.precision],
        "data": "synthetic (seeded jittered fcc Al; starting density from the guess network trained on the "
                "solver's own converged 2x2x2-cell densities)" if guesser is not None else
                "synthetic (seeded jittered fcc Al, uniform initial density)",
        "config": {"workload": "al256_128_wt", "natoms": st.nat, "grid": list(st.nr),
                   "functional": "KEDF WT(5/6,5/6)+LDA+Hartree+analytic PP (PME order 10)",
                   "method": "TN econv 1e-7 Ha, maxfun 50", "precision": args.precision,
                   "guess": ("learned (BF16 tcgen05 network, dftpy_gb300/data/guessnet_al_wt.npz; inference "
                             "inside the timed step)") if guesser is not None else "uniform",
                   "l2": "512 MB buffer written between timed steps",
                   "seed_per_rank": "rank"},
        "accuracy": {"max_err_ev_per_atom": err, "tolerance_ev_per_atom": TOL_EV_PER_ATOM,
                     "ok": None if err is None else err <= TOL_EV_PER_ATOM,
                     "energy": energies[-1], "reference_energy": e_ref},
        "evaluations": evals[-1],
        "plain_fp64": plain,
        "speedup_vs_plain": (plain["value"] / t_step) if plain else None,
        "mixed_uniform_guess": uniform,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_kind": peak_kind,
                     "traffic": traffic.get("bytes_per_eval") if traffic else None,
                     "kernel": "FP32 potential evaluation (rows / plane-convolution / rows pipeline, autotuned "
                               "schedule), 128^3",
                     "t_eval_us": t_eval * 1e6, "n_evals_timed": live[1],
                     "timing": "CUDA events around each FP32 potential evaluation inside the timed solves",
                     "t_eval_isolated_us": t_iso * 1e6, "algorithmic_bytes": b_eval},
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_v, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
