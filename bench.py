#!/usr/bin/env python3
"""Benchmark: wall-seconds to converged OF-DFT energies, learned + mixed
precision against the plain FP64 method.

Workload (``--workload alloy64``, the default): the batched Al/Mg alloy
workload -- 64 random-substitution snapshots (``systems.config_alloy``, seeds
0-63: 108-500 atoms, cubic and orthorhombic cells, grids 96^3-160^3 at 0.24
Bohr spacing, Mg fraction U(0, 0.3), jitter 0.15 Bohr), KEDF TF + vW + WGC
(second-order density-dependent kernel) + LDA + Hartree + analytic local
pseudopotentials (PME), econv 1e-8 Ha/atom.  One "step" optimises all 64:
each structure's starting density comes from the guess network
(``dftpy_gb300/data/guessnet.npz``: 4-level encoder-decoder, 32-128 channels,
1.5 M parameters, run on 4x pooled features; trained on the solver's own
converged densities of 2000 other snapshots, seeds 1000-2999; inference on the
tensor cores inside the step, with the fallback check against the uniform
density's residual), then FP32 truncated Newton and the FP64 refinement, 6
structures in flight on their own streams.  The evaluators' set-up (pseudopotentials, Ewald, kernel
tables, plans) is done before the timed steps, as the reference's timing
excludes it.  ``value`` is the wall time of one step.  Beside it: the plain
FP64 batch (the reference's method: uniform start, unpreconditioned TN, FP64
throughout) and the mixed batch from the uniform density; every energy is
checked against the plain FP64 one (<= 1e-5 eV/atom) and against the CPU
oracle's own solves (``tests/golden/alloy64_oracle.npz``).

``--workload al256`` times one 256-atom Al cell (128^3, Wang-Teter) the same
way; the default run also reports it as ``al256`` (and the FP32 evaluation
roofline is measured inside its single-stream solves).

Under torchrun with N ranks the 64 structures are split by longest
processing time on the grid size (``batch.shard``); each rank solves its
share, no collective on the data path, ``value`` = the slowest rank's time
(strong scaling).  ``--impl reference`` times the reference algorithm's CPU
implementation (the numpy oracle) on the host cores for the same workload.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

HA_EV = 27.211386024367243


def _plain(o):
    """json.dumps default: numpy scalars and arrays as Python numbers and lists."""
    if hasattr(o, "tolist"):
        return o.tolist()
    if hasattr(o, "item"):
        return o.item()
    raise TypeError("%s is not JSON serializable" % type(o).__name__)
TOL_EV_PER_ATOM = 1e-5
METRIC = "wall-s to converged OFDFT energy (<=1e-5 eV/atom vs FP64), learned+mixed vs plain"
ECONV_PER_ATOM = 1e-8
N_ALLOY = 64


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=3)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gbofdft", choices=["gbofdft", "reference"])
    p.add_argument("--workload", default="alloy64", choices=["alloy64", "al256"])
    p.add_argument("--n", type=int, default=N_ALLOY, help="alloy snapshots in the batch (seeds 0..n-1)")
    p.add_argument("--workers", type=int, default=6, help="structures in flight on the GPU")
    p.add_argument("--precision", default="mixed", choices=["mixed", "fp64", "fp32"])
    p.add_argument("--no-plain", action="store_true", help="skip timing the FP64 plain path")
    p.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline")
    p.add_argument("--no-al256", action="store_true", help="skip the 256-atom single-cell section")
    p.add_argument("--guess", default="learned", choices=["learned", "uniform"],
                   help="starting density of the timed solves (learned: the trained network's guess)")
    return p.parse_args()


def rank_info():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


def rank_seed(rank):
    """Seed of the single-cell workload on each rank: the rank."""
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


def oracle_fixture():
    """The CPU oracle's full solves of the 64 alloy snapshots (energies and
    evaluation counts), or None."""
    import numpy as np
    path = os.path.join(ROOT, "tests", "golden", "alloy64_oracle.npz")
    if not os.path.exists(path):
        return None
    return dict(np.load(path))


# ---------------------------------------------------------------------------
# the batched alloy workload
# ---------------------------------------------------------------------------
ALLOY_WEIGHTS = os.path.join(ROOT, "dftpy_gb300", "data", "guessnet.npz")
AL_WEIGHTS = os.path.join(ROOT, "dftpy_gb300", "data", "guessnet_al_wt.npz")


def load_guess(path):
    from dftpy_gb300 import guess as G
    return G.LearnedGuess(G.GuessNet.load(path))


def alloy_jobs(seeds):
    """(evaluator, uniform density) per seed, with the evaluator's set-up on
    the device (PP, Ewald, plans, kernel tables of both precisions)."""
    import torch
    from dftpy_gb300 import batch, systems
    jobs = []
    for s in seeds:
        st = systems.config_alloy(s)
        total, rho0 = batch.build_evaluator(st, kedf="WGC")
        total.PSEUDO.local_PP()
        total.ewald.energy
        for dt in (torch.float32, torch.float64):
            total.spec(rho0.to(dt))
        jobs.append((total, rho0))
    torch.cuda.synchronize()
    return jobs


def batch_step(jobs, precision, guess, workers, extra=None):
    """One step: optimise every job; returns (wall s, results)."""
    import torch
    from dftpy_gb300 import batch
    opts = {"precision": precision, "econv_per_atom": ECONV_PER_ATOM}
    opts.update(extra or {})
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    t0 = time.perf_counter()
    res = batch.optimize_batch(jobs, workers=workers, options=opts, guess=guess)
    e1.record()
    torch.cuda.synchronize()
    wall = time.perf_counter() - t0
    return max(wall, e0.elapsed_time(e1) / 1000.0), res


def timed_batches(jobs, precision, guess, steps, warmup, flush, world, workers, extra=None):
    from dftpy_gb300 import _lib
    for _ in range(warmup):
        batch_step(jobs, precision, guess, workers, extra)
    times, last = [], None
    l0 = _lib.launch_count()
    for _ in range(steps):
        flush.zero_()                      # 512 MB write: evicts L2 between steps
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
        t, last = batch_step(jobs, precision, guess, workers, extra)
        times.append(t)
    return times, last, _lib.launch_count() - l0


def n_evals(r):
    return sum(s["n_eval_ev"] + s["n_eval_v"] + s.get("n_eval_hess", 0) for s in r.stats["stages"])


def e2e_batch(seeds, jobs, precision, guess, workers, steps, warmup):
    """Through the public API with host buffers: the structures' host
    positions go to the device inside the step (the guess features are made
    from them), and every converged density and energy comes back to pinned
    host memory."""
    import numpy as np
    import torch
    from dftpy_gb300 import batch, systems
    outs = [torch.empty(tuple(int(x) for x in j[1].grid.nrR), dtype=torch.float64).pin_memory() for j in jobs]
    times = []
    for i in range(warmup + steps):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res = batch.optimize_batch(jobs, workers=workers, options={"precision": precision,
                                                                     "econv_per_atom": ECONV_PER_ATOM}, guess=guess)
        for r, o in zip(res, outs):
            o.copy_(r.rho.as_subclass(torch.Tensor).to(torch.float64), non_blocking=True)
        torch.cuda.synchronize()
        energies = [float(r.energy) for r in res]
        dt = time.perf_counter() - t0
        if i >= warmup:
            times.append(dt)
    h2d = sum(systems.config_alloy(s).nat * 3 * 8 for s in seeds)
    d2h = sum(int(np.prod(o.shape)) * 8 + 8 for o in outs)
    return statistics.mean(times), h2d, d2h, energies


def eval_roofline_wgc(total, rho0, reps=50):
    """CUDA-event time of one FP32 potential-only evaluation of the batch's
    functional on one 128^3 snapshot, back to back on one stream."""
    import torch
    from dftpy_gb300 import _lib
    r = rho0.to(torch.float32)
    f = total.spec(r).ctypes()
    plan = r.grid.plan(torch.float32)
    x = r.as_subclass(torch.Tensor).contiguous()
    pot = torch.empty_like(x)
    L = _lib.load()
    s = _lib.stream_ptr()
    for _ in range(5):
        _lib.check(L.gbofdft_eval(plan.handle, _lib.ptr(x), f, _lib.ptr(pot), None, _lib.CALC_V, s))
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        L.gbofdft_eval(plan.handle, _lib.ptr(x), f, _lib.ptr(pot), None, _lib.CALC_V, s)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / 1000.0 / reps


# ---------------------------------------------------------------------------
# the 256-atom single cell (one stream; the live evaluation roofline)
# ---------------------------------------------------------------------------
def build_al256(seed):
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
        total.spec(rho0.to(dt))
    torch.cuda.synchronize()
    return st, grid, total, rho0


def solve(total, rho0, precision, time_evals=False, guesser=None):
    from dftpy_gb300.optimization import Optimization
    if guesser is not None:
        rho0 = guesser.guess(total, rho0.grid)
    opt = Optimization(EnergyEvaluator=total, optimization_method="TN",
                       optimization_options={"econv": 1e-7, "maxfun": 50, "maxiter": 100, "precision": precision,
                                             "time_evals": time_evals})
    rho = opt.optimize_rho(guess_rho=rho0)
    return opt, rho


def timed_solves(total, rho0, precision, steps, warmup, flush, guesser=None, time_evals=True):
    import torch
    for _ in range(warmup):
        solve(total, rho0, precision, guesser=guesser)
    torch.cuda.synchronize()
    times, energies, evals = [], [], []
    t_ev, n_ev = 0.0, 0
    for _ in range(steps):
        flush.zero_()
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record()
        opt, rho = solve(total, rho0, precision, time_evals=time_evals, guesser=guesser)
        e1.record()
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) / 1000.0)
        for st in opt.stats["stages"]:
            t_ev += st.get("t_eval_timed", 0.0)
            n_ev += st.get("n_eval_timed", 0)
        energies.append(opt.energy)
        evals.append([{"precision": st["precision"], "n_eval_ev": st["n_eval_ev"], "n_eval_v": st["n_eval_v"],
                       "n_eval_hess_f32": st.get("n_eval_hess", 0), "converged": st["converged"],
                       "n_iter": st["n_iter"], "n_sync": st["n_sync"]} for st in opt.stats["stages"]])
    return times, energies, evals, (t_ev, n_ev)


def al256_section(flush, steps, warmup, do_plain):
    """Learned + mixed solve of the 256-atom cell, the mixed solve from the
    uniform density and the plain FP64 solve; the FP32 potential evaluations
    inside the timed solves are timed with CUDA events (single stream)."""
    import numpy as np
    st, grid, total, rho0 = build_al256(0)
    g = load_guess(AL_WEIGHTS)
    lt, le, lev, live = timed_solves(total, rho0, "mixed", steps, warmup, flush, guesser=g)
    ut, ue, _, _ = timed_solves(total, rho0, "mixed", max(1, min(steps, 2)), 1, flush, time_evals=False)
    out = {"workload": "al256_128_wt", "natoms": st.nat, "grid": list(st.nr),
           "learned_mixed_s": statistics.mean(lt), "mixed_uniform_s": statistics.mean(ut),
           "evaluations": lev[-1], "live_eval": live}
    try:
        ref = float(np.load(os.path.join(ROOT, "tests", "golden", "al256.npz"))["E_final"])
        out["max_err_ev_per_atom_vs_reference"] = max(abs(e - ref) for e in le + ue) * HA_EV / st.nat
    except Exception:
        pass
    if do_plain:
        pt, pe, pev, _ = timed_solves(total, rho0, "fp64", 1, 1, flush, time_evals=False)
        out["plain_fp64_s"] = statistics.mean(pt)
        out["plain_evaluations"] = pev[-1]
        out["speedup_learned_mixed_vs_plain"] = out["plain_fp64_s"] / out["learned_mixed_s"]
    return out, total, rho0


def eval_roofline(total, rho0, reps=50):
    """Isolated back-to-back FP32 potential-only evaluations (128^3, WT)."""
    import torch
    from dftpy_gb300 import _lib
    r = rho0.to(torch.float32)
    f = total.spec(r).ctypes()
    plan = r.grid.plan(torch.float32)
    x = r.as_subclass(torch.Tensor).contiguous()
    pot = torch.empty_like(x)
    L = _lib.load()
    s = _lib.stream_ptr()
    for _ in range(5):
        _lib.check(L.gbofdft_eval(plan.handle, _lib.ptr(x), f, _lib.ptr(pot), None, _lib.CALC_V, s))
    torch.cuda.synchronize()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        L.gbofdft_eval(plan.handle, _lib.ptr(x), f, _lib.ptr(pot), None, _lib.CALC_V, s)
    e1.record()
    torch.cuda.synchronize()
    t = e0.elapsed_time(e1) / 1000.0 / reps
    # algorithmic bytes per evaluation (WT + LDA + H + PP): s N (R + W + 2F),
    # R = 2 (rho, v_loc), W = 1 (V), F = 6 transforms the reference performs
    return t, 4 * int(r.numel()) * (2 + 1 + 2 * 6)


# ---------------------------------------------------------------------------
# CPU: the reference algorithm's numpy implementation (the oracle)
# ---------------------------------------------------------------------------
def _cpu_worker_init():
    os.environ.setdefault("OMP_NUM_THREADS", "1")
    sys.path.insert(0, ROOT)


_CPU_EVAL = {}


def _cpu_sample(seed):
    """One E+V and one V-only evaluation of snapshot ``seed`` by the oracle
    (TF + vW + WGC + LDA + Hartree + PP), 1 thread; set-up excluded and kept
    for the next step.  Returns (seed, t_EV, t_V)."""
    import numpy as np
    from dftpy_gb300 import systems
    from oracle import ofdft as O
    from oracle import wgc as W
    ev = _CPU_EVAL.get(seed)
    if ev is None:
        st = systems.config_alloy(seed)
        base = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")
        nl = W.WGCNL()
        rho = np.full(st.nr, st.nelec / st.volume)
        rho = rho * (1.0 + 0.01 * np.random.default_rng(seed).standard_normal(st.nr))
        ev = _CPU_EVAL[seed] = (base, nl, rho)
        nl(rho, base.grid, True)           # the WGC kernels of this grid (set-up)
    base, nl, rho = ev
    t0 = time.perf_counter()
    base(rho, True)
    nl(rho, base.grid, True)
    t1 = time.perf_counter()
    base(rho, False)
    nl(rho, base.grid, False)
    t2 = time.perf_counter()
    return seed, t1 - t0, t2 - t1


def lpt_makespan(costs, cores):
    from dftpy_gb300.batch import partition_lpt
    _, loads = partition_lpt(costs, cores)
    return max(loads)


def cpu_extrapolate(samples, fix):
    """Per snapshot t_EV * n_EV + t_V * n_V with the oracle's own evaluation
    counts of its full solve of that snapshot."""
    idx = {int(s): i for i, s in enumerate(fix["seed"])}
    out = {}
    for seed, t_ev, t_v in samples:
        i = idx[int(seed)]
        out[int(seed)] = t_ev * int(fix["n_ev"][i]) + t_v * int(fix["n_v"][i])
    return out


def cpu_baseline_1core(seeds, fix):
    """One thread: one snapshot per grid shape sampled, the rest take their
    shape's per-evaluation times; the batch's solves one after another."""
    from dftpy_gb300 import systems
    by_shape = {}
    for s in seeds:
        by_shape.setdefault(systems.config_alloy(s).nr, s)
    t0 = time.perf_counter()
    samp = {systems.config_alloy(s).nr: _cpu_sample(s) for s in by_shape.values()}
    t_sample = time.perf_counter() - t0
    rows = [(s,) + samp[systems.config_alloy(s).nr][1:] for s in seeds]
    per = cpu_extrapolate(rows, fix)
    _CPU_EVAL.clear()
    return sum(per.values()), len(by_shape), t_sample


def _ref_worker(conn, seeds):
    """One host core of the reference arm: owns ``seeds`` (their oracle
    set-up stays here) and answers ("sample", seed) with its evaluation
    times until ("stop",)."""
    _cpu_worker_init()
    while True:
        msg = conn.recv()
        if msg[0] == "stop":
            break
        conn.send(_cpu_sample(msg[1]))
    conn.close()


def run_reference(args):
    """--impl reference: the reference algorithm's CPU implementation (the
    numpy oracle, one single-threaded process per core) on the host, same
    workload, metric and unit.  The snapshots are split over min(n, cores)
    worker processes (longest processing time on the grid size); a set-up
    pass (not timed, as the reference's timing excludes set-up) builds every
    snapshot's oracle and times one E+V and one V-only evaluation of it; each
    step then times again one snapshot per worker, in rotation.  A snapshot's
    solve time is its latest evaluation times times the evaluation counts of
    the oracle's own full solve of it (``tests/golden/alloy64_oracle.npz``);
    ``value`` is the batch's wall time on the cores: the longest-processing-
    time makespan of those solves."""
    rank, world, _ = rank_info()
    if rank != 0:
        return 0
    import multiprocessing as mp
    from dftpy_gb300 import batch, systems
    fix = oracle_fixture()
    if fix is None:
        print(json.dumps({"impl": "reference", "unavailable": "tests/golden/alloy64_oracle.npz is missing"},
                         default=_plain))
        return 0
    seeds = list(range(args.n))
    cores = os.cpu_count() or 1
    workers = max(1, min(len(seeds), cores))
    parts, _ = batch.partition_lpt([int(fix["nr"][s].prod()) for s in seeds], workers)
    parts = [[seeds[i] for i in p] for p in parts]
    ctx = mp.get_context("spawn")
    pipes, procs = [], []
    for part in parts:
        a, b = ctx.Pipe()
        pr = ctx.Process(target=_ref_worker, args=(b, part), daemon=True)
        pr.start()
        pipes.append(a)
        procs.append(pr)
    latest = {}
    try:
        # set-up pass: every snapshot's oracle, and a first sample of each
        for k in range(max(len(p) for p in parts)):
            busy = [(c, p[k]) for c, p in zip(pipes, parts) if k < len(p)]
            for c, sd in busy:
                c.send(("sample", sd))
            for c, _ in busy:
                sd, t_ev, t_v = c.recv()
                latest[sd] = (t_ev, t_v)
        values, walls = [], []
        for i in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            busy = [(c, p[i % len(p)]) for c, p in zip(pipes, parts) if p]
            for c, sd in busy:
                c.send(("sample", sd))
            for c, _ in busy:
                sd, t_ev, t_v = c.recv()
                latest[sd] = (t_ev, t_v)
            wall = time.perf_counter() - t0
            per = cpu_extrapolate([(sd,) + latest[sd] for sd in seeds], fix)
            if i >= args.warmup:
                values.append(lpt_makespan([per[sd] for sd in seeds], workers))
                walls.append(wall)
    finally:
        for c in pipes:
            try:
                c.send(("stop",))
            except Exception:
                pass
        for pr in procs:
            pr.join(timeout=30)
    value = statistics.mean(values)
    nat = [systems.config_alloy(s).nat for s in seeds]
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": 0, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": statistics.mean(walls) * 1000.0, "higher_is_better": False,
        "scaling": "strong", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded Al/Mg alloy snapshots)",
        "config": {"workload": "alloy64_wgc", "structures": len(seeds), "natoms_range": [min(nat), max(nat)],
                   "grids": "96^3-160^3", "functional": "TF+vW+WGC(second order)+LDA+Hartree+analytic PP (PME)",
                   "method": "TN econv 1e-8 Ha/atom, uniform start (the reference's method)"},
        "value_kind": "extrapolated: measured evaluation times x the oracle's full-solve evaluation counts",
        "cpu_baseline": {"value": value, "unit": "s", "cores": workers, "kind": "port",
                         "sample": "%d single-threaded numpy-oracle worker processes; per step each times one "
                                   "E+V and one V-only evaluation of one of its snapshots (in rotation; %.1f s of "
                                   "wall per step); each snapshot's solve = its latest times x its E+V / V-only "
                                   "counts in the oracle's own full TN solve (tests/golden/alloy64_oracle.npz); "
                                   "value = the longest-processing-time makespan of the %d solves on %d cores; "
                                   "set-up excluded" % (workers, statistics.mean(walls), len(seeds), workers)},
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line, default=_plain), flush=True)
    return 0


# ---------------------------------------------------------------------------
def main_al256(args):
    """--workload al256: the 256-atom cell alone (one solve per step)."""
    import torch
    rank, world, local = rank_info()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    st, grid, total, rho0 = build_al256(rank_seed(rank))
    g = load_guess(AL_WEIGHTS) if args.guess == "learned" else None
    clocks = ClockSampler(local)
    clocks.start()
    times, energies, evals, live = timed_solves(total, rho0, args.precision, args.steps, args.warmup, flush, guesser=g)
    clk = clocks.stop()
    t_step = max_over_ranks(statistics.mean(times), world)
    t_iso, b_eval = eval_roofline(total, rho0)
    t_eval = live[0] / live[1] if live[1] else t_iso
    peak, peak_kind = measured_peaks()
    if rank != 0:
        return 0
    print(json.dumps({"metric": METRIC, "value": t_step, "unit": "s", "n_gpus": world, "steps": args.steps,
                      "warmup": args.warmup, "ms_per_step": t_step * 1e3, "higher_is_better": False,
                      "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
                      "config": {"workload": "al256_128_wt"}, "evaluations": evals[-1],
                      "roofline": {"bound": "hbm", "achieved": b_eval / t_eval / 1e9, "peak": peak, "unit": "GB/s",
                                   "frac": b_eval / t_eval / 1e9 / peak, "peak_kind": peak_kind},
                      "clocks": clk}, default=_plain), flush=True)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    import numpy as np
    import torch
    rank, world, local = rank_info()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import __graft_entry__
    __graft_entry__.build()
    if args.workload == "al256":
        return main_al256(args)
    from dftpy_gb300 import batch, systems
    seeds_all = list(range(args.n))
    idx, _ = batch.shard([systems.config_alloy(s) for s in seeds_all], rank, world)
    seeds = [seeds_all[i] for i in idx]
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    jobs = alloy_jobs(seeds)
    guess = load_guess(ALLOY_WEIGHTS) if args.guess == "learned" else None
    clocks = ClockSampler(local)
    clocks.start()
    times, res, launches = timed_batches(jobs, args.precision, guess, args.steps, args.warmup, flush, world,
                                         args.workers)
    clk = clocks.stop()
    t_step = max_over_ranks(statistics.mean(times), world)
    nat = [systems.config_alloy(s).nat for s in seeds]
    energies = [float(r.energy) for r in res]
    uni = None
    if guess is not None:
        ut, ures, _ = timed_batches(jobs, args.precision, None, max(1, min(args.steps, 2)), 1, flush, world,
                                    args.workers)
        uni = {"value": max_over_ranks(statistics.mean(ut), world), "evaluations": sum(n_evals(r) for r in ures),
               "converged": sum(r.converged == 0 for r in ures)}
    plain = None
    e_plain = None
    if not args.no_plain:
        pt, pres, _ = timed_batches(jobs, "fp64", None, 1, 0, flush, world, args.workers)
        e_plain = [float(r.energy) for r in pres]
        plain = {"value": max_over_ranks(pt[0], world), "evaluations": sum(n_evals(r) for r in pres),
                 "converged": sum(r.converged == 0 for r in pres), "guess": "uniform",
                 "method": "FP64 TN, unpreconditioned inner CG, the reference's line search (its method)"}
        # the same FP64 solves with the mixed path's preconditioner: how much of
        # the speed-up is the preconditioner and how much the precision split
        qt, qres, _ = timed_batches(jobs, "fp64", None, 1, 0, flush, world, args.workers, {"precond": True})
        plain["fp64_preconditioned"] = {"value": max_over_ranks(qt[0], world),
                                        "evaluations": sum(n_evals(r) for r in qres),
                                        "converged": sum(r.converged == 0 for r in qres)}
    acc = {"tolerance_ev_per_atom": TOL_EV_PER_ATOM}
    if e_plain is not None:
        err = [abs(a - b) * HA_EV / n for a, b, n in zip(energies, e_plain, nat)]
        acc.update(max_err_ev_per_atom_vs_plain_fp64=max(err), ok=max(err) <= TOL_EV_PER_ATOM,
                   n_within=sum(e <= TOL_EV_PER_ATOM for e in err))
    fix = oracle_fixture()
    if fix is not None:
        eo = {int(s): float(e) for s, e in zip(fix["seed"], fix["energy"])}
        err_o = [abs(a - eo[s]) * HA_EV / n for a, s, n in zip(energies, seeds, nat) if s in eo]
        if err_o:
            acc["max_err_ev_per_atom_vs_cpu_oracle"] = max(err_o)
    # the evaluation the batch spends its time in, in isolation (128^3 snapshot)
    roof_wgc = None
    j128 = [j for j in jobs if tuple(int(x) for x in j[1].grid.nrR) == (128, 128, 128)]
    if j128:
        t_w = eval_roofline_wgc(*j128[0])
        # s N (R + W + 2 F): R = 2 (rho, v_loc), W = 1, F = 16 transforms (vW 2, Hartree 2, WGC 6 + 6: the
        # WGC term has no reference, so this is this implementation's own count)
        b_w = 4 * 128 ** 3 * (2 + 1 + 2 * 16)
        peak_w, _ = measured_peaks()
        roof_wgc = {"t_eval_us": t_w * 1e6, "grid": [128, 128, 128], "algorithmic_bytes": b_w,
                    "achieved_gbs": b_w / t_w / 1e9, "frac": b_w / t_w / 1e9 / peak_w,
                    "functional": "TF+vW+WGC+LDA+Hartree+PP, FP32 potential only, isolated loop (one stream)"}
    e2e_v, h2d, d2h, _ = e2e_batch(seeds, jobs, args.precision, guess, args.workers, 1 if args.steps < 2 else 2, 1)
    al = None
    live, t_iso, b_eval = (0.0, 0), None, None
    if not args.no_al256 and rank == 0:
        al, tot256, rho256 = al256_section(flush, 3, 2, not args.no_plain)
        live = al.pop("live_eval")
        t_iso, b_eval = eval_roofline(tot256, rho256)
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu and fix is not None:
        v, nshape, t_samp = cpu_baseline_1core(seeds, fix)
        cpu = {"value": v, "unit": "s", "cores": 1, "kind": "port",
               "sample": "one E+V and one V-only numpy-oracle evaluation of one snapshot per grid shape (%d "
                         "shapes, %.1f s), 1 thread; each of the %d snapshots' solves = its shape's times x "
                         "its evaluation counts in the oracle's own full solve; the solves one after another"
                         % (nshape, t_samp, len(seeds))}
    if rank != 0:
        if world > 1:
            import torch.distributed as dist
            dist.barrier()
            dist.destroy_process_group()
        return 0
    peak, peak_kind = measured_peaks()
    roofline = None
    if b_eval is not None:
        t_eval = live[0] / live[1] if live[1] else t_iso
        achieved = b_eval / t_eval / 1e9
        traffic = profile_traffic()
        roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                    "peak_kind": peak_kind, "traffic": traffic.get("bytes_per_eval") if traffic else None,
                    "kernel": "FP32 potential evaluation (rows / plane-convolution / rows pipeline), 128^3, "
                              "WT + LDA + Hartree + PP",
                    "t_eval_us": t_eval * 1e6, "n_evals_timed": live[1],
                    "timing": "CUDA events around each FP32 potential evaluation inside the al256 timed solves "
                              "(one stream)", "t_eval_isolated_us": t_iso * 1e6, "algorithmic_bytes": b_eval,
                    "batch_functional_eval": roof_wgc}
    n_conv = sum(r.converged == 0 for r in res)
    line = {
        "metric": METRIC, "value": t_step, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": t_step * 1000.0, "higher_is_better": False, "scaling": "strong",
        "vs_baseline": None, "dtype": {"mixed": "f32+f64", "fp64": "f64", "fp32": "f32"}[args.precision],
        "data": "synthetic (seeded Al/Mg alloy snapshots; starting densities from the guess network trained on "
                "the solver's own converged densities of other seeds)" if guess is not None else
                "synthetic (seeded Al/Mg alloy snapshots, uniform initial density)",
        "config": {"workload": "alloy64_wgc", "structures": len(seeds_all), "structures_this_rank": len(seeds),
                   "natoms_range": [min(nat), max(nat)], "grids": sorted({tuple(j[1].grid.nrR) for j in jobs}),
                   "functional": "TF+vW+WGC(second order)+LDA+Hartree+analytic PP (PME order 10)",
                   "method": "TN econv 1e-8 Ha/atom, maxfun 50", "precision": args.precision,
                   "guess": ("learned (BF16 tcgen05 network dftpy_gb300/data/guessnet.npz, 1.5 M parameters on "
                             "4x pooled features; inference and its fallback check inside the step)")
                            if guess is not None else "uniform",
                   "in_flight": args.workers, "l2": "512 MB buffer written between timed steps",
                   "sharding": "longest-processing-time on grid points over ranks"},
        "converged": n_conv,
        "evaluations": sum(n_evals(r) for r in res),
        "accuracy": acc,
        "plain_fp64": plain,
        "speedup_vs_plain": (plain["value"] / t_step) if plain else None,
        "mixed_uniform_guess": uni,
        "al256": al,
        "roofline": roofline,
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_v, "unit": "s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": launches,
        "clocks": clk,
    }
    print(json.dumps(line, default=_plain), flush=True)
    if world > 1:
        import torch.distributed as dist
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
