"""Many structures optimised together on one GPU.

The reference optimises one structure per process.  Here a batch of
independent structures (uneven cells and grids) shares the GPU: each
structure gets its own grid, plans, workspaces and CUDA stream, and a pool of
host threads drives the solves concurrently -- the truncated-Newton driver is
native code that releases the interpreter while it runs, so one thread per
in-flight structure keeps that many streams busy and small grids fill the
device together.  Results do not depend on the concurrency: every structure's
arithmetic is the same as in a solve on its own.

``optimize_batch(jobs, workers)`` takes ``(EnergyEvaluator, guess_rho)``
pairs (or ``systems.Structure`` objects, for which the evaluator and a uniform
guess are built here) and returns one ``BatchResult`` per job, in order.
"""
import concurrent.futures as cf
import threading
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from . import _lib, systems
from . import functional as F
from .field import DirectField
from .grid import DirectGrid
from .ions import Ions
from .optimization import Optimization

# energy tolerance per atom (Ha): 1e-8 Ha/atom, well inside the 1e-5 eV/atom
# (3.7e-7 Ha/atom) accuracy the mixed-precision solves are held to
DEFAULT_OPTIONS = {"econv_per_atom": 1e-8, "maxfun": 50, "maxiter": 100, "precision": "mixed"}

# worker streams, kept from batch to batch: PyTorch's caching allocator
# reuses a freed block only on the stream it was allocated on, so new streams
# per batch would leave every earlier batch's blocks reserved and unused
_STREAMS = {}
_STREAMS_LOCK = threading.Lock()


def worker_streams(n):
    """``n`` CUDA streams of the current device, the same ones on every call."""
    dev = torch.cuda.current_device()
    with _STREAMS_LOCK:
        pool = _STREAMS.setdefault(dev, [])
        while len(pool) < n:
            pool.append(torch.cuda.Stream(device=dev))
        return pool[:n]


@dataclass
class BatchResult:
    rho: object
    energy: float
    converged: int
    stats: dict
    wall_s: float
    name: str = ""
    extra: dict = field(default_factory=dict)


def build_evaluator(st, kedf="WGC", pme=True, full=False, **kedf_options):
    """TotalFunctional (KEDF + LDA + Hartree + analytic local PP) and a
    uniform guess density for a ``systems.Structure``."""
    grid = DirectGrid(st.lattice, st.nr, full=full)
    ions = Ions(st.symbols, positions=st.positions, cell=st.lattice)
    pp = {s: F.AnalyticPP(*systems.SPECIES[s]) for s in set(st.symbols)}
    ps = F.LocalPseudo(grid=grid, ions=ions, PP_list=pp, PME=pme)
    total = F.TotalFunctional(KineticEnergyFunctional=F.Functional(type="KEDF", name=kedf, **kedf_options),
                              XCFunctional=F.Functional(type="XC", name="LDA"),
                              HARTREE=F.Functional(type="HARTREE"), PSEUDO=ps)
    rho0 = DirectField(grid)
    rho0[:] = st.nelec / st.volume
    return total, rho0


def _natoms(total):
    for f in total.funcDict.values():
        if getattr(f, "type", None) == "PSEUDO":
            return f.ions.nat
    return 1


def _solve_one(job, options, stream, guess=None):
    total, rho0, name = job
    t0 = time.perf_counter()
    o = dict(options)
    per_atom = o.pop("econv_per_atom", None)
    if "econv" not in o:
        o["econv"] = per_atom * _natoms(total)
    extra = {}
    with torch.cuda.stream(stream):
        start = rho0
        if guess is not None:
            # the guess's residual check is left to the optimiser's first
            # evaluation (no evaluation of its own); a rejected guess starts
            # the solve again from the job's density
            start = guess.guess(total, rho0.grid, defer_check=True)
            lim = getattr(start, "start_residual_max", None)
            if lim:
                o["start_residual_max"] = float(lim)
        opt = Optimization(EnergyEvaluator=total, optimization_method="TN", optimization_options=o)
        rho = opt.optimize_rho(guess_rho=start)
        if opt.converged == 3:
            rejected = opt.stats
            o["start_residual_max"] = 0.0
            opt = Optimization(EnergyEvaluator=total, optimization_method="TN", optimization_options=o)
            rho = opt.optimize_rho(guess_rho=rho0)
            opt.stats["stages"] = rejected["stages"] + opt.stats["stages"]
            extra["guess_rejected"] = True
        energy = float(opt.energy)
        stream.synchronize()
    return BatchResult(rho=rho, energy=energy, converged=int(opt.converged), stats=opt.stats,
                       wall_s=time.perf_counter() - t0, name=name, extra=extra)


def optimize_batch(jobs, workers=None, options=None, kedf="WGC", guess=None, **kedf_options):
    """Optimise every job; ``workers`` structures are in flight at a time
    (default: all of them, at most 6 -- on the 64-snapshot alloy batch 6
    streams beat 16 by 3 %: fewer structures' spectra compete for L2, and six
    already hide each other's host synchronisations).  Jobs are ``(evaluator, guess_rho)``
    pairs or ``systems.Structure`` objects.  ``guess``: a
    ``guess.LearnedGuess`` whose starting density replaces each job's (made
    on the job's stream)."""
    _lib.require_cuda()
    opts = dict(DEFAULT_OPTIONS)
    opts.update(options or {})
    prepared = []
    for j in jobs:
        if isinstance(j, systems.Structure):
            total, rho0 = build_evaluator(j, kedf=kedf, **kedf_options)
            prepared.append((total, rho0, j.name))
        else:
            total, rho0 = j
            prepared.append((total, rho0, ""))
    if not prepared:
        return []
    n = len(prepared)
    workers = min(n, 6) if workers is None else max(1, min(int(workers), n))
    streams = worker_streams(workers)
    slots = list(range(workers))
    lock = threading.Lock()
    if guess is not None:
        # the network's packed weights and the per-grid-shape feature tables
        # are made here, once per grid shape, not by racing worker threads
        shapes = {}
        for total, rho0, _ in prepared:
            shapes.setdefault(tuple(int(x) for x in rho0.grid.nrR), (total, rho0.grid))
        for total, grid in shapes.values():
            guess.prepare(total, grid)
    # set-up work queued on the default stream (device copies of the inputs)
    # must be complete before other streams read it
    torch.cuda.synchronize()

    def run(job):
        with lock:
            k = slots.pop()
        try:
            return _solve_one(job, opts, streams[k], guess)
        finally:
            with lock:
                slots.append(k)

    with cf.ThreadPoolExecutor(max_workers=workers) as ex:
        results = list(ex.map(run, prepared))
    return results


def alloy_batch(n=64, seed0=0, **kw):
    """The batched workload: ``n`` Al/Mg alloy snapshots (``systems.config_alloy``)."""
    return [systems.config_alloy(seed0 + i, **kw) for i in range(n)]


def structure_cost(st):
    """Work estimate of one structure's solve: its number of grid points."""
    return int(np.prod(st.nr))


def partition_lpt(costs, nparts):
    """Longest-processing-time assignment of independent items to ``nparts``
    ranks: items in decreasing cost (ties by index), each to the rank with
    the smallest load so far (ties to the lower rank).  Deterministic, so
    every rank computes the same partition without communicating.  Returns
    (parts, loads): per rank the item indices in increasing order, and its
    total cost.  The largest load is at most 4/3 of the optimum."""
    nparts = int(nparts)
    if nparts < 1:
        raise ValueError("nparts must be >= 1")
    costs = [float(c) for c in costs]
    if any(c < 0 for c in costs):
        raise ValueError("costs must be non-negative")
    order = sorted(range(len(costs)), key=lambda i: (-costs[i], i))
    parts = [[] for _ in range(nparts)]
    loads = [0.0] * nparts
    for i in order:
        k = min(range(nparts), key=lambda r: (loads[r], r))
        parts[k].append(i)
        loads[k] += costs[i]
    return [sorted(p) for p in parts], loads


def shard(structures, rank, world, cost=structure_cost):
    """The structures rank ``rank`` of ``world`` optimises (``partition_lpt``
    on ``cost``), with their indices in the batch.  Structures are
    independent, so ranks need no collective on the data path; results are
    gathered by index on the host."""
    parts, _ = partition_lpt([cost(s) for s in structures], world)
    idx = parts[int(rank)]
    return idx, [structures[i] for i in idx]


def main():
    import argparse
    import json
    p = argparse.ArgumentParser(description="batched optimisation of Al/Mg alloy snapshots")
    p.add_argument("--n", type=int, default=64)
    p.add_argument("--workers", type=int, default=16)
    p.add_argument("--kedf", default="WGC")
    p.add_argument("--precision", default="mixed")
    p.add_argument("--sequential", type=int, default=8, help="also time this many jobs one after another")
    p.add_argument("--check", type=int, default=4, help="solve this many in plain FP64 and report the error")
    p.add_argument("--guess", default="uniform", choices=["uniform", "learned"],
                   help="starting densities (learned: data/guessnet.npz, trained on Al/Mg WGC cells)")
    a = p.parse_args()
    sts = alloy_batch(a.n)
    opts = {"precision": a.precision}
    lg = None
    if a.guess == "learned":
        import os
        from .guess import GuessNet, LearnedGuess
        lg = LearnedGuess(GuessNet.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                                                     "guessnet.npz")))
    # warm-up: one small solve per distinct grid (plans, tables, kernels)
    seen = set()
    warm = []
    for st in sts:
        if st.nr not in seen:
            seen.add(st.nr)
            warm.append(st)
    optimize_batch(warm, workers=len(warm), options=opts, kedf=a.kedf, guess=lg)
    jobs = [build_evaluator(st, kedf=a.kedf) for st in sts]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    res = optimize_batch(jobs, workers=a.workers, options=opts, guess=lg)
    torch.cuda.synchronize()
    t_batch = time.perf_counter() - t0
    seq = None
    if a.sequential:
        jobs2 = [build_evaluator(st, kedf=a.kedf) for st in sts[:a.sequential]]
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        res2 = optimize_batch(jobs2, workers=1, options=opts, guess=lg)
        t_seq = time.perf_counter() - t1
        same = all(r.energy == q.energy for r, q in zip(res2, res[:a.sequential]))
        seq = {"n": a.sequential, "wall_s": t_seq, "per_structure_s": t_seq / a.sequential,
               "energies_identical_to_batch": same}
    check = None
    if a.check:
        ref = optimize_batch(sts[:a.check], workers=a.check, options={"precision": "fp64"}, kedf=a.kedf)
        err = [abs(r.energy - q.energy) / st.nat * 27.211386024367243 for r, q, st in zip(res, ref, sts)]
        check = {"n": a.check, "max_abs_dE_eV_per_atom": max(err), "fp64_converged": sum(q.converged == 0 for q in ref)}
    print(json.dumps({"n": a.n, "workers": a.workers, "kedf": a.kedf, "precision": a.precision, "guess": a.guess,
                      "evaluations": sum(sum(s_["n_eval_ev"] + s_["n_eval_v"] + s_.get("n_eval_hess", 0)
                                             for s_ in r.stats["stages"]) for r in res),
                      "wall_s": t_batch, "structures_per_s": a.n / t_batch,
                      "converged": sum(1 for r in res if r.converged == 0),
                      "natoms": [len(st.symbols) for st in sts], "grids": sorted({st.nr for st in sts}),
                      "sequential": seq, "vs_fp64": check}))


if __name__ == "__main__":
    main()
