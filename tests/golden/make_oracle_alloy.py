"""Oracle solves of the 64 Al/Mg alloy snapshots (the batched WGC workload).

Run from the repository root:
``python tests/golden/make_oracle_alloy.py [--workers 7] [--cache DIR] [--n 64]``

The reference has no WGC functional, so these fixtures come from the numpy
oracle (``oracle/ofdft.py`` + ``oracle/wgc.py``), not from the reference
itself: for every snapshot ``systems.config_alloy(seed)``, seed 0..63, the
oracle's restatement of the reference TN (``optimization.py:281-520``, the
unpreconditioned inner CG and the Moré-Thuente line search) minimises
TF + vW + WGC + LDA + Hartree + analytic PP (PME) from the uniform density to
econv = 1e-8 Ha/atom x nat.  Each solve runs in its own process on one core.

alloy64_oracle.npz holds, per seed: grid, atom count, the converged energy,
the number of E+V and V-only evaluations, TN iterations, the convergence flag
and the single-core wall time of the solve in the container that ran this
script (``host``).  The GPU tests compare the batch's energies with these; the
benchmark's CPU arm uses the evaluation counts.
"""
import argparse
import multiprocessing as mp
import os
import pathlib
import platform
import sys
import time

import numpy as np

HERE = pathlib.Path(__file__).resolve().parent
ROOT = HERE.parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

ECONV_PER_ATOM = 1e-8


def wgc_evaluator(st):
    """(evaluator, grid) of TF + vW + WGC + LDA + Hartree + PP for ``st``;
    the evaluator counts its E+V and V-only calls."""
    from oracle import ofdft as O
    from oracle import wgc as W
    base = O.OFDFT(st.lattice, st.nr, st.positions, st.symbols, kedf="TFVW")
    nl = W.WGCNL()
    g = base.grid
    count = {"EV": 0, "V": 0}

    def evaluator(rho, calc_e):
        count["EV" if calc_e else "V"] += 1
        e, v = base(rho, calc_e)
        e2, v2 = nl(rho, g, calc_e)
        return (None if e is None else e + e2), v + v2
    return evaluator, g, count


def solve_one(args):
    seed, cache = args
    out = os.path.join(cache, "alloy_%03d.npz" % seed)
    if os.path.exists(out):
        return seed
    from dftpy_gb300 import systems
    from oracle import ofdft as O
    st = systems.config_alloy(seed)
    t0 = time.perf_counter()
    ev, g, count = wgc_evaluator(st)
    t1 = time.perf_counter()
    rho0 = np.full(st.nr, st.nelec / st.volume)
    r = O.optimize_tn(ev, rho0, g, econv=ECONV_PER_ATOM * st.nat, maxfun=50, maxiter=100)
    t2 = time.perf_counter()
    np.savez(out + ".tmp.npz", seed=seed, nr=np.array(st.nr), nat=st.nat, energy=r["energy"], n_ev=count["EV"],
             n_v=count["V"], n_iter=r["n_iter"], converged=r["converged"], t_solve=t2 - t1, t_setup=t1 - t0)
    os.replace(out + ".tmp.npz", out)
    return seed


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--n", type=int, default=64)
    p.add_argument("--workers", type=int, default=max(1, (os.cpu_count() or 2) - 1))
    p.add_argument("--cache", default="/tmp/gbofdft_alloy_oracle")
    a = p.parse_args()
    os.makedirs(a.cache, exist_ok=True)
    from dftpy_gb300 import systems
    seeds = list(range(a.n))
    # largest grids first (longest-processing-time order)
    seeds.sort(key=lambda s: -int(np.prod(systems.config_alloy(s).nr)))
    ctx = mp.get_context("spawn")
    with ctx.Pool(a.workers) as pool:
        for s in pool.imap_unordered(solve_one, [(s, a.cache) for s in seeds]):
            print("done", s, flush=True)
    rows = [np.load(os.path.join(a.cache, "alloy_%03d.npz" % s)) for s in range(a.n)]
    keys = ["seed", "nr", "nat", "energy", "n_ev", "n_v", "n_iter", "converged", "t_solve", "t_setup"]
    data = {k: np.array([r[k] for r in rows]) for k in keys}
    data["econv_per_atom"] = ECONV_PER_ATOM
    data["host"] = "%s, %d cores, numpy %s" % (platform.machine(), os.cpu_count() or 0, np.__version__)
    np.savez(HERE / "alloy64_oracle.npz", **data)
    print("wrote", HERE / "alloy64_oracle.npz", "total single-core solve time %.0f s" % data["t_solve"].sum())


if __name__ == "__main__":
    main()
