"""Repeat the learned guess of the 256-atom / 128^3 WT workload, or one of
its convolution layers, for profiling.

``python -m dftpy_gb300.profile_guess --conv 16,16,128 --reps 3`` runs the
tensor-core convolution C_in -> C_out on an n^3 grid (SiLU fused) ``reps``
times after two warm-up calls and prints the CUDA-event time per call;
``python -m dftpy_gb300.profile_guess`` computes the learned guess (features,
network, normalisation) after two warm-up guesses, once inside an NVTX
range named ``guess`` (select it with ``--nvtx --nvtx-include guess/``).
"""
import argparse
import os


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--conv", default=None, help="C_in,C_out,n: time one tensor-core layer on an n^3 grid")
    p.add_argument("--up", action="store_true", help="with --conv: the input is the n/2 grid, read upsampled")
    p.add_argument("--reps", type=int, default=3)
    a = p.parse_args()
    import numpy as np
    import torch
    from . import guess as G
    if a.conv:
        cin, cout, n = (int(v) for v in a.conv.split(","))
        rng = np.random.default_rng(0)
        layer = G.Conv(cin, cout, rng)
        sh = (n, n, n)
        ish = tuple(s // 2 for s in sh) if a.up else sh
        x = torch.randn((cin,) + ish, device="cuda")
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        for _ in range(2):
            layer.forward_tc(x, sh, True, err, up=a.up)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(a.reps):
            layer.forward_tc(x, sh, True, err, up=a.up)
        e1.record()
        torch.cuda.synchronize()
        t = e0.elapsed_time(e1) / a.reps * 1e-3
        flop = 2.0 * 27 * cin * cout * n ** 3
        print("conv %d -> %d on %d^3%s: %.1f us per call, %.1f TFLOP/s, error flag %d"
              % (cin, cout, n, " (upsampled input)" if a.up else "", t * 1e6, flop / t / 1e12, int(err.item())))
        return
    from . import systems
    from .batch import build_evaluator
    st = systems.config_al256(0)
    total, rho_u = build_evaluator(st, kedf="WT")
    here = os.path.dirname(os.path.abspath(__file__))
    lg = G.LearnedGuess(G.GuessNet.load(os.path.join(here, "data", "guessnet_al_wt.npz")))
    for _ in range(2):
        lg.guess(total, rho_u.grid)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("guess")
    e0.record()
    g = lg.guess(total, rho_u.grid)
    e1.record()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    print("learned guess al256 128^3: %.3f ms, integral %.6f" % (e0.elapsed_time(e1),
                                                                 float(g.as_subclass(torch.Tensor).sum()) * rho_u.grid.dV))


if __name__ == "__main__":
    main()
