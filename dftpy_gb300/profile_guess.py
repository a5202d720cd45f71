"""Repeat the learned guess of the 256-atom / 128^3 WT workload, or one of
its convolution layers, for profiling.

``python -m dftpy_gb300.profile_guess --conv 16,16,128 --reps 3`` runs the
tensor-core convolution C_in -> C_out on an n^3 grid (SiLU fused) ``reps``
times after two warm-up calls and prints the CUDA-event time per call;
``python -m dftpy_gb300.profile_guess`` computes the learned guess (features,
network, normalisation, the fallback's two residuals) after two warm-up
guesses, once inside an NVTX range named ``guess`` (select it with ``--nvtx
--nvtx-include guess/``), then times its parts one by one
(``--workload alloy --seed S``: the alloy network on one snapshot of the
batched workload).
"""
import argparse
import os


def main():
    p = argparse.ArgumentParser()
    p.add_argument("--conv", default=None, help="C_in,C_out,n: time one tensor-core layer on an n^3 grid")
    p.add_argument("--up", action="store_true", help="with --conv: the input is the n/2 grid, read upsampled")
    p.add_argument("--reps", type=int, default=3)
    p.add_argument("--workload", default="al256", choices=["al256", "alloy"],
                   help="al256: the WT network on the 256-atom cell; alloy: the alloy network on one snapshot")
    p.add_argument("--seed", type=int, default=0, help="alloy snapshot seed")
    p.add_argument("--net", default=None, help="network file (default: the workload's committed network)")
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
    here = os.path.dirname(os.path.abspath(__file__))
    if a.workload == "alloy":
        st = systems.config_alloy(a.seed)
        total, rho_u = build_evaluator(st, kedf="WGC")
        net = a.net or os.path.join(here, "data", "guessnet.npz")
    else:
        st = systems.config_al256(0)
        total, rho_u = build_evaluator(st, kedf="WT")
        net = a.net or os.path.join(here, "data", "guessnet_al_wt.npz")
    lg = G.LearnedGuess(G.GuessNet.load(net))
    grid = rho_u.grid
    for _ in range(2):
        lg.guess(total, grid)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("guess")
    e0.record()
    g = lg.guess(total, grid)
    e1.record()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    # the parts of one guess, each timed alone
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
    ev[0].record()
    x, phib, rho0 = G.features(total, grid)
    ev[1].record()
    out = lg.net.forward(x)
    ev[2].record()
    r1 = G.residual(total, g)
    ev[3].record()
    r2 = G.uniform_residual(total, grid)
    ev[4].record()
    torch.cuda.synchronize()
    parts = [ev[i].elapsed_time(ev[i + 1]) for i in range(4)]
    print("learned guess %s %s: %.3f ms (choice %s), integral %.6f; features %.3f ms, network %.3f ms, "
          "residual of the guess %.3f ms, of the uniform density (from v_loc) %.3f ms (residuals %.3e / %.3e)"
          % (a.workload, "x".join(str(int(n)) for n in grid.nrR), e0.elapsed_time(e1), lg.last_choice,
             float(g.as_subclass(torch.Tensor).sum()) * grid.dV, *parts, r1, r2))


if __name__ == "__main__":
    main()
