"""The learned-guess network kernels against the numpy oracle (FP64, the
same BF16-rounded weights), whole-network gradients against finite
differences of the oracle's loss, and the trained network's gain."""
import os

import numpy as np
import pytest

from oracle import guessnet as G

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gn():
    from dftpy_gb300 import _lib
    _lib.require_cuda()
    from dftpy_gb300 import guess
    return guess


def _bf16_round(a):
    import torch
    return torch.tensor(a, dtype=torch.float32).to(torch.bfloat16).to(torch.float64).numpy()


@pytest.mark.parametrize("shape,cin,cout", [((4, 6, 8), 3, 37), ((8, 8, 8), 16, 32), ((2, 4, 2), 5, 1),
                                             ((16, 32, 160), 3, 37)])
def test_conv_kernels(gn, shape, cin, cout):
    """The CUDA-core convolution against the oracle: small grids run one CTA
    per (channel, 64 voxels) with the input channels split over four thread
    groups (``k_conv3d_ks``), the 81920-voxel grid the voxel-tile kernel
    (``k_conv3d``)."""
    import torch
    rng = np.random.default_rng(2)
    layer = gn.Conv(cin, cout, rng)
    layer.b.copy_(torch.tensor(rng.standard_normal(cout), dtype=torch.float32))
    x = rng.standard_normal((cin,) + shape).astype(np.float32)
    g = rng.standard_normal((cout,) + shape).astype(np.float32)
    xd = torch.tensor(x, device="cuda")
    gd = torch.tensor(g, device="cuda")
    w = _bf16_round(layer.w.cpu().numpy())
    b = layer.b.cpu().numpy().astype(np.float64)
    y = layer.forward(xd, shape).cpu().numpy()
    yr = G.conv3d(x.astype(np.float64), w, b)
    assert np.abs(y - yr).max() <= 1e-5 * np.abs(yr).max()
    gx = layer.backward(xd, gd, shape).cpu().numpy()
    gxr = G.conv3d_input_grad(g.astype(np.float64), w)
    assert np.abs(gx - gxr).max() <= 1e-5 * np.abs(gxr).max()
    gwr, gbr = G.conv3d_weight_grad(x.astype(np.float64), g.astype(np.float64))
    assert np.abs(layer.gw.cpu().numpy() - gwr).max() <= 1e-5 * np.abs(gwr).max()
    assert np.abs(layer.gb.cpu().numpy() - gbr).max() <= 1e-5 * np.abs(gbr).max()


@pytest.mark.parametrize("cin,cout", [(16, 16), (32, 48), (48, 64), (64, 64), (64, 48), (16, 1)])
@pytest.mark.parametrize("act", [0, 1])
def test_conv_tensor_core(gn, cin, cout, act):
    """tcgen05 convolution (BF16 activations and weights, FP32 accumulation)
    against the oracle on the same BF16-rounded operands: within 2e-5 of
    max |y|.  (3, 32, 24): odd depth, two y tiles, three x tiles, periodic
    wrap in every direction; (64, 64) and (64, 48) stream the weights in
    three slabs; (16, 1), the head, runs 16 wide with zero weights and
    stores one channel."""
    import torch
    from dftpy_gb300 import _lib
    shape = (3, 32, 24)
    rng = np.random.default_rng(7)
    layer = gn.Conv(cin, cout, rng)
    layer.b.copy_(torch.tensor(rng.standard_normal(cout), dtype=torch.float32))
    assert layer.tc_supported(shape)
    x = rng.standard_normal((cin,) + shape).astype(np.float32)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    y = layer.forward_tc(torch.tensor(x, device="cuda"), shape, act, err).cpu().numpy()
    assert int(err.item()) == 0
    w = _bf16_round(layer.w.cpu().numpy())
    b = layer.b.cpu().numpy().astype(np.float64)
    yr = G.conv3d(_bf16_round(x), w, b)
    if act:
        yr = G.silu(yr)
    assert np.abs(y - yr).max() <= 2e-5 * np.abs(yr).max()
    # shapes without a kernel are reported, not run
    assert not layer.tc_supported((3, 8, 24)) and not layer.tc_supported((3, 32, 12))
    assert not _lib.load().gbofdft_nn_conv3d_tc_supported(2, 16, 4, 16, 16)


@pytest.mark.parametrize("cin,cout,shape", [(48, 32, (4, 32, 16)), (32, 16, (6, 32, 16)), (16, 32, (2, 16, 8))])
def test_conv_tensor_core_fused_up_skip(gn, cin, cout, shape):
    """The decoder form: input read as the 2x nearest upsampling of a
    half-size grid, SiLU, then a skip tensor added, against the oracle's
    up2 -> conv -> silu -> add on the same BF16-rounded operands.  (48, 32)
    streams its weights per tile; (32, 16) and (16, 32) keep them and walk
    columns of tiles along z (one and several planes per CTA)."""
    import torch
    rng = np.random.default_rng(8)
    layer = gn.Conv(cin, cout, rng)
    layer.b.copy_(torch.tensor(rng.standard_normal(cout), dtype=torch.float32))
    xc = rng.standard_normal((cin,) + tuple(s // 2 for s in shape)).astype(np.float32)
    sk = rng.standard_normal((cout,) + shape).astype(np.float32)
    err = torch.zeros(1, dtype=torch.int32, device="cuda")
    y = layer.forward_tc(torch.tensor(xc, device="cuda"), shape, True, err, skip=torch.tensor(sk, device="cuda"),
                         up=True).cpu().numpy()
    assert int(err.item()) == 0
    w = _bf16_round(layer.w.cpu().numpy())
    b = layer.b.cpu().numpy().astype(np.float64)
    yr = G.silu(G.conv3d(G.up2(_bf16_round(xc)), w, b)) + sk
    assert np.abs(y - yr).max() <= 2e-5 * np.abs(yr).max()


def test_network_inference_tensor_cores(gn):
    """The tensor-core inference path of the whole network against the FP32
    CUDA-core forward: BF16 activations move the output by < 2 % of its
    range."""
    import torch
    net = gn.GuessNet(channels=(16, 32, 48, 64), seed=3)
    rng = np.random.default_rng(4)
    x = torch.tensor(rng.standard_normal((2, 16, 32, 16)).astype(np.float32), device="cuda")
    ref = net.forward(x, keep=True).cpu().numpy()
    net._tape = None
    fast = net.forward(x).cpu().numpy()
    slow = net.forward(x, tc=False).cpu().numpy()
    np.testing.assert_allclose(slow, ref, rtol=0, atol=1e-5 * np.abs(ref).max())
    assert np.abs(fast - ref).max() <= 2e-2 * (np.abs(ref).max() + 1e-30)


def test_pointwise_kernels(gn):
    import torch
    rng = np.random.default_rng(3)
    x = rng.standard_normal((3, 4, 6, 8)).astype(np.float32)
    c = rng.standard_normal((3, 2, 3, 4)).astype(np.float32)
    xd, cd = torch.tensor(x, device="cuda"), torch.tensor(c, device="cuda")
    np.testing.assert_allclose(gn.silu(xd).cpu().numpy(), G.silu(x.astype(np.float64)), rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(gn.silu_bwd(xd, xd).cpu().numpy(), x * G.silu_grad(x.astype(np.float64)),
                               rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(gn.pool2(xd).cpu().numpy(), G.pool2(x), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(gn.pool2_bwd(cd, (4, 6, 8)).cpu().numpy(), G.pool2_adjoint(c), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(gn.up2(cd).cpu().numpy(), G.up2(c), rtol=0, atol=0)
    np.testing.assert_allclose(gn.up2_bwd(xd).cpu().numpy(), G.up2_adjoint(x), rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(gn.uplin(cd).cpu().numpy(), G.uplin(c.astype(np.float64)), rtol=1e-6, atol=1e-6)
    np.testing.assert_allclose(gn.uplin_bwd(xd).cpu().numpy(), G.uplin_adjoint(x.astype(np.float64)), rtol=1e-5,
                               atol=1e-5)


def _oracle_weights(net):
    def wb(l):
        return _bf16_round(l.w.cpu().numpy()), l.b.cpu().numpy().astype(np.float64)
    enc = [wb(a) + wb(b) for a, b in net.enc]
    dec = [wb(a) + wb(b) for a, b in net.dec]
    return enc, dec, wb(net.head)


def test_network_forward_and_gradients(gn):
    """Forward equals the oracle's; the weight gradients of the loss
    sum(out * c) equal the oracle's central differences (FP64)."""
    import torch
    net = gn.GuessNet(channels=(4, 6, 8), seed=1)
    rng = np.random.default_rng(4)
    for l in net.layers:     # non-zero biases exercise every path
        l.b.copy_(torch.tensor(0.1 * rng.standard_normal(l.cout), dtype=torch.float32))
    x = rng.standard_normal((2, 8, 8, 12)).astype(np.float32)
    c = rng.standard_normal((1, 8, 8, 12)).astype(np.float32)
    out = net.forward(torch.tensor(x, device="cuda"), keep=True).cpu().numpy()
    enc, dec, head = _oracle_weights(net)
    ref = G.net_forward(x.astype(np.float64), enc, dec, head)
    assert np.abs(out - ref).max() <= 1e-4 * np.abs(ref).max()
    net.backward(torch.tensor(c, device="cuda"))
    e = 1e-4
    checks = [("enc", 0, 0, (1, 0, 13)), ("enc", 2, 2, (3, 5, 0)), ("dec", 0, 0, (2, 7, 26)), ("dec", 1, 2, (0, 3, 4)),
              ("head", 0, 0, (0, 2, 13))]
    for kind, lvl, which, idx in checks:
        if kind == "head":
            layer = net.head
        else:
            layer = (net.enc if kind == "enc" else net.dec)[lvl][which // 2]
        g_gpu = float(layer.gw.cpu().numpy()[idx])

        def loss(delta):
            enc2, dec2, head2 = _oracle_weights(net)
            if kind == "head":
                w = head2[0].copy()
                w[idx] += delta
                head2 = (w, head2[1])
            else:
                lst = enc2 if kind == "enc" else dec2
                t = list(lst[lvl])
                w = t[which].copy()
                w[idx] += delta
                t[which] = w
                lst[lvl] = tuple(t)
            return float((G.net_forward(x.astype(np.float64), enc2, dec2, head2) * c).sum())
        fd = (loss(e) - loss(-e)) / (2 * e)
        assert abs(g_gpu - fd) <= 2e-3 * max(1.0, abs(fd)), (kind, lvl, which, idx, g_gpu, fd)


def test_training_reduces_loss(gn):
    """A few Adam steps on one synthetic cell lower the normalised error."""
    import torch
    net = gn.GuessNet(channels=(4, 8), seed=0)
    rng = np.random.default_rng(5)
    x = torch.tensor(rng.standard_normal((2, 8, 8, 8)).astype(np.float32), device="cuda")
    phib = torch.full((8, 8, 8), 0.15, dtype=torch.float32, device="cuda")
    phit = (phib + 0.02 * x[0].tanh()).contiguous()
    hist = gn.train(net, [(x, phib, phit, 0.02)], epochs=60, lr=3e-3, lr_min=3e-4)
    assert hist[-1] < 0.5 * hist[0]


TRAINED = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "dftpy_gb300", "data",
                       "guessnet.npz")


@pytest.mark.skipif(not os.path.exists(TRAINED), reason="no trained network committed")
def test_trained_network_gain(gn):
    """On held-out Al/Mg cells (seeds outside the training set) the learned
    guess needs fewer TN evaluations than the uniform start and reaches the
    same energy (within 1e-5 eV/atom)."""
    net = gn.GuessNet.load(TRAINED)
    cells = [gn.training_cell(s) for s in (5000, 5001, 5002)]
    rows = gn.evaluate_guesses(net, cells)
    for r in rows:
        assert r["learned"]["converged"] == 0 and r["uniform"]["converged"] == 0
        assert abs(r["learned"]["energy"] - r["uniform"]["energy"]) / r["nat"] * 27.211386 < 1e-5
    assert sum(r["learned"]["evals"] for r in rows) < 0.8 * sum(r["uniform"]["evals"] for r in rows)


def test_al_network_gain_on_al256(gn):
    """The network trained on pure-Al 2x2x2 WT cells (the benchmark's
    functional) applied to the 256-atom 128^3 cell: from its guess the mixed
    TN needs fewer than 85 % of the evaluations it needs from the uniform
    density and ends at the same energy (1e-8 eV/atom: both stop within the
    1e-7 Ha energy tolerance of the same minimum)."""
    import torch
    from dftpy_gb300 import systems
    from dftpy_gb300.batch import build_evaluator
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    net = gn.GuessNet.load(os.path.join(here, "dftpy_gb300", "data", "guessnet_al_wt.npz"))
    st = systems.config_al256(0)
    total, rho_u = build_evaluator(st, kedf="WT")
    o_u, _ = gn._solve(total, rho_u, econv_per_atom=1e-7 / st.nat)
    g = gn.LearnedGuess(net).guess(total, rho_u.grid)
    assert abs(float(g.as_subclass(torch.Tensor).sum()) * rho_u.grid.dV - st.nelec) < 1e-8 * st.nelec
    o_l, _ = gn._solve(total, g, econv_per_atom=1e-7 / st.nat)
    n_u = sum(s["n_eval_ev"] + s["n_eval_v"] + s.get("n_eval_hess", 0) for s in o_u.stats["stages"])
    n_l = sum(s["n_eval_ev"] + s["n_eval_v"] + s.get("n_eval_hess", 0) for s in o_l.stats["stages"])
    assert n_l < 0.85 * n_u, (n_l, n_u)
    assert abs(o_l.energy - o_u.energy) / st.nat * 27.211386 < 1e-8


def test_fallback_to_uniform_when_the_network_is_worse(gn):
    """``LearnedGuess`` keeps the network's density when its FP32 residual is
    below the uniform density's and starts from the uniform density
    otherwise: the trained WT network on the 256-atom cell is kept, an
    untrained network (random weights, head scaled 50x) is replaced.
    ``residual`` equals a float64 numpy restatement of ||(V - mu) phi||, and
    ``uniform_residual`` (from v_loc alone) the evaluated one."""
    import torch
    from dftpy_gb300 import systems
    from dftpy_gb300.batch import build_evaluator
    here = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    st = systems.config_al256(0)
    total, rho_u = build_evaluator(st, kedf="WT")
    good = gn.LearnedGuess(gn.GuessNet.load(os.path.join(here, "dftpy_gb300", "data", "guessnet_al_wt.npz")))
    g = good.guess(total, rho_u.grid)
    assert good.last_choice == "network"
    r_net, r_uni = gn.residual(total, g), gn.residual(total, rho_u)
    assert r_net < r_uni
    # at the uniform density the potential is a constant plus v_loc
    assert abs(gn.uniform_residual(total, rho_u.grid) - r_uni) <= 1e-4 * r_uni
    v = total(g.to(torch.float32), calcType={"V"}).potential.as_subclass(torch.Tensor).double().cpu().numpy()
    r = g.as_subclass(torch.Tensor).float().double().cpu().numpy()
    mu = (v * r).sum() / r.sum()
    ref = np.sqrt(((v - mu) ** 2 * np.maximum(r, 0)).sum() * rho_u.grid.dV)
    assert abs(r_net - ref) <= 1e-9 * ref
    bad_net = gn.GuessNet(channels=(16, 32, 48, 64), seed=11)
    bad_net.head.w.mul_(50.0)
    bad_net.head.sync_bf16()
    bad = gn.LearnedGuess(bad_net)
    b = bad.guess(total, rho_u.grid)
    assert bad.last_choice == "uniform"
    # a ratio below the network's own residual ratio rejects even the good guess
    strict = gn.LearnedGuess(good.net, fallback_ratio=0.5 * r_net / r_uni)
    strict.guess(total, rho_u.grid)
    assert strict.last_choice == "uniform"
    assert torch.allclose(b.as_subclass(torch.Tensor), rho_u.as_subclass(torch.Tensor).to(b.dtype), rtol=1e-13,
                          atol=0.0)


def test_tensor_core_training_matches_fp32(gn):
    """Training on the tensor cores (forward and input-gradient convolutions
    with BF16 operands where a layer's shape has a kernel, weight gradients on
    the CUDA cores) against the FP32 CUDA-core path on a 32^3 cell with the
    16-64 channel network: the output within 2e-2 of its norm and every
    layer's weight gradient within 5e-2 of the FP32 gradient's norm (BF16
    operands carry 8 mantissa bits)."""
    import torch
    net = gn.GuessNet(channels=(16, 32, 48, 64), seed=3)
    rng = np.random.default_rng(8)
    x = torch.tensor(rng.standard_normal((2, 32, 32, 32)).astype(np.float32), device="cuda")
    c = torch.tensor(rng.standard_normal((1, 32, 32, 32)).astype(np.float32), device="cuda")
    assert any(l.tc_supported((32, 32, 32)) for l in net.layers)
    res = {}
    for tc in (False, True):
        out = net.forward(x, keep=True, tc_train=tc)
        net.backward(c)
        res[tc] = (out.clone(), [l.gw.clone() for l in net.layers])
    o32, g32 = res[False]
    otc, gtc = res[True]
    assert float((otc - o32).norm() / o32.norm()) < 2e-2
    for i, (a, b) in enumerate(zip(gtc, g32)):
        assert float((a - b).norm() / b.norm()) < 5e-2, i
    assert int(net._err_train.item()) == 0


def test_half_resolution_network_gradients(gn):
    """res 2: the network on the pooled features, its output upsampled back;
    the weight gradients of sum(out * c) equal central differences of the
    oracle's composition pool2 -> network -> uplin (FP64)."""
    import torch
    net = gn.GuessNet(channels=(4, 6), seed=2, res=2)
    rng = np.random.default_rng(6)
    x = rng.standard_normal((2, 8, 8, 12)).astype(np.float32)
    c = rng.standard_normal((1, 8, 8, 12)).astype(np.float32)
    out = net.forward(torch.tensor(x, device="cuda"), keep=True).cpu().numpy()
    enc, dec, head = _oracle_weights(net)

    def full(enc2, dec2, head2):
        return G.uplin(G.net_forward(G.pool2(x.astype(np.float64)), enc2, dec2, head2))
    ref = full(enc, dec, head)
    assert out.shape == (1, 8, 8, 12)
    assert np.abs(out - ref).max() <= 1e-4 * np.abs(ref).max()
    net.backward(torch.tensor(c, device="cuda"))
    e = 1e-4
    for lvl, which, idx in [(0, 0, (1, 0, 13)), (1, 2, (3, 5, 0))]:
        layer = net.enc[lvl][which // 2]
        g_gpu = float(layer.gw.cpu().numpy()[idx])

        def loss(delta):
            enc2, dec2, head2 = _oracle_weights(net)
            t = list(enc2[lvl])
            w = t[which].copy()
            w[idx] += delta
            t[which] = w
            enc2[lvl] = tuple(t)
            return float((full(enc2, dec2, head2) * c).sum())
        fd = (loss(e) - loss(-e)) / (2 * e)
        assert abs(g_gpu - fd) <= 2e-3 * max(1.0, abs(fd)), (lvl, which, idx, g_gpu, fd)


def test_batch_leaves_the_guess_check_to_the_optimiser(gn):
    """In ``optimize_batch`` the guess's residual check is the TN's own first
    evaluation: a start whose residual is above ``start_residual_max``
    returns at once (converged 3, density unchanged) and the batch starts
    again from the uniform density.  A broken network (head scaled 50x) is
    rejected and its solve ends where the uniform start's does; the
    option alone rejects any start below its residual."""
    import torch
    from dftpy_gb300 import batch as B
    from dftpy_gb300 import systems
    from dftpy_gb300.optimization import Optimization
    st = systems.fcc_supercell((2, 2, 2), sigma=0.15, seed=6, nr=(64, 64, 64), mg_fraction=0.2, name="defer")
    total, rho_u = B.build_evaluator(st, kedf="WGC")
    o = {"econv": 1e-8 * st.nat, "maxfun": 50, "maxiter": 100, "precision": "mixed",
         "start_residual_max": 1e-12}
    opt = Optimization(EnergyEvaluator=total, optimization_method="TN", optimization_options=o)
    r = opt.optimize_rho(guess_rho=rho_u)
    assert opt.converged == 3
    assert torch.equal(r.as_subclass(torch.Tensor), rho_u.as_subclass(torch.Tensor))
    bad_net = gn.GuessNet(channels=(16, 32, 48, 64), seed=11)
    bad_net.head.w.mul_(50.0)
    bad_net.head.sync_bf16()
    opts = {"precision": "mixed", "econv_per_atom": 1e-8}
    ref = B.optimize_batch([(total, rho_u)], workers=1, options=opts)[0]
    res = B.optimize_batch([(total, rho_u)], workers=1, options=opts, guess=gn.LearnedGuess(bad_net))[0]
    assert res.extra.get("guess_rejected") and res.converged == 0
    assert abs(res.energy - ref.energy) * 27.211386 / st.nat <= 1e-8
