"""Learned initial guess: a 3-D convolutional encoder-decoder that maps the
superposed atomic densities and the local pseudopotential on the grid to a
starting sqrt(rho).

No reference counterpart: the reference starts from a uniform density or
superposed atomic densities (``density/density.py:151-319``); those remain
the network's inputs and its baseline.  The network predicts the correction
to sqrt(rho_atom) (in units of sqrt(rho0), rho0 the mean density); the
truncated-Newton optimiser always finishes from the guess, so the guess
changes how many evaluations a solve takes, not where it ends.

Architecture (all convolutions 3x3x3 and periodic, SiLU activations):
``levels`` resolutions, two convolutions per level on the way down (2x
average pooling between levels), 2x nearest upsampling, one convolution,
an additive skip from the encoder and a second convolution per level on the
way up, and a 1-channel head.  The network is fully convolutional at the
grid spacing of the workloads (0.24 Bohr), so a net trained on small cells
applies to any cell whose grid extents are divisible by its stride,
2^(levels-1) times ``res``: with ``res`` 2 or 4 it runs on the 2x or 4x
average-pooled features and its output is brought back by periodic
trilinear 2x steps.  The alloy network (``data/guessnet.npz``) has 32-128
channels on 4x pooled features; the Al network for Wang-Teter
(``data/guessnet_al_wt.npz``) 16-64 channels at full resolution.
Weights are BF16 for the arithmetic with FP32 master copies; every kernel
(forward, input and weight gradients, pooling, activations, loss, Adam) is
the project's own (``gbofdft_nn_*``).
"""
import ctypes
import gc
import math
import threading
import time

import numpy as np
import torch

from . import _lib, systems

SQRT_CLAMP = 1e-30

_PACK_LOCK = threading.Lock()


def _L():
    return _lib.load()


class Conv:
    """One 3x3x3 periodic convolution layer with FP32 master weights, a BF16
    copy, gradients and Adam moments."""

    def __init__(self, cin, cout, rng):
        self.cin, self.cout = cin, cout
        std = math.sqrt(2.0 / (27 * cin))
        w = rng.normal(0.0, std, size=(cout, cin, 27)).astype(np.float32)
        self.w = torch.tensor(w, device="cuda")
        self.b = torch.zeros(cout, dtype=torch.float32, device="cuda")
        self.wb = torch.empty((cout, cin, 27), dtype=torch.bfloat16, device="cuda")
        self.gw = torch.zeros_like(self.w)
        self.gb = torch.zeros_like(self.b)
        self.mw, self.vw = torch.zeros_like(self.w), torch.zeros_like(self.w)
        self.mb, self.vb = torch.zeros_like(self.b), torch.zeros_like(self.b)
        self.wtc = None            # BF16 weights packed for the tensor-core kernel (made on first use)
        self.wtc_t = None          # ... of the input-gradient convolution (training)
        self.sync_bf16()

    def sync_bf16(self):
        _lib.check(_L().gbofdft_nn_to_bf16(_lib.ptr(self.w), _lib.ptr(self.wb), self.w.numel(), _lib.stream_ptr()))
        self.wtc = None
        self.wtc_t = None

    def _tc_cout(self):
        """Output width of the tensor-core kernel (a layer narrower than 16
        channels runs 16 wide with zero weights and stores its own)."""
        return 16 if self.cout < 16 else self.cout

    def pack_tc(self, publish=True):
        """Pack the BF16 weights for the tensor-core kernel.  publish: the
        packed copy is made visible only once the packing has finished on this
        stream, so guesses on other threads and streams may use it right away
        (training, on one stream, skips that wait)."""
        with _PACK_LOCK:
            if self.wtc is not None:
                return
            cw = self._tc_cout()
            wb = self.wb
            if cw != self.cout:
                wb = torch.zeros((cw, self.cin, 27), dtype=torch.bfloat16, device="cuda")
                wb[:self.cout] = self.wb
            wtc = torch.empty(27 * self.cin * cw, dtype=torch.bfloat16, device="cuda")
            _lib.check(_L().gbofdft_nn_conv3d_tc_pack(_lib.ptr(wb), self.cin, cw, _lib.ptr(wtc),
                                                      _lib.stream_ptr()), "nn_conv3d_tc_pack")
            if publish:
                torch.cuda.current_stream().synchronize()
            self.wtc = wtc

    def _tc_cin_t(self):
        """Output width of the transposed convolution on the tensor cores."""
        return 16 if self.cin < 16 else self.cin

    def pack_tc_t(self):
        """Packed weights of the input-gradient convolution: the transposed,
        tap-reversed kernel (C_out -> C_in) of this periodic convolution."""
        if self.wtc_t is None:
            cw = self._tc_cin_t()
            wt = torch.zeros((cw, self.cout, 27), dtype=torch.bfloat16, device="cuda")
            wt[:self.cin] = self.wb.permute(1, 0, 2).flip(2)
            wtc = torch.empty(27 * self.cout * cw, dtype=torch.bfloat16, device="cuda")
            _lib.check(_L().gbofdft_nn_conv3d_tc_pack(_lib.ptr(wt), self.cout, cw, _lib.ptr(wtc),
                                                      _lib.stream_ptr()), "nn_conv3d_tc_pack")
            self.wtc_t = wtc
        return self.wtc_t

    def tc_dgrad_supported(self, shape):
        D, H, W = shape
        return bool(_L().gbofdft_nn_conv3d_tc_supported(self.cout, self._tc_cin_t(), D, H, W))

    def forward_z(self, x, shape, err, tc):
        """conv + bias without activation (the training forward): on the
        tensor cores (BF16 operands, FP32 accumulation) where the layer shape
        has a kernel and tc is set, else on the CUDA cores in FP32."""
        if tc and self.tc_supported(shape):
            if self.wtc is None:
                self.pack_tc(publish=False)
            return self.forward_tc(x, shape, False, err)
        return self.forward(x, shape)

    def tc_channels(self):
        """The tensor-core kernel has this layer's channel pair."""
        return bool(_L().gbofdft_nn_conv3d_tc_supported(self.cin, self._tc_cout(), 16, 16, 16))

    def tc_supported(self, shape):
        D, H, W = shape
        return bool(_L().gbofdft_nn_conv3d_tc_supported(self.cin, self._tc_cout(), D, H, W))

    def forward_tc(self, x, shape, act, err, skip=None, up=False):
        """conv + bias (then SiLU when act, then + skip) on the tensor cores,
        activations rounded to BF16; up: x is the half-size grid, read as its
        2x nearest upsampling; err: device int32 flag of timed-out waits."""
        D, H, W = shape
        cw = self._tc_cout()
        if self.wtc is None:
            self.pack_tc()
        z = torch.empty((self.cout, D, H, W), dtype=torch.float32, device="cuda")
        _lib.check(_L().gbofdft_nn_conv3d_tc(_lib.ptr(x), self.cin, _lib.ptr(self.wtc), _lib.ptr(self.b), _lib.ptr(z),
                                             cw, self.cout, D, H, W, 1 if act else 0,
                                             _lib.ptr(skip) if skip is not None else None, 1 if up else 0,
                                             _lib.ptr(err), _lib.stream_ptr()), "nn_conv3d_tc")
        return z

    def forward_act(self, x, shape, err, tc=True, skip=None, up=False):
        """silu(conv(x)) (+ skip) for inference, x upsampled 2x first when up:
        the tensor-core kernel with all of it fused where the layer shape has
        one, else the CUDA-core kernel and separate passes."""
        if tc and self.tc_supported(shape):
            return self.forward_tc(x, shape, True, err, skip=skip, up=up)
        a = silu(self.forward(up2(x) if up else x, shape))
        return add(a, skip) if skip is not None else a

    @property
    def nparams(self):
        return self.w.numel() + self.b.numel()

    def forward(self, x, shape):
        D, H, W = shape
        z = torch.empty((self.cout, D, H, W), dtype=torch.float32, device="cuda")
        _lib.check(_L().gbofdft_nn_conv3d(_lib.ptr(x), self.cin, _lib.ptr(self.wb), _lib.ptr(self.b), _lib.ptr(z),
                                          self.cout, D, H, W, 0, _lib.stream_ptr()), "nn_conv3d")
        return z

    def backward(self, x, gz, shape, need_input_grad=True, tc=False, err=None):
        """Weight and bias gradients (overwritten) and the input gradient (on
        the tensor cores where tc is set and the shape has a kernel)."""
        D, H, W = shape
        _lib.check(_L().gbofdft_nn_conv3d_wgrad(_lib.ptr(x), self.cin, _lib.ptr(gz), self.cout, D, H, W,
                                                _lib.ptr(self.gw), _lib.ptr(self.gb), _lib.stream_ptr()),
                   "nn_conv3d_wgrad")
        if not need_input_grad:
            return None
        if tc and err is not None and self.tc_dgrad_supported(shape):
            gx = torch.empty((self.cin, D, H, W), dtype=torch.float32, device="cuda")
            _lib.check(_L().gbofdft_nn_conv3d_tc(_lib.ptr(gz), self.cout, _lib.ptr(self.pack_tc_t()), None,
                                                 _lib.ptr(gx), self._tc_cin_t(), self.cin, D, H, W, 0, None, 0,
                                                 _lib.ptr(err), _lib.stream_ptr()), "nn_conv3d_tc_dgrad")
            return gx
        gx = torch.empty((self.cin, D, H, W), dtype=torch.float32, device="cuda")
        _lib.check(_L().gbofdft_nn_conv3d(_lib.ptr(gz), self.cout, _lib.ptr(self.wb), None, _lib.ptr(gx), self.cin,
                                          D, H, W, 1, _lib.stream_ptr()), "nn_conv3d_t")
        return gx

    def adam(self, lr, step, b1=0.9, b2=0.999, eps=1e-8):
        L = _L()
        s = _lib.stream_ptr()
        _lib.check(L.gbofdft_nn_adam(_lib.ptr(self.w), _lib.ptr(self.gw), _lib.ptr(self.mw), _lib.ptr(self.vw),
                                     _lib.ptr(self.wb), self.w.numel(), lr, b1, b2, eps, step, s))
        self.wtc = None
        self.wtc_t = None
        _lib.check(L.gbofdft_nn_adam(_lib.ptr(self.b), _lib.ptr(self.gb), _lib.ptr(self.mb), _lib.ptr(self.vb),
                                     None, self.b.numel(), lr, b1, b2, eps, step, s))


def _pw(op, a, b, out, C, shape):
    D, H, W = shape
    _lib.check(_L().gbofdft_nn_pointwise(op, _lib.ptr(a), _lib.ptr(b) if b is not None else None, _lib.ptr(out), C,
                                         D, H, W, _lib.stream_ptr()), "nn_pointwise")
    return out


SILU, SILU_BWD, ADD, POOL2, POOL2_BWD, UP2, UP2_BWD, UPLIN, UPLIN_BWD = range(9)


def silu(z):
    return _pw(SILU, z, None, torch.empty_like(z), z.shape[0], tuple(z.shape[1:]))


def silu_bwd(z, ga):
    return _pw(SILU_BWD, z, ga, torch.empty_like(z), z.shape[0], tuple(z.shape[1:]))


def pool2(x):
    C, D, H, W = x.shape
    return _pw(POOL2, x, None, torch.empty((C, D // 2, H // 2, W // 2), dtype=x.dtype, device="cuda"), C, (D, H, W))


def pool2_bwd(g, fine_shape):
    C = g.shape[0]
    return _pw(POOL2_BWD, g, None, torch.empty((C,) + tuple(fine_shape), dtype=g.dtype, device="cuda"), C,
               fine_shape)


def up2(x):
    C, D, H, W = x.shape
    fine = (2 * D, 2 * H, 2 * W)
    return _pw(UP2, x, None, torch.empty((C,) + fine, dtype=x.dtype, device="cuda"), C, fine)


def up2_bwd(g):
    C, D, H, W = g.shape
    return _pw(UP2_BWD, g, None, torch.empty((C, D // 2, H // 2, W // 2), dtype=g.dtype, device="cuda"), C,
               (D, H, W))


def uplin(x):
    """Periodic 2x trilinear upsampling (cell-centred)."""
    C, D, H, W = x.shape
    fine = (2 * D, 2 * H, 2 * W)
    return _pw(UPLIN, x, None, torch.empty((C,) + fine, dtype=x.dtype, device="cuda"), C, fine)


def uplin_bwd(g):
    C, D, H, W = g.shape
    return _pw(UPLIN_BWD, g, None, torch.empty((C, D // 2, H // 2, W // 2), dtype=g.dtype, device="cuda"), C,
               (D, H, W))


def add(a, b):
    return _pw(ADD, a, b, torch.empty_like(a), a.shape[0], tuple(a.shape[1:]))


class GuessNet:
    """The encoder-decoder (see module doc); ``channels`` per level."""

    IN_CHANNELS = 2

    def __init__(self, channels=(16, 32, 48, 64), seed=0, res=1):
        """res 2 (4): the network runs on the 2x (twice 2x) average-pooled
        features and its output is upsampled back by periodic trilinear 2x
        steps -- 8x (64x) less work."""
        if int(res) not in (1, 2, 4):
            raise ValueError("res must be 1, 2 or 4")
        self.res = int(res)
        self.mix = 1.0          # the LearnedGuess mixing factor this network was evaluated with
        rng = np.random.default_rng(seed)
        self.channels = tuple(int(c) for c in channels)
        c = self.channels
        self.enc = []
        cin = self.IN_CHANNELS
        for ch in c:
            self.enc.append((Conv(cin, ch, rng), Conv(ch, ch, rng)))
            cin = ch
        self.dec = []
        for lvl in range(len(c) - 2, -1, -1):
            self.dec.append((Conv(c[lvl + 1], c[lvl], rng), Conv(c[lvl], c[lvl], rng)))
        self.head = Conv(c[0], 1, rng)
        self.step_count = 0
        self._tape = None

    @property
    def layers(self):
        out = []
        for a, b in self.enc + self.dec:
            out += [a, b]
        return out + [self.head]

    @property
    def nparams(self):
        return sum(l.nparams for l in self.layers)

    @property
    def stride(self):
        return 2 ** (len(self.channels) - 1) * self.res

    def forward(self, x, keep=False, tc=True, tc_train=False):
        """x: (2, D, H, W) FP32 -> (1, D, H, W) (see ``_forward``); with res 2
        (4) the network sees pool2(x) (twice) and its output is upsampled."""
        shape = tuple(x.shape[1:])
        if any(s % self.stride for s in shape):
            raise ValueError("grid %s not divisible by %d" % (shape, self.stride))
        for _ in range(self._halvings):
            x = pool2(x)
        out = self._forward(x, keep, tc, tc_train)
        for _ in range(self._halvings):
            out = uplin(out)
        return out

    @property
    def _halvings(self):
        return {1: 0, 2: 1, 4: 2}[self.res]

    def _forward(self, x, keep=False, tc=True, tc_train=False):
        """x: (2, D, H, W) FP32 -> (1, D, H, W).  keep: record what backward
        needs; its convolutions run in FP32 on the CUDA cores, or with
        tc_train on the tensor cores where the layer shape has a kernel (BF16
        operands, FP32 pre-activations kept).  Without keep the inner layers
        run on the tensor cores (BF16 activations) when tc is set."""
        shape = tuple(x.shape[1:])
        if not keep:
            return self._infer(x, shape, tc)
        # one device flag of timed-out tensor-core waits for the whole
        # training run (read once per epoch)
        if tc_train and getattr(self, "_err_train", None) is None:
            self._err_train = torch.zeros(1, dtype=torch.int32, device="cuda")
        err = self._err_train if tc_train else None
        self._err = err
        tape = []
        skips = []
        h = x
        for lvl, (c1, c2) in enumerate(self.enc):
            sh = tuple(h.shape[1:])
            z1 = c1.forward_z(h, sh, err, tc_train)
            a1 = silu(z1)
            z2 = c2.forward_z(a1, sh, err, tc_train)
            a2 = silu(z2)
            tape.append(("enc", lvl, h, z1, a1, z2))
            skips.append(a2)
            h = pool2(a2) if lvl < len(self.enc) - 1 else a2
        for k, (c1, c2) in enumerate(self.dec):
            lvl = len(self.channels) - 2 - k
            u = up2(h)
            sh = tuple(u.shape[1:])
            z1 = c1.forward_z(u, sh, err, tc_train)
            a1 = silu(z1)
            s = add(a1, skips[lvl])
            z2 = c2.forward_z(s, sh, err, tc_train)
            h = silu(z2)
            tape.append(("dec", lvl, u, z1, s, z2))
        out = self.head.forward(h, shape)
        tape.append(("head", 0, h))
        self._tape = tape if keep else None
        return out

    def _infer(self, x, shape, tc):
        err = torch.zeros(1, dtype=torch.int32, device="cuda")
        skips = []
        h = x
        for lvl, (c1, c2) in enumerate(self.enc):
            sh = tuple(h.shape[1:])
            a1 = c1.forward_act(h, sh, err, tc)
            a2 = c2.forward_act(a1, sh, err, tc)
            skips.append(a2)
            h = pool2(a2) if lvl < len(self.enc) - 1 else a2
        for k, (c1, c2) in enumerate(self.dec):
            lvl = len(self.channels) - 2 - k
            sh = tuple(skips[lvl].shape[1:])
            s = c1.forward_act(h, sh, err, tc, skip=skips[lvl], up=True)
            h = c2.forward_act(s, sh, err, tc)
        # the head stays on the CUDA cores with FP32 activations: rounding its
        # input to BF16 costs the Al256 solve ~25 % more evaluations
        out = self.head.forward(h, shape)
        self._tape = None
        if int(err.item()) != 0:
            raise RuntimeError("tensor-core convolution: a wait timed out (code %d)" % int(err.item()))
        return out

    def backward(self, gout):
        """Gradients of every layer from d loss / d out (the last forward's tape)."""
        tape = self._tape
        if tape is None:
            raise RuntimeError("forward(keep=True) must precede backward")
        for _ in range(self._halvings):
            gout = uplin_bwd(gout.contiguous())
        _, _, h = tape[-1]
        shape = tuple(h.shape[1:])
        err = getattr(self, "_err", None)
        tc = err is not None
        g = self.head.backward(h, gout, shape)
        gskip = {}
        for k in range(len(self.dec) - 1, -1, -1):
            _, lvl, u, z1, s, z2 = tape[len(self.enc) + k]
            c1, c2 = self.dec[k]
            sh = tuple(u.shape[1:])
            gz2 = silu_bwd(z2, g)
            gs = c2.backward(s, gz2, sh, tc=tc, err=err)
            gskip[lvl] = gs
            gz1 = silu_bwd(z1, gs)
            gu = c1.backward(u, gz1, sh, tc=tc, err=err)
            g = up2_bwd(gu)
        for lvl in range(len(self.enc) - 1, -1, -1):
            _, _, hin, z1, a1, z2 = tape[lvl]
            c1, c2 = self.enc[lvl]
            sh = tuple(hin.shape[1:])
            if lvl < len(self.enc) - 1:
                g = pool2_bwd(g, sh)
            if lvl in gskip:
                g = add(g, gskip[lvl])
            gz2 = silu_bwd(z2, g)
            ga1 = c2.backward(a1, gz2, sh, tc=tc, err=err)
            gz1 = silu_bwd(z1, ga1)
            g = c1.backward(hin, gz1, sh, need_input_grad=lvl > 0, tc=tc, err=err)
        self._tape = None

    def adam_step(self, lr):
        self.step_count += 1
        for l in self.layers:
            l.adam(lr, self.step_count)

    def state(self):
        return {"channels": np.array(self.channels), "res": np.array(self.res), "mix": np.array(self.mix),
                **{"w%d" % i: l.w.cpu().numpy() for i, l in enumerate(self.layers)},
                **{"b%d" % i: l.b.cpu().numpy() for i, l in enumerate(self.layers)}}

    def save(self, path):
        np.savez_compressed(path, **self.state())

    @classmethod
    def load(cls, path):
        d = np.load(path)
        net = cls(channels=tuple(int(c) for c in d["channels"]), res=int(d["res"]) if "res" in d.files else 1)
        net.mix = float(d["mix"]) if "mix" in d.files else 1.0
        for i, l in enumerate(net.layers):
            l.w.copy_(torch.tensor(d["w%d" % i]))
            l.b.copy_(torch.tensor(d["b%d" % i]))
            l.sync_bf16()
        return net


# --------------------------------------------------------------------------
# features, targets, the guess
# --------------------------------------------------------------------------

def features(total, grid):
    """Network input (2, D, H, W): superposed Gaussian atomic densities over
    the mean minus one, and v_loc; plus sqrt(rho_atom) and rho0."""
    from .density import get_3d_value_recipe
    from .field import DirectField
    ps = total.PSEUDO
    ions = ps.ions
    tabs = {s: systems.atomic_density_table(systems.SPECIES[s][0], systems.ATOMIC_SIGMA[s]) for s in set(ions.symbols)}
    r = {s: t[0] for s, t in tabs.items()}
    arho = {s: t[1] for s, t in tabs.items()}
    # the network input is FP32: superpose in FP32 (the FP64 transforms of
    # the superposition cost ten times more on this part)
    ratom = get_3d_value_recipe(r, arho, ions, grid, dtol=1e-12, rho=DirectField(grid, dtype=torch.float32))
    rho0 = float(ions.get_ncharges()) / grid.volume
    ra = ratom.as_subclass(torch.Tensor).to(torch.float32)
    vloc = ps.vreal_of(torch.float32).reshape(ra.shape)
    x = torch.stack([ra / rho0 - 1.0, vloc]).contiguous()
    phib = torch.sqrt(torch.clamp(ra, min=SQRT_CLAMP))
    return x, phib, rho0


def residual(total, rho):
    """||(V - mu) sqrt(rho)|| (L2 over the cell) of the FP32 potential at
    ``rho``, mu = int V rho / int rho: the square root of the residual norm
    the reference TN prints at its first step (``optimization.py:318-340``,
    residual = (V - mu) phi)."""
    from .field import DirectField
    grid = rho.grid
    x = DirectField(grid, data=rho.as_subclass(torch.Tensor).to(torch.float32))
    v = total(x, calcType={"V"}).potential.as_subclass(torch.Tensor).reshape(-1).to(torch.float64)
    r = x.as_subclass(torch.Tensor).reshape(-1).clamp(min=0.0).to(torch.float64)
    # one pass of sums: int r, int V r, int V^2 r; then
    # int (V - mu)^2 r = int V^2 r - mu int V r
    vr = v * r
    s0, s1, s2 = (float(t) for t in torch.stack([r.sum(), vr.sum(), (vr * v).sum()]).tolist())
    mu = s1 / s0
    return math.sqrt(max(s2 - mu * s1, 0.0) * grid.dV)


def uniform_residual(total, grid):
    """``residual`` at the uniform density.  When every member of ``total``
    is one of this package's functionals the potential there is a constant
    plus v_loc (the semilocal terms are constant, vW and Hartree vanish, the
    nonlocal kernels act on a constant), so the residual is
    sqrt(rho0) ||v_loc - <v_loc>||, a reduction without an evaluation."""
    from .field import DirectField
    nel = float(total.PSEUDO.ions.get_ncharges())
    rho0 = nel / grid.volume
    fusable = getattr(total, "fusable", None)
    if fusable is not None and fusable():
        # a set-up quantity of the structure, like v_loc itself: kept with it
        ps = total.PSEUDO
        cache = ps.__dict__.setdefault("_uniform_residual", {})
        key = (id(grid), id(ps.vreal_of(torch.float64)))
        if key not in cache:
            v = ps.vreal_of(torch.float64)
            dv = v - v.mean()
            cache.clear()
            cache[key] = float(torch.sqrt((dv * dv).sum() * (rho0 * grid.dV)))
        return cache[key]
    uni = DirectField(grid, data=torch.full(tuple(int(n) for n in grid.nrR), rho0, dtype=torch.float64,
                                            device="cuda"))
    return residual(total, uni)


class LearnedGuess:
    """Starting density from a trained ``GuessNet``: the network's density,
    mixed with the uniform density when ``mix`` < 1 (rho0 + mix (rho_net -
    rho0); None: the value saved with the network, else 1).

    fallback: compare the FP32 residual (``residual``) of the network's
    density with the uniform density's (``uniform_residual``) and start from
    the uniform density when the network's is not below ``fallback_ratio``
    times it, or is not finite (one FP32 potential evaluation per guess);
    ``last_choice`` records the pick.  The default ratio 2 catches a broken
    guess, not a merely different one: this residual does not rank good
    starts (the 4000-atom LMGP cell's network density has 1.17x the uniform
    density's residual yet needs far fewer evaluations from it).

    ``guess(..., defer_check=True)`` leaves the residual comparison to the
    optimiser: the density carries ``start_residual_max`` (fallback_ratio
    times the uniform density's residual), which the TN compares with the
    residual of its own first evaluation (``optimization`` option
    ``start_residual_max``); ``batch.optimize_batch`` does this and starts
    again from the uniform density when the TN rejects the guess."""

    def __init__(self, net, mix=None, fallback=True, fallback_ratio=2.0):
        self.net = net
        self.mix = float(mix) if mix is not None else float(getattr(net, "mix", 1.0))
        self.fallback = bool(fallback)
        self.fallback_ratio = float(fallback_ratio)
        self.last_choice = None

    def prepare(self, total, grid=None):
        """Make the network's packed tensor-core weights (every layer whose
        channel pair has a tensor-core kernel, whatever the grid) and the
        cached set-up of the features by one guess on the current stream;
        callers that guess from several threads call this first, once per
        grid shape."""
        for layer in self.net.layers:
            if layer.wtc is None and layer.tc_channels():
                layer.pack_tc()
        self.guess(total, grid)
        torch.cuda.synchronize()

    def guess(self, total, grid=None, dtype=torch.float64, defer_check=False):
        from .field import DirectField
        grid = grid or total.PSEUDO.grid
        x, phib, rho0 = features(total, grid)
        out = self.net.forward(x)[0]
        phi = phib + math.sqrt(rho0) * out
        rho = (phi * phi).to(torch.float64)
        nel = float(total.PSEUDO.ions.get_ncharges())
        rho = rho * (nel / (float(rho.sum()) * grid.dV))
        rho0_u = nel / grid.volume
        if self.mix != 1.0:
            rho = rho0_u + self.mix * (rho - rho0_u)
        out = DirectField(grid, data=rho.to(dtype))
        choice = "network"
        if self.fallback:
            if not bool(torch.isfinite(rho).all()):
                out = DirectField(grid, data=torch.full_like(rho, rho0_u).to(dtype))
                choice = "uniform"
            elif defer_check:
                out.start_residual_max = self.fallback_ratio * uniform_residual(total, grid)
            elif not residual(total, out) < self.fallback_ratio * uniform_residual(total, grid):
                out = DirectField(grid, data=torch.full_like(rho, rho0_u).to(dtype))
                choice = "uniform"
        self.last_choice = choice
        return out


def _solve(total, guess, precision="mixed", econv_per_atom=1e-8):
    from .optimization import Optimization
    nat = total.PSEUDO.ions.nat
    opt = Optimization(EnergyEvaluator=total, optimization_method="TN",
                       optimization_options={"econv": econv_per_atom * nat, "maxfun": 50, "maxiter": 100,
                                             "precision": precision})
    rho = opt.optimize_rho(guess_rho=guess)
    return opt, rho


def training_cell(seed, reps=(2, 2, 2), nr=(64, 64, 64), mg_max=0.3, sigmas=(0.15,)):
    """Training / validation cell: an Al/Mg snapshot as the batched workload
    draws them (Mg fraction U(0, mg_max), jitter sigmas[seed % len(sigmas)]
    Bohr) on a small cell; mg_max = 0 gives pure Al."""
    f = float(np.random.default_rng(10_000 + seed).random() * mg_max)
    sigma = float(sigmas[seed % len(sigmas)])
    return systems.fcc_supercell(reps, sigma=sigma, seed=seed, nr=nr, mg_fraction=f, name="train_%d" % seed)


def make_dataset(seeds, kedf="WGC", precision="mixed", reps=(2, 2, 2), nr=(64, 64, 64), workers=16, chunk=64,
                 mg_max=0.3, sigmas=(0.15,), cells="small", store="cuda"):
    """(x, sqrt(rho_atom), sqrt(rho converged), rho0) per seed from the
    solver's own converged densities (solved as batches).  cells "small":
    ``training_cell`` (2x2x2 cells at 64^3); "alloy": the batched workload's
    own generator (``systems.config_alloy``, 108-500 atoms, 96^3-160^3).
    store "cpu" keeps the samples in pinned host memory (``train`` copies
    each to the device when it is used)."""
    from .batch import build_evaluator, optimize_batch
    data = []
    seeds = list(seeds)
    for c0 in range(0, len(seeds), chunk):
        make = (lambda s: systems.config_alloy(s)) if cells == "alloy" else \
            (lambda s: training_cell(s, reps, nr, mg_max, sigmas))
        jobs = [build_evaluator(make(s), kedf=kedf) for s in seeds[c0:c0 + chunk]]
        res = optimize_batch(jobs, workers=workers, options={"precision": precision})
        for (total, rho_u), r in zip(jobs, res):
            if r.converged != 0:
                continue
            x, phib, rho0 = features(total, rho_u.grid)
            phit = torch.sqrt(torch.clamp(r.rho.as_subclass(torch.Tensor).to(torch.float32), min=SQRT_CLAMP))
            if store == "cpu":
                x, phib, phit = (t.cpu().pin_memory() for t in (x, phib, phit))
            data.append((x, phib, phit, rho0))
        # the chunk's evaluators (plans, workspaces) go before the next chunk's
        del jobs, res
        gc.collect()
    return data


def train(net, data, epochs=10, lr=1e-3, lr_min=1e-5, seed=0, log=None, tc=True):
    """Adam on the normalised squared error of sqrt(rho) (one cell per step),
    random periodic translations; cosine learning-rate decay.  tc: forward and
    input-gradient convolutions on the tensor cores where a layer's shape has
    a kernel (BF16 operands, FP32 accumulation); weight gradients on the CUDA
    cores."""
    L = _L()
    nb = ctypes.c_int64()
    _lib.check(L.gbofdft_nn_sqerr_work_bytes(ctypes.byref(nb)))
    work = torch.empty(int(nb.value) // 8 + 8, dtype=torch.float64, device="cuda")
    loss_d = torch.zeros(1, dtype=torch.float64, device="cuda")
    rng = np.random.default_rng(seed)
    nsteps = epochs * len(data)
    hist = []
    k = 0
    for ep in range(epochs):
        order = rng.permutation(len(data))
        tot = 0.0
        for i in order:
            x, phib, phit, rho0 = data[i]
            if not x.is_cuda:
                x, phib, phit = (t.to("cuda", non_blocking=True) for t in (x, phib, phit))
            sh = [int(rng.integers(n)) for n in x.shape[1:]]
            x_ = torch.roll(x, shifts=sh, dims=(1, 2, 3)).contiguous()
            pb = torch.roll(phib, shifts=sh, dims=(0, 1, 2)).contiguous()
            pt = torch.roll(phit, shifts=sh, dims=(0, 1, 2)).contiguous()
            out = net.forward(x_, keep=True, tc_train=tc)
            s0 = math.sqrt(rho0)
            pred = (pb + s0 * out[0]).contiguous()
            grad = torch.empty_like(pred)
            _lib.check(L.gbofdft_nn_sqerr(_lib.ptr(pred), _lib.ptr(pt), pred.numel(), _lib.ptr(grad),
                                          _lib.ptr(loss_d), _lib.aligned_ptr(work, 16), _lib.stream_ptr()))
            net.backward((grad * s0).reshape(out.shape).contiguous())
            t = k / max(1, nsteps - 1)
            net.adam_step(lr_min + 0.5 * (lr - lr_min) * (1.0 + math.cos(math.pi * t)))
            k += 1
            tot += float(loss_d)
        hist.append(tot / len(data))
        if log:
            log("epoch %d loss %.3e" % (ep, hist[-1]))
        err = getattr(net, "_err", None)
        if err is not None and int(err.item()) != 0:
            raise RuntimeError("tensor-core convolution: a wait timed out (code %d)" % int(err.item()))
    return hist


def evaluate_guesses(net, structures, kedf="WGC", precision="mixed"):
    """TN from the uniform density, from the superposed atomic densities and
    from the learned guess; per structure the evaluations, iterations, wall
    time (guess included) and energy."""
    from .batch import build_evaluator
    from .field import DirectField
    rows = []
    lg = LearnedGuess(net)
    for st in structures:
        res = {}
        for mode in ("uniform", "atomic", "learned"):
            total, rho_u = build_evaluator(st, kedf=kedf)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            if mode == "uniform":
                g = rho_u
            elif mode == "atomic":
                x, phib, rho0 = features(total, rho_u.grid)
                g = DirectField(rho_u.grid, data=(phib * phib).to(torch.float64))
                g = g * (st.nelec / (float(g.sum()) * rho_u.grid.dV))
            else:
                g = lg.guess(total, rho_u.grid)
            opt, rho = _solve(total, g, precision)
            torch.cuda.synchronize()
            t = time.perf_counter() - t0
            ev = sum(s["n_eval_ev"] + s["n_eval_v"] for s in opt.stats["stages"])
            it = sum(s["n_iter"] for s in opt.stats["stages"])
            res[mode] = {"wall_s": t, "evals": ev, "iters": it, "energy": float(opt.energy),
                         "converged": int(opt.converged)}
        rows.append({"name": st.name, "nr": list(st.nr), "nat": st.nat, **res})
    return rows


def evaluate_batched(net, structures, kedf="WGC", chunk=64, workers=16, mix=None):
    """Mixed-precision batches of ``structures`` from the uniform density and
    from the learned guess (with its fallback check): per start the wall time
    of the solves (the evaluators' set-up -- plans, tables, PME -- done by an
    untimed pass first, as the benchmark does; the guess is inside the timed
    region), TN iterations and evaluations, converged count, and the largest
    energy difference to the uniform start (eV/atom)."""
    from .batch import build_evaluator, optimize_batch
    lg = LearnedGuess(net, mix=mix)
    modes = (("uniform", None), ("learned", lg))
    out = {m: {"wall_s": 0.0, "iters": 0, "evals": 0, "converged": 0} for m, _ in modes}
    energies = {m: [] for m, _ in modes}
    for c0 in range(0, len(structures), chunk):
        jobs = [build_evaluator(st, kedf=kedf) for st in structures[c0:c0 + chunk]]
        optimize_batch(jobs, workers=workers, options={"precision": "mixed"}, guess=lg)
        for mode, guess in modes:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            res = optimize_batch(jobs, workers=workers, options={"precision": "mixed"}, guess=guess)
            torch.cuda.synchronize()
            o = out[mode]
            o["wall_s"] += time.perf_counter() - t0
            for r in res:
                o["iters"] += sum(st_["n_iter"] for st_ in r.stats["stages"])
                o["evals"] += sum(st_["n_eval_ev"] + st_["n_eval_v"] + st_.get("n_eval_hess", 0)
                                  for st_ in r.stats["stages"])
                o["converged"] += int(r.converged == 0)
                energies[mode].append(float(r.energy))
        del jobs
        gc.collect()
    nat = np.array([st.nat for st in structures])
    out["learned"]["max_dE_eV_per_atom_vs_uniform"] = float(
        np.max(np.abs(np.array(energies["learned"]) - np.array(energies["uniform"])) / nat * 27.211386024367243))
    return out


def main():
    import argparse
    import json
    p = argparse.ArgumentParser(description="train the learned-guess network on the solver's own densities")
    p.add_argument("--train", type=int, default=400, help="training cells (seeds 1000 ...)")
    p.add_argument("--epochs", type=int, default=8)
    p.add_argument("--lr", type=float, default=1e-3)
    p.add_argument("--channels", default="16,32,48,64")
    p.add_argument("--res", type=int, default=1, choices=[1, 2, 4],
                   help="2 (4): the network runs on 2x (4x) pooled features")
    p.add_argument("--mix", type=float, default=1.0, help="mixing factor with the uniform density saved with the "
                                                           "network")
    p.add_argument("--cells", default="small", choices=["small", "alloy"],
                   help="training cells: small 2x2x2 cells at 64^3, or the batched workload's snapshots")
    p.add_argument("--store", default=None, choices=["cuda", "cpu"],
                   help="where the training samples are kept (default: host memory for alloy cells)")
    p.add_argument("--eval", type=int, default=8, help="held-out cells (seeds 5000 ...)")
    p.add_argument("--out", default=None)
    p.add_argument("--kedf", default="WGC", help="KEDF of the training solves (WGC: the batched workload's; "
                                                  "WT: the 256-atom benchmark's)")
    p.add_argument("--mg-max", type=float, default=0.3, help="Mg fraction drawn from U(0, mg_max); 0: pure Al")
    p.add_argument("--sigma", default="0.15", help="position jitter(s) in Bohr, alternating over seeds")
    p.add_argument("--evaluate", default=None, metavar="NET",
                   help="no training: evaluate this saved network on --eval held-out alloy snapshots")
    a = p.parse_args()
    sigmas = tuple(float(v) for v in a.sigma.split(","))
    if a.evaluate:
        net = GuessNet.load(a.evaluate)
        held = [systems.config_alloy(s) for s in range(5000, 5000 + a.eval)]
        print(json.dumps({"network": a.evaluate, "params": net.nparams, "channels": list(net.channels),
                          "res": net.res, "heldout_seeds": [5000, 5000 + a.eval - 1],
                          "heldout": evaluate_batched(net, held, kedf=a.kedf)}))
        return
    t0 = time.perf_counter()
    store = a.store or ("cpu" if a.cells == "alloy" else "cuda")
    data = make_dataset(range(1000, 1000 + a.train), kedf=a.kedf, mg_max=a.mg_max, sigmas=sigmas, cells=a.cells,
                        store=store)
    torch.cuda.synchronize()
    t_data = time.perf_counter() - t0
    net = GuessNet(channels=tuple(int(c) for c in a.channels.split(",")), seed=0, res=a.res)
    net.mix = float(a.mix)
    t1 = time.perf_counter()
    hist = train(net, data, epochs=a.epochs, lr=a.lr, log=lambda s: print(s, flush=True))
    torch.cuda.synchronize()
    t_train = time.perf_counter() - t1
    if a.out:
        net.save(a.out)
    report = {"params": net.nparams, "channels": list(net.channels), "res": net.res, "mix": net.mix,
              "cells": a.cells, "train_cells": len(data), "epochs": a.epochs, "loss": hist,
              "data_s": t_data, "train_s": t_train}
    del data
    if a.cells == "alloy":
        held = [systems.config_alloy(s) for s in range(5000, 5000 + a.eval)]
        report["heldout"] = evaluate_batched(net, held, kedf=a.kedf)
    else:
        held = [training_cell(s, mg_max=a.mg_max, sigmas=sigmas) for s in range(5000, 5000 + a.eval)]
        report["rows"] = evaluate_guesses(net, held, kedf=a.kedf)
    print(json.dumps(report))


if __name__ == "__main__":
    main()
