"""numpy FP64 restatement of the learned-guess network's operations.

TEST INFRASTRUCTURE ONLY: the checker for the GPU kernels (``gbofdft_nn_*``).
No reference counterpart (the reference has no learned guess).  Arrays are
[C][D][H][W]; weights [C_out][C_in][27] with tap = (dz+1)*9 + (dy+1)*3 + (dx+1);
the grid is periodic.
"""
import numpy as np

TAPS = [(dz, dy, dx) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def shift(x, d):
    """x[v + d] on the periodic grid (last three axes)."""
    dz, dy, dx = d
    return np.roll(x, shift=(-dz, -dy, -dx), axis=(-3, -2, -1))


def conv3d(x, w, b=None):
    cout = w.shape[0]
    out = np.zeros((cout,) + x.shape[1:])
    for t, d in enumerate(TAPS):
        xs = shift(x, d)
        out += np.einsum("oi,i...->o...", w[:, :, t], xs)
    if b is not None:
        out += b[:, None, None, None]
    return out


def conv3d_input_grad(g, w):
    gx = np.zeros((w.shape[1],) + g.shape[1:])
    for t, d in enumerate(TAPS):
        gx += shift(np.einsum("oi,o...->i...", w[:, :, t], g), (-d[0], -d[1], -d[2]))
    return gx


def conv3d_weight_grad(x, g):
    gw = np.zeros((g.shape[0], x.shape[0], 27))
    for t, d in enumerate(TAPS):
        gw[:, :, t] = np.tensordot(g, shift(x, d), axes=([1, 2, 3], [1, 2, 3]))
    return gw, g.sum(axis=(1, 2, 3))


def silu(z):
    return z / (1.0 + np.exp(-z))


def silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def pool2(x):
    C, D, H, W = x.shape
    return x.reshape(C, D // 2, 2, H // 2, 2, W // 2, 2).mean(axis=(2, 4, 6))


def pool2_adjoint(g):
    return np.repeat(np.repeat(np.repeat(g, 2, axis=1), 2, axis=2), 2, axis=3) / 8.0


def up2(x):
    return np.repeat(np.repeat(np.repeat(x, 2, axis=1), 2, axis=2), 2, axis=3)


def up2_adjoint(g):
    C, D, H, W = g.shape
    return g.reshape(C, D // 2, 2, H // 2, 2, W // 2, 2).sum(axis=(2, 4, 6))


def uplin(x):
    """Periodic 2x linear upsampling, cell-centred: fine point i of an axis
    takes 3/4 of coarse point i // 2 and 1/4 of its neighbour on the side
    of i (the inverse pairing of the average pool)."""
    out = x
    for ax in (1, 2, 3):
        even = 0.75 * out + 0.25 * np.roll(out, 1, axis=ax)     # 2j: j and j - 1
        odd = 0.75 * out + 0.25 * np.roll(out, -1, axis=ax)     # 2j + 1: j and j + 1
        shape = list(out.shape)
        shape[ax] *= 2
        new = np.empty(shape)
        sl_e = [slice(None)] * 4
        sl_o = [slice(None)] * 4
        sl_e[ax] = slice(0, None, 2)
        sl_o[ax] = slice(1, None, 2)
        new[tuple(sl_e)] = even
        new[tuple(sl_o)] = odd
        out = new
    return out


def uplin_adjoint(g):
    out = g
    for ax in (1, 2, 3):
        sl_e = [slice(None)] * 4
        sl_o = [slice(None)] * 4
        sl_e[ax] = slice(0, None, 2)
        sl_o[ax] = slice(1, None, 2)
        e, o = out[tuple(sl_e)], out[tuple(sl_o)]
        out = 0.75 * (e + o) + 0.25 * (np.roll(e, -1, axis=ax) + np.roll(o, 1, axis=ax))
    return out


def net_forward(x, enc, dec, head):
    """The encoder-decoder of the product (weights as lists of (w, b) pairs
    per level; enc: [(w1, b1, w2, b2)], dec: the same from the deepest
    decoder level up, head: (w, b))."""
    skips = []
    h = x
    for lvl, (w1, b1, w2, b2) in enumerate(enc):
        a1 = silu(conv3d(h, w1, b1))
        a2 = silu(conv3d(a1, w2, b2))
        skips.append(a2)
        h = pool2(a2) if lvl < len(enc) - 1 else a2
    for k, (w1, b1, w2, b2) in enumerate(dec):
        lvl = len(enc) - 2 - k
        a1 = silu(conv3d(up2(h), w1, b1))
        h = silu(conv3d(a1 + skips[lvl], w2, b2))
    return conv3d(h, *head)
