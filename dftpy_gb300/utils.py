"""Moving fields between grids (``utils/utils.py``): Fourier interpolation by
copying the spectrum of one grid into another (``grid_map_index``,
``grid_map_data``, ``:51-129``) and ``field2distrib`` (``:218-287``), the
coarse-to-fine step of the multi-grid density optimisation.

The spectra come from the GPU transforms (``DirectField.fft``,
``ReciprocalField.ifft``); the copy is a strided device gather.
"""
import numpy as np
import torch

from .field import DirectField, ReciprocalField
from .grid import DirectGrid, ReciprocalGrid


def grid_map_index(nr, nr2, full=False):
    """Where the coarse spectrum's entries sit in the fine one
    (``grid_map_index``, ``utils.py:51-78``).  ``nr`` and ``nr2`` are the two
    spectra's shapes (``nrG``).  Returns one index vector per axis (the
    mapping is separable) and ``lfine``: True when ``nr2`` is the fine
    spectrum.  Entries above half the coarse size (negative frequencies) move
    to the top of the fine axis; the half axis of a half spectrum keeps its
    indices."""
    nr_coarse = np.array(nr, dtype=int)
    nr_fine = np.array(nr2, dtype=int)
    lfine = True
    if np.all(nr_fine < nr_coarse):
        nr_coarse, nr_fine = nr_fine, nr_coarse
        lfine = False
    elif np.all(nr_fine > nr_coarse) or np.prod(nr_fine) > np.prod(nr_coarse):
        pass
    else:
        lfine = False
        nr_coarse, nr_fine = nr_fine, nr_coarse
    nr_coarse = np.minimum(nr_fine, nr_coarse)
    dnr = nr_coarse.copy()
    if full:
        dnr[:3] = nr_coarse[:3] // 2
    else:
        dnr[:2] = nr_coarse[:2] // 2
    index = []
    for i in range(3):
        idx = np.arange(nr_coarse[i])
        idx[idx > dnr[i]] += nr_fine[i] - nr_coarse[i]
        index.append(idx)
    return index, lfine


def _hermitian_planes(X, n2):
    """Make the k2 = 0 (and, for even n2, k2 = n2/2) planes of a half
    spectrum Hermitian: X(k0, k1) <- (X(k0, k1) + conj X(-k0, -k1)) / 2.  A
    real inverse transform keeps only that part of those planes, so this is
    what a C2R transform of the unsymmetrised spectrum computes."""
    planes = [0] + ([n2 // 2] if n2 % 2 == 0 and n2 // 2 < X.shape[2] else [])
    for p in planes:
        P = X[:, :, p]
        partner = torch.roll(torch.flip(P, dims=(0, 1)), shifts=(1, 1), dims=(0, 1)).conj()
        X[:, :, p] = 0.5 * (P + partner)
    return X


def grid_map_data(data, nr=None, direct=True, index=None, grid=None):
    """Spectrum of ``data`` copied onto a grid of ``nr`` points (or onto
    ``grid``) (``grid_map_data``, ``utils.py:80-129``): zero-padding when the
    new grid is finer, truncation when coarser.  Returns the real-space field
    (``direct=True``) or the reciprocal field on the new grid."""
    value = data.fft() if isinstance(data, DirectField) else data
    src_grid = value.grid
    if value.rank != 1:
        return [grid_map_data(v, nr, direct, index, grid) for v in value]
    full = src_grid.full
    if grid is not None:
        dgrid = grid.get_direct() if isinstance(grid, ReciprocalGrid) else grid
    else:
        dgrid = DirectGrid(lattice=src_grid.get_direct().lattice, nr=nr, full=full)
    if dgrid.full != full:
        raise AttributeError("Cannot mapping half and full grid.")
    rgrid = dgrid.get_reciprocal()
    nr1_g, nr2_g = np.array(src_grid.nrG), np.array(rgrid.nrG)
    idx, lfine = grid_map_index(nr1_g, nr2_g, full=full)
    bd = np.minimum(nr1_g, nr2_g)
    X = value.as_subclass(torch.Tensor)
    out = torch.zeros(tuple(int(x) for x in nr2_g), dtype=X.dtype, device=X.device)
    ix = [torch.as_tensor(i, device=X.device) for i in idx]
    if lfine:
        out[ix[0][:, None, None], ix[1][None, :, None], ix[2][None, None, :]] = X[:bd[0], :bd[1], :bd[2]]
    else:
        out[:bd[0], :bd[1], :bd[2]] = X[ix[0][:, None, None], ix[1][None, :, None], ix[2][None, None, :]]
    if not full:
        out = _hermitian_planes(out, int(dgrid.nrR[2]))
    value2 = ReciprocalField(rgrid, data=out)
    return value2.ifft(force_real=True) if direct else value2


def field2distrib(data, out, root=None, tol=1e-30):
    """Copy ``data`` into ``out`` (``field2distrib``, ``utils.py:218-287``, one
    process): equal grids copy (summing or splitting spin channels when the
    ranks differ); different grids interpolate the spectrum
    (``grid_map_data``) and clamp the result below at ``tol``."""
    rank, rank_in = out.rank, data.rank
    same = np.all(np.asarray(out.grid.nrR) == np.asarray(data.grid.nrR))
    if not same:
        if rank == 1 and rank_in > 1:
            data = DirectField(data.grid, data=data.as_subclass(torch.Tensor).sum(dim=0))
            rank_in = 1
        items = [data] if rank_in == 1 else [DirectField(data.grid, data=d) for d in data.as_subclass(torch.Tensor)]
        mapped = []
        for item in items:
            v = grid_map_data(item, grid=out.grid).as_subclass(torch.Tensor)
            mapped.append(torch.clamp(v, min=tol))
        data = mapped[0] if rank_in == 1 else torch.stack(mapped)
    else:
        data = data.as_subclass(torch.Tensor)
    dst = out.as_subclass(torch.Tensor)
    if rank == rank_in:
        dst.copy_(data.to(dst.dtype))
    elif rank == 1 and rank_in > 1:
        dst.copy_(data.sum(dim=0).to(dst.dtype))
    elif rank_in == 1 and rank > 1:
        for i in range(rank):
            dst[i].copy_((data / rank).to(dst.dtype))
    else:
        raise AttributeError("The two fields with different rank can not interpolate({})".format(tuple(out.shape)))
    return out
