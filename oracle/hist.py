"""Oracle: electron-weighted histogram -> rfftn -> |F|^2 -> FP64 frame sum.

TEST INFRASTRUCTURE ONLY -- see ``oracle/__init__.py``.

The reference deposits a Gaussian per atom (dens.py:283-311); the plain
method of this build bins each atom's integer electron count into the voxel
that ``numpy.histogramdd`` assigns it to and then follows the reference's
FFT path unchanged (dens.py:313-318: ``np.fft.rfftn``, ``conj(F)*F``,
``sf += dmag`` with no division by the frame count).

Binning semantics are numpy's (``numpy/lib/_histograms_impl.py``,
``histogramdd``): per axis the edges are ``np.linspace(0, L, n+1)`` in
float64, the bin is ``searchsorted(edges, x, side='right') - 1``, a value
equal to the last edge goes to the last bin, and values below 0, above L or
NaN are dropped.  Optional pre-processing follows the reference:
``rescale`` (dens.py:46-62) when a per-frame box is given and ``wrap``
(dens.py:204-221) when asked.
"""
from __future__ import annotations

import numpy as np


def frame_scale(box):
    """Per-frame rescale factors and the mean box, as dens.py:52-53.

    ``box`` is (3,) (returns scale ones) or (T, 3).
    """
    box = np.asarray(box, dtype=np.float64)
    if box.ndim == 1:
        return None, box
    avg = np.average(box, axis=0)
    return avg / box, avg


def prepare(pos_t, scale_t, L, wrap):
    """FP64 positions of one frame after the reference's rescale and wrap."""
    x = np.asarray(pos_t).astype(np.float64)
    if scale_t is not None:
        x = x * scale_t
    if wrap:
        x = np.where(x < L, x, x - L)
        x = np.where(x > 0.0, x, x + L)
    return x


def hist_grid(pos_t, L, weights, dims, scale_t=None, wrap=False):
    """int64 grid of one frame: ``np.histogramdd`` with electron weights."""
    x = prepare(pos_t, scale_t, L, wrap)
    H, _ = np.histogramdd(x, bins=[int(d) for d in dims],
                          range=[(0.0, float(L[i])) for i in range(3)],
                          weights=np.asarray(weights, dtype=np.float64))
    return H.astype(np.int64)


def bin_index(x, L, n):
    """Per-axis bin of FP64 values with histogramdd semantics (-1 = dropped)."""
    edges = np.linspace(0.0, float(L), int(n) + 1)
    b = np.searchsorted(edges, x, side='right')
    b = np.where(x == edges[-1], b - 1, b)
    b = b - 1
    return np.where((b >= 0) & (b < n) & ~np.isnan(x), b, -1)


def power(grid):
    """|rfftn(grid)|^2 in FP64, dens.py:313-316."""
    F = np.fft.rfftn(np.asarray(grid, dtype=np.float64))
    return (F.real * F.real + F.imag * F.imag)


def hist_sf(positions, box, weights, dims, wrap=False, return_grids=False):
    """Sum over frames of |F|^2 of the weighted histogram (dens.py:277-318).

    positions (T, N, 3) or (N, 3); box (3,) or (T, 3); weights (N,) ints.
    """
    pos = np.asarray(positions)
    if pos.ndim == 2:
        pos = pos[None]
    scale, L = frame_scale(box)
    dims = [int(d) for d in dims]
    sf = np.zeros((dims[0], dims[1], dims[2] // 2 + 1))
    grids = []
    for t in range(pos.shape[0]):
        g = hist_grid(pos[t], L, weights, dims, None if scale is None else scale[t], wrap)
        if return_grids:
            grids.append(g)
        sf += power(g)
    if return_grids:
        return sf, grids
    return sf
