"""(r, z) histograms of the structure factor: measure_intensity.py.

``measure_intensity.py`` (lines 58-125) re-expresses the centred q grid in
the reciprocal basis of the cell, interpolates S there, bins every voxel by
r = sqrt(qx^2 + qy^2) and qz with ``numpy.histogram2d`` (edges: the grid's
own x and z axes), divides the weighted histogram by the counts and mirrors
the r < 0 half; plot2d.py:1035-1147 repeats the steps (with a
nearest-neighbour interpolator for non-orthorhombic cells) after an
``exit()``.  The per-voxel work runs in libmsf (``msf_rz_hist``); the host
does the 3x3 basis, the edge checks and the small 2-D post-processing.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from ._lib import c_p, call
from .api import _ptr, check_axes, to_device
from .plan import stream_ptr

WEIGHTS = {"linear": 0, "self": 1}


def reciprocal_rows(ucell):
    """b1, b2, b3 of measure_intensity.py:51-53 (plot2d.py:1037-1039)."""
    u = np.asarray(ucell, np.float64)
    a1, a2, a3 = u[0], u[1], u[2]
    b1 = (np.cross(a2, a3)) / (np.dot(a1, np.cross(a2, a3)))
    b2 = (np.cross(a3, a1)) / (np.dot(a2, np.cross(a3, a1)))
    b3 = (np.cross(a1, a2)) / (np.dot(a3, np.cross(a1, a2)))
    return np.ascontiguousarray(np.vstack((b1, b2, b3)))


def _edges(e, name):
    e = np.ascontiguousarray(np.asarray(e, np.float64))
    if e.ndim != 1 or e.size < 2:
        raise ValueError(f"{name} edges must be a 1-D array of at least 2 values")
    if np.any(e[:-1] > e[1:]):
        raise ValueError(f"`bins[{0 if name == 'r' else 1}]` must be monotonically increasing, when an array")
    return e


def rz_histogram(S, X, Y, Z, ucell, r_edges=None, z_edges=None, weights="linear", density=False):
    """(Hval, Hcount, r_edges, z_edges): numpy.histogram2d(r, qz, bins=(r_edges,
    z_edges), weights=w, density=density) and the unweighted counts, over
    every voxel of the centred S (p0, p1, p2) CUDA float64 with axes X, Y, Z
    moved to the reciprocal basis of ``ucell``.  weights="linear": S
    interpolated there (measure_intensity.py:92, plot2d.py:1080); "self":
    each voxel's own S (plot2d.py:1093-1101 at its own nodes).  Default edges
    (X, Z) as measure_intensity.py:114."""
    if weights not in WEIGHTS:
        raise ValueError("weights must be 'linear' or 'self'")
    X = np.ascontiguousarray(np.asarray(X, np.float64))
    Y = np.ascontiguousarray(np.asarray(Y, np.float64))
    Z = np.ascontiguousarray(np.asarray(Z, np.float64))
    if weights == "linear":
        check_axes(X, Y, Z)
    re = _edges(X if r_edges is None else r_edges, "r")
    ze = _edges(Z if z_edges is None else z_edges, "z")
    dev = S.device
    S = S.to(torch.float64).contiguous()
    p0, p1, p2 = S.shape
    if (len(X), len(Y), len(Z)) != (p0, p1, p2):
        raise ValueError("axes must match the grid shape")
    b = reciprocal_rows(ucell)
    nr, nz = len(re) - 1, len(ze) - 1
    with torch.cuda.device(dev):
        hval = torch.zeros((nr, nz), dtype=torch.float64, device=dev)
        hcount = torch.zeros((nr, nz), dtype=torch.int64, device=dev)
        Xd, Yd, Zd, red, zed = (to_device(a, dev) for a in (X, Y, Z, re, ze))
        call("msf_rz_hist", _ptr(S), p0, p1, p2, _ptr(Xd), _ptr(Yd), _ptr(Zd), c_p(b.ctypes.data),
             WEIGHTS[weights], _ptr(red), len(re), _ptr(zed), len(ze), _ptr(hval), _ptr(hcount), stream_ptr(dev))
        H = hval.cpu().numpy()
        C = hcount.cpu().numpy().astype(np.float64)   # histogramdd returns float counts
    if density:
        H = to_density(H, re, ze)
    return H, C, re, ze


def to_density(H, re, ze):
    """numpy.histogramdd(density=True) from the raw sums: divided by the bin
    widths along r, then along z, then by the total."""
    s = H.sum()
    H = H / np.diff(re).reshape(len(re) - 1, 1)
    H = H / np.diff(ze).reshape(1, len(ze) - 1)
    H /= s
    return H


def rz_average(Hval, Hcount, mirror=True):
    """Hrz of measure_intensity.py:118-125: Hval / max(Hcount, 1) per bin,
    then row nr//2 - i := row nr//2 + 1 + i for i < nr//2 (r < 0 mirrored
    from r > 0)."""
    Hcount = np.where(Hcount == 0, 1, Hcount)
    Hrz = Hval / Hcount
    if mirror:
        h = Hrz.shape[0] // 2
        for ir in range(h):
            Hrz[-ir + h, :] = Hrz[ir + 1 + h, :]
    return Hrz


MI_THETA = math.pi / 3.0   # measure_intensity.py:41


def measure_intensity(kgridplt, box=(63, 73, 60, 40), full=False, device=None):
    """measure_intensity.py run non-interactively (``-y``): the (r, z) map of
    the kgridplt array (numpy (p0, p1, p2, 4)) in the theta = 60 degree cell
    of measure_intensity.py:41-42, normed as the script asks
    (``histogram2d(..., normed=True)``, numpy's density), and the average
    and maximum of Hrz.T inside the crop box (left, right, top, bottom) or
    the whole map (``full``).  Returns (Iavg, Imax, Hrz)."""
    D = np.asarray(kgridplt, np.float64)
    X = D[:, 0, 0, 0].copy()
    Y = D[0, :, 0, 1].copy()
    Z = D[0, 0, :, 2].copy()
    ucell = np.array([[1, 0, 0], [np.cos(MI_THETA), np.sin(MI_THETA), 0], [0, 0, 1]])
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    S = to_device(np.ascontiguousarray(D[..., 3]), dev)
    Hval, Hcount, re, ze = rz_histogram(S, X, Y, Z, ucell, weights="linear")
    with np.errstate(invalid="ignore", divide="ignore"):
        Hrz = rz_average(to_density(Hval, re, ze), Hcount)
    if full:
        lx, by, rx, ty = 0, 0, Hrz.shape[0], Hrz.shape[1]
    else:
        lx, rx, ty, by = (int(v) for v in box)
    crop = Hrz.T[by:ty, lx:rx]
    with np.errstate(invalid="ignore"):
        return np.mean(crop), np.amax(crop), Hrz


def lattice_params(X, Y, Z, ucell):
    """The 28 doubles msf_nearest_sheared takes: reciprocal rows (9), the
    first node (3), the inverse of the step lattice M (rows dX b1, dY b2,
    dZ b3; 9), a bound on how far a node lies from its uniform-lattice model
    (the axes' largest deviations from equal steps times |b_a|, summed, with
    a margin for the rounding of the node arithmetic; 1), and the upper
    Cholesky factor R of M M^T = R^T R (R00 R01 R02 R11 R12 R22; 6)."""
    X, Y, Z = (np.asarray(a, np.float64) for a in (X, Y, Z))
    b = reciprocal_rows(ucell)
    o = (X[0] * b[0] + Y[0] * b[1]) + Z[0] * b[2]
    axes = (X, Y, Z)
    steps = [(a[-1] - a[0]) / (len(a) - 1) if len(a) > 1 else 1.0 for a in axes]
    M = np.vstack([steps[i] * b[i] for i in range(3)])
    minv = np.linalg.inv(M)
    dev = sum(np.max(np.abs(a - (a[0] + np.arange(len(a)) * steps[i]))) * np.linalg.norm(b[i])
              for i, a in enumerate(axes))
    scale = sum(np.max(np.abs(a)) * np.linalg.norm(b[i]) for i, a in enumerate(axes))
    delta = 2.0 * dev + 1e-12 * scale
    R = np.linalg.cholesky(M @ M.T).T
    r = [R[0, 0], R[0, 1], R[0, 2], R[1, 1], R[1, 2], R[2, 2]]
    return np.ascontiguousarray(np.concatenate([b.ravel(), o, minv.ravel(), [delta], r]))


def nearest_sheared(S, X, Y, Z, ucell, points, return_index=False):
    """NearestNDInterpolator(transformed nodes, S.ravel())(points) of
    plot2d.py:1087-1101 on the GPU: S (p0, p1, p2) CUDA float64 with axes
    X, Y, Z, nodes moved to the reciprocal basis of ``ucell``; points (m, 3)
    numpy or CUDA float64.  Returns a CUDA float64 (m,) tensor (and the
    nodes' flat indices)."""
    dev = S.device
    S = S.to(torch.float64).contiguous()
    p0, p1, p2 = S.shape
    if (len(X), len(Y), len(Z)) != (p0, p1, p2):
        raise ValueError("axes must match the grid shape")
    lat = lattice_params(X, Y, Z, ucell)
    if not np.all(np.isfinite(lat)):
        raise ValueError("the sheared lattice is singular or not finite")
    with torch.cuda.device(dev):
        q = to_device(points, dev, torch.float64).reshape(-1, 3).contiguous()
        m = q.shape[0]
        out = torch.empty(m, dtype=torch.float64, device=dev)
        idx = torch.empty(m, dtype=torch.int64, device=dev) if return_index else None
        Xd, Yd, Zd = (to_device(np.ascontiguousarray(np.asarray(a, np.float64)), dev) for a in (X, Y, Z))
        call("msf_nearest_sheared", _ptr(S), p0, p1, p2, _ptr(Xd), _ptr(Yd), _ptr(Zd), c_p(lat.ctypes.data),
             _ptr(q), m, _ptr(out), _ptr(idx) if idx is not None else c_p(0), stream_ptr(dev))
    return (out, idx) if return_index else out
