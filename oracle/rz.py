"""Oracle: the (r, z) histograms of measure_intensity.py.

TEST INFRASTRUCTURE ONLY -- see ``oracle/__init__.py``.

Restates measure_intensity.py:45-125: axes X, Y, Z of the kgridplt array;
reciprocal rows b1, b2, b3 of ``ucell`` (lines 51-53); every voxel moved to
X b1 + Y b2 + Z b3, accumulated per axis in the script's order (lines
55-64); S interpolated there by ``RegularGridInterpolator((X, Y, Z), S,
bounds_error=False)`` (line 92); r = sqrt(x^2 + y^2) (line 112);
``histogram2d(r, z, bins=(X, Z))`` counts and weighted sums (lines
114-116); Hrz = sums / counts with empty bins counted as 1; the r < 0 rows
mirrored (lines 124-125).  The script passes ``normed=``, which numpy removed
in 1.24; ``density=`` is the same histogramdd option under its current name.
``weights="self"`` takes each voxel's own S instead: what plot2d.py's
NearestNDInterpolator over the transformed grid (plot2d.py:1093-1101)
returns at its own nodes.
"""
from __future__ import annotations

import numpy as np
from scipy.interpolate import RegularGridInterpolator


def reciprocal_rows(ucell):
    a1, a2, a3 = ucell[0], ucell[1], ucell[2]
    b1 = (np.cross(a2, a3)) / (np.dot(a1, np.cross(a2, a3)))
    b2 = (np.cross(a3, a1)) / (np.dot(a2, np.cross(a3, a1)))
    b3 = (np.cross(a1, a2)) / (np.dot(a3, np.cross(a1, a2)))
    return b1, b2, b3


def transformed_points(D, ucell):
    """measure_intensity.py:45-64, 95-107: (N, 3) points in C order."""
    X = D[:, 0, 0, 0].copy()
    Y = D[0, :, 0, 1].copy()
    Z = D[0, 0, :, 2].copy()
    b1, b2, b3 = reciprocal_rows(np.asarray(ucell, np.float64))
    Dnew = np.zeros_like(D)
    for ix in range(D.shape[0]):
        Dnew[ix, :, :, 0:3] += X[ix] * b1
    for iy in range(D.shape[1]):
        Dnew[:, iy, :, 0:3] += Y[iy] * b2
    for iz in range(D.shape[2]):
        Dnew[:, :, iz, 0:3] += Z[iz] * b3
    return Dnew[..., :3].reshape(-1, 3), (X, Y, Z)


def rz_histogram(D, ucell, r_edges=None, z_edges=None, weights="linear", density=False):
    """(Hval, Hcount, rpts, zpts, w): the two histogram2d results and their inputs."""
    pts, (X, Y, Z) = transformed_points(D, ucell)
    SF = D[:, :, :, 3]
    if weights == "linear":
        w = RegularGridInterpolator((X, Y, Z), SF, bounds_error=False)(pts)
    else:
        w = SF.reshape(-1).copy()
    rpts = np.sqrt(pts[:, 0] ** 2.0 + pts[:, 1] ** 2.0)
    bins = (X if r_edges is None else r_edges, Z if z_edges is None else z_edges)
    Hcount, _, _ = np.histogram2d(rpts, pts[:, 2], bins=bins)
    Hval, _, _ = np.histogram2d(rpts, pts[:, 2], weights=w, density=density, bins=bins)
    return Hval, Hcount, rpts, pts[:, 2], w


def rz_average(Hval, Hcount):
    """measure_intensity.py:118-125."""
    Hcount = np.where(Hcount == 0, 1, Hcount)
    Hrz = Hval / Hcount
    for ir in range(Hrz.shape[0] // 2):
        Hrz[-ir + Hrz.shape[0] // 2, :] = Hrz[ir + 1 + Hrz.shape[0] // 2, :]
    return Hrz


def nearest_sheared(D, ucell, points):
    """plot2d.py:1087-1101: NearestNDInterpolator over the transformed nodes
    (the non-orthorhombic branch), evaluated at ``points``; also the nodes'
    flat indices from the same KD-tree query."""
    from scipy.interpolate import NearestNDInterpolator
    pts, _ = transformed_points(D.copy(), ucell)
    coords = list(zip(pts[:, 0], pts[:, 1], pts[:, 2]))
    ES = NearestNDInterpolator(coords, D[:, :, :, 3].ravel())
    vals = ES(points)
    _, idx = ES.tree.query(points)
    return vals, idx
