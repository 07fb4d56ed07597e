"""Oracle: Ewald-sphere slices of the centred structure factor.

TEST INFRASTRUCTURE ONLY -- see ``oracle/__init__.py``.

Restates ``plot2d.Plot_Ewald_Sphere_Correction`` (plot2d.py:218-267) without
its plotting: a linear ``scipy.interpolate.RegularGridInterpolator`` over the
``kgridplt`` axes (NaN outside, plot2d.py:234) is sampled, for every point
(a, b) of the xy, xz and yz planes, at the point of the Ewald sphere of
radius K = 2*pi/lambda above it: theta = atan(sqrt(a^2+b^2)/K), in-plane
coordinates scaled by cos(theta), the third coordinate K*(1-cos(theta))
(plot2d.py:236-255).
"""
from __future__ import annotations

import math

import numpy as np
from scipy.interpolate import RegularGridInterpolator


def slice_points(X, Y, Z, K):
    """The three point lists of plot2d.py:236-255, as (n, 3) arrays."""
    xy, xz, yz = [], [], []
    for ix in range(len(X)):
        xsq = X[ix] ** 2.0
        for iy in range(len(Y)):
            th = np.arctan(np.sqrt(xsq + Y[iy] ** 2.0) / K)
            xy.append((X[ix] * np.cos(th), Y[iy] * np.cos(th), K * (1.0 - np.cos(th))))
    for ix in range(len(X)):
        xsq = X[ix] ** 2.0
        for iz in range(len(Z)):
            th = np.arctan(np.sqrt(xsq + Z[iz] ** 2.0) / K)
            xz.append((X[ix] * np.cos(th), K * (1.0 - np.cos(th)), Z[iz] * np.cos(th)))
    for iy in range(len(Y)):
        ysq = Y[iy] ** 2.0
        for iz in range(len(Z)):
            th = np.arctan(np.sqrt(ysq + Z[iz] ** 2.0) / K)
            yz.append((K * (1.0 - np.cos(th)), Y[iy] * np.cos(th), Z[iz] * np.cos(th)))
    return np.asarray(xy), np.asarray(xz), np.asarray(yz)


def slice_points_vec(X, Y, Z, K):
    """Vectorised form of :func:`slice_points` (same formulas, same order)."""
    def plane(A, B):
        th = np.arctan(np.sqrt((A[:, None] ** 2.0) + B[None, :] ** 2.0) / K)
        c = np.cos(th)
        return A[:, None] * c, B[None, :] * c, K * (1.0 - c)
    a, b, h = plane(X, Y)
    xy = np.stack([a, b, h], -1).reshape(-1, 3)
    a, b, h = plane(X, Z)
    xz = np.stack([a, h, b], -1).reshape(-1, 3)
    a, b, h = plane(Y, Z)
    yz = np.stack([h, a, b], -1).reshape(-1, 3)
    return xy, xz, yz


def ewald_slices(D, wavelength, vectorised=True):
    """(EWDxy, EWDxz, EWDyz) from D = kgridplt, plot2d.py:227-267."""
    X = D[:, 0, 0, 0]
    Y = D[0, :, 0, 1]
    Z = D[0, 0, :, 2]
    SF = D[:, :, :, 3]
    K = 2.0 * math.pi / wavelength
    ES = RegularGridInterpolator((X, Y, Z), SF, bounds_error=False)
    pts = (slice_points_vec if vectorised else slice_points)(X, Y, Z, K)
    xy, xz, yz = (ES(p) for p in pts)
    return (xy.reshape(D.shape[0], D.shape[1]),
            xz.reshape(D.shape[0], D.shape[2]),
            yz.reshape(D.shape[1], D.shape[2]))
