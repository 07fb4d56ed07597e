"""Oracle: cylindrical (r, z) average of the structure factor.

TEST INFRASTRUCTURE ONLY -- see ``oracle/__init__.py``.

Restates the averaging part of ``plot2d.PLOT_RAD_NEW`` (plot2d.py:559-640),
the step the reference CLI runs after ``compute_sf`` (main_gromacs.py:231 ->
plot2d.py:1008-1011): the centred S(q) of ``kgridplt`` is interpolated
(linear, NaN outside, plot2d.py:584) on rings of 400 radii up to 0.95 of
half the smaller in-plane q extent, with max(int(20 * 2 pi r), 1) angles per
ring, at every z of the grid; points are mapped through the inverse of the
reciprocal basis of ``ucell`` (plot2d.py:595-603, 631); each ring's values
are averaged over angle; NaNs become the smallest average; the array is
divided by its mean unless ``format``; and it is mirrored to (-r, r).
"""
from __future__ import annotations

import numpy as np
from scipy.interpolate import RegularGridInterpolator

THETA_BINS_PER_INV_ANG = 20.0   # plot2d.py:586
MIN_THETA_BINS = 1              # plot2d.py:587
RBINS = 400                     # plot2d.py:588


def b_inverse(ucell):
    """Inverse of the stacked reciprocal vectors, plot2d.py:591-599."""
    a1, a2, a3 = ucell[0], ucell[1], ucell[2]
    b1 = (np.cross(a2, a3)) / (np.dot(a1, np.cross(a2, a3)))
    b2 = (np.cross(a3, a1)) / (np.dot(a2, np.cross(a3, a1)))
    b3 = (np.cross(a1, a2)) / (np.dot(a3, np.cross(a1, a2)))
    return np.linalg.inv(np.vstack((b1, b2, b3)))


def rings(X, Y, Z, ucell):
    """Radii, z values and angle counts, plot2d.py:601-618."""
    XR = (X[-1] - X[0]) * ucell[0][0]
    YR = (Y[-1] - Y[0]) * ucell[1][1]
    Rmax = min(XR, YR) / 2.0
    Rmax *= 0.95
    rarr, _ = np.linspace(0.0, Rmax, RBINS, retstep=True)
    zar = np.linspace(Z[0], Z[-1], Z.shape[0])
    circ = 2. * np.pi * rarr
    nth = np.array([max(int(THETA_BINS_PER_INV_ANG * c), MIN_THETA_BINS) for c in circ])
    return rarr, zar, nth


def cylindrical_average(D, ucell, format=False):
    """(final, rfin, zfin, oa) as PLOT_RAD_NEW builds them (plot2d.py:578-645)."""
    X = D[:, 0, 0, 0]
    Y = D[0, :, 0, 1]
    Z = D[0, 0, :, 2]
    ES = RegularGridInterpolator((X, Y, Z), D[..., 3], bounds_error=False)
    b_inv = b_inverse(np.asarray(ucell, dtype=np.float64))
    rarr, zar, nth = rings(X, Y, Z, ucell)
    oa = np.zeros((rarr.shape[0], zar.shape[0]))
    for ir in range(rarr.shape[0]):
        thetas = np.linspace(0.0, np.pi * 2.0, nth[ir], endpoint=False)
        t, r, z = np.meshgrid(thetas, rarr[ir], zar)
        pts = np.vstack(((r * np.cos(t)).ravel(), (r * np.sin(t)).ravel(), z.ravel())).T
        oa[ir, :] = np.average(ES(np.matmul(pts, b_inv)).reshape(r.shape), axis=1)
    mn = np.nanmin(oa)
    oa = np.where(np.isnan(oa), mn, oa)
    if not format:
        oa /= np.average(oa)
    final = np.append(oa[::-1, :], oa[1:], axis=0)
    rfin = np.append(-rarr[::-1], rarr[1:])
    return final, rfin, zar, oa
