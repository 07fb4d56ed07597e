"""The sheared-grid nearest-node search of msf_post.cu (k_nearest: a
Fincke-Pohst enumeration of the lattice points within the distance bound,
intersected with the grid), modelled in numpy and checked against the
KD-tree of plot2d.py:1087-1101 (scipy's NearestNDInterpolator) for queries
inside, around and far outside the grid, with equal and unequal axis steps.
No GPU."""
import math

import numpy as np
import pytest

from mdsf import rz as mrz
from mdsf.api import plot_axes
from oracle import rz as orz

K_REL, K_ABS = 1.0 + 1e-9, 1e-6


def cell(theta_deg):
    th = theta_deg * np.pi / 180.0
    return np.array([[1, 0, 0], [np.cos(th), np.sin(th), 0], [0, 0, 1]])


def clamp(r, n):
    return 0 if not r >= 0.0 else (n - 1 if r >= n - 1 else int(r))


def model_nearest(q, nodes, shape, lat):
    """k_nearest for one query: (flat index, candidates evaluated)."""
    o, minv, delta = lat[9:12], lat[12:21].reshape(3, 3), lat[21]
    R00, R01, R02, R11, R12, R22 = lat[22:28]
    n = shape
    f = (q - o) @ minv
    c = [clamp(float(np.rint(f[k])), n[k]) for k in range(3)]

    def d2(i, j, k):
        d = nodes[i, j, k] - q
        return (d[0] * d[0] + d[1] * d[1]) + d[2] * d[2]
    best = d2(*c)
    bi = (c[0] * n[1] + c[1]) * n[2] + c[2]
    rad = math.sqrt(best) + delta
    count = 0
    w2 = rad * K_REL / R22
    for i2 in range(clamp(math.floor(f[2] - w2 - K_ABS), n[2]), clamp(math.ceil(f[2] + w2 + K_ABS), n[2]) + 1):
        u2 = i2 - f[2]
        t2 = R22 * u2
        r1sq = rad * rad * K_REL - t2 * t2
        if r1sq < 0:
            continue
        r1 = math.sqrt(r1sq)
        cen1 = f[1] - R12 * u2 / R11
        for i1 in range(clamp(math.floor(cen1 - r1 / R11 - K_ABS), n[1]),
                        clamp(math.ceil(cen1 + r1 / R11 + K_ABS), n[1]) + 1):
            u1 = i1 - f[1]
            t1 = R11 * u1 + R12 * u2
            r0sq = rad * rad * K_REL - t2 * t2 - t1 * t1
            if r0sq < 0:
                continue
            r0 = math.sqrt(r0sq)
            cen0 = f[0] - (R01 * u1 + R02 * u2) / R00
            for i0 in range(clamp(math.floor(cen0 - r0 / R00 - K_ABS), n[0]),
                            clamp(math.ceil(cen0 + r0 / R00 + K_ABS), n[0]) + 1):
                count += 1
                dd = d2(i0, i1, i2)
                fi = (i0 * n[1] + i1) * n[2] + i2
                if dd < best or (dd == best and fi < bi):
                    best, bi = dd, fi
                    rad = math.sqrt(best) + delta
    return bi, count


@pytest.mark.parametrize("theta", [120.0, 60.0, 90.0, 45.0])
@pytest.mark.parametrize("jitter", [0.0, 0.3])
def test_enumeration_finds_the_kdtree_node(theta, jitter):
    shape = (14, 16, 11)
    rng = np.random.default_rng(int(theta) + int(10 * jitter))
    X, Y, Z = plot_axes((shape[0] + 2, shape[1] + 2, (shape[2] + 3) // 2), np.array([9.0, 8.0, 6.0]))
    if jitter:   # unequal steps: the radius widens by the axes' deviation
        X = np.sort(X + rng.uniform(-jitter, jitter, len(X)) * (X[1] - X[0]))
    D = np.zeros(shape + (4,))
    D[..., 0], D[..., 1], D[..., 2] = X[:, None, None], Y[None, :, None], Z[None, None, :]
    uc = cell(theta)
    pts, _ = orz.transformed_points(D.copy(), uc)
    nodes = pts.reshape(shape + (3,))
    lo, hi = pts.min(axis=0), pts.max(axis=0)
    span = hi - lo
    q = np.concatenate([rng.uniform(lo, hi, (600, 3)),                            # inside and around
                        rng.uniform(lo - 1.5 * span, hi + 1.5 * span, (600, 3)),  # far outside too
                        pts[rng.integers(0, len(pts), 100)]])                     # on nodes
    _, idx = orz.nearest_sheared(D, uc, q)
    lat = mrz.lattice_params(X, Y, Z, uc)
    counts = []
    for k in range(len(q)):
        bi, cnt = model_nearest(q[k], nodes, shape, lat)
        assert bi == idx[k]
        counts.append(cnt)
    if not jitter:
        assert np.median(counts[:600]) <= 27
