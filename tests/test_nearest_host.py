"""The candidate box of the sheared-grid nearest-node search (msf_post.cu,
k_nearest), modelled in numpy: for every query the KD-tree's nearest node
of plot2d.py:1087-1101 lies inside the box, so the exhaustive search over
the box returns it.  No GPU."""
import numpy as np
import pytest

from mdsf import rz as mrz
from mdsf.api import plot_axes
from oracle import rz as orz


def cell(theta_deg):
    th = theta_deg * np.pi / 180.0
    return np.array([[1, 0, 0], [np.cos(th), np.sin(th), 0], [0, 0, 1]])


@pytest.mark.parametrize("theta", [120.0, 60.0, 90.0, 100.0, 75.0, 45.0])
@pytest.mark.parametrize("jitter", [0.0, 0.2])
def test_search_box_holds_the_kdtree_answer(theta, jitter):
    shape = (22, 26, 15)
    rng = np.random.default_rng(int(theta))
    X, Y, Z = plot_axes((shape[0] + 2, shape[1] + 2, (shape[2] + 3) // 2), np.array([9.0, 8.0, 6.0]))
    if jitter:   # unequal steps: the box must widen by the axes' deviation
        X = np.sort(X + rng.uniform(-jitter, jitter, len(X)) * (X[1] - X[0]))
    D = np.zeros(shape + (4,))
    D[..., 0], D[..., 1], D[..., 2] = X[:, None, None], Y[None, :, None], Z[None, None, :]
    D[..., 3] = rng.uniform(0, 1, shape)
    uc = cell(theta)
    nodes, _ = orz.transformed_points(D.copy(), uc)
    lo, hi = nodes.min(axis=0), nodes.max(axis=0)
    q = rng.uniform(lo - 0.2 * (hi - lo), hi + 0.2 * (hi - lo), (20000, 3))
    _, idx = orz.nearest_sheared(D, uc, q)
    lat = mrz.lattice_params(X, Y, Z, uc)
    o, minv, cn, delta = lat[9:12], lat[12:21].reshape(3, 3), lat[21:24], lat[24]
    n = np.array(shape)
    f = (q - o) @ minv
    c0 = np.clip(np.rint(f), 0, n - 1).astype(int)
    p0 = nodes.reshape(shape + (3,))[c0[:, 0], c0[:, 1], c0[:, 2]]
    rho = np.sqrt(((p0 - q) ** 2).sum(axis=1))
    w = (rho[:, None] + delta) * cn[None, :] * (1.0 + 1e-9) + 1e-6
    blo = np.clip(np.floor(f - w), 0, n - 1)
    bhi = np.clip(np.ceil(f + w), 0, n - 1)
    ijk = np.stack(np.unravel_index(idx, shape), axis=1)
    assert np.all((ijk >= blo) & (ijk <= bhi))
    # with equal steps the boxes stay small for queries inside the node cloud
    if not jitter:
        inside = np.all((q >= lo) & (q <= hi), axis=1)
        assert np.median(np.prod(bhi[inside] - blo[inside] + 1, axis=1)) <= 64
