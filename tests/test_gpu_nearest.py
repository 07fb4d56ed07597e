"""Nearest node of the sheared grid (plot2d.py:1087-1101,
NearestNDInterpolator over the transformed kgridplt) on the GPU against
scipy's KD-tree: the same node for every query (random queries: no ties)."""
import numpy as np
import pytest
import torch

from mdsf import rz as mrz
from mdsf.api import plot_axes
from oracle import rz as orz

pytestmark = pytest.mark.gpu


def cell(theta_deg, c=1.0):
    th = theta_deg * np.pi / 180.0
    return np.array([[1, 0, 0], [np.cos(th), np.sin(th), 0], [0, 0, c]])


@pytest.mark.parametrize("theta", [120.0, 60.0, 90.0, 100.0, 75.0])
@pytest.mark.parametrize("shape,L", [((20, 24, 17), (9.0, 8.0, 6.0)), ((46, 38, 29), (15.0, 13.0, 10.0))])
def test_nearest_matches_scipy(theta, shape, L):
    rng = np.random.default_rng(int(theta) + shape[0])
    X, Y, Z = plot_axes((shape[0] + 2, shape[1] + 2, (shape[2] + 3) // 2), np.asarray(L))
    S = rng.gamma(2.0, 5.0, shape)
    D = np.zeros(shape + (4,))
    D[..., 0], D[..., 1], D[..., 2] = X[:, None, None], Y[None, :, None], Z[None, None, :]
    D[..., 3] = S
    uc = cell(theta)
    nodes, _ = orz.transformed_points(D.copy(), uc)
    lo, hi = nodes.min(axis=0), nodes.max(axis=0)
    span = hi - lo
    q = np.concatenate([rng.uniform(lo - 0.1 * span, hi + 0.1 * span, (4000, 3)),   # inside and around
                        rng.uniform(lo - 1.5 * span, hi + 1.5 * span, (1000, 3)),   # far outside
                        nodes[rng.integers(0, len(nodes), 500)] + rng.normal(0, 1e-3, (500, 3)),
                        nodes[rng.integers(0, len(nodes), 200)]])                     # on nodes
    want, widx = orz.nearest_sheared(D, uc, q)
    got, gidx = mrz.nearest_sheared(torch.from_numpy(S).cuda(), X, Y, Z, uc, q, return_index=True)
    np.testing.assert_array_equal(gidx.cpu().numpy(), widx)
    np.testing.assert_array_equal(got.cpu().numpy(), want)


def test_nearest_with_unequal_axis_steps():
    """Axes with unequal steps: the candidate box widens by their deviation
    from the uniform lattice and still holds scipy's node."""
    rng = np.random.default_rng(12)
    shape = (24, 20, 17)
    X, Y, Z = plot_axes((26, 22, 10), np.array([9.0, 8.0, 6.0]))
    X = np.sort(X + rng.uniform(-0.3, 0.3, len(X)) * (X[1] - X[0]))
    Z = np.sort(Z + rng.uniform(-0.2, 0.2, len(Z)) * (Z[1] - Z[0]))
    S = rng.uniform(0, 1, shape)
    D = np.zeros(shape + (4,))
    D[..., 0], D[..., 1], D[..., 2] = X[:, None, None], Y[None, :, None], Z[None, None, :]
    D[..., 3] = S
    uc = cell(120.0)
    nodes, _ = orz.transformed_points(D.copy(), uc)
    lo, hi = nodes.min(axis=0), nodes.max(axis=0)
    q = rng.uniform(lo, hi, (5000, 3))
    want, widx = orz.nearest_sheared(D, uc, q)
    got, gidx = mrz.nearest_sheared(torch.from_numpy(S).cuda(), X, Y, Z, uc, q, return_index=True)
    np.testing.assert_array_equal(gidx.cpu().numpy(), widx)
    np.testing.assert_array_equal(got.cpu().numpy(), want)


def test_nearest_at_own_nodes_is_identity_and_nan_query():
    shape = (12, 10, 9)
    X, Y, Z = plot_axes((14, 12, 6), np.array([6.0, 5.0, 4.0]))
    S = np.arange(np.prod(shape), dtype=np.float64).reshape(shape)
    D = np.zeros(shape + (4,))
    D[..., 0], D[..., 1], D[..., 2] = X[:, None, None], Y[None, :, None], Z[None, None, :]
    D[..., 3] = S
    nodes, _ = orz.transformed_points(D, cell(120.0))
    got = mrz.nearest_sheared(torch.from_numpy(S).cuda(), X, Y, Z, cell(120.0), nodes).cpu().numpy()
    np.testing.assert_array_equal(got, S.ravel())
    bad = np.array([[np.nan, 0.0, 0.0], [0.0, np.inf, 0.0], [0.0, 0.0, -np.inf], [0.1, 0.2, 0.3]])
    got, idx = mrz.nearest_sheared(torch.from_numpy(S).cuda(), X, Y, Z, cell(120.0), bad, return_index=True)
    got, idx = got.cpu().numpy(), idx.cpu().numpy()
    assert np.all(np.isnan(got[:3])) and np.all(idx[:3] == -1)
    want, widx = orz.nearest_sheared(D, cell(120.0), bad[3:])
    assert got[3] == want[0] and idx[3] == widx[0]


def test_singular_cell_raises():
    X, Y, Z = plot_axes((8, 8, 5), np.array([4.0, 4.0, 4.0]))
    S = torch.zeros((6, 6, 7), dtype=torch.float64, device="cuda")
    flat = np.array([[1, 0, 0], [1, 0, 0], [0, 0, 1.0]])
    with pytest.raises(Exception):
        mrz.nearest_sheared(S, X, Y, Z, flat, np.zeros((1, 3)))
