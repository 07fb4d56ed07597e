"""radial_integrate (plot2d.py:160-173) on the host, no GPU: the oracle
against the reference's own outputs, and the float16 range/edge/bin-search
arithmetic that the CUDA kernels implement, modelled in numpy and checked
against numpy.histogram itself."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from mdsf import radial as mrad
from oracle import radial as orad

CASES = ["ortho", "tcl", "corner", "wide", "flat"]


def radial_input(name):
    z = np.load(os.path.join(GOLDEN, "radial_" + name + ".npz"))
    if "source" in z.files:
        D = np.load(os.path.join(GOLDEN, str(z["source"]) + ".npz"))["out_kgridplt"]
    elif "D" in z.files:
        D = z["D"]
    else:
        X, Y, Z, S = z["X"], z["Y"], z["Z"], z["S"]
        D = np.zeros(S.shape + (4,))
        D[..., 0], D[..., 1], D[..., 2] = X[:, None, None], Y[None, :, None], Z[None, None, :]
        D[..., 3] = S
    return D, int(z["nbins"]), z


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference(name):
    D, nb, z = radial_input(name)
    E, H = orad.radial_integrate(D, nb)
    assert E.dtype == np.float16
    np.testing.assert_array_equal(E, z["E"])
    np.testing.assert_array_equal(H, z["H"])


def f16_op(a, b, op):
    """One float32 op on float16 operands, rounded to float16: the kernels'
    (and numpy's) float16 arithmetic."""
    return np.float16(op(np.asarray(a, np.float16).astype(np.float32), np.asarray(b, np.float16).astype(np.float32)))


def model_index(R, edges):
    """The CUDA bin search (msf_radial.cu, BinCtx::index) in numpy."""
    n = len(edges) - 1
    first = edges[0]
    den = f16_op(edges[n], first, np.subtract)
    fn = np.float16(np.float32(n))
    t = f16_op(R, first, np.subtract)
    t = f16_op(t, den, np.divide)
    t = f16_op(t, fn, np.multiply)
    i = t.astype(np.float32).astype(np.int64)
    i[i == n] -= 1
    i[R < edges[i]] -= 1
    inc = (R >= edges[i + 1]) & (i != n - 1)
    i[inc] += 1
    return i


def test_float16_add_is_float32_add_rounded():
    rng = np.random.default_rng(0)
    a = rng.uniform(0, 300, 200000).astype(np.float16)
    b = rng.uniform(0, 300, 200000).astype(np.float16) * np.float16(rng.choice([1, 1e-3, 1e-5], 200000))
    np.testing.assert_array_equal(a + b, f16_op(a, b, np.add))
    np.testing.assert_array_equal(a / b[b > 0].max(), f16_op(a, b[b > 0].max(), np.divide))


@pytest.mark.parametrize("nbins", [1, 7, 100, 750, 2048])
@pytest.mark.parametrize("scale", [0.3, 30.0, 400.0])
def test_bin_model_matches_numpy_histogram(nbins, scale):
    rng = np.random.default_rng(nbins + int(scale))
    q = rng.uniform(-1, 1, (60000, 3)) * np.sqrt(scale)
    R = (q[:, 0] ** 2).astype(np.float16) + (q[:, 1] ** 2).astype(np.float16) + (q[:, 2] ** 2).astype(np.float16)
    w = rng.uniform(0, 1, len(R))
    try:
        H, E = np.histogram(R, bins=nbins, weights=w)
    except ValueError:
        with pytest.raises(ValueError):
            mrad._edges(R.min(), R.max(), nbins)
        return
    edges = mrad._edges(R.min(), R.max(), nbins)
    np.testing.assert_array_equal(edges, E)
    i = model_index(R, edges)
    np.testing.assert_array_equal(np.bincount(i, minlength=nbins), np.histogram(R, bins=nbins)[0])
    np.testing.assert_array_equal(np.bincount(i, weights=w, minlength=nbins), H)


def test_edges_of_an_empty_range_and_sample():
    R = np.full(10, np.float16(0.25))
    np.testing.assert_array_equal(mrad._edges(R.min(), R.max(), 12), np.histogram(R, bins=12)[1])
    np.testing.assert_array_equal(mrad._edges(0, 1, 9), np.histogram(np.zeros(0, np.float16), bins=9)[1])
    with pytest.raises(ValueError):
        mrad._edges(np.float16(0.25), np.float16(0.25), 2000)


def test_grid_range_from_axis_extremes():
    """max/min of R over a product grid = R of the per-axis extremes."""
    rng = np.random.default_rng(3)
    X, Y, Z = (np.sort(rng.uniform(-15, 15, n)) for n in (17, 13, 11))
    tabs = [(a ** 2).astype(np.float16) for a in (X, Y, Z)]
    R = (tabs[0][:, None, None] + tabs[1][None, :, None]) + tabs[2][None, None, :]
    assert (tabs[0].min() + tabs[1].min()) + tabs[2].min() == R.min()
    assert (tabs[0].max() + tabs[1].max()) + tabs[2].max() == R.max()
