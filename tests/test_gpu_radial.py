"""radial_integrate (plot2d.py:160-173) on the GPU: against the reference's
own outputs (tests/golden/radial_*.npz) and the numpy oracle.  Counts and
edges bit-exact; the S sums (FP64, atomics in a different order than
numpy's bincount) within 1e-12 relative."""
import numpy as np
import pytest
import torch

from mdsf import radial as mrad
from mdsf.api import plot_axes
from oracle import radial as orad
from test_radial_host import CASES, radial_input

pytestmark = pytest.mark.gpu
RTOL = 1e-12


def assert_h(got, want):
    np.testing.assert_allclose(got, want, rtol=RTOL, atol=RTOL * np.nanmax(np.abs(want)), equal_nan=True)


@pytest.mark.parametrize("name", CASES)
def test_radial_integrate_vs_reference(name):
    D, nb, z = radial_input(name)
    E, H = mrad.radial_integrate(D, nb)
    np.testing.assert_array_equal(E, z["E"])
    assert_h(H, z["H"])
    hist, count, edges = mrad.radial_histograms(D, nb)
    oh, oc, oe = orad.radial_counts(D, nb)
    np.testing.assert_array_equal(count.cpu().numpy(), oc)
    np.testing.assert_array_equal(edges, oe)
    assert_h(hist.cpu().numpy(), oh)


def kgrid(shape, L, rng):
    X, Y, Z = plot_axes((shape[0] + 2, shape[1] + 2, (shape[2] + 3) // 2), L)
    S = rng.gamma(2.0, 5.0, shape)
    D = np.zeros(shape + (4,))
    D[..., 0], D[..., 1], D[..., 2] = X[:, None, None], Y[None, :, None], Z[None, None, :]
    D[..., 3] = S
    return D, S, (X, Y, Z)


@pytest.mark.parametrize("shape,L,nb", [((62, 62, 63), (20.0, 17.0, 9.0), 750),
                                        ((126, 94, 61), (6.0, 8.0, 5.0), 1500),
                                        ((30, 254, 17), (40.0, 30.0, 12.0), 1)])
def test_points_and_grid_forms_vs_oracle(shape, L, nb):
    rng = np.random.default_rng(sum(shape))
    D, S, (X, Y, Z) = kgrid(shape, np.array(L), rng)
    oh, oc, oe = orad.radial_counts(D, nb)
    for hist, count, edges in (mrad.radial_histograms(torch.from_numpy(D).cuda(), nb),
                               mrad.radial_histograms_grid(torch.from_numpy(S).cuda(), X, Y, Z, nb)):
        np.testing.assert_array_equal(edges, oe)
        np.testing.assert_array_equal(count.cpu().numpy(), oc)
        assert_h(hist.cpu().numpy(), oh)
    E, H = mrad.radial_integrate_grid(torch.from_numpy(S).cuda(), X, Y, Z, nb)
    oE, oH = orad.radial_integrate(D, nb)
    np.testing.assert_array_equal(E, oE)
    assert_h(H, oH)


def test_scattered_points_not_on_a_grid():
    rng = np.random.default_rng(9)
    D = np.zeros((5000, 1, 1, 4))
    D[..., :3] = rng.standard_normal((5000, 1, 1, 3)) * 4.0
    D[..., 3] = rng.uniform(0, 1, (5000, 1, 1))
    D[:7, 0, 0, :3] = 0.0                      # the minimum many times over
    oh, oc, oe = orad.radial_counts(D, 300)
    hist, count, edges = mrad.radial_histograms(D, 300)
    np.testing.assert_array_equal(count.cpu().numpy(), oc)
    assert_h(hist.cpu().numpy(), oh)


def test_non_finite_range_raises_like_numpy():
    D = np.zeros((4, 4, 4, 4))
    D[..., 3] = 1.0
    D[1, 2, 3, 0] = 300.0                      # 300^2 overflows float16
    with pytest.raises(ValueError):
        orad.radial_integrate(D, 10)
    with pytest.raises(ValueError):
        mrad.radial_integrate(D, 10)
    D[1, 2, 3, 0] = np.nan
    with pytest.raises(ValueError):
        mrad.radial_integrate(D, 10)


def test_float16_overflow_in_the_grid_form_raises():
    """|q| > 255.9: q^2 overflows float16 in the reference too."""
    D, S, (X, Y, Z) = kgrid((30, 254, 17), np.array([40.0, 3.0, 12.0]), np.random.default_rng(1))
    with pytest.raises(ValueError):
        orad.radial_integrate(D, 10)
    with pytest.raises(ValueError):
        mrad.radial_integrate_grid(torch.from_numpy(S).cuda(), X, Y, Z, 10)
    with pytest.raises(ValueError):
        mrad.radial_integrate(D, 10)


def test_too_many_bins_and_empty_input():
    D = np.zeros((3, 4, 5, 4))
    D[..., 0] = 0.5
    with pytest.raises(ValueError):
        orad.radial_integrate(D, 2000)
    with pytest.raises(ValueError):
        mrad.radial_integrate(D, 2000)
    E, H = mrad.radial_integrate(np.zeros((0, 4)), 9)
    oE = np.histogram(np.zeros(0, np.float16), bins=9)[1][:-1]
    np.testing.assert_array_equal(E, oE)
    assert np.all(np.isnan(H))
