"""get_dplot and Ewald slices on the GPU against the reference's outputs."""
import os

import numpy as np
import pytest
import torch

import mdsf
from conftest import GOLDEN
from oracle import ewald as oewald

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["gauss_ortho", "gauss_tcl", "gauss_corner"])
def test_sfplt_bit_exact_vs_reference(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    got = mdsf.get_dplot(torch.from_numpy(z["out_sf"]).cuda()).cpu().numpy()
    np.testing.assert_array_equal(got, z["out_sfplt"])


@pytest.mark.parametrize("name", ["ortho", "tcl", "corner"])
def test_ewald_vs_reference(name):
    z = np.load(os.path.join(GOLDEN, "ewald_" + name + ".npz"))
    D = z["D"]
    xy, xz, yz = mdsf.ewald_slices(torch.from_numpy(np.ascontiguousarray(D[..., 3])).cuda(),
                                   D[:, 0, 0, 0], D[0, :, 0, 1], D[0, 0, :, 2], float(z["wavelength"]))
    for a, b in ((xy, z["xy"]), (xz, z["xz"]), (yz, z["yz"])):
        np.testing.assert_allclose(a.cpu().numpy(), b, rtol=1e-12, atol=1e-12 * np.nanmax(np.abs(b)),
                                   equal_nan=True)


def test_ewald_nan_outside_and_asymmetric_axes():
    rng = np.random.default_rng(4)
    X = np.linspace(-3.0, 1.0, 21)
    Y = np.linspace(-0.5, 2.0, 17)
    Z = np.linspace(0.2, 0.9, 9)
    S = rng.uniform(0, 10, (21, 17, 9))
    D = np.zeros((21, 17, 9, 4))
    D[..., 0] = X[:, None, None]
    D[..., 1] = Y[None, :, None]
    D[..., 2] = Z[None, None, :]
    D[..., 3] = S
    ref = oewald.ewald_slices(D, 2.0)
    got = mdsf.ewald_slices(torch.from_numpy(S).cuda(), X, Y, Z, 2.0)
    for a, b in zip(got, ref):
        a = a.cpu().numpy()
        assert np.isnan(b).any()
        np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=1e-12, equal_nan=True)


def test_ewald_from_sf_chain():
    z = np.load(os.path.join(GOLDEN, "gauss_tcl.npz"))
    e = np.load(os.path.join(GOLDEN, "ewald_tcl.npz"))
    xy, xz, yz = mdsf.ewald_from_sf(torch.from_numpy(z["out_sf"]).cuda(), z["out_L"], 1.54)
    np.testing.assert_allclose(xy.cpu().numpy(), e["xy"], rtol=1e-12)
    np.testing.assert_allclose(yz.cpu().numpy(), e["yz"], rtol=1e-12)


@pytest.mark.parametrize("name", ["ortho", "tcl"])
def test_cylindrical_average_vs_reference(name):
    """PLOT_RAD_NEW's (r, z) ring average on the GPU against the reference's own output."""
    z = np.load(os.path.join(GOLDEN, "cyl_" + name + ".npz"))
    D = z["D"]
    final, rfin, zfin, oa = mdsf.cylindrical_average(torch.from_numpy(np.ascontiguousarray(D[..., 3])).cuda(),
                                                     D[:, 0, 0, 0], D[0, :, 0, 1], D[0, 0, :, 2], z["ucell"])
    np.testing.assert_array_equal(rfin, z["rfin"])
    np.testing.assert_array_equal(zfin, z["zfin"])
    np.testing.assert_allclose(final, z["final"], rtol=1e-11, atol=0)


def test_axes_checked_before_the_gpu():
    S = torch.zeros((5, 6, 7), dtype=torch.float64, device="cuda")
    X, Y, Z = np.linspace(-1, 1, 5), np.linspace(-1, 1, 6), np.linspace(-1, 1, 7)
    with pytest.raises(ValueError):
        mdsf.ewald_slices(S, X[:4], Y, Z, 1.5)          # shorter than the grid
    with pytest.raises(ValueError):
        mdsf.ewald_slices(S, X[::-1], Y, Z, 1.5)        # descending
    with pytest.raises(ValueError):
        mdsf.cylindrical_average(S, X, np.zeros(6), Z, np.eye(3))
