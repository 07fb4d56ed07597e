"""(r, z) histograms (measure_intensity.py:45-125, plot2d.py:1035-1147) on
the GPU against the script's own run and the oracle.  Counts bit-exact; the
FP64 sums (atomics, another order than numpy's bincount) within 1e-12
relative; NaN bins where the reference has them."""
import numpy as np
import pytest
import torch

from mdsf import rz as mrz
from mdsf.api import plot_axes
from oracle import rz as orz
from test_rz_host import MI_UCELL, rz_case

pytestmark = pytest.mark.gpu
RTOL = 1e-12
TH = 120 * np.pi / 180.0
UCELLS = {"ortho": np.eye(3), "tcl120": np.array([[1, 0, 0], [np.cos(TH), np.sin(TH), 0], [0, 0, 1]]),
          "mi60": MI_UCELL}


def close(a, b):
    fin = np.isfinite(b)
    scale = np.nanmax(np.abs(b)) if fin.any() else 1.0
    np.testing.assert_allclose(a, b, rtol=RTOL, atol=RTOL * scale, equal_nan=True)


@pytest.mark.parametrize("name", ["ortho", "tcl"])
def test_measure_intensity_vs_script(name):
    D, z = rz_case(name)
    iavg, imax, Hrz = mrz.measure_intensity(D, full=True)
    close(Hrz.T, z["HrzT"])
    line = "{:<5d}{:6.5f}\n".format(7, imax)
    assert line == str(z["line"])


def grid(shape, L, seed):
    rng = np.random.default_rng(seed)
    X, Y, Z = plot_axes((shape[0] + 2, shape[1] + 2, (shape[2] + 3) // 2), np.asarray(L))
    S = rng.gamma(2.0, 5.0, shape)
    D = np.zeros(shape + (4,))
    D[..., 0], D[..., 1], D[..., 2] = X[:, None, None], Y[None, :, None], Z[None, None, :]
    D[..., 3] = S
    return D, S, (X, Y, Z)


@pytest.mark.parametrize("ucell", sorted(UCELLS))
@pytest.mark.parametrize("weights", ["linear", "self"])
@pytest.mark.parametrize("shape,L", [((30, 26, 21), (9.0, 8.0, 6.0)), ((62, 62, 63), (20.0, 17.0, 9.0))])
def test_rz_histogram_vs_oracle(ucell, weights, shape, L):
    D, S, (X, Y, Z) = grid(shape, L, sum(shape))
    oH, oC, _, _, _ = orz.rz_histogram(D, UCELLS[ucell], weights=weights)
    H, C, _, _ = mrz.rz_histogram(torch.from_numpy(S).cuda(), X, Y, Z, UCELLS[ucell], weights=weights)
    np.testing.assert_array_equal(C, oC)
    close(H, oH)
    close(mrz.rz_average(H, C), orz.rz_average(oH, oC))


def test_custom_edges_density_and_duplicate_edges():
    D, S, (X, Y, Z) = grid((40, 36, 33), (12.0, 10.0, 7.0), 5)
    re = np.concatenate([np.sqrt(np.linspace(0, 1, 50)) * X[-1], [X[-1]]])   # last edge repeated
    ze = np.linspace(Z[0] * 0.8, Z[-1] * 0.7, 19)
    for density in (False, True):
        oH, oC, _, _, _ = orz.rz_histogram(D, UCELLS["tcl120"], r_edges=re, z_edges=ze, density=density)
        with np.errstate(divide="ignore", invalid="ignore"):
            H, C, _, _ = mrz.rz_histogram(torch.from_numpy(S).cuda(), X, Y, Z, UCELLS["tcl120"], r_edges=re,
                                          z_edges=ze, density=density)
        np.testing.assert_array_equal(C, oC)
        close(H, oH)


def test_decreasing_edges_raise():
    D, S, (X, Y, Z) = grid((8, 8, 9), (5.0, 5.0, 5.0), 1)
    with pytest.raises(ValueError):
        mrz.rz_histogram(torch.from_numpy(S).cuda(), X, Y, Z, np.eye(3), r_edges=X[::-1])
