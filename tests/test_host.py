"""Host-side logic of the drop-in module against the reference's outputs
(no GPU): grid sizing, rescale and wrap side effects, type tables and the
kgrid / kgridplt writers."""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from mdsf import dens as mdens
from mdsf import synth
from mdsf import tune as _tune
from mdsf.api import plot_axes

GAUSS = ["gauss_ortho", "gauss_tcl", "gauss_corner"]


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"))


@pytest.mark.parametrize("name", GAUSS)
def test_host_preprocessing_matches_reference(name):
    z = load(name)
    r = z["r"].copy()
    r, Lm = mdens.rescale(r, z["L_in"].copy())
    N = mdens.grid_dims(Lm, float(z["Sres"]))
    mdens.wrap_positions(r, Lm)
    np.testing.assert_array_equal(N, z["out_N"])
    np.testing.assert_array_equal(Lm, z["out_L"])
    np.testing.assert_array_equal(r, z["r_after"])
    np.testing.assert_array_equal(mdens.kgrid(z["out_sf"].shape, Lm), z["out_kgrid"])
    np.testing.assert_array_equal(mdens.kgridplt(z["out_sfplt"], Lm), z["out_kgridplt"])
    ax = plot_axes(z["out_sf"].shape, Lm)
    kp = z["out_kgridplt"]
    np.testing.assert_array_equal(ax[0], kp[:, 0, 0, 0])
    np.testing.assert_array_equal(ax[2], kp[0, 0, :, 2])


def test_load_radii(tmp_path):
    f = tmp_path / "radii.txt"
    f.write_bytes(b"1   R3  90\r\n1\tH\t53\r\n8\tO\t60\n8       O       61      \r\n")
    assert mdens.load_radii(str(f)) == {"R3": (1.0, 0.9), "H": (1.0, 0.53), "O": (8.0, 0.61)}


def test_type_table():
    rad = {"O": (8.0, 0.6), "H": (1.0, 0.53)}
    dr = np.array([0.5, 0.55, 0.6])
    names, tidx, tab, nb = mdens._type_table(rad, np.array(["O", "H", "H"], object), dr)
    assert names == ["H", "O"] and list(tidx) == [1, 0, 0]
    bd = mdens.get_borders(rad, dr, ["O", "H"])
    assert nb == int(max(max(v) for v in bd.values()))
    np.testing.assert_array_equal(tab[1, 2:], bd["O"].astype(int))
    assert tab[1, 0] == 8.0 / np.power(0.6, 3.) and tab[1, 1] == 2 * np.power(0.6, 2.)


def test_wrap_buffered_branch_quirk():
    """>= BUFFSIZE atoms: only atoms [0, n_frames) are wrapped (dens.py:214-221)."""
    old = mdens.BUFFSIZE
    mdens.BUFFSIZE = 10
    try:
        r = np.full((2, 12, 3), -0.5)
        mdens.wrap_positions(r, np.array([4.0, 4.0, 4.0]))
        assert np.all(r[:, :2] == 3.5) and np.all(r[:, 2:] == -0.5)
    finally:
        mdens.BUFFSIZE = old


def test_generators_shapes_and_bounds():
    p, b, w = synth.columnar(n_atoms=5000, frames=2)
    assert p.shape == (2, 5000, 3) and p.dtype == np.float32
    assert np.all(p >= 0) and np.all(p.astype(np.float64) < b)
    assert set(np.unique(w)) <= {1, 6, 7, 8}
    p, b, w = synth.water_box(n_waters=50, frames=2)
    assert p.shape == (2, 150, 3) and np.all(p < b)
    d = np.linalg.norm(p[0, 1::3] - p[0, 0::3], axis=1)
    ok = np.abs(d - 0.09572) < 1e-9
    assert ok.mean() > 0.8            # molecules not cut by the wrap keep the bond length
    assert 48 in synth.smooth_sizes() and 243 in synth.smooth_sizes() and 49 not in synth.smooth_sizes()


def test_candidates_cover_the_fused_and_generic_chains():
    assert {c["variant"] for c in _tune.candidates((256, 256, 128))} == {3, 4}
    assert {c["variant"] for c in _tune.candidates((75, 48, 81))} == {4}
    assert {c["variant"] for c in _tune.candidates((74, 64, 26))} <= {1, 2}


def test_host_chunks_lead_short_then_balanced():
    from mdsf.api import _chunk_sizes
    assert _chunk_sizes(100, 64) == [16, 42, 42]
    assert _chunk_sizes(64, 64) == [64]
    assert _chunk_sizes(100, 64, lead=False) == [64, 36]
    for T in range(1, 300, 7):
        for c in (1, 4, 16, 50, 64):
            z = _chunk_sizes(T, c)
            assert sum(z) == T and max(z) <= c and min(z) >= 1
            if T > c:
                assert z[0] == max(1, c // 4) and max(z[1:]) - min(z[1:]) <= 1
