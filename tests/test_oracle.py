"""The oracle against the reference's own outputs (golden fixtures).

The fixtures in tests/golden were produced by running the reference's
``dens.compute_sf`` and ``plot2d.Plot_Ewald_Sphere_Correction``
(tests/golden/make_golden.py).  These tests pin the numpy restatements in
``oracle/`` before anything is compared against them.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN
from oracle import dens as odens
from oracle import ewald as oewald
from oracle import hist as ohist

GAUSS = ["gauss_ortho", "gauss_tcl", "gauss_corner"]


def load(name):
    return np.load(os.path.join(GOLDEN, name + ".npz"), allow_pickle=False)


def rad_of(z):
    """The type table entries the fixture was made with (from the reference's radii.txt)."""
    return {str(n): (float(e), float(s)) for n, e, s in zip(z["rad_names"], z["rad_nel"], z["rad_sigma"])}


def test_load_radii_format(tmp_path):
    """Lines are 'Nel name sigma_pm'; later duplicates win; pm -> Angstrom."""
    f = tmp_path / "radii.txt"
    f.write_bytes(b"1   R3  90\r\n1\tH\t53\r\n8\tO\t60\n8       O       61      \r\n")
    rad = odens.load_radii(str(f))
    assert rad == {"R3": (1.0, 0.9), "H": (1.0, 0.53), "O": (8.0, 0.61)}


@pytest.mark.parametrize("name", GAUSS)
def test_compute_sf_restatement_matches_reference(name):
    z = load(name)
    rad = rad_of(z)
    r = z["r"].copy()
    L = z["L_in"].copy()
    out = odens.compute_sf(r, L, z["typ"].astype(object), rad, z["ucell"], float(z["Sres"]))
    np.testing.assert_array_equal(out["N"], z["out_N"])
    np.testing.assert_array_equal(out["L"], z["out_L"])
    # the reference mutates its input array: same positions after rescale + wrap
    np.testing.assert_array_equal(r, z["r_after"])
    smax = z["out_sf"].max()
    np.testing.assert_allclose(out["sf"], z["out_sf"], rtol=0, atol=1e-11 * smax)
    np.testing.assert_allclose(out["sfplt"], z["out_sfplt"], rtol=0, atol=1e-11 * smax)
    np.testing.assert_array_equal(out["kgrid"], z["out_kgrid"])
    np.testing.assert_array_equal(out["kgridplt"][..., :3], z["out_kgridplt"][..., :3])


def _sha(a):
    import hashlib
    return hashlib.sha256(np.ascontiguousarray(a, np.float64).tobytes()).hexdigest()


def test_compute_sf_restatement_water_box():
    """The 4,500-atom water box at 64^3 (2 frames) run by the reference: sf
    and sfplt stored in float32, so the bar is that rounding (6e-8 of each
    value) instead of 1e-11."""
    z = load("gauss_water")
    rad = rad_of(z)
    r = z["r"].copy()
    out = odens.compute_sf(r, z["L_in"].copy(), np.array(["O", "H", "H"] * 1500, dtype=object), rad, np.eye(3),
                           float(z["Sres"]))
    np.testing.assert_array_equal(out["N"], z["out_N"])
    np.testing.assert_array_equal(out["L"], z["out_L"])
    np.testing.assert_array_equal(r, z["r_after"])
    assert out["sf"].max() == z["out_sf_max"]
    np.testing.assert_allclose(out["sf"], z["out_sf32"], rtol=1e-7, atol=1e-12 * float(z["out_sf_max"]))
    np.testing.assert_allclose(out["sfplt"], z["out_sfplt32"], rtol=1e-7, atol=1e-12 * float(z["out_sf_max"]))
    assert _sha(out["kgrid"]) == str(z["kgrid_sha256"])
    assert _sha(out["kgridplt"][..., :3]) == str(z["kgridplt_q_sha256"])


@pytest.mark.parametrize("name", GAUSS)
def test_get_dplot_exact(name):
    z = load(name)
    np.testing.assert_array_equal(odens.get_dplot(z["out_sf"]), z["out_sfplt"])


def test_corner_quirk_is_visible():
    """The fold must differ from a plain periodic fold when corners are populated."""
    z = load("gauss_corner")
    rad = rad_of(z)
    r = z["r"].copy()
    r, Lm = odens.rescale(r, z["L_in"].copy())
    N = odens.grid_dims(Lm, float(z["Sres"]))
    dr = Lm / N
    odens.wrap(r, Lm)
    typ = z["typ"].astype(object)
    bdict, Nb = odens.borders(rad, dr, set(typ))
    d0 = odens.deposit_frame(r[0], typ, rad, bdict, Nb, N, dr, z["ucell"])
    quirk = odens.fold_tcl(d0, N, Nb)
    plain = np.zeros(tuple(int(n) for n in N))
    idx = [(np.arange(int(N[a]) + 2 * Nb) - Nb) % int(N[a]) for a in range(3)]
    np.add.at(plain, np.ix_(*idx), d0)
    assert abs(quirk.sum() - plain.sum()) < 1e-9 * plain.sum()
    assert np.abs(quirk - plain).max() > 1e-3 * plain.max()


@pytest.mark.parametrize("name", ["ortho", "tcl", "corner"])
def test_ewald_restatement_matches_reference(name):
    z = load("ewald_" + name)
    xy, xz, yz = oewald.ewald_slices(z["D"], float(z["wavelength"]))
    for a, b in ((xy, z["xy"]), (xz, z["xz"]), (yz, z["yz"])):
        np.testing.assert_allclose(a, b, rtol=1e-12, atol=0, equal_nan=True)
    xy2, _, _ = oewald.ewald_slices(z["D"], float(z["wavelength"]), vectorised=False)
    np.testing.assert_array_equal(xy2, z["xy"])


def test_hist_oracle_pinned():
    z = load("hist_edges")
    g = ohist.hist_grid(z["pos"], z["L"], z["weights"], z["dims"])
    np.testing.assert_array_equal(g, z["grid"])
    g32 = ohist.hist_grid(z["pos32"], z["L"], z["weights"], z["dims"])
    np.testing.assert_array_equal(g32, z["grid32"])
    np.testing.assert_allclose(ohist.power(g), z["sf"], rtol=1e-12, atol=1e-9)


def test_bin_index_matches_histogramdd():
    z = load("hist_edges")
    pos = z["pos"]
    b = [ohist.bin_index(pos[:, a], z["L"][a], z["dims"][a]) for a in range(3)]
    ok = (b[0] >= 0) & (b[1] >= 0) & (b[2] >= 0)
    g = np.zeros(tuple(z["dims"]), np.int64)
    np.add.at(g, (b[0][ok], b[1][ok], b[2][ok]), z["weights"][ok])
    np.testing.assert_array_equal(g, z["grid"])


def test_hist_single_atom_kat():
    """One atom: |F|^2 = w^2 at every q."""
    sf = ohist.hist_sf(np.array([[[0.3, 0.7, 1.1]]]), np.array([2.0, 2.0, 2.0]), [7], (8, 6, 4))
    np.testing.assert_allclose(sf, 49.0, rtol=1e-12)


def test_hist_two_atoms_kat():
    """Two atoms one voxel apart in x: S = w1^2 + w2^2 + 2 w1 w2 cos(2 pi k/n0)."""
    n = (8, 4, 4)
    pos = np.array([[[0.1, 0.1, 0.1], [0.35, 0.1, 0.1]]])
    sf = ohist.hist_sf(pos, np.array([2.0, 1.0, 1.0]), [3, 5], n)
    k = np.arange(n[0])
    expect = 9 + 25 + 30 * np.cos(2 * np.pi * k / n[0])
    np.testing.assert_allclose(sf[:, 0, 0], expect, rtol=1e-12, atol=1e-9)


@pytest.mark.parametrize("name", ["ortho", "tcl"])
def test_cylindrical_average_restatement_matches_reference(name):
    from oracle import cyl as ocyl
    z = load("cyl_" + name)
    final, rfin, zfin, _ = ocyl.cylindrical_average(z["D"], z["ucell"])
    np.testing.assert_array_equal(rfin, z["rfin"])
    np.testing.assert_array_equal(zfin, z["zfin"])
    np.testing.assert_allclose(final, z["final"], rtol=1e-12, atol=0)
