"""Trajectory ingest (.gro) on the host: the native reader of libmsf
(``msf_gro_scan`` / ``msf_gro_read``) against the oracle's restatement of
load_traj.py, bit for bit, plus the npz layout of process_gro_mdtraj and the
monoclinic transform of main_gromacs.py:204-207.  No GPU."""
import os

import numpy as np
import pytest

from mdsf import traj
from oracle import gro as ogro

# the reference's own test data, read in place from the checkout named by
# MSF_REFERENCE (its test/ directory); skipped when that is not set
REF_ROOT = os.environ.get("MSF_REFERENCE", "")


def ref_file(name):
    p = os.path.join(REF_ROOT, "test", name)
    if not REF_ROOT or not os.path.isfile(p):
        pytest.skip("reference checkout not given (MSF_REFERENCE)")
    return p


def synth_traj(rng, frames, atoms, box=(3.1, 2.7, 4.4)):
    box = np.asarray(box)
    coords = rng.uniform(-0.2, 1.0, (frames, atoms, 3)) * box
    boxes = np.tile(box, (frames, 1)) * (1.0 + 0.01 * rng.standard_normal((frames, 1)))
    names = [["OW", "HW1", "HW2"][i % 3] + ("" if i % 7 else str(i % 10)) for i in range(atoms)]
    return coords, boxes, names


def assert_same(path):
    x, d, nm = traj.read_gro(path)
    ox, od, onm = ogro.read_gro(path)
    assert x.dtype == np.float32 and d.dtype == np.float32
    np.testing.assert_array_equal(x, ox)
    np.testing.assert_array_equal(d, od)
    assert list(nm) == onm
    return x, d, nm


def test_reference_water_names_golden():
    """load_traj.py:11-20 with the assertions of test/test_load_traj.py:16-25."""
    p = ref_file("water.gro")
    want = ["OW1", "HW2", "HW3", "OW1", "HW2", "HW3"]
    assert ogro.load_gro(p)[:6] == want
    assert traj.load_gro(p)[:6] == want
    x, d, _ = assert_same(p)
    assert x.shape == (1, 6, 3)
    np.testing.assert_array_equal(d[0], np.float32(1.82060) * np.float32(10.0))


def test_reference_triclinic_system():
    """55680 atoms with velocities and a 9-number (120 degree) box line."""
    p = ref_file("test_system.gro")
    x, d, nm = assert_same(p)
    assert x.shape == (1, 55680, 3)
    assert nm[0] == "C" and nm[-1] == "HW2"
    assert abs(d[0, 0] - d[0, 1]) < 1e-3     # |v2| = |v1| for the hexagonal cell
    assert traj.load_gro(p) == ogro.load_gro(p)


@pytest.mark.parametrize("decimals", [3, 4, 5])
@pytest.mark.parametrize("frames,atoms", [(1, 1), (4, 37), (9, 300)])
def test_round_trip_matches_oracle(tmp_path, decimals, frames, atoms):
    rng = np.random.default_rng(frames * 1000 + atoms + decimals)
    coords, boxes, names = synth_traj(rng, frames, atoms)
    p = str(tmp_path / "t.gro")
    ogro.write_gro(p, coords, boxes, names, decimals=decimals)
    assert traj.scan_gro(p) == (atoms, frames)
    x, d, nm = assert_same(p)
    # the file holds the coordinates rounded to `decimals` nm
    np.testing.assert_allclose(x, coords * 10, atol=10 * 0.51 * 10.0 ** -decimals + 1e-4)
    assert list(nm) == [s[:5] for s in names]


def test_triclinic_box_and_velocities(tmp_path):
    rng = np.random.default_rng(7)
    coords, _, names = synth_traj(rng, 3, 40)
    b9 = np.array([[8.65915, 7.49905, 8.34313, 0, 0, -4.32958, 0, 0, 0]] * 3)
    b9[1, 5] = -4.0
    b9[2, 7], b9[2, 8] = 0.5, -0.25
    p = str(tmp_path / "tcl.gro")
    ogro.write_gro(p, coords, b9, names, velocities=rng.standard_normal(coords.shape))
    x, d, _ = assert_same(p)
    np.testing.assert_allclose(d[1, 1], 10 * np.hypot(4.0, 7.49905), rtol=1e-6)
    np.testing.assert_allclose(d[2, 2], 10 * np.sqrt(8.34313 ** 2 + 0.5 ** 2 + 0.25 ** 2), rtol=1e-6)


def test_threads_do_not_change_results(tmp_path):
    rng = np.random.default_rng(3)
    coords, boxes, names = synth_traj(rng, 13, 50)
    p = str(tmp_path / "t.gro")
    ogro.write_gro(p, coords, boxes, names)
    a = traj.read_gro(p, threads=1)
    for t in (2, 5, 64):
        b = traj.read_gro(p, threads=t)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])


def test_trailing_blank_lines_and_crlf(tmp_path):
    rng = np.random.default_rng(5)
    coords, boxes, names = synth_traj(rng, 2, 9)
    p = str(tmp_path / "t.gro")
    ogro.write_gro(p, coords, boxes, names)
    ref = traj.read_gro(p)
    with open(p) as f:
        text = f.read()
    q = str(tmp_path / "crlf.gro")
    with open(q, "w", newline="") as f:
        f.write(text.replace("\n", "\r\n") + "\r\n\r\n")
    got = traj.read_gro(q)
    np.testing.assert_array_equal(ref[0], got[0])
    np.testing.assert_array_equal(ref[1], got[1])


@pytest.mark.parametrize("bad", ["missing", "truncated", "count", "box", "changing"])
def test_malformed_files_raise(tmp_path, bad):
    rng = np.random.default_rng(11)
    coords, boxes, names = synth_traj(rng, 2, 5)
    p = str(tmp_path / "t.gro")
    ogro.write_gro(p, coords, boxes, names)
    lines = open(p).read().splitlines()
    if bad == "missing":
        p = str(tmp_path / "nope.gro")
    elif bad == "truncated":
        lines = lines[:-3]
    elif bad == "count":
        lines[1] = "  abc"
    elif bad == "box":
        lines[7] = " 1.0 2.0"
    elif bad == "changing":
        lines[9] = "    4"
    if bad != "missing":
        with open(p, "w") as f:
            f.write("\n".join(lines) + "\n")
    with pytest.raises(Exception):
        traj.read_gro(p)


def test_process_gro_npz_layout(tmp_path):
    """load_traj.py:96-109: dims, coords (Angstrom), name, mass, typ = name,
    loadable without pickles as main_gromacs.py:200-202 reads it."""
    rng = np.random.default_rng(1)
    coords, boxes, names = synth_traj(rng, 3, 12)
    p = str(tmp_path / "t.gro")
    ogro.write_gro(p, coords, boxes, names)
    out = str(tmp_path / "out_t_traj")
    traj.process_gro(p, out)
    z = np.load(out + ".npz")
    assert set(z.files) == {"dims", "coords", "name", "mass", "typ"}
    ox, od, onm = ogro.read_gro(p)
    np.testing.assert_array_equal(z["coords"], ox)
    np.testing.assert_array_equal(z["dims"], od)
    assert list(z["typ"]) == onm and list(z["name"]) == onm
    assert z["mass"][0] == pytest.approx(15.999) and z["mass"][1] == pytest.approx(1.008)


def test_monoclinic_transform():
    """main_gromacs.py:204-207 in place."""
    rng = np.random.default_rng(2)
    T = rng.uniform(0, 50, (3, 20, 3)).astype(np.float32)
    theta = 120 * np.pi / 180.0
    want = T.copy()
    want[..., 1] = want[..., 1] / np.sin(theta)
    want[..., 0] = want[..., 0] - want[..., 1] * np.cos(theta)
    got = traj.monoclinic(T, theta)
    assert got is T
    np.testing.assert_array_equal(got, want)


def test_frames_without_atoms(tmp_path):
    p = str(tmp_path / "empty.gro")
    with open(p, "w") as f:
        f.write("empty t=0\n    0\n   1.00000   1.00000   1.00000\n"
                "empty t=1\n    0\n   2.00000   2.00000   2.00000\n")
    x, d, nm = assert_same(p)
    assert x.shape == (2, 0, 3) and len(nm) == 0
    np.testing.assert_array_equal(d[:, 0], np.float32([10.0, 20.0]))
