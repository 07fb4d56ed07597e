"""Trajectory ingest (.trr): the native reader of libmsf (``msf_trr_scan`` /
``msf_trr_read``) against the oracle's restatement of the frame layout, bit
for bit, and the .gro topology + .trr trajectory pair of the reference CLI
(main_gromacs.py:95-101 -> load_traj.process_gro_mdtraj).  No GPU."""
import numpy as np
import pytest

from mdsf import traj
from oracle import gro as ogro
from oracle import trr as otrr


def boxes(rng, T, theta=90.0):
    th = np.deg2rad(theta)
    L = np.array([3.1, 2.7, 4.4])
    b = np.zeros((T, 3, 3))
    for t in range(T):
        s = 1.0 + 0.01 * rng.standard_normal()
        b[t] = s * np.array([[L[0], 0, 0], [L[1] * np.cos(th), L[1] * np.sin(th), 0], [0, 0, L[2]]])
    return b


@pytest.mark.parametrize("double", [False, True])
@pytest.mark.parametrize("frames,atoms", [(1, 1), (5, 37), (7, 1000)])
@pytest.mark.parametrize("theta", [90.0, 120.0])
def test_round_trip_matches_oracle(tmp_path, double, frames, atoms, theta):
    rng = np.random.default_rng(frames + atoms + int(double))
    x = rng.uniform(-0.5, 3.5, (frames, atoms, 3))
    b = boxes(rng, frames, theta)
    p = str(tmp_path / "t.trr")
    otrr.write_trr(p, x, b, double=double)
    assert traj.scan_trr(p) == (atoms, frames)
    got, dims = traj.read_trr(p)
    want, wdims = otrr.read_trr(p)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(dims, wdims)
    np.testing.assert_allclose(got, x * 10, rtol=1e-6, atol=1e-5)


def test_velocities_forces_and_no_box(tmp_path):
    rng = np.random.default_rng(3)
    x = rng.uniform(0, 3, (4, 20, 3))
    p = str(tmp_path / "vf.trr")
    otrr.write_trr(p, x, boxes(rng, 4), velocities=rng.standard_normal(x.shape),
                   forces=rng.standard_normal(x.shape))
    got, dims = traj.read_trr(p)
    want, wdims = otrr.read_trr(p)
    np.testing.assert_array_equal(got, want)
    np.testing.assert_array_equal(dims, wdims)
    q = str(tmp_path / "nobox.trr")
    otrr.write_trr(q, x, None, with_box=False)
    got, dims = traj.read_trr(q)
    assert np.all(dims == 0)
    np.testing.assert_array_equal(got, otrr.read_trr(q)[0])


def test_threads_do_not_change_results(tmp_path):
    rng = np.random.default_rng(5)
    x = rng.uniform(0, 3, (11, 300, 3))
    p = str(tmp_path / "t.trr")
    otrr.write_trr(p, x, boxes(rng, 11))
    a = traj.read_trr(p, threads=1)
    for t in (2, 4, 32):
        b = traj.read_trr(p, threads=t)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])


@pytest.mark.parametrize("bad", ["magic", "truncated", "changing"])
def test_malformed_files_raise(tmp_path, bad):
    rng = np.random.default_rng(8)
    p = str(tmp_path / "t.trr")
    if bad == "changing":
        otrr.write_trr(p, rng.uniform(0, 3, (1, 10, 3)), boxes(rng, 1))
        with open(p, "ab") as f:
            q = str(tmp_path / "u.trr")
            otrr.write_trr(q, rng.uniform(0, 3, (1, 11, 3)), boxes(rng, 1))
            f.write(open(q, "rb").read())
    else:
        otrr.write_trr(p, rng.uniform(0, 3, (2, 10, 3)), boxes(rng, 2))
        data = bytearray(open(p, "rb").read())
        if bad == "magic":
            data[3] ^= 0xFF
        else:
            data = data[:-7]
        open(p, "wb").write(bytes(data))
    with pytest.raises(Exception):
        traj.read_trr(p)


def test_gro_topology_with_trr_trajectory(tmp_path):
    """process_gro_mdtraj(top.gro, traj.trr, out): names from the topology,
    coordinates and box lengths from the trajectory."""
    rng = np.random.default_rng(9)
    n, T = 30, 6
    names = [["OW", "HW1", "HW2"][i % 3] for i in range(n)]
    x = rng.uniform(0, 2.5, (T, n, 3))
    b = boxes(rng, T, 120.0)
    top = str(tmp_path / "top.gro")
    ogro.write_gro(top, x[:1], b[:1, [0, 1, 2], [0, 1, 2]], names)
    trr = str(tmp_path / "run.trr")
    otrr.write_trr(trr, x, b)
    out = str(tmp_path / "out_run_traj")
    traj.process_gro_trr(top, trr, out)
    z = np.load(out + ".npz")
    want, wdims = otrr.read_trr(trr)
    np.testing.assert_array_equal(z["coords"], want)
    np.testing.assert_array_equal(z["dims"], wdims)
    assert list(z["typ"]) == names and z["coords"].shape == (T, n, 3)
