"""The bucketed chain (variant 3: per-x-plane atom lists, shared-memory
deposit inside the plane FFT kernel) against the oracle.

The bucket contents are checked bit-exactly as an int32 grid (the in-chain
binning), and S(q) at 1e-5 * max(S); a sparse system makes a single misplaced
atom visible far above that bar."""
import os

import numpy as np
import pytest
import torch

import mdsf
from mdsf import synth
from mdsf._lib import c_p, call
from conftest import GOLDEN
from oracle import hist as ohist

pytestmark = pytest.mark.gpu
TOL = 1e-5


def bucket_grid(pos, box, w, dims, layout, scale=None, wrap=False):
    n = pos.shape[0]
    plan = mdsf.get_plan(dims, box, max_atoms=max(n, 1), variant=3)
    g = torch.zeros(dims, dtype=torch.int32, device="cuda")
    p = torch.from_numpy(np.ascontiguousarray(pos)).cuda()
    wd = torch.from_numpy(np.asarray(w, np.int32)).cuda()
    sc = torch.from_numpy(np.asarray(scale, np.float64)).cuda() if scale is not None else None
    call("msf_hist_bucket_grid", plan.handle, layout, c_p(p.data_ptr()), c_p(wd.data_ptr()), n,
         c_p(sc.data_ptr()) if sc is not None else c_p(0), 1 if wrap else 0, c_p(g.data_ptr()),
         c_p(torch.cuda.current_stream().cuda_stream))
    return g.cpu().numpy()


def test_bucket_grid_golden_edges_bit_exact():
    z = np.load(os.path.join(GOLDEN, "hist_edges.npz"))
    dims = (32, 32, 32)   # power-of-two grid over the fixture box
    L, w = z["L"], z["weights"]
    ref = ohist.hist_grid(z["pos"], L, w, dims)
    np.testing.assert_array_equal(bucket_grid(z["pos"], L, w, dims, 1), ref)
    ref32 = ohist.hist_grid(z["pos32"], L, w, dims)
    np.testing.assert_array_equal(bucket_grid(z["pos32"], L, w, dims, 2), ref32)
    np.testing.assert_array_equal(bucket_grid(synth.pack_float4(z["pos32"], w), L, w, dims, 0), ref32)


@pytest.mark.parametrize("wrap", [False, True])
def test_bucket_grid_columnar_rescaled(wrap):
    pos, box, w = synth.columnar(n_atoms=60_000, frames=1)
    p = pos[0].copy()
    p[:100] += 0.5            # some atoms beyond the box (wrapped or dropped)
    scale = np.array([1.002, 0.997, 1.0])
    ref = ohist.hist_grid(p, box, w, (128, 128, 64), scale_t=scale, wrap=wrap)
    np.testing.assert_array_equal(bucket_grid(p, box, w, (128, 128, 64), 2, scale=scale, wrap=wrap), ref)


@pytest.mark.parametrize("dims", [(64, 64, 64), (256, 256, 128), (32, 512, 64), (128, 64, 256), (512, 32, 32)])
def test_bucketed_chain_vs_oracle(dims):
    box = np.array([3.0, 2.5, 2.8])
    pos, _, w = synth.uniform_system(20_000, box, frames=3, seed=sum(dims))
    ref = ohist.hist_sf(pos, box, w, dims)
    got = mdsf.structure_factor(pos, box, w, dims, tuning=dict(variant=3, batch=2)).cpu().numpy()
    assert np.abs(got - ref).max() / ref.max() < TOL


def test_bucketed_sparse_system_exact_enough():
    """300 atoms on a 64^3 grid: one misplaced atom would show at ~1e-3."""
    pos, box, w = synth.uniform_system(300, (2.0, 2.0, 2.0), frames=4, seed=99)
    ref = ohist.hist_sf(pos, box, w, (64, 64, 64))
    got = mdsf.structure_factor(pos, box, w, (64, 64, 64), tuning=dict(variant=3)).cpu().numpy()
    assert np.abs(got - ref).max() / ref.max() < 2e-6


@pytest.mark.parametrize("batch", [1, 3, 8])
def test_bucketed_headline_grid_batches(batch):
    pos, box, w = synth.columnar(frames=5)
    ref = ohist.hist_sf(pos, box, w, (256, 256, 128))
    got = mdsf.structure_factor(synth.pack_float4(pos, w), box, None, (256, 256, 128),
                                tuning=dict(variant=3, batch=batch)).cpu().numpy()
    e = np.abs(got - ref).max() / ref.max()
    rms = np.sqrt(np.mean((got - ref) ** 2)) / ref.max()
    print(f"bucketed batch {batch}: max err {e:.2e}, rms {rms:.2e} of max(S)")
    assert e < TOL


@pytest.fixture(scope="module")
def headline_five_frames():
    pos, box, w = synth.columnar(frames=5, seed=4)
    return pos, box, w, ohist.hist_sf(pos, box, w, (256, 256, 128))


@pytest.mark.parametrize("tile_w", [8, 16, 32])
@pytest.mark.parametrize("options", [0, 1])
def test_headline_grid_x_tiles_and_overlap(headline_five_frames, tile_w, options):
    """Batches of 2 over 5 frames: with the overlap (options 0) the x passes
    of the first two batches run beside the next plane FFT (8-column tiles on
    two 128-thread CTAs per SM, 16- and 32-column ones on 256-thread CTAs) and
    the last alone; the plane kernel hands its planes out by its counter."""
    pos, box, w, ref = headline_five_frames
    got = mdsf.structure_factor(synth.pack_float4(pos, w), box, None, (256, 256, 128),
                                tuning=dict(variant=3, batch=2, tile_w=tile_w, options=options)).cpu().numpy()
    assert np.abs(got - ref).max() / ref.max() < TOL


def test_power_accum_ct_grids():
    rng = np.random.default_rng(3)
    for dims in [(64, 64, 64), (256, 128, 64), (32, 128, 256)]:
        g = rng.integers(0, 9, (2,) + dims).astype(np.int32)
        ref = sum(ohist.power(g[k]) for k in range(2))
        plan = mdsf.get_plan(dims, (1.0, 1.0, 1.0), variant=3, batch=2)
        sf = torch.zeros(plan.half_shape, dtype=torch.float64, device="cuda")
        gd = torch.from_numpy(g).cuda()
        call("msf_power_accum_i32", plan.handle, c_p(gd.data_ptr()), 2, c_p(sf.data_ptr()),
             c_p(torch.cuda.current_stream().cuda_stream))
        got = sf.cpu().numpy()
        assert np.abs(got - ref).max() / ref.max() < TOL, dims


def test_too_many_atoms_for_the_plan():
    plan = mdsf.get_plan((64, 64, 64), (1.0, 1.0, 1.0), max_atoms=10, variant=3)
    p = torch.zeros((1, 20, 4), dtype=torch.float32, device="cuda")
    sf = torch.zeros(plan.half_shape, dtype=torch.float64, device="cuda")
    with pytest.raises(mdsf.MsfError, match="MSF_E_WORKSPACE"):
        call("msf_hist_sf_f32", plan.handle, c_p(p.data_ptr()), 20, 1, c_p(0), 0, c_p(sf.data_ptr()),
             c_p(torch.cuda.current_stream().cuda_stream))


def test_headline_plan_uses_tma_x_pass():
    """The default x tile of 256-point lines: 8 columns (2048 values, two
    128-thread CTAs beside the plane FFT)."""
    plan = mdsf.get_plan((256, 256, 128), (16.0, 13.856, 8.0), max_atoms=1000, variant=3, batch=4)
    assert plan.tma and plan.tile_w == 8
    for dims, w in (((128, 64, 32), 16), ((64, 64, 64), 32), ((512, 64, 64), 8)):
        assert mdsf.get_plan(dims, (1.0, 1.0, 1.0), max_atoms=1000, variant=3, batch=2).tile_w == w, dims


@pytest.mark.parametrize("dims", [(64, 64, 64), (128, 64, 32), (256, 32, 64)])
@pytest.mark.parametrize("options", [0, 1])
def test_tma_x_pass_many_frames_per_launch(dims, options):
    """12 frames per launch through the TMA x pass; options=1 (no overlap)
    launches more x-pass CTAs per SM."""
    box = np.array([2.0, 2.2, 1.9])
    pos, _, w = synth.uniform_system(3_000, box, frames=12, seed=7 + options)
    ref = ohist.hist_sf(pos, box, w, dims)
    tuning = dict(batch=12, variant=3, options=options)
    assert mdsf.get_plan(dims, box, max_atoms=3_000, **tuning).tma
    got = mdsf.structure_factor(pos, box, w, dims, tuning=tuning).cpu().numpy()
    assert np.abs(got - ref).max() / ref.max() < TOL
