"""Histogram deposit and the fused chain on the GPU against the oracle.

Bar: the int32 grid is bit-exact with numpy.histogramdd; S(q) is within
1e-5 * max(S) of the FP64 numpy path (FP32 FFT, FP64 frame sum)."""
import os
import time

import numpy as np
import pytest
import torch

import mdsf
from mdsf import synth
from conftest import GOLDEN
from oracle import hist as ohist

pytestmark = pytest.mark.gpu
TOL = 1e-5


def rel_err(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


def test_hist_grid_golden_edges_all_layouts():
    z = np.load(os.path.join(GOLDEN, "hist_edges.npz"))
    dims, L, w = tuple(z["dims"]), z["L"], z["weights"]
    g = mdsf.hist_grid(z["pos"], L, w, dims).cpu().numpy()
    np.testing.assert_array_equal(g, z["grid"])
    g32 = mdsf.hist_grid(z["pos32"], L, w, dims).cpu().numpy()
    np.testing.assert_array_equal(g32, z["grid32"])
    p4 = synth.pack_float4(z["pos32"], w)
    g4 = mdsf.hist_grid(p4, L, None, dims).cpu().numpy()
    np.testing.assert_array_equal(g4, z["grid32"])


@pytest.mark.parametrize("dims,box", [((64, 64, 64), (2.5, 2.5, 2.5)), ((256, 256, 128), (16.0, 13.856, 8.0)),
                                      ((75, 48, 81), (3.3, 4.1, 5.9)), ((2, 3, 5), (1.0, 1.0, 1.0))])
@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_hist_grid_random_outliers(dims, box, dtype):
    rng = np.random.default_rng(11)
    n = 50_000
    box = np.asarray(box)
    pos = (rng.uniform(-0.05, 1.05, (n, 3)) * box).astype(dtype)
    pos[:50] = np.nan
    pos[50:60] = box.astype(dtype)
    pos[60:70, 0] = 0.0
    w = rng.integers(1, 9, n).astype(np.int32)
    ref = ohist.hist_grid(pos, box, w, dims)
    got = mdsf.hist_grid(pos, box, w, dims).cpu().numpy()
    np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("wrap", [False, True])
def test_hist_grid_scale_and_wrap(wrap):
    rng = np.random.default_rng(5)
    box = np.array([3.0, 2.0, 2.5])
    pos = (rng.uniform(-0.3, 1.3, (20_000, 3)) * box).astype(np.float32)
    w = rng.integers(1, 9, 20_000).astype(np.int32)
    scale = np.array([1.01, 0.98, 1.003])
    ref = ohist.hist_grid(pos, box, w, (40, 30, 36), scale_t=scale, wrap=wrap)
    got = mdsf.hist_grid(pos, box, w, (40, 30, 36), scale=scale, wrap=wrap).cpu().numpy()
    np.testing.assert_array_equal(got, ref)


def test_hist_sf_water_box_f64():
    """Water box: 4,500 atoms, 2.5 nm, 64^3, 10 frames, float64 positions."""
    pos, box, w = synth.water_box(frames=10)
    ref = ohist.hist_sf(pos, box, w, (64, 64, 64))
    got = mdsf.structure_factor(pos, box, w, (64, 64, 64)).cpu().numpy()
    assert rel_err(got, ref) < TOL


@pytest.mark.parametrize("layout", ["xyz", "float4"])
@pytest.mark.parametrize("variant", [1, 2])
def test_hist_sf_columnar_headline_grid(layout, variant):
    """Columnar system at the headline size (200k atoms, 256x256x128), 3 frames."""
    pos, box, w = synth.columnar(frames=3)
    ref = ohist.hist_sf(pos, box, w, (256, 256, 128))
    arg = pos if layout == "xyz" else synth.pack_float4(pos, w)
    got = mdsf.structure_factor(arg, box, w, (256, 256, 128), tuning=dict(variant=variant, batch=2)).cpu().numpy()
    e = rel_err(got, ref)
    rms = float(np.sqrt(np.mean((got - ref) ** 2)) / ref.max())
    print(f"columnar {layout} variant {variant}: max err {e:.2e} rms {rms:.2e} of max(S)")
    assert e < TOL


def test_hist_sf_rescaled_frames_and_wrap():
    rng = np.random.default_rng(9)
    T, N = 4, 3000
    boxes = np.array([[3.0, 3.2, 2.9]]) * (1 + 0.01 * rng.standard_normal((T, 1)))
    pos = rng.uniform(-0.1, 1.1, (T, N, 3)) * boxes[:, None, :]
    w = rng.integers(1, 9, N).astype(np.int32)
    ref = ohist.hist_sf(pos, boxes, w, (32, 36, 30), wrap=True)
    got = mdsf.structure_factor(pos, boxes, w, (32, 36, 30), wrap=True).cpu().numpy()
    assert rel_err(got, ref) < TOL
    got32 = mdsf.structure_factor(pos.astype(np.float32), boxes, w, (32, 36, 30), wrap=True).cpu().numpy()
    ref32 = ohist.hist_sf(pos.astype(np.float32), boxes, w, (32, 36, 30), wrap=True)
    assert rel_err(got32, ref32) < TOL


def test_empty_and_mean():
    box = np.array([1.0, 1.0, 1.0])
    sf = mdsf.structure_factor(np.zeros((3, 0, 3), np.float32), box, np.zeros(0, np.int32), (8, 8, 8))
    assert float(sf.abs().max()) == 0.0
    pos, box, w = synth.uniform_system(100, (1.0, 1.0, 1.0), frames=4)
    s1 = mdsf.structure_factor(pos, box, w, (8, 8, 8)).cpu().numpy()
    s2 = mdsf.structure_factor(pos, box, w, (8, 8, 8), mean=True).cpu().numpy()
    np.testing.assert_allclose(s2 * 4, s1, rtol=1e-12)
    # accumulate into `out`, frame by frame == all frames at once
    out = torch.zeros_like(torch.from_numpy(s1)).cuda()
    for t in range(4):
        mdsf.structure_factor(pos[t], box, w, (8, 8, 8), out=out)
    np.testing.assert_allclose(out.cpu().numpy(), s1, rtol=1e-6)


def test_single_atom_kat():
    pos = np.array([[[0.31, 0.77, 0.12]]], np.float32)
    sf = mdsf.structure_factor(pos, (1.0, 1.0, 1.0), np.array([7], np.int32), (16, 12, 10)).cpu().numpy()
    np.testing.assert_allclose(sf, 49.0, rtol=1e-6)


def test_large_grid_512_cubed():
    """The stress-test grid (512^3, planes larger than shared memory): one frame
    of a 6 x 6 column system in a 25 nm box against numpy."""
    pos, box, w = synth.columnar(n_atoms=30_000, box=(25.0, 25.0, 25.0), n_cols=(6, 6), lattice=25.0 / 6,
                                 frames=1, seed=4)
    ref = ohist.hist_sf(pos, box, w, (512, 512, 512))
    got = mdsf.structure_factor(pos, box, w, (512, 512, 512), tuning=dict(batch=1)).cpu().numpy()
    assert rel_err(got, ref) < TOL


@pytest.mark.parametrize("chunk", [3, 4, 8])
def test_host_streamed_chunks(chunk):
    """Host positions streamed to the device in chunks (double-buffered on a
    side stream, one chain call per chunk, uneven last chunk) equal the
    oracle."""
    pos, box, w = synth.uniform_system(4000, (2.0, 2.2, 1.8), frames=23, seed=31)
    ref = ohist.hist_sf(pos, box, w, (64, 64, 32))
    got = mdsf.structure_factor(pos.astype(np.float32), box, w, (64, 64, 32),
                                tuning=dict(batch=4), stream_chunk=chunk, zero_copy=False).cpu().numpy()
    assert mdsf.get_plan((64, 64, 32), box, max_atoms=4000, batch=4).tuning()["variant"] == "bucketed"
    assert rel_err(got, ref) < TOL


def test_host_streamed_calls_back_to_back():
    """Two host-streamed calls on different trajectories, issued back to
    back without a synchronisation: each sf equals the same call run alone,
    bit for bit (the second call's chunk copies must not overwrite staging
    memory the first call's kernels have still to read)."""
    dims, tun = (256, 256, 128), dict(batch=16)
    a = [synth.columnar(frames=40, seed=s) for s in (21, 22)]
    hs = [torch.from_numpy(synth.pack_float4(p, w)).pin_memory() for p, _, w in a]
    box = a[0][1]
    alone = []
    for h in hs:
        alone.append(mdsf.structure_factor(h, box, None, dims, tuning=tun))
        torch.cuda.synchronize()
    for _ in range(3):
        got = [mdsf.structure_factor(h, box, None, dims, tuning=tun) for h in hs]
        torch.cuda.synchronize()
        for g, r in zip(got, alone):
            assert torch.equal(g, r)


def test_host_streamed_staging_outlives_a_stalled_stream():
    """The caller's stream is held up (a sleep kernel) while a two-chunk
    call's copies finish at once on the copy stream; a second call issued
    then must not copy into staging memory the first call's kernels have
    still to read: both results equal the calls run alone."""
    dims, tun = (256, 256, 128), dict(batch=16)
    a = [synth.columnar(frames=40, seed=s) for s in (31, 32)]
    hs = [torch.from_numpy(synth.pack_float4(p, w)).pin_memory() for p, _, w in a]
    box = a[0][1]
    alone = []
    for h in hs:
        alone.append(mdsf.structure_factor(h, box, None, dims, tuning=tun, stream_chunk=20))
        torch.cuda.synchronize()
    torch.cuda._sleep(400_000_000)
    first = mdsf.structure_factor(hs[0], box, None, dims, tuning=tun, stream_chunk=20)
    time.sleep(0.05)
    second = mdsf.structure_factor(hs[1], box, None, dims, tuning=tun, stream_chunk=20)
    torch.cuda.synchronize()
    assert torch.equal(first, alone[0])
    assert torch.equal(second, alone[1])
    mdsf.release_staging()
    again = mdsf.structure_factor(hs[0], box, None, dims, tuning=tun, stream_chunk=20)
    assert torch.equal(again, alone[0])


@pytest.mark.parametrize("variant", [3, 4])
def test_zero_copy_host_positions(variant):
    """Pinned host positions read in place by the kernels give the same sf,
    bit for bit, as the same call on a device copy; an unpinned array is
    pinned first; pageable memory passed straight to the C ABI is refused
    before any launch."""
    from mdsf._lib import MsfError, c_p, call
    pos, box, w = synth.uniform_system(5000, (2.0, 2.2, 1.8), frames=13, seed=41)
    p4 = synth.pack_float4(pos.astype(np.float32), w)
    dims = (64, 64, 32) if variant == 3 else (48, 60, 30)
    tun = dict(batch=4, variant=variant)
    dev = mdsf.structure_factor(torch.from_numpy(p4).cuda(), box, None, dims, tuning=tun)
    pinned = torch.from_numpy(p4).pin_memory()
    zc = mdsf.structure_factor(pinned, box, None, dims, tuning=tun, zero_copy=True)
    torch.cuda.synchronize()
    assert torch.equal(dev, zc)
    zc2 = mdsf.structure_factor(p4, box, None, dims, tuning=tun, zero_copy=True)   # numpy: pinned copy
    assert torch.equal(dev, zc2)
    plan = mdsf.get_plan(dims, box, max_atoms=5000, **tun)
    sf = torch.zeros(plan.half_shape, dtype=torch.float64, device="cuda")
    with pytest.raises(MsfError):
        call("msf_hist_sf_f32", plan.handle, c_p(p4.ctypes.data), 5000, 13, c_p(0), 0, c_p(sf.data_ptr()),
             c_p(torch.cuda.current_stream().cuda_stream))
    ref = ohist.hist_sf(pos.astype(np.float32), box, w, dims)
    assert rel_err(zc.cpu().numpy(), ref) < TOL


def test_continue_flag_equals_one_call():
    """Three calls (MSF_CONTINUE, MSF_CONTINUE, plain) on one plan and sf give
    the same sf as one call over all frames, bit for bit (chunks on batch
    boundaries, so the FP32 batch sums are the same)."""
    from mdsf._lib import MSF_CONTINUE, c_p, call
    pos, box, w = synth.uniform_system(3000, (2.0, 2.0, 2.0), frames=11, seed=5)
    p4 = torch.from_numpy(synth.pack_float4(pos.astype(np.float32), w)).cuda()
    plan = mdsf.get_plan((64, 64, 64), box, max_atoms=3000, batch=2, variant=3)
    st = c_p(torch.cuda.current_stream().cuda_stream)
    one = torch.zeros(plan.half_shape, dtype=torch.float64, device="cuda")
    call("msf_hist_sf_f32", plan.handle, c_p(p4.data_ptr()), 3000, 11, c_p(0), 0, c_p(one.data_ptr()), st)
    three = torch.zeros_like(one)
    for f0, f1, fl in ((0, 4, MSF_CONTINUE), (4, 8, MSF_CONTINUE), (8, 11, 0)):
        call("msf_hist_sf_f32", plan.handle, c_p(p4[f0:f1].data_ptr()), 3000, f1 - f0, c_p(0), fl,
             c_p(three.data_ptr()), st)
    torch.cuda.synchronize()
    assert torch.equal(one, three)
    ref = ohist.hist_sf(pos.astype(np.float32), box, w, (64, 64, 64))
    assert rel_err(one.cpu().numpy(), ref) < TOL


@pytest.mark.parametrize("priority", [0, -1])
def test_overlapped_chain_on_a_caller_stream(priority):
    """The overlapped chain forks its two plan-owned streams from the
    caller's stream and joins them back: called on a non-default stream (of
    default or raised priority), the sf is complete on that stream when the
    call returns, across MSF_CONTINUE calls too, and equals the oracle's."""
    from mdsf._lib import MSF_CONTINUE, c_p, call
    pos, box, w = synth.uniform_system(4000, (2.0, 2.0, 2.0), frames=7, seed=8)
    p4 = torch.from_numpy(synth.pack_float4(pos.astype(np.float32), w)).cuda()
    plan = mdsf.get_plan((64, 64, 64), box, max_atoms=4000, batch=2, variant=3)
    s = torch.cuda.Stream(priority=priority)
    torch.cuda.synchronize()
    with torch.cuda.stream(s):
        st = c_p(s.cuda_stream)
        sf = torch.zeros(plan.half_shape, dtype=torch.float64, device="cuda")
        for f0, f1, fl in ((0, 3, MSF_CONTINUE), (3, 7, 0)):
            call("msf_hist_sf_f32", plan.handle, c_p(p4[f0:f1].data_ptr()), 4000, f1 - f0, c_p(0), fl,
                 c_p(sf.data_ptr()), st)
        host = sf.to("cpu", non_blocking=False)   # ordered on s only
    ref = ohist.hist_sf(pos.astype(np.float32), box, w, (64, 64, 64))
    assert rel_err(host.numpy(), ref) < TOL


def test_full_workload_properties():
    """The headline workload itself (columnar 200k atoms, 100 frames,
    256x256x128, the plan's default batch), checked through properties that
    hold at any size against exact integer references: the DC term is the
    squared electron count of each frame (no atom lost or doubled), Parseval
    over the full spectrum equals V * sum of the exact int32 grid squared,
    S is finite and non-negative, and two calls split at the boundary of the
    chain's first (near-equal) batch add up to one call bit for bit."""
    pos, box, w = synth.columnar(frames=100, seed=2)
    p4 = torch.from_numpy(synth.pack_float4(pos, w)).cuda()
    dims = (256, 256, 128)
    sf = mdsf.structure_factor(p4, box, None, dims)
    dc = 0.0
    sumsq = 0
    g = torch.zeros(dims, dtype=torch.int32, device="cuda")
    for t in range(p4.shape[0]):
        g.zero_()
        mdsf.hist_grid(p4[t], box, None, dims, out=g)
        gl = g.to(torch.int64)
        dc += float(int(gl.sum())) ** 2
        sumsq += int((gl * gl).sum())
    V = dims[0] * dims[1] * dims[2]
    s = sf.cpu().numpy()
    assert abs(s[0, 0, 0] - dc) <= 1e-5 * dc
    full = s[:, :, 0].sum() + s[:, :, -1].sum() + 2.0 * s[:, :, 1:-1].sum()
    assert abs(full - V * float(sumsq)) <= 1e-5 * V * float(sumsq)
    assert np.all(np.isfinite(s)) and s.min() >= 0.0
    batch = mdsf.get_plan(dims, box, max_atoms=p4.shape[1]).batch
    T = p4.shape[0]
    assert batch < T
    first = -(-T // -(-T // batch))   # the chain's near-equal batches: the first one's end
    a = mdsf.structure_factor(p4[:first], box, None, dims)
    b = mdsf.structure_factor(p4[first:], box, None, dims)
    assert torch.equal(a + b, sf)


def test_sharded_frames_sum_to_the_one_call_sf():
    """structure_factor_sharded's two shards (rank 0 and 1 of 2, run one
    after another without a process group) with per-frame boxes: every shard
    bins in the trajectory's mean box, so their sum is the one-call sf."""
    from mdsf.shard import structure_factor_sharded
    rng = np.random.default_rng(12)
    T, N = 7, 20_000
    boxes = np.array([3.0, 2.6, 2.8]) * (1 + 0.02 * rng.standard_normal((T, 1)))
    pos = (rng.uniform(0, 1, (T, N, 3)) * np.array([3.0, 2.6, 2.8])).astype(np.float32)
    w = rng.integers(1, 9, N).astype(np.int32)
    one = mdsf.structure_factor(pos, boxes, w, (64, 48, 56)).cpu().numpy()
    parts = [structure_factor_sharded(pos, boxes, w, (64, 48, 56), rank=r, world=2).cpu().numpy() for r in (0, 1)]
    assert rel_err(parts[0] + parts[1], one) < 1e-6
    ref = ohist.hist_sf(pos, boxes, w, (64, 48, 56))
    assert rel_err(parts[0] + parts[1], ref) < TOL
