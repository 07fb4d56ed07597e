"""msf_hist_sf_f32_noalloc: the chain for callers that cannot allocate device
memory, called through the C ABI and compared with msf_hist_sf_f32 (plan +
caller workspace) on two calls in a row with different inputs and grids.

Collected last on purpose (file name), so that a run stopping at the first
failure has run every other test before this one."""
import ctypes as C

import numpy as np
import pytest
import torch

import mdsf
from mdsf import synth
from mdsf._lib import c_p

pytestmark = pytest.mark.gpu
TOL = 1e-5   # the S(q) tolerance used by every chain test


def _ref_sf(p4, box, dims):
    plan = mdsf.get_plan(dims, box, max_atoms=p4.shape[1])
    sf = torch.zeros(plan.half_shape, dtype=torch.float64, device="cuda")
    lib = mdsf.load()
    st = lib.msf_hist_sf_f32(plan.handle, c_p(p4.data_ptr()), p4.shape[1], p4.shape[0], None, 0,
                             c_p(sf.data_ptr()), c_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0
    return sf


def _stream():
    return c_p(torch.cuda.current_stream().cuda_stream)


def _noalloc_into(sf, p4, box, dims, flags=0):
    lib = mdsf.load()
    bx = (C.c_double * 3)(*box)
    return lib.msf_hist_sf_f32_noalloc(c_p(p4.data_ptr()), p4.shape[1], p4.shape[0], C.cast(bx, c_p),
                                       dims[0], dims[1], dims[2], flags, c_p(sf.data_ptr()), _stream())


def _noalloc_sf(p4, box, dims):
    lib = mdsf.load()
    sf = torch.zeros((dims[0], dims[1], dims[2] // 2 + 1), dtype=torch.float64, device="cuda")
    assert lib.msf_noalloc_init(dims[0], dims[1], dims[2], c_p(sf.data_ptr()), _stream()) == 0
    st = _noalloc_into(sf, p4, box, dims)
    assert st == 0, lib.msf_strerror(st)
    assert lib.msf_noalloc_status(_stream()) == 0
    return sf


def test_noalloc_matches_plan_entry_point_on_two_calls():
    lib = mdsf.load()
    assert lib.msf_noalloc_scratch_bytes() == 32 << 20
    cases = [((96, 80, 64), (3.0, 2.5, 2.0), 30_000, 5, 21),
             ((128, 128, 128), (4.0, 4.0, 4.0), 50_000, 3, 22)]
    for dims, box, n, t, seed in cases:
        pos, bx, w = synth.uniform_system(n, box, frames=t, seed=seed)
        p4 = torch.from_numpy(synth.pack_float4(pos, w)).cuda()
        ref = _ref_sf(p4, bx, dims)
        got = _noalloc_sf(p4, bx, dims)
        torch.cuda.synchronize()
        err = float((got - ref).abs().max() / ref.abs().max())
        assert err < TOL, (dims, err)


def test_noalloc_call_after_init_takes_no_device_memory():
    """After msf_noalloc_init (and one call) on a grid, further calls leave
    the device's free memory unchanged: nothing is allocated, not even by
    loading."""
    lib = mdsf.load()
    dims, box = (64, 64, 64), (2.0, 2.0, 2.0)
    pos, bx, w = synth.uniform_system(8000, box, frames=4, seed=23)
    p4 = torch.from_numpy(synth.pack_float4(pos, w)).cuda()
    sf = torch.zeros((64, 64, 33), dtype=torch.float64, device="cuda")
    assert lib.msf_noalloc_init(64, 64, 64, c_p(sf.data_ptr()), _stream()) == 0
    torch.cuda.synchronize()
    assert float(sf.abs().max()) == 0.0          # the init's placeholder atom adds nothing
    assert _noalloc_into(sf, p4, bx, dims) == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for flags in (0, 1):                           # both binning modes were loaded by the init
        assert _noalloc_into(sf, p4, bx, dims, flags) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert lib.msf_noalloc_status(_stream()) == 0


def test_noalloc_refuses_continue():
    lib = mdsf.load()
    sf = torch.zeros((8, 8, 5), dtype=torch.float64, device="cuda")
    p4 = torch.zeros((1, 10, 4), dtype=torch.float32, device="cuda")
    assert _noalloc_into(sf, p4, (1.0, 1.0, 1.0), (8, 8, 8), flags=2) == -1   # MSF_CONTINUE: MSF_E_INVALID
    assert lib.msf_noalloc_status(_stream()) == 0


def test_noalloc_rejects_grids_beyond_the_scratch():
    lib = mdsf.load()
    sf = torch.zeros((256, 256, 65), dtype=torch.float64, device="cuda")
    p4 = torch.zeros((1, 10, 4), dtype=torch.float32, device="cuda")
    bx = (C.c_double * 3)(16.0, 13.856, 8.0)
    st = lib.msf_hist_sf_f32_noalloc(c_p(p4.data_ptr()), 10, 1, C.cast(bx, c_p), 256, 256, 128, 0,
                                     c_p(sf.data_ptr()), c_p(torch.cuda.current_stream().cuda_stream))
    assert st == -3  # MSF_E_WORKSPACE
