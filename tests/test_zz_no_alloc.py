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


def _noalloc_sf(p4, box, dims):
    lib = mdsf.load()
    sf = torch.zeros((dims[0], dims[1], dims[2] // 2 + 1), dtype=torch.float64, device="cuda")
    bx = (C.c_double * 3)(*box)
    st = lib.msf_hist_sf_f32_noalloc(c_p(p4.data_ptr()), p4.shape[1], p4.shape[0], C.cast(bx, c_p),
                                     dims[0], dims[1], dims[2], 0, c_p(sf.data_ptr()),
                                     c_p(torch.cuda.current_stream().cuda_stream))
    assert st == 0, lib.msf_strerror(st)
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


def test_noalloc_rejects_grids_beyond_the_scratch():
    lib = mdsf.load()
    sf = torch.zeros((256, 256, 65), dtype=torch.float64, device="cuda")
    p4 = torch.zeros((1, 10, 4), dtype=torch.float32, device="cuda")
    bx = (C.c_double * 3)(16.0, 13.856, 8.0)
    st = lib.msf_hist_sf_f32_noalloc(c_p(p4.data_ptr()), 10, 1, C.cast(bx, c_p), 256, 256, 128, 0,
                                     c_p(sf.data_ptr()), c_p(torch.cuda.current_stream().cuda_stream))
    assert st == -3  # MSF_E_WORKSPACE
