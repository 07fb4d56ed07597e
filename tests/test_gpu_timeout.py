"""The bounded waits' error path, made to happen without any fault: a plan
with MSF_PLAN_DIAG_STALL arms the plane kernel's first wait for bytes that no
copy delivers, so the wait runs out, MSF_E_TIMEOUT is latched and read by
msf_plan_status, and the context stays usable for the next (normal) call."""
import time

import numpy as np
import pytest
import torch

import mdsf
from mdsf import synth
from mdsf._lib import c_p, call
from mdsf.api import _ptr
from oracle import hist as ohist

pytestmark = pytest.mark.gpu
MSF_PLAN_DIAG_STALL = 2
MSF_E_TIMEOUT = -7


def test_stalled_wait_reports_timeout_and_context_survives():
    dims, n = (64, 64, 64), 5000
    pos, box, w = synth.uniform_system(n, (2.0, 2.0, 2.0), frames=3, seed=4)
    p4 = torch.from_numpy(synth.pack_float4(pos, w)).cuda()
    lib = mdsf.load()
    stream = c_p(torch.cuda.current_stream().cuda_stream)
    plan = mdsf.get_plan(dims, box, max_atoms=n, variant=3, options=MSF_PLAN_DIAG_STALL)
    sf = torch.zeros(plan.half_shape, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    call("msf_hist_sf_f32", plan.handle, _ptr(p4), n, 3, c_p(0), 0, _ptr(sf), stream)
    st = lib.msf_plan_status(plan.handle, stream)
    dt = time.perf_counter() - t0
    print(f"stalled chain returned after {dt * 1e3:.1f} ms (2 x 2^14 polls per waiting thread)")
    assert st == MSF_E_TIMEOUT
    assert lib.msf_plan_status(plan.handle, stream) == 0      # read and cleared
    # the same process and context: a normal chain gives the oracle's answer
    got = mdsf.structure_factor(p4, box, None, dims, tuning=dict(variant=3)).cpu().numpy()
    ref = ohist.hist_sf(pos, box, w, dims)
    assert np.abs(got - ref).max() / ref.max() < 1e-5
