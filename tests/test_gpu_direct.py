"""Direct-sum S(q) and its adjoint against the FP64 oracle and central FD."""
import numpy as np
import pytest
import torch

import mdsf
from oracle import direct as odirect

pytestmark = pytest.mark.gpu


def system(n=2000, m=3000, L=6.0, seed=0):
    rng = np.random.default_rng(seed)
    r = rng.uniform(0, L, (n, 3)).astype(np.float32)
    f = rng.choice(np.array([1, 6, 7, 8], np.float32), n)
    d = rng.standard_normal((m, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    q = (d * rng.uniform(5, 15, (m, 1))).astype(np.float32)
    return r, f, q


def test_forward_matches_fp64():
    r, f, q = system()
    S = mdsf.direct_sf(torch.from_numpy(r).cuda(), torch.from_numpy(f).cuda(), torch.from_numpy(q).cuda())
    ref = odirect.sf(r, f, q)
    err = np.linalg.norm(S.cpu().numpy() - ref) / np.linalg.norm(ref)
    assert err < 2e-5, err


def test_adjoint_matches_fp64_gradient_and_fd():
    r, f, q = system(n=400, m=2000, seed=1)
    rng = np.random.default_rng(2)
    target = odirect.sf(r + rng.normal(0, 0.05, r.shape), f, q)
    rt = torch.from_numpy(r).cuda().requires_grad_(True)
    ft = torch.from_numpy(f).cuda().requires_grad_(True)
    S = mdsf.direct_sf(rt, ft, torch.from_numpy(q).cuda())
    tt = torch.from_numpy(target).cuda().float()
    loss = torch.mean((torch.log1p(S) - torch.log1p(tt)) ** 2)
    loss.backward()
    S64 = odirect.sf(r, f, q)
    _, dLdS = odirect.loss_log1p_mse(S64, target)
    gr_ref, gf_ref = odirect.grad(r, f, q, dLdS)
    gr = rt.grad.cpu().numpy()
    err = np.linalg.norm(gr - gr_ref) / np.linalg.norm(gr_ref)
    assert err < 1e-4, err
    errf = np.linalg.norm(ft.grad.cpu().numpy() - gf_ref) / np.linalg.norm(gf_ref)
    assert errf < 1e-4, errf
    atoms = [0, 7, 123]
    fd = odirect.fd_grad(r, f, q, target, h=1e-5, atoms=atoms)
    np.testing.assert_allclose(gr_ref[atoms], fd, rtol=1e-4, atol=1e-4 * np.abs(gr_ref).max())
    err_fd = np.linalg.norm(gr[atoms] - fd) / np.linalg.norm(fd)
    assert err_fd < 1e-4, err_fd


def test_batched_systems_shared_and_per_system_q():
    rs, fs = [], []
    for s in range(3):
        r, f, q = system(n=500, m=700, seed=10 + s)
        rs.append(r)
        fs.append(f)
    R = torch.from_numpy(np.stack(rs)).cuda()
    Fw = torch.from_numpy(np.stack(fs)).cuda()
    Q = torch.from_numpy(q).cuda()
    S = mdsf.direct_sf(R, Fw, Q).cpu().numpy()
    for s in range(3):
        ref = odirect.sf(rs[s], fs[s], q)
        assert np.linalg.norm(S[s] - ref) / np.linalg.norm(ref) < 2e-5
    Qs = Q.unsqueeze(0).expand(3, -1, -1).contiguous()
    S2 = mdsf.direct_sf(R, Fw, Qs).cpu().numpy()
    np.testing.assert_allclose(S2, S, rtol=1e-6)
