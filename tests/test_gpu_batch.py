"""Batched systems (one CUDA graph over systems of uneven size and grid
shape) against the oracle, system by system."""
import numpy as np
import pytest
import torch

import mdsf
from mdsf.batch import BatchedSystems, random_batch
from oracle import hist as ohist

pytestmark = pytest.mark.gpu
TOL = 1e-5


def _oracle(s):
    p = s["pos_w"].cpu().numpy()
    return ohist.hist_sf(p[..., :3], np.asarray(s["box"]), p[0, :, 3].astype(np.int32), s["dims"])


def test_batched_systems_match_oracle_and_accumulate():
    dev = torch.device("cuda")
    g = torch.Generator(device=dev)
    g.manual_seed(3)
    specs = [((64, 64, 64), 3000, 3), ((48, 50, 54), 5000, 2), ((32, 128, 64), 1000, 4),
             ((75, 81, 45), 2000, 2), ((128, 96, 160), 4000, 1)]
    systems = []
    for dims, n, t in specs:
        L = np.array([2.0 + 0.1 * dims[0] / 16, 2.5, 1.9])
        p = torch.rand((t, n, 4), generator=g, device=dev)
        p[..., :3] *= torch.tensor(L, dtype=torch.float32, device=dev)
        p[..., 3] = torch.randint(1, 9, (n,), generator=g, device=dev).float()
        systems.append(dict(pos_w=p, box=L, dims=dims))
    b = BatchedSystems(systems, n_streams=3)
    b.run()
    torch.cuda.synchronize()
    refs = [_oracle(s) for s in systems]
    for i, (s, ref) in enumerate(zip(systems, refs)):
        got = b.sf[i].cpu().numpy()
        assert np.abs(got - ref).max() / ref.max() < TOL, (i, s["dims"])
    b.run()                                  # replay accumulates
    torch.cuda.synchronize()
    for i, ref in enumerate(refs):
        got = b.sf[i].cpu().numpy()
        assert np.abs(got - 2 * ref).max() / ref.max() < 2 * TOL
    # power-of-two grid: bucketed chain; 2^a 3^b 5^c grid: smooth (mixed-radix) chain
    assert b.tuning(0)["variant"] == 3 and b.tuning(1)["variant"] == 4


def test_random_batch_generator_shapes():
    systems = random_batch(n_systems=3, atoms=(100, 200), frames=(1, 2))
    for s in systems:
        assert s["pos_w"].shape[-1] == 4 and len(s["dims"]) == 3
        assert all(48 <= d <= 256 for d in s["dims"])
