"""Frame sharding and the FP64 sum across ranks, as two gloo processes on CPU.

Each rank computes the oracle power of its own frames (CPU), the sums are
combined with mdsf.shard.reduce_sf and must equal the single-process sum."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from mdsf.shard import reduce_sf, shard_range


def test_shard_range_partitions():
    for n in (0, 1, 7, 100, 101):
        for world in (1, 2, 3, 8):
            got = [shard_range(n, r, world) for r in range(world)]
            assert got[0][0] == 0 and got[-1][1] == n
            assert all(got[i][1] == got[i + 1][0] for i in range(world - 1))
            sizes = [b - a for a, b in got]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard_range(10, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out):
    import torch.distributed as dist
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "md-structure-factor_gb300")]
    from oracle import hist as ohist
    from mdsf import synth
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pos, box, w = synth.uniform_system(300, (1.0, 1.2, 0.9), frames=5, seed=8)
    a, b = shard_range(5, rank, world)
    sf = torch.from_numpy(ohist.hist_sf(pos[a:b], box, w, (8, 10, 6)) if b > a else np.zeros((8, 10, 4)))
    reduce_sf(sf)
    if rank == 0:
        torch.save(sf, out)
    dist.destroy_process_group()


def test_two_rank_sum_equals_single(tmp_path):
    out = str(tmp_path / "sf.pt")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    from oracle import hist as ohist
    from mdsf import synth
    pos, box, w = synth.uniform_system(300, (1.0, 1.2, 0.9), frames=5, seed=8)
    ref = ohist.hist_sf(pos, box, w, (8, 10, 6))
    np.testing.assert_allclose(torch.load(out).numpy(), ref, rtol=1e-12)
