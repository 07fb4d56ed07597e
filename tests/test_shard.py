"""Frame sharding and the FP64 sum across ranks, as two gloo processes on CPU.

Each rank computes the oracle power of its own frames (CPU) with the inputs
mdsf.shard.shard_inputs gives it, the sums are combined with
mdsf.shard.reduce_sf and must equal the single-process sum -- also with
per-frame boxes, where every rank must rescale to and bin in the mean box of
the whole trajectory (dens.py:50-58), not of its own frames."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.multiprocessing as mp

from mdsf.shard import reduce_sf, shard_inputs, shard_range


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


def _boxes(T, seed=4):
    """Per-frame boxes that differ by a few percent (an NPT trajectory)."""
    rng = np.random.default_rng(seed)
    return np.array([1.0, 1.2, 0.9]) * (1 + 0.03 * rng.standard_normal((T, 1)))


def _system(per_frame_box):
    from mdsf import synth
    pos, box, w = synth.uniform_system(300, (1.0, 1.2, 0.9), frames=5, seed=8, dtype=np.float64)
    if per_frame_box:
        box = _boxes(5)
        pos = pos * (box / np.array([1.0, 1.2, 0.9]))[:, None, :]
    return pos, box, w


def _shard_sf(pos, box, w, dims, rank, world):
    """The oracle power of one rank's frames, binned as shard_inputs says."""
    from oracle import hist as ohist
    a, b, scale, L = shard_inputs(pos.shape[0], box, rank, world)
    sf = np.zeros((dims[0], dims[1], dims[2] // 2 + 1))
    for k, t in enumerate(range(a, b)):
        sf += ohist.power(ohist.hist_grid(pos[t], L, w, dims, None if scale is None else scale[k]))
    return sf


def _worker(rank, world, port, out, per_frame_box):
    import torch.distributed as dist
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path[:0] = [root, os.path.join(root, "md-structure-factor_gb300")]
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    pos, box, w = _system(per_frame_box)
    sf = torch.from_numpy(_shard_sf(pos, box, w, (8, 10, 6), rank, world))
    reduce_sf(sf)
    if rank == 0:
        torch.save(sf, out)
    dist.destroy_process_group()


@pytest.mark.parametrize("per_frame_box", [False, True])
def test_two_rank_sum_equals_single(tmp_path, per_frame_box):
    out = str(tmp_path / "sf.pt")
    mp.spawn(_worker, args=(2, _free_port(), out, per_frame_box), nprocs=2, join=True)
    from oracle import hist as ohist
    pos, box, w = _system(per_frame_box)
    ref = ohist.hist_sf(pos, box, w, (8, 10, 6))
    np.testing.assert_allclose(torch.load(out).numpy(), ref, rtol=1e-12)


def test_shard_inputs_use_the_trajectory_mean_box():
    box = _boxes(7)
    avg = box.mean(axis=0)
    rows = []
    for rank in range(3):
        a, b, scale, L = shard_inputs(7, box, rank, 3)
        np.testing.assert_array_equal(L, np.average(box, axis=0))
        np.testing.assert_array_equal(scale, np.average(box, axis=0) / box[a:b])
        rows.append(scale)
    np.testing.assert_allclose(np.concatenate(rows) * box, np.broadcast_to(avg, box.shape), rtol=1e-15)
    a, b, scale, L = shard_inputs(5, np.array([1.0, 2.0, 3.0]), 1, 2)
    assert scale is None and (a, b) == (3, 5) and list(L) == [1.0, 2.0, 3.0]
    with pytest.raises(ValueError):
        shard_inputs(6, box, 0, 2)

