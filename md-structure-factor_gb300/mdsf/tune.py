"""Autotuner: per grid shape, time the FFT variant, x/y tile width, z-pass
rows per block and frames per batch on the live GPU and cache the winner.

The cache is a JSON file keyed by GPU name and grid shape
(``$MSF_TUNE_CACHE``, default ``~/.cache/mdsf_gb300/tune.json``);
:func:`lookup` reads it, :func:`tune` measures and writes it.  Candidates
are timed with CUDA events on the full chain (deposit + FFT + |F|^2 + sum)
over a synthetic frame batch of the requested atom count.
"""
from __future__ import annotations

import itertools
import json
import os
import threading

import numpy as np

_lock = threading.Lock()


def cache_path():
    return os.environ.get("MSF_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "mdsf_gb300", "tune.json"))


def _gpu_name():
    import torch
    return torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"


def _key(dims):
    return "%s|%dx%dx%d" % (_gpu_name(), *dims)


def _read():
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def lookup(dims):
    """Cached tuning dict for this GPU and grid, or None."""
    with _lock:
        return _read().get(_key(dims), {}).get("tuning")


def _pow2(n):
    return n >= 16 and n & (n - 1) == 0


def _smooth(n):
    if n == 512:
        return True
    if not 16 <= n <= 256:
        return False
    for f in (2, 3, 5):
        while n % f == 0:
            n //= f
    return n == 1


def candidates(dims):
    """Bucketed chain (power-of-two axes, batches up to 64), the smooth
    mixed-radix chain (2^a 3^b 5^c axes), and the generic engine's plane and
    split variants with their tile widths and z rows per block."""
    n0, n1, n2 = dims
    if all(_pow2(n) for n in dims):
        for b in (16, 32, 64):
            yield dict(variant=3, batch=b)
    if all(_smooth(n) for n in dims):
        for b in (4, 8, 16, 32):
            yield dict(variant=4, batch=b)
    variants = [1, 2] if n1 % 2 == 0 else [2]
    tiles = [w for w in (4, 8, 16, 32) if max(n0, n1) * w <= 4096]
    rows = sorted({max(2, min(32, 2048 // n2)), max(2, min(32, 1024 // n2)), max(2, min(32, 4096 // n2))})
    batches = [4, 8, 16, 32]
    for v, w, b in itertools.product(variants, tiles, batches):
        for g in (rows if v == 2 else rows[:1]):
            yield dict(variant=v, tile_w=w, rows_per_block=g, batch=b)


def time_config(dims, box, n_atoms, tuning, frames=None, reps=3, device=None):
    import torch
    from . import synth
    from .api import structure_factor
    from .plan import Plan
    try:
        Plan(dims, box, device=device, **tuning)
    except Exception:
        return None
    if frames is None:   # two batches at least, so that batching and overlap show
        frames = max(16, 2 * int(tuning.get("batch", 4)))
    pos, _, w = synth.uniform_system(n_atoms, box, frames=frames, seed=17)
    p4 = torch.from_numpy(synth.pack_float4(pos, w)).cuda(device)
    out = torch.zeros((dims[0], dims[1], dims[2] // 2 + 1), dtype=torch.float64, device=p4.device)
    structure_factor(p4, box, None, dims, out=out, tuning=tuning)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        structure_factor(p4, box, None, dims, out=out, tuning=tuning)
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / (reps * frames)


def tune(dims, box=None, n_atoms=200_000, max_candidates=None, device=None, verbose=False):
    """Time every candidate, store and return the fastest tuning."""
    dims = tuple(int(d) for d in dims)
    box = box if box is not None else (1.0, 1.0, 1.0)
    results = []
    for i, c in enumerate(candidates(dims)):
        if max_candidates and i >= max_candidates:
            break
        ms = time_config(dims, box, n_atoms, c, device=device)
        if ms is not None:
            results.append((ms, c))
            if verbose:
                print("%8.4f ms/frame  %s" % (ms, c))
    if not results:
        return None
    results.sort(key=lambda r: r[0])
    best_ms, best = results[0]
    with _lock:
        data = _read()
        data[_key(dims)] = {"tuning": best, "ms_per_frame": best_ms, "n_atoms": n_atoms,
                            "tried": len(results)}
        path = cache_path()
        os.makedirs(os.path.dirname(path), exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    return best
