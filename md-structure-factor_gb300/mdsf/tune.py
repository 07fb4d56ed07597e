"""Autotuner: per grid shape, time the chain's variants and their tile and
batch sizes on the live GPU and cache the fastest.

What is tuned (each knob is a field of ``msf_plan_desc``):

* ``variant`` -- the FFT chain: the bucketed power-of-two chain (atoms binned
  per x-plane, deposit fused into the plane FFT), the smooth mixed-radix chain
  (2^a 3^b 5^c axes), or the generic plane / split engines;
* ``batch`` -- frames per pass (spectra held per batch);
* ``tile_w`` -- columns per x-pass tile (pencils per block of the x FFT);
* ``rows_per_block`` -- z-pass row pairs per block (split engine);
* ``deposit_block`` -- threads per histogram-deposit block.

The cache is a JSON file keyed by GPU name and grid shape
(``$MSF_TUNE_CACHE``, default ``~/.cache/mdsf_gb300/tune.json``).
:func:`lookup` reads it; :func:`tune` measures every candidate and writes the
winner; :func:`tune_for` returns the cached tuning of a shape, tuning it
first when the cache has none.  :func:`mdsf.structure_factor` and
:class:`mdsf.batch.BatchedSystems` use the cached tuning of a shape when the
caller gives none.  Candidates are timed with CUDA events on the whole chain
(deposit + FFT + |F|^2 + FP64 sum) over synthetic uniform frames of the
requested atom count.
"""
from __future__ import annotations

import json
import os
import threading

_lock = threading.Lock()


def cache_path():
    return os.environ.get("MSF_TUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "mdsf_gb300", "tune.json"))


def _gpu_name():
    import torch
    return torch.cuda.get_device_name() if torch.cuda.is_available() else "cpu"


def key(dims):
    """Cache key of a grid shape on this GPU."""
    return "%s|%dx%dx%d" % (_gpu_name_cached(), *dims)


_memo = {}


def _read():
    """The cache file's contents (re-read only when the file changed)."""
    path = cache_path()
    try:
        st = os.stat(path)
    except OSError:
        return {}
    stamp = (path, st.st_mtime_ns, st.st_size)
    if _memo.get("stamp") != stamp:
        try:
            with open(path) as f:
                _memo["data"] = json.load(f)
        except (OSError, ValueError):
            _memo["data"] = {}
        _memo["stamp"] = stamp
    return _memo["data"]


_names = {}


def _gpu_name_cached():
    import torch
    d = torch.cuda.current_device() if torch.cuda.is_available() else -1
    if d not in _names:
        _names[d] = _gpu_name()
    return _names[d]


def entry(dims):
    """The cache entry of a grid shape on this GPU (tuning, ms_per_frame,
    candidates tried), or None."""
    with _lock:
        return _read().get(key(tuple(int(d) for d in dims)))


def lookup(dims):
    """Cached tuning dict for this GPU and grid, or None."""
    e = entry(dims)
    return None if e is None else dict(e["tuning"])


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
    """Candidate tunings of a grid shape, the fused chains first.

    Power-of-two grids: the bucketed chain with 16/32/64-frame batches, the
    x tiles instantiated for n0, and the x pass of one batch overlapped with
    the next batch's plane FFT or not (``options=1``), then the smooth chain.  2^a 3^b 5^c grids:
    the smooth chain with 4-32-frame batches and 256/512-thread deposit
    blocks.  Other grids (a prime factor above 5, an odd n1): the generic
    plane and split engines with their tile widths, z rows per block and
    batches."""
    n0, n1, n2 = dims
    fused = False
    if all(_pow2(n) for n in dims):
        fused = True
        tiles = [w for w in (8, 16, 32) if n0 * w <= 8192]
        for b in (64, 32, 16):
            for w in tiles:
                for o in (0, 1):
                    yield dict(variant=3, batch=b, tile_w=w, options=o)
    if all(_smooth(n) for n in dims):
        fused = True
        for b in (8, 4, 16, 32):
            for db in (256, 512):
                yield dict(variant=4, batch=b, deposit_block=db)
    if fused:
        return
    variants = [1, 2] if n1 % 2 == 0 else [2]
    tiles = [w for w in (4, 8, 16, 32) if max(n0, n1) * w <= 4096]
    rows = sorted({max(2, min(32, 2048 // n2)), max(2, min(32, 1024 // n2)), max(2, min(32, 4096 // n2))})
    for v in variants:
        for w in tiles:
            for b in (4, 8, 16):
                for g in (rows if v == 2 else rows[:1]):
                    yield dict(variant=v, tile_w=w, rows_per_block=g, batch=b)


def _frames(dims, n_atoms, frames, device):
    """Uniform synthetic frames (float4, electrons in .w) made on the device."""
    import torch
    g = torch.Generator(device=device)
    g.manual_seed(17)
    p = torch.rand((frames, n_atoms, 4), generator=g, device=device)
    p[..., 3] = torch.tensor([1.0, 6.0, 7.0, 8.0], device=device)[
        torch.randint(0, 4, (n_atoms,), generator=g, device=device)]
    return p


def time_config(dims, n_atoms, tuning, frames=64, reps=3, device=None, positions=None):
    """Milliseconds per frame of the chain under `tuning` (None if the plan
    refuses it).  Box (1, 1, 1): positions are uniform in the unit cube."""
    import torch
    from ._lib import MsfError
    from .api import structure_factor
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    box = (1.0, 1.0, 1.0)
    p4 = positions if positions is not None else _frames(dims, n_atoms, frames, dev)
    out = torch.zeros((dims[0], dims[1], dims[2] // 2 + 1), dtype=torch.float64, device=dev)
    try:
        structure_factor(p4, box, None, dims, out=out, tuning=tuning, device=dev)
    except MsfError:          # a tuning the plan refuses for this shape
        return None
    torch.cuda.synchronize(dev)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        structure_factor(p4, box, None, dims, out=out, tuning=tuning, device=dev)
    e1.record()
    torch.cuda.synchronize(dev)
    return e0.elapsed_time(e1) / (reps * p4.shape[0])


def tune(dims, n_atoms=200_000, max_candidates=None, frames=128, device=None, verbose=False):
    """Time the candidates of `dims` (at most `max_candidates`) on `frames`
    frames, store the fastest in the cache and return it.  The default of
    128 frames spans several batches, so the overlap of one batch's x pass
    with the next batch's plane FFT is part of what is timed."""
    import torch
    from . import plan as _plan
    dims = tuple(int(d) for d in dims)
    before = set(_plan._cache)
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    p4 = _frames(dims, n_atoms, frames, dev)
    results = []
    for i, c in enumerate(candidates(dims)):
        if max_candidates and i >= max_candidates:
            break
        ms = time_config(dims, n_atoms, c, device=dev, positions=p4)
        if ms is not None:
            results.append((ms, c))
            if verbose:
                print("%8.4f ms/frame  %s" % (ms, c))
    del p4
    with _plan._cache_lock:      # drop the candidates' plans (and workspaces)
        for k in set(_plan._cache) - before:
            del _plan._cache[k]
    if not results:
        return None
    results.sort(key=lambda r: r[0])
    best_ms, best = results[0]
    with _lock:
        data = dict(_read())
        data[key(dims)] = {"tuning": best, "ms_per_frame": best_ms, "n_atoms": int(n_atoms), "frames": int(frames),
                           "tried": len(results),
                           "results": [{"tuning": c, "ms_per_frame": ms} for ms, c in results]}
        path = cache_path()
        os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
        tmp = path + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, path)
    return dict(best)


def tune_for(dims, n_atoms=200_000, max_candidates=None, frames=128, device=None):
    """The cached tuning of `dims` on this GPU, tuning the shape first if the
    cache has no entry for it."""
    t = lookup(dims)
    if t is None:
        t = tune(dims, n_atoms=n_atoms, max_candidates=max_candidates, frames=frames, device=device)
    return t
