"""The autotuner on the GPU: it times candidates of a grid shape, caches the
fastest per GPU and shape, and structure_factor then runs that tuning (and
still gives the oracle's S(q))."""
import json

import numpy as np
import pytest

import mdsf
from mdsf import synth, tune
from oracle import hist as ohist

pytestmark = pytest.mark.gpu


def test_tune_caches_and_is_used(tmp_path, monkeypatch):
    cache = tmp_path / "tune.json"
    monkeypatch.setenv("MSF_TUNE_CACHE", str(cache))
    dims = (64, 64, 64)
    assert tune.lookup(dims) is None
    best = tune.tune_for(dims, n_atoms=20_000, max_candidates=4, frames=32)
    assert best is not None and best["variant"] in (3, 4)
    data = json.loads(cache.read_text())
    e = data[tune.key(dims)]
    assert 1 <= e["tried"] <= 4 and e["tuning"] == best     # tunings a plan refuses are skipped
    assert min(r["ms_per_frame"] for r in e["results"]) == e["ms_per_frame"]
    assert tune.lookup(dims) == best
    assert tune.tune_for(dims) == best                 # cached: no second tuning
    # structure_factor without a tuning runs the cached one
    pos, box, w = synth.uniform_system(20_000, (2.0, 2.0, 2.0), frames=5, seed=31)
    got = mdsf.structure_factor(pos, box, w, dims).cpu().numpy()
    plan = mdsf.get_plan(dims, box, max_atoms=20_000, **best)
    assert plan.tuning()["batch"] == best["batch"]
    ref = ohist.hist_sf(pos, box, w, dims)
    assert np.abs(got - ref).max() / ref.max() < 1e-5

