"""Shared test set-up: import paths, the ``gpu`` marker and a process pool
for the oracle."""
import multiprocessing as mp
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_DIR = os.path.join(ROOT, "md-structure-factor_gb300")
for p in (ROOT, PKG_DIR):
    if p not in sys.path:
        sys.path.insert(0, p)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libmsf.so")


@pytest.fixture(scope="session")
def oracle_pool():
    """Spawned worker processes (safe after CUDA is initialised) that run
    oracle functions on the host's cores, for checks at full workload sizes."""
    n = max(1, min(16, os.cpu_count() or 1))
    with mp.get_context("spawn").Pool(n) as pool:
        yield pool
