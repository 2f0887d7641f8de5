"""Shared fixtures.  `-m gpu` tests need a GB300 and the built library; everything else runs on
the CPU (oracle checks, host logic, ABI exports)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 GPU and the built CUDA library")


@pytest.fixture(scope="session")
def built_lib():
    from slemm_gb300 import build
    build.build()
    from slemm_gb300 import _lib
    return _lib.load()


@pytest.fixture(scope="session")
def gpu(built_lib):
    from slemm_gb300 import api
    api.init(0)
    return built_lib


def make_case(n_fam, m, seed=1, missing=0.0, keep_frac=1.0):
    """Synthetic .bed rows plus the oracle's decoded counts of the kept individuals."""
    from oracle import slemm_np as orc
    from slemm_gb300 import synth
    counts, _ = synth.simulate_counts(n_fam, m, seed=seed)
    rows = synth.encode_bed(counts, missing=missing, seed=seed + 11)
    keep_idx = None
    keep_mask = None
    if keep_frac < 1.0:
        rng = np.random.default_rng(seed + 5)
        keep_mask = (rng.random(n_fam) < keep_frac).astype(np.uint8)
        keep_idx = np.nonzero(keep_mask)[0].astype(np.int64)
    dec = orc.bed_decode(rows, n_fam, keep_mask)
    return rows, keep_idx, dec
