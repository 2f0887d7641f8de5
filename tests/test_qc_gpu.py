"""GPU marker QC: the exact HWE test against the reference's SNPHWE2 outputs
(tests/golden/hwe_ref.json, from src/snphwe.cpp compiled unmodified), MAF and HWE p per SNP against
the oracle (src/input.cpp:388-394), and decoded count rows (src/option.cpp:471-472)."""
import json
import os

import numpy as np
import pytest

from conftest import make_case
from oracle import slemm_np as orc
from slemm_gb300 import api

pytestmark = pytest.mark.gpu
GOLD = os.path.join(os.path.dirname(__file__), "golden")


def test_hwe_exact_matches_reference_snphwe2(gpu):
    cases = json.load(open(os.path.join(GOLD, "hwe_ref.json")))["cases"]
    for midp in (0, 1):
        sel = [c for c in cases if c[3] == midp]
        het = np.array([c[0] for c in sel])
        h1 = np.array([c[1] for c in sel])
        h2 = np.array([c[2] for c in sel])
        ref = np.array([c[4] for c in sel])
        p = api.hwe_exact(het, h1, h2, midp)
        assert np.all(np.abs(p - ref) <= 1e-12 * ref), np.max(np.abs(p - ref) / ref)


@pytest.mark.parametrize("n_fam,m,missing,keep,midp", [
    (1000, 300, 0.0, 1.0, 0),
    (1001, 257, 0.02, 1.0, 1),
    (777, 1030, 0.01, 0.8, 0),
    (5000, 64, 0.05, 1.0, 1),
])
def test_marker_qc_vs_oracle(gpu, n_fam, m, missing, keep, midp):
    rows, keep_idx, dec = make_case(n_fam, m, seed=29, missing=missing, keep_frac=keep)
    with api.Genotypes(rows, n_fam, keep_idx) as g:
        maf, hwep = g.marker_qc(midp)
    rmaf, rhwe = orc.marker_qc(dec, midp)
    assert np.array_equal(maf, rmaf)
    # FP32-stored p-values: the FP64 values agree to ~1e-15, so the roundings agree
    assert np.allclose(hwep, rhwe, rtol=1e-6, atol=0)


def test_genotype_rows_decode(gpu):
    rows, keep_idx, dec = make_case(1537, 700, seed=31, missing=0.02, keep_frac=0.9)
    sel = np.array([0, 5, 127, 128, 699, 300], np.int64)
    with api.Genotypes(rows, 1537, keep_idx) as g:
        out = g.genotype_rows(sel)
    assert np.array_equal(out, dec[sel].T.astype(np.float32))


@pytest.mark.parametrize("keep", [1.0, 0.7])
def test_pinned_rows_upload_matches_pageable(gpu, keep):
    """.bed rows in pinned host memory take the upload path that first touches every host page
    from the device (geno.cu touch_host_pages_kernel) and a strided view of them the same path
    with a row stride: counts and decoded rows bit-exact against the oracle and the pageable
    upload."""
    import torch
    n_fam, m = 4097, 3001
    rows, keep_idx, dec = make_case(n_fam, m, seed=31, missing=0.01, keep_frac=keep)
    wide = np.zeros((m, rows.shape[1] + 13), np.uint8)
    wide[:, :rows.shape[1]] = rows
    pinned = torch.from_numpy(wide).pin_memory()
    strided = pinned.numpy()[:, :rows.shape[1]]
    assert not strided.flags["C_CONTIGUOUS"]
    idx = np.array([0, 5, 1500, m - 1], np.int64)
    with api.Genotypes(rows, n_fam, keep_idx) as ga:
        want = ga.counts()
        want_rows = ga.genotype_rows(idx)
    contiguous = torch.from_numpy(rows.copy()).pin_memory()
    for src in (contiguous.numpy(), strided):
        with api.Genotypes(src, n_fam, keep_idx) as gb:
            got = gb.counts()
            assert all(np.array_equal(a, b) for a, b in zip(got, want))
            assert np.array_equal(gb.genotype_rows(idx), want_rows)
    assert np.array_equal(want[0], orc.popcounts(dec))
