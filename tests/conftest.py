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


def gss_margins(trace):
    """|fc − fd| at each golden-section iteration, from the evaluations in order (c₀, d₀, then one
    new point per iteration), with the reference's bookkeeping (src/reml.cpp:526-541)."""
    pts = [p for p, _ in trace]
    f = [v for _, v in trace]
    c, fc, d, fd = pts[0], f[0], pts[1], f[1]
    out = []
    for i in range(2, len(pts)):
        out.append(abs(fc - fd))
        if fc > fd:
            d, fd = c, fc
            c, fc = pts[i], f[i]
        else:
            c, fc = d, fd
            d, fd = pts[i], f[i]
    return out


def check_gss_branches(got, want, f_tol):
    """A GPU golden-section trace against the oracle's: the same h² points until the first branch
    the oracle itself took by a criterion margin of at most 2·f_tol, and 2logLL within f_tol at
    every common point.  Returns the number of common points."""
    want = [(float(p), float(v)) for p, v in want]
    assert len(got) == len(want)
    margins = gss_margins(want)
    k = next((i for i, (a, b) in enumerate(zip(got, want)) if a[0] != b[0]), len(want))
    if k < len(want):
        assert k >= 2 and margins[k - 2] <= 2 * f_tol, (k, margins[k - 2])
    for i in range(k):
        assert abs(got[i][1] - want[i][1]) <= f_tol, (i, got[i][1], want[i][1])
    return k


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


def load_gwa_case(d):
    """Inputs of bin/slemm_gwa.py for a golden case, parsed as the script does (:137-260): Py,
    covariates and R from .reml.py.txt; model SNPs of chromosome 1 (.reml.snp.csv order mapped to
    .bim indices); block size and cfactor = mean(xBx/xPx) from .gstat.txt; Vg/Ve and the model SNP
    count from .reml.vc.csv; the .bed rows and decoded A2 counts.  Returns a dict."""
    import os
    from oracle import slemm_np as orc
    fam = [l.split() for l in open(os.path.join(d, "geno.fam"))]
    bim = [l.split() for l in open(os.path.join(d, "geno.bim"))]
    n_fam = len(fam)
    raw = np.fromfile(os.path.join(d, "geno.bed"), dtype=np.uint8)[3:]
    rows = raw.reshape(-1, (n_fam + 3) // 4)
    py = [l.split() for l in open(os.path.join(d, "s1.reml.py.txt")).read().splitlines()[1:]]
    y = np.array([float(r[1]) for r in py], np.float32)
    covar = np.array([[float(v) for v in r[2:-1]] for r in py], np.float32)
    R = np.array([float(r[-1]) for r in py], np.float32)
    gs = [l.split() for l in open(os.path.join(d, "s1.gstat.txt")).read().splitlines()[1:]]
    cfactor = sum(float(r[8]) / float(r[7]) for r in gs) / len(gs)
    block_size = int(gs[-1][10])
    vc = open(os.path.join(d, "s1.reml.vc.csv")).read().splitlines()
    model_snp_ct = int(vc[1].split(",")[1])
    snp_var = float(vc[2].split(",")[1])
    err_var = float(vc[3].split(",")[1])
    ksnp = {l.split(",")[0] for l in open(os.path.join(d, "s1.reml.snp.csv")).read().splitlines()[1:]
            if l.split(",")[1] == "1"}
    ksnp_idx = [j for j, b in enumerate(bim) if b[1] in ksnp]
    chr_idx = [j for j, b in enumerate(bim) if b[0] == "1"]
    dec = orc.bed_decode(rows, n_fam)
    out = [l.split("\t") for l in open(os.path.join(d, "gwa.txt")).read().splitlines()[1:]]
    ref = {k: np.array([float(r[i]) for r in out]) for k, i in (("beta", 6), ("se", 7), ("chisq", 8), ("p", 9))}
    return dict(rows=rows, n_fam=n_fam, a2=dec, y=y, covar=covar, R=R, cfactor=cfactor, block_size=block_size,
                model_snp_ct=model_snp_ct, snp_var=snp_var, tau=err_var / snp_var, ksnp_idx=ksnp_idx,
                chr_start=min(chr_idx), chr_end=max(chr_idx), ref=ref, mac=20)
