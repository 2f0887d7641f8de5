"""REML parity at the benchmark's CPU-sized configuration: n = 2,000 individuals, m = 10,000 SNPs,
Binomial(2, p) genotypes with p ~ U(0.05, 0.5), 1 % missing calls, y = Z_std·β + e with 1,000
causal SNPs and h² = 0.5, 30 Rademacher probes, seed 1 — against the FP64 oracle and the FP32
oracle (the reference's arithmetic, src/reml.cpp) on the same inputs and probes.

Tolerances:
  h² vs the FP64 oracle                         |Δ| ≤ 1e-4  (DF-REML and MC-REML, every precision)
  DF-REML golden-section branches               identical to the FP64 oracle's wherever the
                                                oracle's two criteria differ by more than 2·F_TOL;
                                                2logLL at common points within F_TOL
  MC-REML secant points                         within 1e-5 of the FP32 and FP64 oracles'
  SNP-BLUP and GEBV correlation with FP64       ≥ 0.99999
The reference's FP32 golden-section search is itself no closer than about 2e-4 to the FP64 one on
this configuration (its float criterion moves by ~1e-4 from point to point), which
test_oracle.test_fp32_reference_gss_spread_at_config1 records on the CPU; so the GPU is held to
1e-4 against FP64 and to the FP32 oracle's own distance from FP64 plus 1e-4.
"""
import numpy as np
import pytest

from conftest import check_gss_branches
from oracle import slemm_np as orc
from slemm_gb300 import _lib, api, synth

pytestmark = pytest.mark.gpu

N, M, N_V, SEED = 2000, 10000, 30, 1
F_TOL = 2e-3
PRECS = [_lib.PREC_BF16X2, _lib.PREC_FP16X2, _lib.PREC_FP32]


@pytest.fixture(scope="module")
def case1():
    counts, _ = synth.simulate_counts(N, M, seed=SEED)
    rows = synth.encode_bed(counts, missing=0.01, seed=SEED + 11)
    dec = orc.bed_decode(rows, N)
    y, _, _ = synth.simulate_phenotype(dec, 0.5, n_causal=1000, seed=SEED)
    y = y.astype(np.float32)
    X = np.ones((N, 1), np.float32)
    persnp = np.ones(M, np.float32)
    out = dict(rows=rows, dec=dec, y=y, X=X, persnp=persnp)
    for dt, key in ((np.float64, "64"), (np.float32, "32")):
        out["sldf" + key] = orc.SLDF_REML(dec, None, X, y, persnp, seed=SEED, n_V=N_V, dtype=dt)
        out["lmc" + key] = orc.LMC_REML(dec, None, X, y, persnp, seed=SEED, n_MC=N_V, dtype=dt)
    return out


@pytest.mark.parametrize("prec", PRECS)
def test_sldf_config1(gpu, case1, prec):
    r64, r32 = case1["sldf64"], case1["sldf32"]
    with api.Genotypes(case1["rows"], N) as g:
        g.set_precision(prec)
        r = g.SLDF_REML(None, case1["X"], case1["y"], case1["persnp"], seed=SEED, n_V=N_V)
        gebv = g.gebv(r["snp_blup"].astype(np.float64))
    assert r["n_criterion"] == len(r64["gss"]) == len(r["trace"])
    # identical points until the first branch the FP64 oracle took by a margin ≤ 2·F_TOL
    check_gss_branches(r["trace"], r64["gss"], F_TOL)
    assert abs(r["h2"] - r64["h2"]) <= 1e-4
    assert abs(r["h2"] - r32["h2"]) <= abs(r32["h2"] - r64["h2"]) + 1e-4
    assert np.corrcoef(r["snp_blup"], r64["snp_blup"])[0, 1] >= 0.99999
    assert np.corrcoef(gebv, orc.gebv(case1["dec"], r64["snp_blup"]))[0, 1] >= 0.99999


@pytest.mark.parametrize("prec", PRECS)
def test_lmc_config1(gpu, case1, prec):
    r64, r32 = case1["lmc64"], case1["lmc32"]
    with api.Genotypes(case1["rows"], N) as g:
        g.set_precision(prec)
        r = g.LMC_REML(None, case1["X"], case1["y"], case1["persnp"], seed=SEED, n_MC=N_V)
    pts = [p for p, _ in r["trace"]]
    assert len(pts) == len(r64["secant"]) == len(r32["secant"])
    assert np.allclose(pts, [p for p, _ in r64["secant"]], rtol=0, atol=1e-5)
    assert np.allclose(pts, [p for p, _ in r32["secant"]], rtol=0, atol=1e-5)
    assert abs(r["h2"] - r64["h2"]) <= 1e-5
    assert abs(r["h2"] - r32["h2"]) <= 1e-5
    assert np.corrcoef(r["snp_blup"], r64["snp_blup"])[0, 1] >= 0.99999


def test_sldf_config1_reorth(gpu, case1):
    """The opt-in reorthogonalised seeds against the FP64 oracle run the same way."""
    r64 = orc.SLDF_REML(case1["dec"], None, case1["X"], case1["y"], case1["persnp"], seed=SEED, n_V=N_V,
                        dtype=np.float64, reorth=True)
    with api.Genotypes(case1["rows"], N) as g:
        g.set_precision(_lib.PREC_FP16X2)
        g.set_lanczos(reorth=True)
        r = g.SLDF_REML(None, case1["X"], case1["y"], case1["persnp"], seed=SEED, n_V=N_V)
    assert tuple(r["iters"]) == tuple(r64["iters"])
    assert abs(r["h2"] - r64["h2"]) <= 1e-4
    assert abs(r["h2"] - case1["sldf64"]["h2"]) <= 1e-4
    assert np.corrcoef(r["snp_blup"], r64["snp_blup"])[0, 1] >= 0.99999
