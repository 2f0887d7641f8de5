"""The opt-in reorthogonalised Lanczos seeds (SLEMM_LANCZOS_REORTH) on the structure of the
window-weighted workload, at reduced size: n = 20,000 individuals, m = 6,000 SNPs with block LD
(AR(1) latent correlation 0.6 within 50-SNP blocks, thresholded to 0/1/2), h² = 0.3,
`--iter_weighting --lrt --window_size 50` (MC-REML equal-weight stage, window weights, clumping,
window-weighted DF-REML) with 30 probes, seed 1 — against the FP64 oracle run the same way with
the same reorthogonalisation.

Tolerances: h² within 1e-4 of the FP64 oracle for the reorthogonalised and the plain seeds at the
FP16 hi+lo and FP32 product paths; the same fixed-effect SNPs; the reorthogonalised step counts
within one of the oracle's; SNP-BLUP correlation ≥ 0.99999.
"""
import numpy as np
import pytest

from oracle import slemm_np as orc
from slemm_gb300 import _lib, api, synth

pytestmark = pytest.mark.gpu

N, M, N_V = 20000, 6000, 30
KW = dict(lrt=True, seed=0, n_V=N_V, window_size=50)


@pytest.fixture(scope="module")
def case():
    rows, y = synth.simulate_bed_torch(N, M, seed=1, h2=0.3, device="cpu", ld_rho=0.6, ld_block=50)
    rows = rows.numpy()
    y = y.astype(np.float32)
    dec = orc.bed_decode(rows, N)
    maf = orc.maf(orc.popcounts(dec), N)
    X = np.ones((N, 1), np.float32)
    ps = np.ones(M, np.float32)
    r64 = orc.REML_iter_weighting(dec, None, X, y, ps, maf, dtype=np.float64, reorth=True, **KW)
    return dict(rows=rows, y=y, maf=maf, X=X, ps=ps, r64=r64)


@pytest.mark.parametrize("prec", [_lib.PREC_FP16X2, _lib.PREC_FP32])
def test_iter_weighting_reorth_vs_oracle(gpu, case, prec):
    r64 = case["r64"]
    with api.Genotypes(case["rows"], N) as g:
        maf, _ = g.marker_qc()
        assert np.array_equal(maf, case["maf"])
        g.set_precision(prec)
        out = {}
        for reorth in (True, False):
            g.set_lanczos(reorth=reorth)
            out[reorth] = g.REML_iter_weighting(None, case["X"], case["y"], case["ps"], maf, **KW)
    for reorth, r in out.items():
        assert r["fixed"] == r64["fixed"]
        assert abs(r["h2"] - r64["h2"]) <= 1e-4, (reorth, r["h2"], r64["h2"])
        assert np.corrcoef(r["snp_blup"], r64["snp_blup"])[0, 1] >= 0.99999
    assert all(abs(a - b) <= 1 for a, b in zip(out[True]["iters"], r64["iters"])), (out[True]["iters"], r64["iters"])
