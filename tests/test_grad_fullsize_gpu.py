"""The REML log-likelihood gradient at its full workload size — n = 200,000 individuals,
m = 100,000 SNPs (5 GB of .bed rows), 2,000 window weights in (0, 2], 64 Rademacher probes —
where the dense FP64 oracle is out of reach (its n × n projection alone would take 320 GB).
Checked through properties that hold at every size:

* homogeneity: V = σ_e²·I + σ_g²·Σ_k w_k·K_k depends on σ_g² and the window weights only through
  the products σ_g²·w_k, so σ_g²·∂ℓ/∂σ_g² = Σ_k w_k·∂ℓ/∂w_k; the estimate keeps this exactly
  when every SNP is in a window (the same per-SNP probe terms enter both sides);
* reparametrisation: (s·w, σ_g²/s) gives the same V, hence ∂ℓ/∂w → ∂ℓ/∂w / s,
  ∂ℓ/∂σ_g² → s·∂ℓ/∂σ_g², ∂ℓ/∂σ_e² unchanged — although the Lanczos recurrence then runs on
  s·(K + τI) with different rounding throughout;
* precision: the BF16 hi+lo products in the solves agree with FP32 ones;
* determinism: the same seed gives the same bits.
"""
import numpy as np
import pytest

from slemm_gb300 import _lib, api, synth

pytestmark = pytest.mark.gpu

N, M, K, NV = 200_000, 100_000, 2000, 64
SG2, SE2 = 0.4, 0.6


@pytest.fixture(scope="module")
def full(gpu):
    rows, y = synth.simulate_bed_torch(N, M, seed=1, h2=0.4)
    window = np.minimum(np.arange(M) // (M // K), K - 1).astype(np.int32)
    wwin = (2.0 - np.random.default_rng(7).uniform(0.0, 2.0, K)).astype(np.float32)
    X = np.ones((N, 1), np.float32)
    persnp = np.ones(M, np.float32)
    g = api.Genotypes(rows.numpy(), N)
    g.set_precision(_lib.PREC_BF16X2)

    def grad(w=wwin, sg2=SG2, seed=0):
        return g.REML_grad(None, X, y.astype(np.float32), persnp, window, w, sg2, SE2, n_V=NV, seed=seed,
                           tol=1e-6)

    yield g, grad, wwin, grad()
    g.close()


def test_homogeneity_identity_full_size(full):
    _, _, wwin, r = full
    lhs = SG2 * r["d_sigma_g2"]
    rhs = float(np.dot(wwin.astype(np.float64), r["d_w"]))
    assert abs(lhs - rhs) <= 1e-6 * abs(lhs)


def test_reparametrisation_full_size(full):
    _, grad, wwin, r = full
    s = 1.7
    r2 = grad(w=(wwin * s).astype(np.float32), sg2=SG2 / s)
    dw = r2["d_w"] * s
    assert np.max(np.abs(dw - r["d_w"])) <= 1e-4 * np.max(np.abs(r["d_w"]))
    assert abs(r2["d_sigma_e2"] - r["d_sigma_e2"]) <= 1e-4 * abs(r["d_sigma_e2"])
    assert abs(r2["d_sigma_g2"] / s - r["d_sigma_g2"]) <= 2e-3 * abs(r["d_sigma_g2"])


def test_mixed_precision_solves_match_fp32_full_size(full):
    g, grad, _, r = full
    g.set_precision(_lib.PREC_FP32)
    try:
        rf = grad()
    finally:
        g.set_precision(_lib.PREC_BF16X2)
    assert np.max(np.abs(rf["d_w"] - r["d_w"])) <= 1e-4 * np.max(np.abs(rf["d_w"]))
    assert abs(rf["d_sigma_e2"] - r["d_sigma_e2"]) <= 1e-4 * abs(rf["d_sigma_e2"])
    # ∂ℓ/∂σ_g² is the difference of two terms a few hundred times larger than itself
    assert abs(rf["d_sigma_g2"] - r["d_sigma_g2"]) <= 2e-3 * abs(rf["d_sigma_g2"])


def test_gradient_is_deterministic_full_size(full):
    _, grad, _, r = full
    r2 = grad()
    assert r2["d_sigma_g2"] == r["d_sigma_g2"] and r2["d_sigma_e2"] == r["d_sigma_e2"]
    assert np.array_equal(r2["d_w"], r["d_w"])
