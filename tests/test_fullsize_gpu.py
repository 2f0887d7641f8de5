"""Size-independent checks at the benchmark's full size: n = 100,000 individuals, m = 50,000 SNPs
(1.25 GB of .bed rows, the plain-FP32-vs-batched configuration), where the dense FP64 oracle is
out of reach:

* per-SNP integer counts bit-exact against the oracle's own decode (src/input.cpp:343-386 and
  :10-22, run chunk by chunk on the CPU);
* the adjoint identity ⟨Z_cᵀu, v⟩ = ⟨u, Z_c v⟩ and linearity of the packed products, both
  precisions;
* a constant column: Z_cᵀ1 = pc − n·gm exactly (the intercept column of the REML blocks, whose
  centring cancels almost completely);
* the metric's own criterion: the mixed-precision batched DF-REML agrees with the plain FP32
  per-vector GPU path to |Δh²| ≤ 1e-4.
"""
import numpy as np
import pytest

from oracle import slemm_np as orc
from slemm_gb300 import _lib, api, synth

pytestmark = pytest.mark.gpu

N, M = 100_000, 50_000


@pytest.fixture(scope="module")
def full(gpu):
    rows, y = synth.simulate_bed_torch(N, M, seed=1, h2=0.4)
    rows_np = rows.numpy()
    g = api.Genotypes(rows_np, N)
    yield rows_np, y.astype(np.float32), g
    g.close()


def _weights(g):
    pc = g.counts()[0]
    gm = orc.genotype_mean(pc, N)
    w = orc.snp_weights(gm, np.ones(M, np.float32))
    return gm, np.where(np.isfinite(w), w, 0).astype(np.float32)


def test_counts_bit_exact_full_size(full):
    rows_np, _, g = full
    pc, n0, n1, n2 = g.counts()
    chunk = 2000
    for j0 in range(0, M, chunk):
        dec = orc.bed_decode(rows_np[j0:j0 + chunk], N)
        want_pc = orc.popcounts(dec)
        w0, w1, w2 = orc.hwe_counts(dec)
        sl = slice(j0, j0 + dec.shape[0])
        assert np.array_equal(pc[sl], want_pc), f"popcounts differ in SNPs {j0}…"
        assert np.array_equal(n0[sl], w0) and np.array_equal(n1[sl], w1) and np.array_equal(n2[sl], w2)


@pytest.mark.parametrize("prec,tol", [(_lib.PREC_BF16X2, 4e-5), (_lib.PREC_FP32, 1e-5)])
def test_adjoint_and_linearity_full_size(full, prec, tol):
    _, _, g = full
    gm, w = _weights(g)
    g.set_weights(gm, w)
    g.set_precision(prec)
    rng = np.random.default_rng(11)
    u = rng.standard_normal((N, 4)).astype(np.float32)
    v = rng.standard_normal((M, 4)).astype(np.float32)
    ztu = g.rmatvec(u)                      # Z_cᵀ u   (m × 4)
    zv = g.matvec(v)                        # Z_c v    (n × 4)
    for c in range(4):
        lhs = float(np.dot(ztu[:, c].astype(np.float64), v[:, c]))
        rhs = float(np.dot(u[:, c].astype(np.float64), zv[:, c]))
        scale = np.linalg.norm(ztu[:, c]) * np.linalg.norm(v[:, c])
        assert abs(lhs - rhs) <= tol * scale, (c, lhs, rhs)
    # linearity: Z_c(v1 + 2 v2) = Z_c v1 + 2 Z_c v2 (each product carries its own rounding)
    both = g.matvec(v[:, :2] + 2.0 * v[:, 2:4])
    sep = zv[:, :2] + 2.0 * zv[:, 2:4]
    assert np.linalg.norm(both - sep) <= 2 * tol * np.linalg.norm(sep)
    g.set_precision(_lib.PREC_BF16X2)


def test_mixed_precision_reml_matches_fp32_per_vector_full_size(full):
    _, y, g = full
    X = np.ones((N, 1), np.float32)
    persnp = np.ones(M, np.float32)
    g.set_precision(_lib.PREC_BF16X2)
    g.set_per_vector(False)
    mixed = g.SLDF_REML(None, X, y, persnp, seed=0, n_V=64)
    g.set_precision(_lib.PREC_FP32)
    g.set_per_vector(True)
    try:
        plain = g.SLDF_REML(None, X, y, persnp, seed=0, n_V=64)
    finally:
        g.set_per_vector(False)
        g.set_precision(_lib.PREC_BF16X2)
    assert abs(mixed["h2"] - plain["h2"]) <= 1e-4, (mixed["h2"], plain["h2"])
    assert abs(mixed["vg"] - plain["vg"]) <= 1e-3 * abs(plain["vg"])
    assert 0.3 < mixed["h2"] < 0.5     # simulated h² = 0.4


@pytest.mark.parametrize("prec", [_lib.PREC_BF16X2, _lib.PREC_FP32])
def test_constant_column_full_size(full, prec):
    """Z_cᵀ(c·1) = c·(pc − n·gm): the product's centring must not leave the FP32 accumulation
    error of Cntᵀ1 (≈ 0.55·n per SNP) in a result that is only the rounding of gm."""
    _, _, g = full
    gm, w = _weights(g)
    g.set_weights(gm, w)
    g.set_precision(prec)
    pc = g.counts()[0]
    want = 0.37 * (pc.astype(np.float64) - N * gm.astype(np.float64))
    got = g.rmatvec(np.full((N, 1), 0.37, np.float32))[:, 0]
    assert np.max(np.abs(got - want)) <= 1e-5 * 0.37 * N ** 0.5 + 1e-6 * np.max(np.abs(want))
    # and mixed with a zero-mean part: linear in the constant
    u = np.random.default_rng(3).standard_normal((N, 1)).astype(np.float32)
    a = g.rmatvec(u)[:, 0]
    b = g.rmatvec(u + 0.37)[:, 0]
    assert np.linalg.norm(b - a - got) <= 4e-5 * np.linalg.norm(a)
    g.set_precision(_lib.PREC_BF16X2)
