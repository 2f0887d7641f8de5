"""GPU parity of the packed-genotype operators against the oracle (reference src/reml.cpp:8-233).

Integer side outputs must be bit-exact.  Floating-point operators are compared with the FP64
restatement of the reference operators; the stated tolerance is on the relative Frobenius
error ‖out − ref‖/‖ref‖:
  FP32 CUDA-core path              ≤ 2e-6
  BF16 hi+lo tensor-core path      ≤ 4e-5
  BF16 hi+mid+lo tensor-core path  ≤ 2e-6
  FP16 hi+lo (column-scaled) path  ≤ 2e-6
"""
import numpy as np
import pytest

from conftest import make_case
from oracle import slemm_np as orc
from slemm_gb300 import _lib, api

pytestmark = pytest.mark.gpu

TOL = {_lib.PREC_FP32: 2e-6, _lib.PREC_BF16X2: 4e-5, _lib.PREC_BF16X3: 2e-6, _lib.PREC_FP16X2: 2e-6}


def relerr(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.mark.parametrize("n_fam,m,missing,keep", [
    (1000, 300, 0.0, 1.0),
    (1001, 257, 0.01, 1.0),
    (777, 1030, 0.01, 0.8),
    (130, 5, 0.0, 0.5),
])
def test_counts_bit_exact(gpu, n_fam, m, missing, keep):
    rows, keep_idx, dec = make_case(n_fam, m, seed=3, missing=missing, keep_frac=keep)
    with api.Genotypes(rows, n_fam, keep_idx) as g:
        pc, n0, n1, n2 = g.counts()
    rpc = orc.popcounts(dec)
    r0, r1, r2 = orc.hwe_counts(dec)
    assert np.array_equal(pc, rpc)
    assert np.array_equal(n0, r0) and np.array_equal(n1, r1) and np.array_equal(n2, r2)


def _setup(n_fam, m, seed, keep=1.0, c=2):
    rows, keep_idx, dec = make_case(n_fam, m, seed=seed, missing=0.01, keep_frac=keep)
    n = dec.shape[1]
    pc = orc.popcounts(dec)
    gm = orc.genotype_mean(pc, n)
    rng = np.random.default_rng(seed)
    persnp = rng.uniform(0.5, 1.5, m).astype(np.float32)
    w = orc.snp_weights(gm, persnp)
    w = np.where(np.isfinite(w), w, 0).astype(np.float32)
    rr = rng.uniform(0.7, 1.3, n).astype(np.float32)
    X = np.column_stack([np.ones(n), rng.standard_normal((n, c - 1))])
    Q, _, _ = orc.qr_colpiv(rr[:, None] * X, dtype=np.float64)
    return rows, keep_idx, dec, gm, w, rr, Q.astype(np.float32)


CASES = [(1000, 700, 1.0), (1537, 1300, 0.9)]


@pytest.mark.parametrize("prec", [_lib.PREC_FP16X2, _lib.PREC_BF16X2, _lib.PREC_BF16X3])
@pytest.mark.parametrize("k", [1, 7, 64, 66, 130])
def test_column_scales_and_piece_layout(gpu, prec, k):
    """Columns of very different magnitudes (1e-30 … 1e30, a zero column, a column with a large
    mean) in one block: FP16 pieces are scaled per column by a power of two, so every column keeps
    its own relative accuracy; k not a multiple of 8 exercises the padding rows between pieces and
    the epilogue's sum of a column's pieces.  Per-column relative error ≤ the path's tolerance."""
    rows, keep_idx, dec, gm, w, rr, Q = _setup(900, 650, seed=19)
    n, m = dec.shape[1], dec.shape[0]
    ref = orc.Operators(dec, gm, w, rr, Q, dtype=np.float64)
    rng = np.random.default_rng(23)
    # BF16 shares FP32's exponent range but its lo piece of a 1e-30 value is near FP32's
    # smallest normal; FP16 columns are rescaled, so they take the whole range
    exps = (-30, -12, -3, 0, 4, 12, 30) if prec == _lib.PREC_FP16X2 else (-12, -3, 0, 4, 12)
    scales = np.array([10.0 ** e for e in exps])
    v = rng.standard_normal((n, k)) * scales[np.arange(k) % scales.size]
    if k > 3:
        v[:, 2] = 0.0
        v[:, 3] += 50.0   # large mean
    u = rng.standard_normal((m, k)) * scales[(np.arange(k) + 3) % scales.size]
    v = v.astype(np.float32)
    u = u.astype(np.float32)
    with api.Genotypes(rows, 900, keep_idx) as g:
        g.set_weights(gm, w, rr)
        g.set_projection(Q)
        g.set_precision(prec)
        tol = TOL[prec]
        for got, want in ((g.rmatvec(v), ref.rmatvec(v)), (g.matvec(u), ref.matvec(u)),
                          (g.H0_ldet_mv(0.5, v), ref.H0_ldet_mv(0.5, v))):
            for c in range(k):
                if np.any(want[:, c] != 0):
                    assert relerr(got[:, c], want[:, c]) < tol, (c, relerr(got[:, c], want[:, c]))
                else:
                    assert np.all(got[:, c] == 0)


@pytest.mark.parametrize("prec", [_lib.PREC_FP32, _lib.PREC_BF16X2, _lib.PREC_BF16X3, _lib.PREC_FP16X2])
@pytest.mark.parametrize("n_fam,m,keep", CASES)
def test_operators_vs_oracle(gpu, prec, n_fam, m, keep):
    rows, keep_idx, dec, gm, w, rr, Q = _setup(n_fam, m, seed=7, keep=keep)
    n = dec.shape[1]
    ref = orc.Operators(dec, gm, w, rr, Q, dtype=np.float64)
    rng = np.random.default_rng(11)
    tau0 = 0.4285714
    with api.Genotypes(rows, n_fam, keep_idx) as g:
        g.set_weights(gm, w, rr)
        g.set_projection(Q)
        g.set_precision(prec)
        for k in (1, 5, 64):
            v = rng.standard_normal((n, k)).astype(np.float32)
            u = rng.standard_normal((m, k)).astype(np.float32)
            tol = TOL[prec]
            assert relerr(g.H0_quadform_mv(tau0, v), ref.H0_quadform_mv(tau0, v)) < tol
            assert relerr(g.H0_ldet_mv(tau0, v), ref.H0_ldet_mv(tau0, v)) < tol
            assert relerr(g.rmatvec(v), ref.rmatvec(v)) < tol
            assert relerr(g.weighted_rmatvec(v), ref.weighted_rmatvec(v)) < tol
            assert relerr(g.matvec(u), ref.matvec(u)) < tol


@pytest.mark.parametrize("prec", [_lib.PREC_BF16X2, _lib.PREC_FP32])
def test_wide_blocks_and_groups(gpu, prec):
    """k beyond one column group (BF16 hi+lo groups 128 columns) and odd widths."""
    rows, keep_idx, dec, gm, w, rr, Q = _setup(700, 390, seed=9)
    n = dec.shape[1]
    ref = orc.Operators(dec, gm, w, rr, Q, dtype=np.float64)
    rng = np.random.default_rng(5)
    with api.Genotypes(rows, 700, keep_idx) as g:
        g.set_weights(gm, w, rr)
        g.set_projection(Q)
        g.set_precision(prec)
        for k in (66, 130):
            v = rng.standard_normal((n, k)).astype(np.float32)
            assert relerr(g.H0_ldet_mv(0.5, v), ref.H0_ldet_mv(0.5, v)) < TOL[prec]


def test_per_vector_fp32_matches_batched(gpu):
    """The per-vector FP32 path does the same arithmetic per column as the batched FP32 path."""
    rows, keep_idx, dec, gm, w, rr, Q = _setup(900, 500, seed=13)
    n = dec.shape[1]
    v = np.random.default_rng(3).standard_normal((n, 7)).astype(np.float32)
    with api.Genotypes(rows, 900, keep_idx) as g:
        g.set_weights(gm, w, rr)
        g.set_projection(Q)
        g.set_precision(_lib.PREC_FP32)
        a = g.H0_quadform_mv(0.3, v)
        g.set_per_vector(True)
        b = g.H0_quadform_mv(0.3, v)
    assert relerr(a, b) < 1e-6


def test_operator_determinism(gpu):
    rows, keep_idx, dec, gm, w, rr, Q = _setup(1200, 800, seed=17)
    n = dec.shape[1]
    v = np.random.default_rng(4).standard_normal((n, 33)).astype(np.float32)
    with api.Genotypes(rows, 1200, keep_idx) as g:
        g.set_weights(gm, w, rr)
        g.set_projection(Q)
        a = g.H0_quadform_mv(0.3, v)
        b = g.H0_quadform_mv(0.3, v)
    assert np.array_equal(a, b)


@pytest.mark.parametrize("n_fam,m", [(1001, 257), (130, 5), (4099, 300), (2048, 384)])
def test_tiled_pack_matches_subset_pack(gpu, n_fam, m):
    """The tiled pack's row-contiguous reads (no individual subset) and its keep-list gather with
    the identity subset build the same tiles: counts and operator outputs agree bit for bit in
    both directions."""
    rows, _, dec = make_case(n_fam, m, seed=23, missing=0.02)
    n = dec.shape[1]
    pc = orc.popcounts(dec)
    gm = orc.genotype_mean(pc, n)
    w = np.where(np.isfinite(orc.snp_weights(gm, np.ones(m, np.float32))), orc.snp_weights(gm, np.ones(m, np.float32)), 0)
    w = w.astype(np.float32)
    rng = np.random.default_rng(2)
    v = rng.standard_normal((n, 5)).astype(np.float32)
    u = rng.standard_normal((m, 5)).astype(np.float32)
    outs = []
    for keep in (None, np.arange(n_fam, dtype=np.int64)):
        with api.Genotypes(rows, n_fam, keep) as g:
            g.set_weights(gm, w, None)
            pcg = g.counts()[0]
            outs.append((pcg, g.H0_ldet_mv(0.2, v), g.matvec(u), g.rmatvec(v)))
    for a, b in zip(outs[0], outs[1]):
        assert np.array_equal(a, b)
    assert np.array_equal(outs[0][0], pc)


def test_errors_are_status_codes(gpu):
    rows, keep_idx, dec, gm, w, rr, Q = _setup(300, 130, seed=19)
    with api.Genotypes(rows, 300, keep_idx) as g:
        with pytest.raises(_lib.SlemmError) as e:
            g.H0_ldet_mv(0.3, np.ones((dec.shape[1], 1), np.float32))   # weights not set
        assert e.value.code == -4
        with pytest.raises(_lib.SlemmError) as e:
            g.set_precision(9)
        assert e.value.code == -1


def test_gwa_windows_rejects_model_snps_outside_the_tested_range(gpu):
    """slemm_gwa's blocks take their share of the tested range from the model SNPs' positions, so
    model SNPs outside [test_begin, test_end] are an argument error (nothing is launched)."""
    rows, _, dec = make_case(600, 400, seed=67)
    y = np.random.default_rng(1).standard_normal(600).astype(np.float32)
    model = np.arange(0, 400, 4, dtype=np.int64)   # up to SNP 396
    with api.Genotypes(rows, 600) as g:
        with pytest.raises(_lib.SlemmError) as e:
            g.gwa_windows(y, None, np.ones((600, 1), np.float32), model, 0, 199, 40, 1.5, model.size, 1.0, 0.5)
        assert e.value.code == -1
        beta, _, _, _ = g.gwa_windows(y, None, np.ones((600, 1), np.float32), model, 0, 399, 40, 1.5, model.size,
                                      1.0, 0.5)
        assert beta.shape == (400,)


def test_create_from_device_rows(gpu):
    """SLEMM_ROWS_DEVICE: .bed rows already in HBM build the same tiles as host rows."""
    import torch
    rows, _, dec = make_case(1001, 257, seed=61, missing=0.02)
    v = np.random.default_rng(3).standard_normal((1001, 3)).astype(np.float32)
    gm = orc.genotype_mean(orc.popcounts(dec), 1001)
    w = np.full(257, 1.0 / 257, np.float32)
    with api.Genotypes(rows, 1001) as g:
        g.set_weights(gm, w)
        a = (g.counts()[0], g.rmatvec(v))
    with api.Genotypes(torch.from_numpy(np.ascontiguousarray(rows)).cuda(), 1001) as g:
        g.set_weights(gm, w)
        b = (g.counts()[0], g.rmatvec(v))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
