"""Trait views (slemm_gpu_genotype_view): several traits with their own missing individuals over one
packed .bed.  The reference analyses each trait on its own individual set (src/input.cpp:287,
src/option.cpp:320); a view shares the parent handle's packed copies and must give exactly what a
handle packed for those individuals gives:

  integer counts, MAF and decoded rows of the view's individuals   bit-exact against the oracle
  operators (all five kinds, projection, rr, FP16 / BF16 / FP32)   the operator tolerances of
                                                                   test_ops_gpu against FP64
  DF-REML per trait                                                h² within 1e-4 of the FP64 oracle
                                                                   with its golden-section branches,
                                                                   SNP-BLUP correlation ≥ 0.99999
"""
import numpy as np
import pytest

from conftest import check_gss_branches
from oracle import slemm_np as orc
from slemm_gb300 import _lib, api, synth

pytestmark = pytest.mark.gpu

TOL = {_lib.PREC_FP32: 2e-6, _lib.PREC_BF16X2: 4e-5, _lib.PREC_FP16X2: 2e-6}


def relerr(a, b):
    return np.linalg.norm(np.asarray(a, np.float64) - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def shared():
    import torch
    n_fam, m = 1600, 1500
    counts, _ = synth.simulate_counts(n_fam, m, seed=43)
    rows = synth.encode_bed(counts, missing=0.01, seed=44)
    dec_all = orc.bed_decode(rows, n_fam)
    rows_dev = torch.from_numpy(rows).cuda()
    return dict(n_fam=n_fam, m=m, rows=rows, rows_dev=rows_dev, dec=dec_all)


def test_view_counts_rows_and_maf_bit_exact(gpu, shared):
    rng = np.random.default_rng(5)
    keep = np.sort(rng.choice(shared["n_fam"], size=1111, replace=False)).astype(np.int64)
    ct = np.ascontiguousarray(shared["dec"][:, keep])
    with api.Genotypes(shared["rows_dev"], shared["n_fam"]) as parent:
        with api.Genotypes.view(parent, keep) as v:
            pc, n0, n1, n2 = v.counts()
            assert np.array_equal(pc, orc.popcounts(ct))
            h0, h1, h2 = orc.hwe_counts(ct)
            assert np.array_equal(n0, h0) and np.array_equal(n1, h1) and np.array_equal(n2, h2)
            maf, _ = v.marker_qc()
            assert np.array_equal(maf, orc.maf(orc.popcounts(ct), keep.size))
            idx = np.array([0, 7, 512, 1499], np.int64)
            assert np.array_equal(v.genotype_rows(idx), ct[idx].T.astype(np.float32))
        # the parent is untouched by its views
        assert np.array_equal(parent.counts()[0], orc.popcounts(shared["dec"]))


@pytest.mark.parametrize("prec", [_lib.PREC_FP16X2, _lib.PREC_BF16X2, _lib.PREC_FP32])
@pytest.mark.parametrize("k", [1, 7, 66])
def test_view_operators_vs_oracle(gpu, shared, prec, k):
    rng = np.random.default_rng(k + 10 * prec)
    keep = np.sort(rng.choice(shared["n_fam"], size=1203, replace=False)).astype(np.int64)
    ct = np.ascontiguousarray(shared["dec"][:, keep])
    n, m = keep.size, shared["m"]
    gm = orc.genotype_mean(orc.popcounts(ct), n)
    w = orc.snp_weights(gm, rng.uniform(0.5, 1.5, m).astype(np.float32))
    rr = rng.uniform(0.7, 1.3, n).astype(np.float32)
    X = np.column_stack([np.ones(n), rng.standard_normal(n)])
    Q, _, _ = orc.qr_colpiv(rr[:, None] * X)
    Q = Q.astype(np.float32)
    ref = orc.Operators(ct, gm, w, rr, Q, dtype=np.float64)
    v = rng.standard_normal((n, k)).astype(np.float32)
    u = rng.standard_normal((m, k)).astype(np.float32)
    with api.Genotypes(shared["rows_dev"], shared["n_fam"]) as parent, api.Genotypes.view(parent, keep) as g:
        g.set_weights(gm, w, rr)
        g.set_projection(Q)
        g.set_precision(prec)
        tol = TOL[prec]
        assert relerr(g.H0_quadform_mv(0.43, v), ref.H0_quadform_mv(0.43, v)) < tol
        assert relerr(g.H0_ldet_mv(0.43, v), ref.H0_ldet_mv(0.43, v)) < tol
        assert relerr(g.rmatvec(v), ref.rmatvec(v)) < tol
        assert relerr(g.weighted_rmatvec(v), ref.weighted_rmatvec(v)) < tol
        assert relerr(g.matvec(u), ref.matvec(u)) < tol


def test_view_per_trait_fits_vs_oracle(gpu, shared):
    """Three traits missing 5 %, 20 % and 40 % of the individuals, each a view of one parent."""
    n_fam, m = shared["n_fam"], shared["m"]
    rng = np.random.default_rng(43)
    persnp = np.ones(m, np.float32)
    with api.Genotypes(shared["rows_dev"], n_fam) as parent:
        for t, frac in enumerate((0.05, 0.2, 0.4)):
            keep = np.sort(rng.choice(n_fam, size=n_fam - int(frac * n_fam), replace=False)).astype(np.int64)
            ct = np.ascontiguousarray(shared["dec"][:, keep])
            y, _, _ = synth.simulate_phenotype(ct, 0.5, n_causal=150, seed=100 + t)
            y = y.astype(np.float32)
            X = np.column_stack([np.ones(keep.size), rng.standard_normal(keep.size)]).astype(np.float32)
            r64 = orc.SLDF_REML(ct, None, X, y, persnp, seed=3, n_V=12, dtype=np.float64)
            with api.Genotypes.view(parent, keep) as g:
                assert np.array_equal(g.counts()[0], orc.popcounts(ct))
                g.set_precision(_lib.PREC_FP16X2)
                r = g.SLDF_REML(None, X, y, persnp, seed=3, n_V=12)
            check_gss_branches(r["trace"], r64["gss"], 2e-3)
            assert abs(r["h2"] - r64["h2"]) <= 1e-4
            assert np.corrcoef(r["snp_blup"], r64["snp_blup"])[0, 1] >= 0.99999


def test_view_rejects_direct_readers(gpu, shared):
    keep = np.arange(0, shared["n_fam"], 3, dtype=np.int64)
    with api.Genotypes(shared["rows_dev"], shared["n_fam"]) as parent, api.Genotypes.view(parent, keep) as g:
        with pytest.raises(_lib.SlemmError) as e:
            g.gebv(np.ones(shared["m"]))
        assert e.value.code == -7 and "trait view" in str(e.value)
    with pytest.raises(_lib.SlemmError):   # indices must increase and lie in the parent
        with api.Genotypes(shared["rows_dev"], shared["n_fam"]) as parent:
            api.Genotypes.view(parent, np.array([3, 2], np.int64))
