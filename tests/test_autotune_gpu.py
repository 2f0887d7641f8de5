"""The split-K autotuner: a handle with autotune on times candidate split counts at the first pass
of each shape, caches the decision for the process, and computes the same operators as the fixed
rule (within the BF16 hi+lo and FP16 hi+lo operator tolerances against the FP64 oracle)."""
import numpy as np
import pytest

from conftest import make_case
from oracle import slemm_np as orc
from slemm_gb300 import _lib, api

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("prec,tol", [(_lib.PREC_FP16X2, 2e-6), (_lib.PREC_BF16X2, 4e-5)])
def test_autotuned_operators_match_oracle(gpu, prec, tol):
    n, m = 9001, 4099
    rows, _, dec = make_case(n, m, seed=83)
    pc = orc.popcounts(dec)
    gm = orc.genotype_mean(pc, n)
    w = orc.snp_weights(gm, np.ones(m, np.float32))
    ref = orc.Operators(dec, gm, w, None, None, dtype=np.float64)
    rng = np.random.default_rng(3)
    with api.Genotypes(rows, n) as g:
        g.set_weights(gm, w)
        g.set_precision(prec)
        g.set_autotune(True)
        for k in (65, 3):
            v = rng.standard_normal((n, k)).astype(np.float32)
            want = ref.H0_ldet_mv(0.43, v)
            got = g.H0_ldet_mv(0.43, v)
            assert np.linalg.norm(got - want) / np.linalg.norm(want) < tol
            table = api.autotune_table()
            again = g.H0_ldet_mv(0.43, v)          # cached: no new decisions, same plan, same bits
            assert len(api.autotune_table()) == len(table)
            assert np.array_equal(again, got)
    kp = {65: 72, 3: 8}
    for k in (65, 3):
        N = -(-2 * kp[k] // 16) * 16
        mine = [t for t in table if t["N"] == N and t["pieces"] == 2]
        assert {t["M_pad"] for t in mine} >= {4352, 9216}   # both directions: m and n padded to 256
        for t in mine:
            assert t["candidates"] >= 1 and t["splits"] >= 1 and t["ms"] > 0
            assert t["plan"] in ((0, 1) if N <= 64 else (0,))
            assert t["candidates"] >= (2 if N <= 64 else 1)             # N ≤ 64 also times the two-CTA plan
            assert t["ms"] <= t["ms_rule"] + 1e-9                        # never slower than the rule's count


@pytest.mark.parametrize("prec,tol", [(_lib.PREC_FP16X2, 2e-6), (_lib.PREC_BF16X2, 4e-5)])
@pytest.mark.parametrize("k", [1, 5, 24])
def test_two_cta_plan_matches_oracle(gpu, prec, tol, k):
    """The narrow plan with one 128-row tile per CTA and two CTAs per SM (256 TMEM columns each),
    forced for every pass with N ≤ 64, in both directions, and a ragged row count."""
    n, m = 7003, 5001
    rows, _, dec = make_case(n, m, seed=85)
    pc = orc.popcounts(dec)
    gm = orc.genotype_mean(pc, n)
    w = orc.snp_weights(gm, np.ones(m, np.float32))
    ref = orc.Operators(dec, gm, w, None, None, dtype=np.float64)
    rng = np.random.default_rng(k)
    v = rng.standard_normal((n, k)).astype(np.float32)
    u = rng.standard_normal((m, k)).astype(np.float32)
    with api.Genotypes(rows, n) as g:
        g.set_weights(gm, w)
        g.set_precision(prec)
        g.set_autotune("two_cta")
        for name, x in (("H0_ldet_mv", v), ("rmatvec", v)):
            got = getattr(g, name)(0.43, x) if name == "H0_ldet_mv" else g.rmatvec(x)
            want = ref.H0_ldet_mv(0.43, x) if name == "H0_ldet_mv" else ref.rmatvec(x)
            assert np.linalg.norm(got - want) / np.linalg.norm(want) < tol, name
        got = g.matvec(u)
        want = ref.matvec(u)
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < tol
