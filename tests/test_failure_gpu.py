"""Failure path of the tensor-core product's bounded waits, without a GPU fault.

slemm_gpu_test_withhold_b_stage makes the next tensor-core launch skip one dense-operand copy in
its first CTA: that CTA's barrier for the stage never fills, exactly like a copy that never
arrives.  Its waits run out after their 2 s budget, the CTA sets the handle's device error word,
drains the copies it has in flight, frees its tensor memory and returns; the call reports
SLEMM_ERR_CUDA and clears the word.  The same handle's next call must then be correct.  Both
kernel shapes are covered: the narrow ring (N ≤ 64, the dense tile rides on the stage barrier)
and the wide one (N > 64, the dense tile has its own barrier).
"""
import time

import numpy as np
import pytest

from conftest import make_case
from oracle import slemm_np as orc
from slemm_gb300 import _lib, api

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("k", [1, 40])
def test_withheld_copy_times_out_and_handle_recovers(gpu, k):
    n, m = 3001, 1537
    rows, _, dec = make_case(n, m, seed=61)
    pc = orc.popcounts(dec)
    gm = orc.genotype_mean(pc, n)
    w = orc.snp_weights(gm, np.ones(m, np.float32))
    v = np.random.default_rng(k).standard_normal((n, k)).astype(np.float32)
    want = orc.Operators(dec, gm, w, None, None, dtype=np.float64).rmatvec(v)
    with api.Genotypes(rows, n) as g:
        g.set_weights(gm, w)
        g.set_precision(_lib.PREC_BF16X2)
        _lib.check(gpu.slemm_gpu_test_withhold_b_stage(0))
        t0 = time.perf_counter()
        with pytest.raises(_lib.SlemmError) as e:
            g.rmatvec(v)
        elapsed = time.perf_counter() - t0
        assert e.value.code == -2                        # SLEMM_ERR_CUDA
        assert "bounded wait" in str(e.value)
        assert 1.5 < elapsed < 30.0                      # the 2 s budget ran out, then the CTA drained
        # the request was one-shot and the error word was cleared: the next call is correct
        got = g.rmatvec(v)
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 4e-5
        got = g.rmatvec(v)
        assert np.linalg.norm(got - want) / np.linalg.norm(want) < 4e-5
    # a pending request can be withdrawn
    _lib.check(gpu.slemm_gpu_test_withhold_b_stage(0))
    _lib.check(gpu.slemm_gpu_test_withhold_b_stage(-1))
    with api.Genotypes(rows, n) as g:
        g.set_weights(gm, w)
        g.set_precision(_lib.PREC_BF16X2)
        got = g.rmatvec(v)
    assert np.linalg.norm(got - want) / np.linalg.norm(want) < 4e-5
