"""slemm_gpu_rmatvec_noalloc: the Z_cᵀv entry point for callers that cannot allocate device memory
(a framework that has reserved the GPU's memory for its own pool, or a loop where cudaMalloc's
device-wide synchronisation is not allowed).  It must give the same product as the allocating
entry point slemm_gpu_op(SLEMM_OP_RMATVEC) on the FP32 path — within that path's operator
tolerance, ‖Δ‖/‖ref‖ ≤ 2e-6 — on consecutive calls that share its static scratch, and refuse sizes
beyond the scratch with an error instead of launching.

This file is collected last so that a run stopping at the first failure has run everything else.
"""
import ctypes

import numpy as np
import pytest

from slemm_gb300 import _lib, api, synth

pytestmark = pytest.mark.gpu
TOL = 2e-6


def _bind(lib):
    f = lib.slemm_gpu_rmatvec_noalloc
    f.restype = ctypes.c_int
    f.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int, ctypes.c_void_p,
                  ctypes.c_int64]
    return f


def test_noalloc_matches_allocating_entry_point_twice(gpu):
    import torch
    from oracle import slemm_np as orc
    n, m = 1537, 1100
    counts, _ = synth.simulate_counts(n, m, seed=61)
    rows = synth.encode_bed(counts, missing=0.01, seed=62)
    dec = orc.bed_decode(rows, n)
    gm = orc.genotype_mean(orc.popcounts(dec), n)
    w = np.ones(m, np.float32)
    noalloc = _bind(gpu)
    with api.Genotypes(rows, n) as g:
        g.set_weights(gm, w)
        g.set_precision(_lib.PREC_FP32)
        stream = torch.cuda.ExternalStream(g.stream())
        for call, k in enumerate((3, 5)):            # two calls in a row, sharing the scratch
            v = torch.randn(k, n, device="cuda", dtype=torch.float32,
                            generator=torch.Generator("cuda").manual_seed(call))
            ref = torch.zeros(k, m, device="cuda", dtype=torch.float32)
            out = torch.full((k, m), float("nan"), device="cuda", dtype=torch.float32)
            torch.cuda.synchronize()   # v, ref and out are written on torch's stream, read on the handle's
            g.op_device(_lib.OP_RMATVEC, v, ref)
            torch.cuda.synchronize()
            st = noalloc(g.h, ctypes.c_void_p(v.data_ptr()), n, k, ctypes.c_void_p(out.data_ptr()), m)
            _lib.check(st)
            stream.synchronize()
            err = (torch.linalg.norm(out.double() - ref.double()) / torch.linalg.norm(ref.double())).item()
            assert err <= TOL, (call, err)


def test_noalloc_constant_column_is_exact(gpu):
    """A constant column gives c·(pc − n·gm) (Z_cᵀ1 from the integer popcounts): the mean is
    removed from the operand and added back exactly, as on the allocating path."""
    import torch
    from oracle import slemm_np as orc
    n, m = 20000, 700
    counts, _ = synth.simulate_counts(n, m, seed=65)
    rows = synth.encode_bed(counts, missing=0.01, seed=66)
    dec = orc.bed_decode(rows, n)
    pc = orc.popcounts(dec)
    gm = orc.genotype_mean(pc, n)
    noalloc = _bind(gpu)
    with api.Genotypes(rows, n) as g:
        g.set_weights(gm, np.ones(m, np.float32))
        stream = torch.cuda.ExternalStream(g.stream())
        v = torch.full((1, n), 0.37, device="cuda", dtype=torch.float32)
        out = torch.zeros(1, m, device="cuda", dtype=torch.float32)
        torch.cuda.synchronize()   # written on torch's stream, read on the handle's
        _lib.check(noalloc(g.h, ctypes.c_void_p(v.data_ptr()), n, 1, ctypes.c_void_p(out.data_ptr()), m))
        stream.synchronize()
    want = np.float32(0.37) * (pc.astype(np.float64) - n * gm.astype(np.float64))
    got = out.cpu().numpy()[0].astype(np.float64)
    assert np.max(np.abs(got - want)) <= 1e-6 * max(1.0, np.max(np.abs(want)))


def test_noalloc_rejects_sizes_beyond_its_scratch(gpu):
    import torch
    n, m = 4096, 512
    counts, _ = synth.simulate_counts(n, m, seed=63)
    rows = synth.encode_bed(counts)
    noalloc = _bind(gpu)
    with api.Genotypes(rows, n) as g:
        g.set_weights(np.full(m, 1.0, np.float32), np.ones(m, np.float32))
        k = 4096                                         # 4·k·n alone is 64 MiB > 32 MiB
        v = torch.zeros(k, n, device="cuda", dtype=torch.float32)
        out = torch.zeros(k, m, device="cuda", dtype=torch.float32)
        st = noalloc(g.h, ctypes.c_void_p(v.data_ptr()), n, k, ctypes.c_void_p(out.data_ptr()), m)
        assert st == -7
        assert b"scratch" in gpu.slemm_gpu_last_error()
