"""slemm_gb300 — GB300-native engine for SLEMM's packed-genotype REML / BLUP / GWAS path.

The compute lives in libslemm_gb300.so (hand-written sm_103a CUDA behind the C ABI of
include/slemm_gpu.h).  This package holds the build script, the ctypes binding and a thin
host-side mirror of the reference's operator interface (``api``), plus a synthetic data
generator (``synth``).
"""
from ._lib import (OP_LDET, OP_MATVEC, OP_QUADFORM, OP_RMATVEC, OP_WRMATVEC, PREC_BF16X2,
                   PREC_BF16X3, PREC_FP32, SlemmError, load)

__all__ = ["load", "SlemmError", "OP_QUADFORM", "OP_LDET", "OP_MATVEC", "OP_RMATVEC",
           "OP_WRMATVEC", "PREC_FP32", "PREC_BF16X2", "PREC_BF16X3"]
