"""ctypes binding of libslemm_gb300.so (the C ABI declared in include/slemm_gpu.h).

The library is the product: there is no Python or CPU fallback.  If the shared object is
missing this module raises instead of degrading.
"""
from __future__ import annotations

import ctypes
import os
import re

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libslemm_gb300.so")
HEADER = os.path.join(os.path.dirname(HERE), "include", "slemm_gpu.h")

OP_QUADFORM, OP_LDET, OP_MATVEC, OP_RMATVEC, OP_WRMATVEC = range(5)
ROWS_DEVICE = 1
PREC_FP32, PREC_BF16X2, PREC_BF16X3, PREC_FP16X2 = range(4)
MEM_HOST, MEM_DEVICE = 0, 1
LANCZOS_REORTH = 1

P = ctypes.c_void_p
I64 = ctypes.c_int64
I32 = ctypes.c_int
F32 = ctypes.c_float


class RemlOpts(ctypes.Structure):
    _fields_ = [("n_V", I32), ("seed", I32), ("tol_L", F32), ("s2max", F32), ("s2min", F32),
                ("tol_VC", F32), ("maxit", I32), ("verbose", I32)]


TRACE_MAX = 64


class RemlResult(ctypes.Structure):
    _fields_ = [("vg", F32), ("ve", F32), ("h2", F32), ("lrt", F32), ("iters_y", I32),
                ("iters_Q", I32), ("iters_V", I32), ("n_criterion", I32), ("seconds", ctypes.c_double),
                ("t_setup", ctypes.c_double), ("t_seed", ctypes.c_double), ("t_search", ctypes.c_double),
                ("t_final", ctypes.c_double), ("n_points", I32), ("h2_points", F32 * TRACE_MAX),
                ("f_points", ctypes.c_double * TRACE_MAX), ("first_iters_V", I32),
                ("first_n_criterion", I32)]

    def trace(self):
        """[(h², criterion)] of the search's evaluations, in order."""
        return [(float(self.h2_points[q]), float(self.f_points[q])) for q in range(self.n_points)]


class WindowOpts(ctypes.Structure):
    _fields_ = [("window_size", I32), ("sig_chisq", F32), ("indep_r2", F32), ("lrt", I32), ("n_MC", I32),
                ("n_MC_final", I32), ("max_fixed", I32)]


_SIGS = {
    "slemm_gpu_last_error": (ctypes.c_char_p, []),
    "slemm_gpu_version": (I32, []),
    "slemm_gpu_init": (I32, [I32]),
    "slemm_gpu_launch_count": (I64, []),
    "slemm_gpu_genotype_create": (I32, [P, I64, I64, I64, P, I64, I32, ctypes.POINTER(P)]),
    "slemm_gpu_genotype_destroy": (I32, [P]),
    "slemm_gpu_genotype_view": (I32, [P, P, I64, ctypes.POINTER(P)]),
    "slemm_gpu_genotype_dims": (I32, [P, ctypes.POINTER(I64), ctypes.POINTER(I64)]),
    "slemm_gpu_set_stream": (I32, [P, P]),
    "slemm_gpu_get_stream": (I32, [P, ctypes.POINTER(P)]),
    "slemm_gpu_genotype_counts": (I32, [P, P, P, P, P]),
    "slemm_gpu_marker_qc": (I32, [P, I32, P, P]),
    "slemm_gpu_hwe_exact": (I32, [P, P, P, I64, I32, P]),
    "slemm_gpu_genotype_rows": (I32, [P, P, I32, P, I64, I32]),
    "slemm_gpu_set_weights": (I32, [P, P, P, P]),
    "slemm_gpu_set_projection": (I32, [P, P, I64, I32]),
    "slemm_gpu_set_precision": (I32, [P, I32]),
    "slemm_gpu_set_per_vector": (I32, [P, I32]),
    "slemm_gpu_set_lanczos": (I32, [P, I32]),
    "slemm_gpu_set_autotune": (I32, [P, I32]),
    "slemm_gpu_autotune_table": (I32, [I32, ctypes.POINTER(I32), P, P, P]),
    "slemm_gpu_op": (I32, [P, I32, F32, P, I64, I32, P, I64, I32]),
    "slemm_gpu_lanczos_seed": (I32, [P, I32, F32, P, I64, I32, F32, I32, I32, ctypes.POINTER(P),
                                     ctypes.POINTER(I32)]),
    "slemm_gpu_lseed_destroy": (I32, [P]),
    "slemm_gpu_lseed_coeffs": (I32, [P, P, P]),
    "slemm_gpu_lanczos_solve": (I32, [P, F32, F32, P, I64, I32]),
    "slemm_gpu_tridiag_eig": (I32, [P, P, I32, I32, P, P]),
    "slemm_gpu_reml_sldf": (I32, [P, P, P, I64, I32, P, P, ctypes.POINTER(RemlOpts), P, P, P, P,
                                  ctypes.POINTER(RemlResult)]),
    "slemm_gpu_reml_lmc": (I32, [P, P, P, I64, I32, P, P, ctypes.POINTER(RemlOpts), P, P, P,
                                 ctypes.POINTER(RemlResult)]),
    "slemm_gpu_reml_grad": (I32, [P, P, P, I64, I32, P, P, P, I32, P, ctypes.c_double, ctypes.c_double, I32, I32,
                                  ctypes.c_float, P]),
    "slemm_gpu_reml_iter_weighting": (I32, [P, P, P, I64, I32, P, P, P, ctypes.POINTER(RemlOpts),
                                            ctypes.POINTER(WindowOpts), P, P, P, P, P, P,
                                            ctypes.POINTER(I32), ctypes.POINTER(RemlResult)]),
    "slemm_gpu_lmm_quadforms": (I32, [P, P, F32, F32, I32, I32, P, P, P, P, P, ctypes.POINTER(I32)]),
    "slemm_gpu_gwa_windows": (I32, [P, P, P, P, I64, I32, P, I64, I64, I64, I32, F32, I64, F32, F32, I32,
                                    P, P, P, P]),
    "slemm_gpu_wls": (I32, [P, P, P, I64, I32, P, P]),
    "slemm_gpu_gebv": (I32, [P, P, P, P]),
    "slemm_gpu_score_terms": (I32, [P, P, I32, P, P]),
    "slemm_gpu_profile": (I32, [P, I32, I32, ctypes.POINTER(I32), P, P, P]),
    "slemm_gpu_test_withhold_b_stage": (I32, [I32]),
    "slemm_gpu_rademacher": (I32, [I32, I64, I32, P, I64, I32]),
}

_LIB = None


class SlemmError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"[{code}] {msg}")
        self.code = code


def header_symbols(path: str = HEADER):
    """Function names declared in the C ABI header."""
    txt = open(path).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(slemm_gpu_\w+)\s*\(", txt)))


def load():
    """Loads the library (built by slemm_gb300.build); raises if it is absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run `python -m slemm_gb300.build` "
                           "(there is no CPU fallback)")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGS.items():
        fn = getattr(lib, name, None)
        if fn is None:
            continue   # reported by the ABI test (every header symbol must be exported)
        fn.restype = res
        fn.argtypes = args
    _LIB = lib
    return lib


def check(status: int):
    if status != 0:
        msg = load().slemm_gpu_last_error().decode(errors="replace")
        raise SlemmError(status, msg)
