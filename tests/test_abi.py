"""The C ABI library builds for sm_103a, loads without a GPU, and exports every symbol that
include/slemm_gpu.h declares (no compute calls are made here)."""
import ctypes

import pytest

from slemm_gb300 import _lib


def test_header_declares_the_boundary():
    syms = _lib.header_symbols()
    for s in ("slemm_gpu_genotype_create", "slemm_gpu_op", "slemm_gpu_lanczos_seed",
              "slemm_gpu_lanczos_solve", "slemm_gpu_reml_sldf", "slemm_gpu_reml_lmc",
              "slemm_gpu_gebv", "slemm_gpu_score_terms", "slemm_gpu_last_error"):
        assert s in syms


def test_library_exports_every_header_symbol(built_lib):
    lib = ctypes.CDLL(_lib.LIB_PATH)
    missing = [s for s in _lib.header_symbols() if not hasattr(lib, s)]
    assert missing == []


def test_version_and_error_reporting_without_gpu(built_lib):
    assert built_lib.slemm_gpu_version() >= 100
    # null handle → argument error, reported through the thread-local message
    st = built_lib.slemm_gpu_set_precision(None, 1)
    assert st == -1
    assert b"null" in built_lib.slemm_gpu_last_error()
