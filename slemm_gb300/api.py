"""Host-side mirror of the reference's operator interface over the C ABI.

Names follow the reference (src/reml.cpp): ``H0_quadform_mv``, ``H0_ldet_mv``, ``matvec``,
``rmatvec``, ``weighted_rmatvec``, ``L_Seed``, ``L_Solve``, ``SLDF_REML``, ``LMC_REML``.
Matrices are NumPy arrays (host; copied through the library) or CUDA tensors (device;
column-major n×k stored as a contiguous (k, n) tensor).  Errors raise ``SlemmError`` carrying
the library's status code — the reference instead exits or throws a C string.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import _lib
from ._lib import (WindowOpts, MEM_DEVICE, MEM_HOST, OP_LDET, OP_MATVEC, OP_QUADFORM, OP_RMATVEC,
                   OP_WRMATVEC, RemlOpts, RemlResult, check)

_OP_OF_NAME = {"quadform": OP_QUADFORM, "ldet": OP_LDET}


def _f32c(a, rows=None):
    """Column-major FP32 copy (Fortran order) of a host matrix/vector; returns (array, k)."""
    a = np.asarray(a, dtype=np.float32)
    if a.ndim == 1:
        a = a[:, None]
    return np.asfortranarray(a), a.shape[1]


def _ptr(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def init(device: int = 0):
    check(_lib.load().slemm_gpu_init(device))


def launch_count() -> int:
    return int(_lib.load().slemm_gpu_launch_count())


class Genotypes:
    """Packed genotypes resident in HBM (replaces the reference's kmat, src/option.cpp:347).

    bed_rows: m×ceil(n_fam/4) uint8 .bed rows (SNP-major, magic skipped) of the analysed SNPs in
    analysis order; keep_idx: indices of kept individuals in .fam order (None = all)."""

    def __init__(self, bed_rows, n_fam: int, keep_idx=None):
        self._lib = _lib.load()
        flags = 0
        if getattr(bed_rows, "is_cuda", False):   # a CUDA tensor of .bed rows: read in HBM
            rows = bed_rows.contiguous()
            ptr = ctypes.c_void_p(rows.data_ptr())
            flags = _lib.ROWS_DEVICE
            stride = rows.shape[1]
        else:
            rows = np.asarray(bed_rows)
            if not (rows.dtype == np.uint8 and rows.ndim == 2 and rows.strides[1] == 1
                    and rows.strides[0] >= rows.shape[1]):
                rows = np.ascontiguousarray(rows, dtype=np.uint8)   # rows with a byte stride pass as they are
            ptr = _ptr(rows)
            stride = rows.strides[0] if rows.shape[0] > 1 else rows.shape[1]
        m, rb = rows.shape
        if rb < (n_fam + 3) // 4:
            raise ValueError(f"rows of {rb} bytes hold fewer than the {n_fam} individuals' {(n_fam + 3) // 4} bytes")
        keep = None if keep_idx is None else np.ascontiguousarray(keep_idx, dtype=np.int64)
        n = n_fam if keep is None else keep.size
        h = ctypes.c_void_p()
        check(self._lib.slemm_gpu_genotype_create(ptr, n_fam, m, stride, _ptr(keep), n, flags,
                                                  ctypes.byref(h)))
        self.h = h
        self.n, self.m = int(n), int(m)

    @classmethod
    def view(cls, parent: "Genotypes", keep_idx):
        """A handle over the parent's individuals keep_idx that shares the parent's packed copies
        (slemm_gpu_genotype_view); the parent must stay open while the view is used."""
        keep = np.ascontiguousarray(keep_idx, dtype=np.int64)
        self = cls.__new__(cls)
        self._lib = _lib.load()
        h = ctypes.c_void_p()
        check(self._lib.slemm_gpu_genotype_view(parent.h, _ptr(keep), keep.size, ctypes.byref(h)))
        self.h = h
        self.n, self.m = int(keep.size), parent.m
        self._parent = parent   # keeps the parent alive as long as the view
        return self

    def close(self):
        if getattr(self, "h", None):
            check(self._lib.slemm_gpu_genotype_destroy(self.h))
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    # ---- integer side outputs -------------------------------------------------------------
    def counts(self):
        """(popcnt int64, n0, n1, n2 int32) per SNP — bit-exact integer work."""
        pc = np.zeros(self.m, np.int64)
        n0 = np.zeros(self.m, np.int32)
        n1 = np.zeros(self.m, np.int32)
        n2 = np.zeros(self.m, np.int32)
        check(self._lib.slemm_gpu_genotype_counts(self.h, _ptr(pc), _ptr(n0), _ptr(n1), _ptr(n2)))
        return pc, n0, n1, n2

    def marker_qc(self, hwe_midp: int = 0):
        """(maf, hwep) float32 per SNP — cal_maf_from_genobits / cal_hwep_from_genobits
        (src/weight.cpp:3-15, src/input.cpp:10-22)."""
        maf = np.zeros(self.m, np.float32)
        hwep = np.zeros(self.m, np.float32)
        check(self._lib.slemm_gpu_marker_qc(self.h, int(hwe_midp), _ptr(maf), _ptr(hwep)))
        return maf, hwep

    def genotype_rows(self, rows):
        """n×len(rows) float32 allele-2 counts (missing = 1) of the given SNP rows."""
        rows = np.ascontiguousarray(rows, np.int64).reshape(-1)
        out = np.zeros((self.n, rows.size), np.float32, order="F")
        check(self._lib.slemm_gpu_genotype_rows(self.h, _ptr(rows), rows.size, _ptr(out), self.n, MEM_HOST))
        return out

    # ---- configuration -----------------------------------------------------------------------
    def set_weights(self, gm, w, rr=None):
        gm = np.ascontiguousarray(gm, np.float32)
        w = np.ascontiguousarray(w, np.float32)
        rr = None if rr is None else np.ascontiguousarray(rr, np.float32)
        check(self._lib.slemm_gpu_set_weights(self.h, _ptr(gm), _ptr(w), _ptr(rr)))

    def set_projection(self, Q):
        if Q is None or np.asarray(Q).size == 0:
            check(self._lib.slemm_gpu_set_projection(self.h, None, self.n, 0))
            return
        Qf, c = _f32c(Q)
        check(self._lib.slemm_gpu_set_projection(self.h, _ptr(Qf), self.n, c))

    def set_precision(self, prec: int):
        check(self._lib.slemm_gpu_set_precision(self.h, prec))

    def set_per_vector(self, flag: bool):
        check(self._lib.slemm_gpu_set_per_vector(self.h, 1 if flag else 0))

    def set_autotune(self, on=True):
        """Split-K counts and ring plans of this handle's tensor-core passes picked by timing at first
        use (True), by the fixed rule (False), or by the fixed rule with the two-CTAs-per-SM plan for
        every pass with N ≤ 64 ("two_cta")."""
        mode = 2 if on == "two_cta" else (1 if on else 0)
        check(self._lib.slemm_gpu_set_autotune(self.h, mode))

    def set_lanczos(self, reorth: bool = False):
        """Lanczos mode of the seeds run on this handle (default: the reference's recurrence)."""
        check(self._lib.slemm_gpu_set_lanczos(self.h, _lib.LANCZOS_REORTH if reorth else 0))

    def set_stream(self, stream_ptr: int | None):
        check(self._lib.slemm_gpu_set_stream(self.h, stream_ptr))

    def stream(self) -> int:
        s = ctypes.c_void_p()
        check(self._lib.slemm_gpu_get_stream(self.h, ctypes.byref(s)))
        return s.value or 0

    # ---- operators (src/reml.cpp:8-233) -----------------------------------------------------------
    def op(self, kind: int, v, tau0: float = 0.0):
        """Host call: NumPy in, NumPy out (column-major semantics, shape rows×k)."""
        vin, k = _f32c(v)
        rows_out = self.m if kind in (OP_RMATVEC, OP_WRMATVEC) else self.n
        out = np.zeros((rows_out, k), np.float32, order="F")
        check(self._lib.slemm_gpu_op(self.h, kind, float(tau0), _ptr(vin), vin.shape[0], k,
                                     _ptr(out), rows_out, MEM_HOST))
        return out

    def op_device(self, kind: int, v_t, out_t, tau0: float = 0.0):
        """Device call on CUDA tensors stored as (k, rows) contiguous (column-major rows×k)."""
        k, rows_in = v_t.shape
        rows_out = out_t.shape[1]
        check(self._lib.slemm_gpu_op(self.h, kind, float(tau0), ctypes.c_void_p(v_t.data_ptr()),
                                     rows_in, k, ctypes.c_void_p(out_t.data_ptr()), rows_out,
                                     MEM_DEVICE))

    def H0_quadform_mv(self, tau0, v):
        return self.op(OP_QUADFORM, v, tau0)

    def H0_ldet_mv(self, tau0, v):
        return self.op(OP_LDET, v, tau0)

    def lnr_op_select(self, lnr: str, tau0, v):
        if lnr not in _OP_OF_NAME:
            raise ValueError("Unknown linear operator in lnr_op_select()")
        return self.op(_OP_OF_NAME[lnr], v, tau0)

    def matvec(self, v):
        return self.op(OP_MATVEC, v)

    def rmatvec(self, v):
        return self.op(OP_RMATVEC, v)

    def weighted_rmatvec(self, v):
        return self.op(OP_WRMATVEC, v)

    # ---- Lanczos (src/reml.cpp:246-431) ------------------------------------------------------------
    def L_Seed(self, lnr: str, tau0, B, tol=5e-4, maxit=600):
        Bf, t = _f32c(B)
        s = ctypes.c_void_p()
        it = ctypes.c_int()
        check(self._lib.slemm_gpu_lanczos_seed(self.h, _OP_OF_NAME[lnr], float(tau0), _ptr(Bf),
                                               Bf.shape[0], t, float(tol), int(maxit), MEM_HOST,
                                               ctypes.byref(s), ctypes.byref(it)))
        return LSeed(self, s, t, it.value)

    # ---- drivers ------------------------------------------------------------------------------------
    def _reml_args(self, rvec, X, y, persnp):
        n = self.n
        rv = None if rvec is None else np.ascontiguousarray(rvec, np.float32)
        Xf, c = _f32c(X)
        yv = np.ascontiguousarray(y, np.float32)
        ps = np.ascontiguousarray(persnp, np.float32)
        assert yv.size == n and Xf.shape[0] == n and ps.size == self.m
        return rv, Xf, c, yv, ps

    def SLDF_REML(self, rvec, X, y, persnp, seed=0, n_V=30, tol_L=5e-4, s2max=0.7, s2min=1e-4,
                  tol_VC=1e-4, maxit=600, verbose=False):
        rv, Xf, c, yv, ps = self._reml_args(rvec, X, y, persnp)
        o = RemlOpts(n_V, seed, tol_L, s2max, s2min, tol_VC, maxit, int(verbose))
        Py = np.zeros(self.n, np.float32)
        b = np.zeros(self.m, np.float32)
        blue = np.zeros(c, np.float32)
        vb = np.zeros((c, c), np.float32, order="F")
        r = RemlResult()
        check(self._lib.slemm_gpu_reml_sldf(self.h, _ptr(rv), _ptr(Xf), self.n, c, _ptr(yv),
                                            _ptr(ps), ctypes.byref(o), _ptr(Py), _ptr(b),
                                            _ptr(blue), _ptr(vb), ctypes.byref(r)))
        return dict(vg=r.vg, ve=r.ve, h2=r.h2, lrt=r.lrt, Py=Py, snp_blup=b, blue=blue,
                    var_blue=vb, iters=(r.iters_y, r.iters_Q, r.iters_V),
                    n_criterion=r.n_criterion, seconds=r.seconds, trace=r.trace(),
                    phases=dict(setup=r.t_setup, seed=r.t_seed, search=r.t_search, final=r.t_final))

    def LMC_REML(self, rvec, X, y, persnp, seed=0, n_MC=3, tol_L=5e-4, s2max=0.7, s2min=1e-4,
                 maxit=600, verbose=False):
        rv, Xf, c, yv, ps = self._reml_args(rvec, X, y, persnp)
        o = RemlOpts(n_MC, seed, tol_L, s2max, s2min, 1e-4, maxit, int(verbose))
        Py = np.zeros(self.n, np.float32)
        b = np.zeros(self.m, np.float32)
        blue = np.zeros(c, np.float32)
        r = RemlResult()
        check(self._lib.slemm_gpu_reml_lmc(self.h, _ptr(rv), _ptr(Xf), self.n, c, _ptr(yv),
                                           _ptr(ps), ctypes.byref(o), _ptr(Py), _ptr(b),
                                           _ptr(blue), ctypes.byref(r)))
        return dict(vg=r.vg, ve=r.ve, h2=r.h2, Py=Py, snp_blup=b, blue=blue, iters=r.iters_V,
                    n_criterion=r.n_criterion, seconds=r.seconds, trace=r.trace(),
                    phases=dict(setup=r.t_setup, seed=r.t_seed, search=r.t_search, final=r.t_final))

    def REML_grad(self, rvec, X, y, persnp, window, wwin, sigma_g2, sigma_e2, n_V=30, seed=0, tol=1e-6):
        """Gradient of the REML log-likelihood with respect to (σ_g², σ_e², per-window SNP
        weights): dict with d_sigma_g2, d_sigma_e2 and d_w (one per window)."""
        rv, Xf, c, yv, ps = self._reml_args(rvec, X, y, persnp)
        win = None if window is None else np.ascontiguousarray(window, np.int32)
        ww = np.ascontiguousarray(np.zeros(0) if wwin is None else wwin, np.float32)
        grad = np.zeros(2 + ww.size, np.float64)
        check(self._lib.slemm_gpu_reml_grad(self.h, _ptr(rv), _ptr(Xf), self.n, c, _ptr(yv), _ptr(ps), _ptr(win),
                                            int(ww.size), _ptr(ww), float(sigma_g2), float(sigma_e2), int(n_V),
                                            int(seed), float(tol), _ptr(grad)))
        return dict(d_sigma_g2=grad[0], d_sigma_e2=grad[1], d_w=grad[2:])

    def REML_iter_weighting(self, rvec, X, y, persnp, maf, lrt=True, seed=0, n_V=30, n_MC=0,
                            n_MC_final=0, tol_L=5e-4, s2max=0.7, window_size=20, sig_chisq=1e6,
                            indep_r2=0.5, max_fixed=64, verbose=False):
        """`--iter_weighting` (src/option.cpp:437-530): equal-weight GREML, window weights from the
        SNP-BLUP, fixed-effect SNPs by clumping, window-weighted GREML."""
        rv, Xf, c, yv, ps = self._reml_args(rvec, X, y, persnp)
        mf = np.ascontiguousarray(maf, np.float32)
        o = RemlOpts(n_V, seed, tol_L, s2max, 1e-4, 1e-4, 600, int(verbose))
        w = WindowOpts(int(window_size), float(sig_chisq), float(indep_r2), int(bool(lrt)), int(n_MC),
                       int(n_MC_final), int(max_fixed))
        Py = np.zeros(self.n, np.float32)
        b = np.zeros(self.m, np.float32)
        blue = np.zeros(c + max_fixed, np.float32)
        vb = np.zeros((c + max_fixed) ** 2, np.float32)
        p2 = np.zeros(self.m, np.float32)
        fixed = np.zeros(max(max_fixed, 1), np.int64)
        nf = ctypes.c_int(0)
        r = RemlResult()
        check(self._lib.slemm_gpu_reml_iter_weighting(self.h, _ptr(rv), _ptr(Xf), self.n, c, _ptr(yv), _ptr(ps),
                                                      _ptr(mf), ctypes.byref(o), ctypes.byref(w), _ptr(Py),
                                                      _ptr(b), _ptr(blue), _ptr(vb), _ptr(p2), _ptr(fixed),
                                                      ctypes.byref(nf), ctypes.byref(r)))
        k = nf.value
        cc = c + k
        out = dict(vg=r.vg, ve=r.ve, h2=r.h2, lrt=r.lrt, Py=Py, snp_blup=b, blue=blue[:cc],
                   fixed=list(fixed[:k]), persnp=p2, iters=(r.iters_y, r.iters_Q, r.iters_V),
                   trace=r.trace(), seconds=r.seconds,
                   first_stage=dict(iters_V=r.first_iters_V, n_criterion=r.first_n_criterion))
        if lrt:
            out["var_blue"] = vb[:cc * cc].reshape(cc, cc, order="F")
        return out

    def LMM_quadforms(self, Py, tau1, num_qf=30, window_size=1000, tol_L=5e-4):
        """--lmm quadratic forms (src/reml.cpp:919-981): dict of variants, xPy, xPx, xBx, xSx."""
        py = np.ascontiguousarray(Py, np.float32)
        var = np.zeros(num_qf, np.int64)
        out = {k: np.zeros(num_qf, np.float32) for k in ("xPy", "xPx", "xBx", "xSx")}
        cnt = ctypes.c_int(0)
        check(self._lib.slemm_gpu_lmm_quadforms(self.h, _ptr(py), float(tau1), float(tol_L), int(num_qf),
                                                int(window_size), _ptr(var), _ptr(out["xPy"]), _ptr(out["xPx"]),
                                                _ptr(out["xBx"]), _ptr(out["xSx"]), ctypes.byref(cnt)))
        k = cnt.value
        res = {key: v[:k] for key, v in out.items()}
        res["variants"] = [int(v) for v in var[:k]]
        return res

    def gwa_windows(self, y, R, covar, model_idx, test_begin, test_end, block_size, tau, model_snp_ct,
                    cfactor, snp_var, mac=20):
        """slemm_gwa.py windowed MLMA (bin/slemm_gwa.py:259-434): beta, se, chisq, p per tested
        variant test_begin … test_end (allele 1 orientation)."""
        yv = np.ascontiguousarray(y, np.float32)
        Rv = None if R is None else np.ascontiguousarray(R, np.float32)
        cv = np.asfortranarray(np.asarray(covar, np.float32).reshape(self.n, -1))
        mi = np.ascontiguousarray(model_idx, np.int64)
        t = test_end - test_begin + 1
        beta, se, chisq = (np.zeros(t, np.float32) for _ in range(3))
        p = np.zeros(t, np.float64)
        check(self._lib.slemm_gpu_gwa_windows(self.h, _ptr(yv), _ptr(Rv), _ptr(cv), self.n, cv.shape[1], _ptr(mi),
                                              mi.size, int(test_begin), int(test_end), int(block_size), float(tau),
                                              int(model_snp_ct), float(cfactor), float(snp_var), int(mac),
                                              _ptr(beta), _ptr(se), _ptr(chisq), _ptr(p)))
        return beta, se, chisq, p

    def weighted_least_squares(self, rvec, X, y):
        """`--wls` SNP effects (src/wls.cpp:4-129), float32 per SNP."""
        rv, Xf, c, yv, _ = self._reml_args(rvec, X, y, np.ones(self.m, np.float32))
        b = np.zeros(self.m, np.float32)
        check(self._lib.slemm_gpu_wls(self.h, _ptr(rv), _ptr(Xf), self.n, c, _ptr(yv), _ptr(b)))
        return b

    def gebv(self, alpha, flip=None):
        """GEBV Σ_j (flip ? 2−count : count)·alpha_j in FP64 (src/pred.cpp:154-172)."""
        a = np.ascontiguousarray(alpha, np.float64)
        f = None if flip is None else np.ascontiguousarray(flip, np.uint8)
        out = np.zeros(self.n, np.float64)
        check(self._lib.slemm_gpu_gebv(self.h, _ptr(a), _ptr(f), _ptr(out)))
        return out

    def score_terms(self, y, mac: int):
        """slemm_gamma per-variant xy and xx (bin/slemm_gamma.py:302-319)."""
        yv = np.ascontiguousarray(y, np.float32)
        xy = np.zeros(self.m, np.float32)
        xx = np.zeros(self.m, np.float32)
        check(self._lib.slemm_gpu_score_terms(self.h, _ptr(yv), int(mac), _ptr(xy), _ptr(xx)))
        return xy, xx


class LSeed:
    """A seed system resident on the GPU (basis + Jacobi coefficients)."""

    def __init__(self, geno: Genotypes, handle, t: int, iters: int):
        self.g, self.s, self.t, self.iters = geno, handle, t, iters

    def coeffs(self):
        beta = np.zeros((self.t, self.iters + 1), np.float64, order="F")
        delta = np.zeros((self.t, max(self.iters, 1)), np.float64, order="F")
        check(self.g._lib.slemm_gpu_lseed_coeffs(self.s, _ptr(beta), _ptr(delta)))
        return beta, delta[:, : self.iters]

    def L_Solve(self, sigma, tol=1e-6):
        X = np.zeros((self.g.n, self.t), np.float32, order="F")
        check(self.g._lib.slemm_gpu_lanczos_solve(self.s, float(sigma), float(tol), _ptr(X),
                                                  self.g.n, MEM_HOST))
        return X

    def close(self):
        if getattr(self, "s", None):
            check(self.g._lib.slemm_gpu_lseed_destroy(self.s))
            self.s = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def hwe_exact(het, hom1, hom2, midp: int = 0) -> np.ndarray:
    """SNPHWE2(het, hom1, hom2, midp) (src/snphwe.cpp:18) for arrays of count triples, FP64."""
    het = np.ascontiguousarray(het, np.int32).reshape(-1)
    hom1 = np.ascontiguousarray(hom1, np.int32).reshape(-1)
    hom2 = np.ascontiguousarray(hom2, np.int32).reshape(-1)
    p = np.zeros(het.size, np.float64)
    check(_lib.load().slemm_gpu_hwe_exact(_ptr(het), _ptr(hom1), _ptr(hom2), het.size, int(midp), _ptr(p)))
    return p


def tridiag_eig(delta, beta):
    """Batched FP64 eigenvalues D and squared first components W² (src/reml.cpp:638-646)."""
    delta = np.asfortranarray(delta, np.float64)
    beta = np.asfortranarray(beta, np.float64)
    t, nld = delta.shape
    D = np.zeros((t, nld), np.float64, order="F")
    W2 = np.zeros((t, nld), np.float64, order="F")
    check(_lib.load().slemm_gpu_tridiag_eig(_ptr(delta), _ptr(beta), t, nld, _ptr(D), _ptr(W2)))
    return D, W2


def autotune_table():
    """The tuner's cached decisions: one dict per shape."""
    lib = _lib.load()
    rows = ctypes.c_int(0)
    check(lib.slemm_gpu_autotune_table(0, ctypes.byref(rows), None, None, None))
    r = rows.value
    info = np.zeros(7 * max(r, 1), np.int32)
    shape = np.zeros(2 * max(r, 1), np.int64)
    ms = np.zeros(2 * max(r, 1), np.float64)
    check(lib.slemm_gpu_autotune_table(r, ctypes.byref(rows), _ptr(info), _ptr(shape), _ptr(ms)))
    return [dict(device=int(info[7 * i]), N=int(info[7 * i + 1]), pieces=int(info[7 * i + 2]),
                 rule_splits=int(info[7 * i + 3]), splits=int(info[7 * i + 4]), plan=int(info[7 * i + 5]),
                 candidates=int(info[7 * i + 6]),
                 K_tiles=int(shape[2 * i]), M_pad=int(shape[2 * i + 1]), ms_rule=float(ms[2 * i]),
                 ms=float(ms[2 * i + 1])) for i in range(r)]
