"""ORACLE — test infrastructure only.

NumPy restatement of the reference's REML / BLUP / prediction / score-test path, used only by
tests/, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg as the checker.  It is
never imported by the product (``slemm_gb300``).  Every function cites the reference file:line
it follows (paths inside jiang18/slemm).

``dtype=np.float32`` follows the reference's FP32 Eigen arithmetic; ``dtype=np.float64`` gives the
FP64 oracle used to state the error of each result.  Integer work (decode, popcounts, class
counts, MAF) goes through the plain-C restatement in ``bedref.c``; the probe draws go through
libstdc++ itself (``rng.cpp``), which is what the reference calls.
"""
from __future__ import annotations

import ctypes
import math
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB = None
_LOCK = threading.Lock()


def _lib():
    """Builds (make) and loads the C part of the oracle."""
    global _LIB
    with _LOCK:
        if _LIB is None:
            so = os.path.join(_HERE, "_build", "liboracle.so")
            srcs = [os.path.join(_HERE, f) for f in ("bedref.c", "rng.cpp")]
            if not os.path.exists(so) or any(os.path.getmtime(s) > os.path.getmtime(so) for s in srcs):
                subprocess.run(["make", "-s", "-C", _HERE, "all"], check=True)
            lib = ctypes.CDLL(so)
            P = ctypes.c_void_p
            I64 = ctypes.c_int64
            lib.oracle_bed_decode.argtypes = [P, I64, I64, I64, P, P, I64]
            lib.oracle_popcounts.argtypes = [P, I64, I64, P]
            lib.oracle_decode_centred_f32.argtypes = [P, I64, I64, I64, P, P]
            lib.oracle_hwe_counts.argtypes = [P, I64, I64, P, P, P]
            lib.oracle_lmm_variants.argtypes = [P, I64, I64, ctypes.c_int, P]
            lib.oracle_lmm_variants.restype = ctypes.c_int
            lib.oracle_libc_rand.argtypes = [ctypes.c_uint, ctypes.c_int, P]
            lib.oracle_maf.argtypes = [P, I64, I64, P]
            lib.oracle_gm.argtypes = [P, I64, I64, P]
            lib.oracle_gebv.argtypes = [P, I64, I64, P, P, P]
            lib.oracle_rademacher.argtypes = [ctypes.c_int, I64, ctypes.c_int, P]
            lib.oracle_lmc_draws.argtypes = [ctypes.c_int, I64, I64, ctypes.c_int, P, P]
            _LIB = lib
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


# ------------------------------------------------------------------------------------------
# integer path (bedref.c)
# ------------------------------------------------------------------------------------------
def bed_decode(rows: np.ndarray, n_fam: int, keep: np.ndarray | None = None) -> np.ndarray:
    """src/input.cpp:343-386 — m×n allele-2 counts (missing→1) of the kept individuals."""
    rows = np.ascontiguousarray(rows, dtype=np.uint8)
    m, rb = rows.shape
    kp = None if keep is None else np.ascontiguousarray(keep, dtype=np.uint8)
    n = n_fam if kp is None else int(kp.astype(bool).sum())
    out = np.zeros((m, n), dtype=np.uint8)
    _lib().oracle_bed_decode(_p(rows), m, n_fam, rb, _p(kp), _p(out), n)
    return out


def popcounts(counts: np.ndarray) -> np.ndarray:
    """src/reml.cpp:613-621 — nz_bits per SNP."""
    counts = np.ascontiguousarray(counts, dtype=np.uint8)
    m, n = counts.shape
    pc = np.zeros(m, dtype=np.int64)
    _lib().oracle_popcounts(_p(counts), m, n, _p(pc))
    return pc


def hwe_counts(counts: np.ndarray):
    """src/input.cpp:10-22 — (n0, n1, n2) with missing counted as heterozygous."""
    counts = np.ascontiguousarray(counts, dtype=np.uint8)
    m, n = counts.shape
    n0 = np.zeros(m, np.int32)
    n1 = np.zeros(m, np.int32)
    n2 = np.zeros(m, np.int32)
    _lib().oracle_hwe_counts(_p(counts), m, n, _p(n0), _p(n1), _p(n2))
    return n0, n1, n2


def maf(pc: np.ndarray, n: int) -> np.ndarray:
    """src/weight.cpp:3-15."""
    pc = np.ascontiguousarray(pc, dtype=np.int64)
    out = np.zeros(pc.size, np.float32)
    _lib().oracle_maf(_p(pc), pc.size, n, _p(out))
    return out


def hwe_exact(het: int, hom1: int, hom2: int, midp: int = 0) -> float:
    """src/snphwe.cpp:18 SNPHWE2 (called as SNPHWE2(n1, n0, n2, midp) at src/input.cpp:20): exact
    Hardy–Weinberg test (Wigginton, Cutler & Abecasis 2005).  Under HWE the het count h (parity of
    the rare-allele count) has P(h+2)/P(h) = 4·hom_r·hom_c / ((h+2)(h+1)); p = Σ P(h) over
    P(h) ≤ P(obs) (relative tie tolerance 1e-7), normalised; mid-p subtracts P(obs)/2.  Terms are
    taken relative to the mode and summed outward with math.fsum."""
    import math
    n = het + hom1 + hom2
    if n == 0:
        return 0.5 if midp else 1.0
    rare = 2 * min(hom1, hom2) + het
    hmax = min(rare, 2 * n - rare)
    par = rare & 1

    def up(h):
        hr = (rare - h) // 2
        hc = n - h - hr
        return 4.0 * hr * hc / ((h + 2) * (h + 1))

    h = int(rare * (2 * n - rare) / (2 * n - 1))
    if (h & 1) != par:
        h += 1 if h + 1 <= hmax else -1
    h = max(par, min(h, hmax))
    while h + 2 <= hmax and up(h) > 1.0:
        h += 2
    while h >= 2 and up(h - 2) < 1.0:
        h -= 2
    probs = {h: 1.0}
    p, k = 1.0, h
    while k + 2 <= hmax and p > 0.0:
        p *= up(k)
        k += 2
        probs[k] = p
    p, k = 1.0, h
    while k >= 2 and p > 0.0:
        p /= up(k - 2)
        k -= 2
        probs[k] = p
    pobs = probs[het]
    tot = math.fsum(probs.values())
    tail = math.fsum(v for v in probs.values() if v <= pobs * (1.0 + 1e-7))
    if midp:
        tail -= 0.5 * pobs
    return min(1.0, tail / tot)


def marker_qc(counts: np.ndarray, midp: int = 0):
    """src/input.cpp:388-394 — per-SNP MAF (src/weight.cpp:3-15, FP32) and HWE p-value stored as
    FP32 (src/input.cpp:10-22: n2 = both bits, n1 = one bit incl. missing, n0 = neither)."""
    counts = np.ascontiguousarray(counts, dtype=np.uint8)
    m, n = counts.shape
    pc = popcounts(counts)
    n0, n1, n2 = hwe_counts(counts)
    maf_v = maf(pc, n)
    hwep = np.array([hwe_exact(int(a), int(b), int(c), midp) for a, b, c in zip(n1, n0, n2)], np.float32)
    return maf_v, hwep


def genotype_mean(pc: np.ndarray, n: int) -> np.ndarray:
    """src/reml.cpp:620 — gm = nz_bits/float(n)."""
    pc = np.ascontiguousarray(pc, dtype=np.int64)
    out = np.zeros(pc.size, np.float32)
    _lib().oracle_gm(_p(pc), pc.size, n, _p(out))
    return out


def snp_weights(gm: np.ndarray, persnp: np.ndarray, dtype=np.float32) -> np.ndarray:
    """src/reml.cpp:622 — gw = 1/(gm(2−gm)/2) / m · persnp/mean(persnp)."""
    gm = gm.astype(dtype)
    persnp = persnp.astype(dtype)
    m = gm.size
    return (dtype(1) / (gm * (dtype(2) - gm) / dtype(2))) / dtype(m) * (persnp / persnp.mean(dtype=dtype))


def rademacher(seed: int, n: int, n_V: int) -> np.ndarray:
    """src/reml.cpp:597-605 — n×n_V normalised Rademacher probes (libstdc++ draws)."""
    V = np.zeros((n_V, n), np.float32)
    _lib().oracle_rademacher(seed, n, n_V, _p(V))
    return V.T.copy()


def lmc_draws(seed: int, m: int, n: int, n_MC: int):
    """src/reml.cpp:795-809 — u (m×n_MC) then e (n×n_MC) from one mt19937 stream."""
    u = np.zeros((n_MC, m), np.float32)
    e = np.zeros((n_MC, n), np.float32)
    _lib().oracle_lmc_draws(seed, m, n, n_MC, _p(u), _p(e))
    return u.T.copy(), e.T.copy()


def gebv(counts: np.ndarray, alpha: np.ndarray, flip: np.ndarray | None = None) -> np.ndarray:
    """src/pred.cpp:154-172 — FP64 GEBV accumulation over SNPs in file order."""
    counts = np.ascontiguousarray(counts, dtype=np.uint8)
    m, n = counts.shape
    alpha = np.ascontiguousarray(alpha, dtype=np.float64)
    fl = None if flip is None else np.ascontiguousarray(flip, dtype=np.uint8)
    out = np.zeros(n, np.float64)
    _lib().oracle_gebv(_p(counts), m, n, _p(alpha), _p(fl), _p(out))
    return out


# ------------------------------------------------------------------------------------------
# operators (src/reml.cpp:8-233)
# ------------------------------------------------------------------------------------------
class Operators:
    """The reference's subset loop: decode `subset_size` SNPs into FP centred columns
    (count − gm), then two GEMMs per subset (src/reml.cpp:28-47)."""

    def __init__(self, counts, gm, w, rr=None, Q=None, subset_size=1000, dtype=np.float32):
        self.G = np.ascontiguousarray(counts, dtype=np.uint8)   # m×n
        self.m, self.n = self.G.shape
        self.dt = dtype
        self.gm = np.asarray(gm, dtype=dtype)
        self.w = np.asarray(w, dtype=dtype)
        self.rr = np.ones(self.n, dtype) if rr is None else np.asarray(rr, dtype=dtype)
        self.Q = np.zeros((self.n, 0), dtype) if Q is None else np.asarray(Q, dtype=dtype)
        self.s = int(subset_size)
        self._lut = np.arange(3, dtype=dtype)

    def _subsets(self):
        for i0 in range(0, self.m, self.s):
            i1 = min(self.m, i0 + self.s)
            Zc = self._lut[self.G[i0:i1]].T - self.gm[i0:i1]   # n×s, (count − gm)
            yield i0, i1, Zc

    def _proj(self, v):
        if self.Q.shape[1] == 0:
            return v
        return v - self.Q @ (self.Q.T @ v)

    def H0_quadform_mv(self, tau0, v):
        """src/reml.cpp:8-50."""
        v = np.asarray(v, self.dt)
        v_adj = self.rr[:, None] * self._proj(v)
        ZPv = np.zeros_like(v)
        for i0, i1, Zc in self._subsets():
            ZPv += Zc @ (self.w[i0:i1, None] * (Zc.T @ v_adj))
        ZPv *= self.rr[:, None]
        return ZPv + self.dt(tau0) * v - (self.Q @ (self.Q.T @ ZPv) if self.Q.shape[1] else 0)

    def H0_ldet_mv(self, tau0, v):
        """src/reml.cpp:52-94."""
        v = np.asarray(v, self.dt)
        rv = self.rr[:, None] * v
        out = np.zeros_like(v)
        for i0, i1, Zc in self._subsets():
            out += Zc @ (self.w[i0:i1, None] * (Zc.T @ rv))
        out *= self.rr[:, None]
        return out + self.dt(tau0) * v

    def op(self, lnr, tau0, v):
        """src/reml.cpp:96-118 lnr_op_select."""
        if lnr == "quadform":
            return self.H0_quadform_mv(tau0, v)
        if lnr == "ldet":
            return self.H0_ldet_mv(tau0, v)
        raise ValueError("Unknown linear operator in lnr_op_select()")

    def weighted_rmatvec(self, v):
        """src/reml.cpp:121-157 — W Z_cᵀ v."""
        v = np.asarray(v, self.dt).reshape(self.n, -1)
        out = np.zeros((self.m, v.shape[1]), self.dt)
        for i0, i1, Zc in self._subsets():
            out[i0:i1] = self.w[i0:i1, None] * (Zc.T @ v)
        return out

    def rmatvec(self, v):
        """src/reml.cpp:160-195 — Z_cᵀ v."""
        v = np.asarray(v, self.dt).reshape(self.n, -1)
        out = np.zeros((self.m, v.shape[1]), self.dt)
        for i0, i1, Zc in self._subsets():
            out[i0:i1] = Zc.T @ v
        return out

    def matvec(self, v):
        """src/reml.cpp:198-233 — Z_c v."""
        v = np.asarray(v, self.dt).reshape(self.m, -1)
        out = np.zeros((self.n, v.shape[1]), self.dt)
        for i0, i1, Zc in self._subsets():
            out += Zc @ v[i0:i1]
        return out


class PackedOperators(Operators):
    """Same operators, decoding each `subset_size` block straight from the packed .bed rows of
    the kept individuals (all individuals here), as the reference decodes kmat bits per subset
    (src/reml.cpp:29-35) — used for the timed CPU baseline at full sizes.  The decode runs in the
    oracle's C restatement over `threads` host threads (ctypes releases the GIL) into one reused
    FP32 subset buffer, and the two products per subset are OpenBLAS SGEMMs, the structure of the
    reference's OpenMP decode + MKL SGEMM loop."""

    def __init__(self, bed_rows, n, gm, w, rr=None, Q=None, subset_size=1000, dtype=np.float32, threads=None):
        self.rows = np.ascontiguousarray(bed_rows, dtype=np.uint8)
        self.m, self.n = self.rows.shape[0], n
        self.dt = dtype
        self.gm = np.asarray(gm, dtype=dtype)
        self.w = np.asarray(w, dtype=dtype)
        self.rr = np.ones(n, dtype) if rr is None else np.asarray(rr, dtype=dtype)
        self.Q = np.zeros((n, 0), dtype) if Q is None else np.asarray(Q, dtype=dtype)
        self.s = int(subset_size)
        self.threads = max(1, int(threads or os.cpu_count() or 1))
        self.subset_limit = None
        self._buf = None

    def _decode(self, i0, i1):
        """(i1 − i0) × n FP32 rows count − gm of SNPs i0 … i1−1."""
        if self.dt != np.float32:
            raise TypeError("the packed C decode writes FP32")
        need = (i1 - i0) * self.n
        if self._buf is None or self._buf.size < need:
            self._buf = np.empty(need, np.float32)
        out = self._buf[:need].reshape(i1 - i0, self.n)
        gm = np.ascontiguousarray(self.gm[i0:i1], np.float32)
        rb = self.rows.shape[1]
        lib = _lib()
        chunks = [c for c in np.array_split(np.arange(i0, i1), self.threads) if c.size]

        def work(c):
            a, b = int(c[0]), int(c[-1]) + 1
            lib.oracle_decode_centred_f32(_p(self.rows[a:b]), b - a, self.n, rb, _p(gm[a - i0:b - i0]),
                                          _p(out[a - i0:b - i0]))

        if len(chunks) == 1:
            work(chunks[0])
        else:
            from concurrent.futures import ThreadPoolExecutor
            with ThreadPoolExecutor(len(chunks)) as ex:
                list(ex.map(work, chunks))
        return out

    def _subsets(self):
        count = 0
        for i0 in range(0, self.m, self.s):
            if self.subset_limit is not None and count >= self.subset_limit:
                return
            i1 = min(self.m, i0 + self.s)
            count += 1
            yield i0, i1, self._decode(i0, i1).T   # n × s view, (count − gm)


# ------------------------------------------------------------------------------------------
# Lanczos seed / solve / SLQ (src/reml.cpp:240-451)
# ------------------------------------------------------------------------------------------
def L_Seed(ops: Operators, lnr, tau0, B, tol=5e-4, maxit=600, reorth=False):
    """src/reml.cpp:246-339 — per-column Lanczos with CG coefficients; returns the basis U
    (list of n×t), beta (t×(j+1)), delta (t×j) and the step count j.

    reorth=True restates the engine's opt-in mode (not in the reference): after the three-term
    update each new vector loses its components along every stored vector of its column
    (one classical Gram–Schmidt pass, coefficients U_iᵀw from the vector before the pass)."""
    dt = ops.dt
    B = np.asarray(B, dt).reshape(ops.n, -1)
    n, t = B.shape
    B_norm = np.sqrt((B * B).sum(axis=0, dtype=dt)).astype(dt)
    rho = np.zeros((t, maxit), dt)
    beta = np.zeros((t, maxit), dt)
    omega = np.zeros((t, maxit), dt)
    gamma = np.ones((t, maxit), dt)
    delta = np.zeros((t, maxit), dt)
    rho[:, 0] = B_norm
    beta[:, 0] = rho[:, 0]
    U = [B / beta[:, 0]]
    j = 0
    while j < maxit - 1:
        tmp = ops.op(lnr, tau0, U[j])
        if j > 0:
            tmp = tmp - U[j - 1] * beta[:, j]
        delta[:, j] = (U[j] * tmp).sum(axis=0, dtype=dt)
        tmp = tmp - U[j] * delta[:, j]
        if reorth:   # classical Gram–Schmidt: all coefficients from w before the pass
            d = [(Ui * tmp).sum(axis=0, dtype=dt) for Ui in U]   # U_i[:,c]ᵀ w[:,c]
            for Ui, di in zip(U, d):
                tmp = tmp - Ui * di
        beta[:, j + 1] = np.sqrt((tmp * tmp).sum(axis=0, dtype=dt))
        U.append(tmp / beta[:, j + 1])
        if j == 0:
            gamma[:, j] = dt(1) / delta[:, j]
        else:
            gamma[:, j] = dt(1) / (delta[:, j] - omega[:, j - 1] / gamma[:, j - 1])
        omega[:, j] = (beta[:, j + 1] * gamma[:, j]) ** 2
        rho[:, j + 1] = -beta[:, j + 1] * gamma[:, j] * rho[:, j]
        R = U[j + 1] * rho[:, j + 1]
        j += 1
        res = (np.sqrt((R * R).sum(axis=0, dtype=dt)) / B_norm).max()
        if res <= tol:
            break
    return {"U": U, "beta": beta[:, : j + 1].copy(), "delta": delta[:, :j].copy(), "iters": j}


def L_Solve(seed, B, sigma, tol=1e-6):
    """src/reml.cpp:369-431 — shifted CG rebuilt from the stored basis."""
    U = seed["U"]
    dt = U[0].dtype.type
    B = np.asarray(B, dt).reshape(U[0].shape)
    B_norm = np.sqrt((B * B).sum(axis=0, dtype=dt))
    delta = seed["delta"] + dt(sigma)
    beta = seed["beta"]
    t = B.shape[1]
    maxit = len(U)
    omega = np.zeros((t, maxit), dt)
    gamma = np.ones((t, maxit), dt)
    rho = np.zeros((t, maxit), dt)
    rho[:, 0] = B_norm
    R = B.copy()
    P = B.copy()
    X = np.zeros_like(B)
    j = 0
    while j < maxit - 1:
        if j == 0:
            gamma[:, j] = dt(1) / delta[:, j]
        else:
            gamma[:, j] = dt(1) / (delta[:, j] - omega[:, j - 1] / gamma[:, j - 1])
        omega[:, j] = (beta[:, j + 1] * gamma[:, j]) ** 2
        rho[:, j + 1] = -beta[:, j + 1] * gamma[:, j] * rho[:, j]
        X = X + P * gamma[:, j]
        R = U[j + 1] * rho[:, j + 1]
        P = R + P * omega[:, j]
        j += 1
        res = (np.sqrt((R * R).sum(axis=0, dtype=dt)) / B_norm).max()
        if res <= tol:
            break
    return X


def jacobi_eig(seed):
    """src/reml.cpp:638-646 — eigenvalues D and first eigenvector components W of each probe's
    Jacobi matrix (delta row, beta row segment 1..nld-1)."""
    from scipy.linalg import eigh_tridiagonal
    delta = np.asarray(seed["delta"], np.float64)
    beta = np.asarray(seed["beta"], np.float64)
    t, nld = delta.shape
    D = np.zeros((t, nld))
    W = np.zeros((t, nld))
    for i in range(t):
        if nld == 1:
            D[i, 0] = delta[i, 0]
            W[i, 0] = 1.0
            continue
        d, v = eigh_tridiagonal(delta[i], beta[i, 1:nld])
        D[i] = d
        W[i] = v[0]
    return D, W


def SLQ_LDet(D, W, n, n_V, sigma=0.0):
    """src/reml.cpp:440-451 — log det(A + σI) ≈ (n/n_V)·Σ W²·log(D+σ)."""
    return float((W ** 2 * np.log(D + sigma)).sum()) * n / n_V


# ------------------------------------------------------------------------------------------
# DF-REML (src/reml.cpp:457-690)
# ------------------------------------------------------------------------------------------
def qr_colpiv(A, dtype=np.float64):
    """Q (n×rank) and qrR = R·Pᵀ of a column-pivoted Householder QR with Eigen's rank rule
    (threshold = eps·min(n,c)·|R00|), src/reml.cpp:583-588."""
    from scipy.linalg import qr
    A = np.asarray(A, np.float64)
    n, c = A.shape
    Qf, R, piv = qr(A, mode="economic", pivoting=True)
    diag = np.abs(np.diag(R))
    thr = np.finfo(np.float32).eps * min(n, c) * (diag[0] if diag.size else 0.0)
    rank = int((diag > thr).sum())
    P = np.eye(c)[:, piv]
    qrR = R[:rank, :rank] @ P[:, :rank].T if rank == c else None
    return Qf[:, :rank].astype(dtype), (None if qrR is None else qrR.astype(dtype)), rank


def REML_criterion(ss, tau0, y_proj, seed_y, Q, seed_Q, D_V, W_V, ySy):
    """src/reml.cpp:457-489 — returns (slogLL, vg, ve, lrt)."""
    n, c = Q.shape
    tau = (1 - ss) / ss
    sigma = tau - tau0
    yPy = float(y_proj @ L_Solve(seed_y, y_proj, sigma)[:, 0])
    M = Q.T @ L_Solve(seed_Q, Q, sigma)
    logdet = float(np.linalg.slogdet(np.asarray(M, np.float64))[1])
    if y_proj.dtype == np.float32:
        # The reference's criterion keeps yPy, v_g, v_e, ldet_H, lrt and slogLL in float
        # variables; its `log` of a float quotient is the C library's double log
        # (src/reml.cpp:470-488), each expression rounded once on assignment.
        f32 = np.float32
        ySy32, yPy32 = f32(ySy), f32(yPy)
        v_g = float(f32(yPy32 / f32(n - c)))
        v_e = float(f32(f32(v_g) * f32(tau)))
        ldet_H = float(f32(SLQ_LDet(D_V, W_V, n, D_V.shape[0], sigma)))
        lq = math.log(float(ySy32 / yPy32))
        lrt = float(f32(n * lq - ldet_H))
        slogLL = float(f32((n - c) * lq - float(f32(logdet)) - ldet_H))
        return slogLL, v_g, v_e, lrt
    v_g = yPy / (n - c)
    v_e = v_g * tau
    ldet_H = SLQ_LDet(D_V, W_V, n, D_V.shape[0], sigma)
    lrt = n * math.log(ySy / yPy) - ldet_H
    slogLL = (n - c) * math.log(ySy / yPy) - logdet - ldet_H
    return slogLL, v_g, v_e, lrt


def gss_point(a, k, h):
    """float(a + k·h) with a, h float32 and k a double constant: the double sum rounded once to
    float32, as the reference's `c = a + invphi2 * h;` does (src/reml.cpp:520-521)."""
    return np.float32(float(a) + k * float(h))


def REML_GSS(a, b, tau0, y_proj, seed_y, Q, seed_Q, D_V, W_V, tol, log=None):
    """src/reml.cpp:493-547 — golden-section search on h²; vg/ve/lrt come from the LAST
    criterion evaluation, as in the reference."""
    invphi = 0.618033988749894848204586834365638117720309179805762862135
    invphi2 = 0.381966011250105151795413165634361882279690820194237137864
    f32 = np.float32
    ySy = float(np.dot(y_proj, y_proj))
    a, b = f32(a), f32(b)
    h = f32(b - a)
    # The reference's points and steps mix float operands with double constants
    # (`c = a + invphi2 * h;`, `h *= invphi;`, src/reml.cpp:520-540): C++ promotes to double,
    # evaluates there and rounds once on assignment to float.  NumPy 2 keeps a float32 times a
    # Python float in float32, so each operand is taken to a Python float (double) first.
    nitr = 1 if h < tol else int(math.ceil(math.log(float(f32(tol) / h)) / math.log(invphi)))
    c = gss_point(a, invphi2, h)
    d = gss_point(a, invphi, h)
    evals = []
    fc, vg, ve, lrt = REML_criterion(c, tau0, y_proj, seed_y, Q, seed_Q, D_V, W_V, ySy)
    fd, vg, ve, lrt = REML_criterion(d, tau0, y_proj, seed_y, Q, seed_Q, D_V, W_V, ySy)
    evals += [(c, fc), (d, fd)]
    for _ in range(nitr):
        if fc > fd:
            b, d, fd = d, c, fc
            h = f32(float(h) * invphi)
            c = gss_point(a, invphi2, h)
            fc, vg, ve, lrt = REML_criterion(c, tau0, y_proj, seed_y, Q, seed_Q, D_V, W_V, ySy)
            evals.append((c, fc))
        else:
            a, c, fc = c, d, fd
            h = f32(float(h) * invphi)
            d = gss_point(a, invphi, h)
            fd, vg, ve, lrt = REML_criterion(d, tau0, y_proj, seed_y, Q, seed_Q, D_V, W_V, ySy)
            evals.append((d, fd))
    if log is not None:
        log.extend(evals)
    return vg, ve, lrt


def SLDF_REML(counts, rvec, X, y, persnp, seed=0, n_V=30, tol_L=5e-4, s2max=0.7, s2min=1e-4,
              tol_VC=1e-4, subset_size=1000, dtype=np.float32, maxit=600, reorth=False):
    """src/reml.cpp:549-690 — DF-REML; returns a dict with vg, ve, h2, lrt, Py, snp_blup, blue,
    var_blue and the Lanczos step counts.  reorth: the engine's opt-in reorthogonalised seeds."""
    dt = dtype
    n = y.size
    rvec = np.ones(n) if rvec is None else rvec
    rr = (1.0 / np.sqrt(np.asarray(rvec, np.float64))).astype(dt)
    Xd = np.asarray(X, dt).reshape(n, -1)
    Q, qrR, rank = qr_colpiv(rr[:, None].astype(np.float64) * Xd, dtype=dt)
    if rank != Xd.shape[1]:
        raise RuntimeError("Fixed-effects design matrix is not of full rank.")
    y_proj = rr * np.asarray(y, dt)
    y_proj = y_proj - Q @ (Q.T @ y_proj)
    V = rademacher(seed, n, n_V).astype(dt)
    pc = popcounts(counts)
    gm = genotype_mean(pc, n)
    gw = snp_weights(gm, persnp, dt)
    ops = Operators(counts, gm, gw, rr, Q, subset_size, dt)
    tau0 = (1 - np.float32(s2max)) / np.float32(s2max)
    seed_y = L_Seed(ops, "quadform", tau0, y_proj, tol_L, maxit, reorth)
    seed_Q = L_Seed(ops, "ldet", tau0, Q, tol_L, maxit, reorth)
    seed_V = L_Seed(ops, "ldet", tau0, V, tol_L, maxit, reorth)
    D_V, W_V = jacobi_eig(seed_V)
    log = []
    vg, ve, lrt = REML_GSS(s2min, s2max, tau0, y_proj, seed_y, Q, seed_Q, D_V, W_V, tol_VC, log)
    tau1 = ve / vg
    Py = L_Solve(seed_y, y_proj, tau1 - tau0)[:, 0]
    Py = Py - Q @ (Q.T @ Py)
    Py = rr * Py
    snp_blup = ops.weighted_rmatvec(Py)[:, 0]
    HinvX = (rr[:, None] * L_Solve(seed_Q, Q, tau1 - tau0)) @ qrR
    XtHinvX = np.asarray(Xd.T @ HinvX, np.float64)
    blue = np.linalg.solve(XtHinvX, np.asarray(HinvX.T @ np.asarray(y, dt), np.float64))
    var_blue = np.linalg.inv(XtHinvX) * vg
    return dict(vg=vg, ve=ve, h2=vg / (vg + ve), lrt=lrt, Py=Py, snp_blup=snp_blup, blue=blue,
                var_blue=var_blue, iters=(seed_y["iters"], seed_Q["iters"], seed_V["iters"]),
                gss=log, gm=gm, gw=gw)


# ------------------------------------------------------------------------------------------
# MC-REML (src/reml.cpp:696-883)
# ------------------------------------------------------------------------------------------
def REML_first_order(ops: Operators, ss, tau0, V, seed_V, gw):
    """src/reml.cpp:696-728 — returns (f, Py) with Py the rr-scaled projected solutions."""
    dt = ops.dt
    n_MC = (V.shape[1] - 1) // 2
    tau = (1 - ss) / ss
    sigma = tau - tau0
    PV = L_Solve(seed_V, V, sigma)
    Py = np.empty((ops.n, 1 + n_MC), dt)
    Py[:, 1:] = PV[:, 1:1 + n_MC] + dt(math.sqrt(tau)) * PV[:, 1 + n_MC:]
    Py[:, 0] = PV[:, 0]
    Py = ops._proj(Py)
    e_BLUP = Py.copy()
    Py = Py * ops.rr[:, None]
    u_BLUP = ops.rmatvec(Py) * np.sqrt(gw)[:, None]
    num = (u_BLUP[:, :1] ** 2).sum() / (e_BLUP[:, :1] ** 2).sum()
    den = (u_BLUP[:, 1:] ** 2).sum() / (e_BLUP[:, 1:] ** 2).sum()
    return math.log(num / den), Py


def LMC_REML(counts, rvec, X, y, persnp, seed=0, n_MC=3, tol_L=5e-4, s2max=0.7, s2min=1e-4,
             subset_size=1000, dtype=np.float32, maxit=600, reorth=False):
    """src/reml.cpp:730-883 — MC-REML with secant iterations on log((1−h²)/h²)."""
    dt = dtype
    n = y.size
    m = counts.shape[0]
    rvec = np.ones(n, dt) if rvec is None else np.asarray(rvec, dt)
    rr = (1.0 / np.sqrt(np.asarray(rvec, np.float64))).astype(dt)
    Xd = np.asarray(X, dt).reshape(n, -1)
    Q, _, rank = qr_colpiv(rr[:, None].astype(np.float64) * Xd, dtype=dt)
    if rank != Xd.shape[1]:
        raise RuntimeError("Fixed-effects design matrix is not of full rank.")
    c = rank
    pc = popcounts(counts)
    gm = genotype_mean(pc, n)
    gw = snp_weights(gm, persnp, dt)
    ops = Operators(counts, gm, gw, rr, Q, subset_size, dt)
    u_MC, e_MC = lmc_draws(seed, m, n, n_MC)
    V = np.empty((n, 1 + 2 * n_MC), dt)
    V[:, 0] = y
    V[:, 1:1 + n_MC] = ops.matvec(u_MC.astype(dt) * np.sqrt(gw)[:, None])
    V[:, 1 + n_MC:] = e_MC
    V[:, :1 + n_MC] *= rr[:, None]
    V = ops._proj(V)
    tau0 = (1 - np.float32(s2max)) / np.float32(s2max)
    seed_V = L_Seed(ops, "quadform", tau0, V, 10 * np.float32(tol_L), maxit, reorth)
    s2 = np.float32(s2max) / 2
    log_tau1 = np.float32(math.log((1 - s2) / s2))
    f1, PyMC = REML_first_order(ops, s2, tau0, V, seed_V, gw)
    f1 = np.float32(f1)
    trace = [(float(s2), float(f1))]
    s2 = np.float32(s2max) / 4 if f1 < 0 else np.float32(s2max)
    log_tau2 = np.float32(math.log((1 - s2) / s2))
    f2, PyMC = REML_first_order(ops, s2, tau0, V, seed_V, gw)
    f2 = np.float32(f2)
    trace.append((float(s2), float(f2)))
    for _ in range(3, 10):
        lt = np.float32((log_tau1 * f2 - log_tau2 * f1) / (f2 - f1))
        lt = np.float32(min(max(lt, -9.0), 9.0))
        if abs(lt - log_tau2) < 0.002:
            break
        s2 = np.float32(1 / (math.exp(lt) + 1))
        f1 = f2
        f2, PyMC = REML_first_order(ops, s2, tau0, V, seed_V, gw)
        f2 = np.float32(f2)
        log_tau1 = log_tau2
        log_tau2 = lt
        trace.append((float(s2), float(f2)))
    Py = PyMC[:, 0].copy()
    vg = float(np.dot(np.asarray(y, dt), Py)) / (n - c)
    tau1 = (1 - s2) / s2
    ve = tau1 * vg
    snp_blup = ops.weighted_rmatvec(Py)[:, 0]
    v0 = ops.matvec(snp_blup)[:, 0] + dt(tau1) * rvec * Py
    v0 = np.asarray(y, dt) - v0
    Xd64 = np.asarray(Xd, np.float64)
    blue = np.linalg.solve(Xd64.T @ Xd64, Xd64.T @ v0.astype(np.float64))
    return dict(vg=vg, ve=ve, h2=float(s2), Py=Py, snp_blup=snp_blup, blue=blue,
                iters=seed_V["iters"], secant=trace, gm=gm, gw=gw, n_MC=n_MC)


def lmm_variants(gm, n: int, num_qf: int = 30) -> list:
    """src/reml.cpp:919-925 — markers with MAC > 20 on both alleles in file order, shuffled by
    libstdc++ std::random_shuffle on the C library's unseeded rand(); the first num_qf."""
    gm = np.ascontiguousarray(gm, np.float32)
    out = np.zeros(max(num_qf, 1), np.int64)
    k = _lib().oracle_lmm_variants(_p(gm), gm.size, n, num_qf, _p(out))
    return [int(v) for v in out[:k]]


def LMM_quadforms(counts, Py, rr, Q, gm, gw, tau1, num_qf=30, window_size=1000, tol_L=5e-4,
                  dtype=np.float64):
    """src/reml.cpp:919-981 (--lmm, real markers): for the sampled markers x (centred counts),
    xPy = xᵀPy; with v = (I − QQᵀ)(rr∘x): xPx = vᵀ(H0 + τ1)⁻¹v by one Lanczos seed and solve,
    xSx = ‖v‖², and xBx = (xSx − zᵀ(ZᵀZ + τ1·diag(1/gw))⁻¹z)/τ1 with Z the projected, rr-scaled
    centred counts of the window_size markers around x (clamped at the ends) and z = Zᵀv."""
    dt = dtype
    counts = np.asarray(counts)
    m, n = counts.shape
    gm = np.asarray(gm, np.float32)
    variants = lmm_variants(gm, n, num_qf)
    rr = np.asarray(rr, dt)
    Q = np.asarray(Q, dt).reshape(n, -1)
    V = counts[variants].T.astype(dt) - gm[variants].astype(dt)
    xPy = V.T @ np.asarray(Py, dt)
    V = rr[:, None] * V
    V = V - Q @ (Q.T @ V)
    ops = Operators(counts, gm, gw, rr, Q, dtype=dt)
    seed_V = L_Seed(ops, "quadform", tau1, V, tol_L)
    X = L_Solve(seed_V, V, 0.0)
    xPx = np.einsum("ij,ij->j", V, X)
    xSx = np.einsum("ij,ij->j", V, V)
    xBx = np.zeros(len(variants), dt)
    gw = np.asarray(gw, dt)
    for i, j in enumerate(variants):
        if j < window_size // 2:
            wds = 0
        elif j > m - window_size // 2:
            wds = m - window_size
        else:
            wds = j - window_size // 2
        Z = counts[wds:wds + window_size].T.astype(dt) - gm[wds:wds + window_size].astype(dt)
        Z = rr[:, None] * Z
        Z = Z - Q @ (Q.T @ Z)
        G = Z.T @ Z + np.diag(tau1 / gw[wds:wds + window_size])
        z = Z.T @ V[:, i]
        xBx[i] = (xSx[i] - z @ np.linalg.solve(G, z)) / tau1
    return dict(variants=variants, xPy=xPy, xPx=xPx, xBx=xBx, xSx=xSx, iters=seed_V["iters"])


def gwa_blocks(ksnp_idx, block_size, chr_start, chr_end):
    """bin/slemm_gwa.py:322-345 — overlapping blocks of model SNPs (step block_size/2) and the
    range of tested variants each block serves."""
    ksnp_idx = np.asarray(ksnp_idx, np.int64)
    ksnp_ct = ksnp_idx.size
    if block_size > ksnp_ct:
        block_size = int(ksnp_ct / 2) * 2
    step = int(block_size / 2)
    ext = int(step / 2)
    block_ct = int((ksnp_ct - step) / step)
    blocks = [ksnp_idx[i * step:i * step + block_size] for i in range(block_ct)]
    if (ksnp_ct - step) % step != 0:
        blocks.append(ksnp_idx[ksnp_ct - block_size:ksnp_ct])
    bounds = np.empty((len(blocks), 2), np.int64)
    bounds[0, 0] = chr_start
    bounds[0, 1] = blocks[0][block_size - ext]
    for i in range(1, len(blocks)):
        bounds[i, 0] = bounds[i - 1, 1]
        bounds[i, 1] = blocks[i][block_size - ext]
    bounds[-1, 1] = chr_end + 1
    return blocks, bounds, block_size


def gwa_windows(a1_counts, y, R, covar, ksnp_idx, chr_start, chr_end, block_size, tau, model_snp_ct,
                cfactor, snp_var, mac):
    """bin/slemm_gwa.py:259-431 — windowed MLMA for the variants chr_start … chr_end.  a1_counts is
    m×n allele-1 counts (pgenlib's convention, 2 − the .bed A2 count); y the Py column of
    .reml.py.txt; R its last column; covar its covariates.  FP32 as the script (numpy float32).
    Returns beta, se, chisq, p (FP32, p FP64) over the tested range; NaN where MAC ≤ mac."""
    from scipy import linalg
    from scipy.stats import chi2
    f32 = np.float32
    n = y.size
    vec_y = np.asarray(y, f32)
    vec_rr = np.asarray(R, f32)
    mat_covar = np.asarray(covar, f32).reshape(n, -1)
    is_one_rr = bool(np.min(vec_rr) > 0.99999 and np.max(vec_rr) < 1.00001)
    is_const_covar = bool(mat_covar.shape[1] == 1 and np.max(mat_covar) == np.min(mat_covar))
    vec_rr = (1.0 / np.sqrt(vec_rr)).astype(f32)
    mat_covar = np.transpose(np.transpose(mat_covar) * vec_rr)
    Q = linalg.qr(mat_covar, mode="economic")[0]
    blocks, bounds, block_size = gwa_blocks(ksnp_idx, block_size, chr_start, chr_end)
    step = int(block_size / 2)
    tested = chr_end - chr_start + 1
    st_xx = np.empty(tested, f32)
    st_xy = np.empty(tested, f32)
    A = np.asarray(a1_counts)

    def prep(rows):
        b = A[rows].astype(f32)
        mean = b.mean(axis=1, keepdims=True)
        rv = ((2. - mean) * mean / 2.)[:, 0]
        b = b - mean
        if not is_one_rr:
            b = b * vec_rr
        if not (is_one_rr and is_const_covar):
            b = b - np.matmul(np.matmul(b, Q), np.transpose(Q))
        return b.astype(f32), rv.astype(f32)

    for i, blk in enumerate(blocks):
        buf2, rvars = prep(blk)
        mat_h = np.matmul(buf2, np.transpose(buf2))
        mat_h.ravel()[::mat_h.shape[1] + 1] += model_snp_ct * tau * rvars
        cf = linalg.cho_factor(mat_h)
        for j in range(bounds[i, 0], bounds[i, 1]):
            x = A[j].astype(f32)
            sx = x.sum()
            if sx <= mac or (2 * n - sx) <= mac:
                st_xx[j - chr_start] = np.nan
                st_xy[j - chr_start] = np.nan
                continue
            x = x - sx / n
            st_xy[j - chr_start] = np.dot(x, vec_y)
            if not is_one_rr:
                x = x * vec_rr
            if not (is_one_rr and is_const_covar):
                x = x - np.dot(Q, np.dot(np.transpose(Q), x))
            zx = np.dot(buf2, x)
            st_xx[j - chr_start] = np.dot(x, x) - np.dot(zx, linalg.cho_solve(cf, zx))
    st_xx /= tau
    beta = st_xy / st_xx * cfactor
    serr = np.sqrt((snp_var * cfactor) / st_xx)
    chisq = np.square(beta / serr)
    pval = chi2.sf(chisq, 1)
    return beta, serr, chisq, pval


def WLS(counts, rvec, X, y, dtype=np.float64):
    """src/wls.cpp:4-129 — SNP effects by weighted least squares: with Z̃ = (I − QQᵀ)(rr∘(Cnt − gm)),
    solve (Z̃ᵀZ̃ + 1e-4·mean(diag(Z̃ᵀZ̃))·I) b = Z̃ᵀ(I − QQᵀ)(rr∘y)."""
    dt = dtype
    counts = np.asarray(counts)
    m, n = counts.shape
    rvec = np.ones(n) if rvec is None else np.asarray(rvec, np.float64)
    rr = (1.0 / np.sqrt(rvec)).astype(dt)
    Xd = np.asarray(X, dt).reshape(n, -1)
    Q, _, rank = qr_colpiv(rr[:, None].astype(np.float64) * Xd, dtype=dt)
    y_proj = rr * np.asarray(y, dt)
    y_proj = y_proj - Q @ (Q.T @ y_proj)
    gm = genotype_mean(popcounts(counts), n).astype(dt)
    Z = counts.T.astype(dt) - gm
    Z = rr[:, None] * Z
    Z = Z - Q @ (Q.T @ Z)
    XtX = Z.T @ Z
    Xty = Z.T @ y_proj
    XtX[np.diag_indices(m)] += 1e-4 * np.mean(np.diag(XtX))
    return np.linalg.solve(XtX, Xty)


def n_mc_rule(n: int) -> int:
    """src/option.cpp:381,414 — n_MC = max(min(int(4e9/n/n), 30), 3)."""
    return max(min(int(4e9 / n / n), 30), 3)


# ------------------------------------------------------------------------------------------
# window weighting (src/option.cpp:458-529)
# ------------------------------------------------------------------------------------------
def window_weights(maf_vals, snp_blup, window_size, sig_idx=()):
    """snpvar = 2·maf(1−maf)·b², normalised to mean 1 (:458-464); sliding mean over
    window_size+1 SNPs with clamped edges (:505-509); logistic map (:511); fixed SNPs get 0
    (:523).  FP32 like the reference."""
    f32 = np.float32
    maf_vals = np.asarray(maf_vals, f32)
    b = np.asarray(snp_blup, f32)
    snpvar = f32(2.0) * maf_vals * (f32(1.0) - maf_vals) * b * b
    snpvar = snpvar / snpvar.mean(dtype=f32)
    m = snpvar.size
    half = window_size // 2
    out = np.empty(m, f32)
    cs = np.concatenate([[0.0], np.cumsum(snpvar.astype(np.float64))])
    for i in range(m):
        if i < half:
            lo, hi = 0, window_size + 1
        elif i > m - half - 1:
            lo, hi = m - window_size - 1, m
        else:
            lo, hi = i - half, i - half + window_size + 1
        out[i] = f32((cs[hi] - cs[lo]) / (hi - lo))
    out = f32(0.001) / (f32(0.001) + f32(0.999) * np.exp(out * f32(-0.5)))
    for j in sig_idx:
        out[j] = 0
    return snpvar, out


def clump_fixed_snps(counts, snpvar, sig_chisq, indep_r2):
    """src/option.cpp:466-497 — repeatedly take the SNP with the largest snpvar (first maximum)
    while it exceeds sig_chisq; its centred count vector joins the fixed effects when it is the
    first, or when its residual after regression on the ones already taken keeps more than
    indep_r2 of its squared norm.  Returns the indices taken and the n×s centred columns."""
    f32 = np.float32
    tmp = np.asarray(snpvar, f32).copy()
    idx, cols = [], []
    while True:
        j = int(np.argmax(tmp))
        if not tmp[j] > sig_chisq:
            break
        tmp[j] = 0
        yv = np.asarray(counts[j], f32)
        yv = yv - f32(yv.astype(np.float64).mean())
        if not idx:
            idx.append(j)
            cols.append(yv)
            continue
        Xs = np.column_stack(cols).astype(np.float64)
        y64 = yv.astype(np.float64)
        coef = np.linalg.solve(Xs.T @ Xs, Xs.T @ y64)
        res = y64 - Xs @ coef
        if (res @ res) / (y64 @ y64) > indep_r2:
            idx.append(j)
            cols.append(yv)
    Xs = np.column_stack(cols).astype(f32) if cols else np.zeros((counts.shape[1], 0), f32)
    return idx, Xs


def REML_iter_weighting(counts, rvec, X, y, persnp, maf_vals, lrt=True, seed=0, n_V=30, n_MC=None,
                        n_MC_final=None, tol_L=5e-4, s2max=0.7, window_size=20, sig_chisq=1e6,
                        indep_r2=0.5, dtype=np.float32, reorth=False):
    """src/option.cpp:437-530 — equal-weight GREML (DF-REML when --lrt and n < 5000, else MC-REML),
    per-SNP variance 2·maf(1−maf)·b² normalised to mean 1, fixed-effect SNPs by clumping, window
    weights, then the window-weighted GREML with those SNPs as covariates; their SNP-BLUP entries
    become their BLUE."""
    f32 = np.float32
    n = y.size
    m = counts.shape[0]
    n_MC = n_mc_rule(n) if n_MC is None else n_MC
    n_MC_final = n_MC if n_MC_final is None else n_MC_final
    ones = np.ones(m, f32)
    if lrt and n < 5000:
        r1 = SLDF_REML(counts, rvec, X, y, ones, seed=seed, n_V=n_V, tol_L=tol_L, s2max=s2max, dtype=dtype,
                       reorth=reorth)
    else:
        r1 = LMC_REML(counts, rvec, X, y, ones, seed=seed, n_MC=n_MC, tol_L=tol_L, s2max=s2max, dtype=dtype,
                      reorth=reorth)
    snpvar, _ = window_weights(maf_vals, r1["snp_blup"], window_size)
    sig, Xs = clump_fixed_snps(counts, snpvar, sig_chisq, indep_r2)
    _, w = window_weights(maf_vals, r1["snp_blup"], window_size, sig)
    p2 = np.asarray(persnp, f32) * w
    p2 = (p2 / f32(p2.astype(np.float64).mean())).astype(f32)
    X2 = np.column_stack([np.asarray(X, f32).reshape(n, -1), Xs])
    if lrt:
        r2 = SLDF_REML(counts, rvec, X2, y, p2, seed=seed, n_V=n_V, tol_L=tol_L, s2max=s2max, dtype=dtype,
                       reorth=reorth)
    else:
        r2 = LMC_REML(counts, rvec, X2, y, p2, seed=seed, n_MC=n_MC_final, tol_L=tol_L, s2max=s2max,
                      dtype=dtype, reorth=reorth)
    c = np.asarray(X).reshape(n, -1).shape[1]
    blup = np.asarray(r2["snp_blup"], f32).copy()
    for i, j in enumerate(sig):
        blup[j] = r2["blue"][c + i]
    r2 = dict(r2)
    r2.update(snp_blup=blup, fixed=sig, persnp=p2, stage1=r1)
    return r2


# ------------------------------------------------------------------------------------------
# GWAS step 2: GRAMMAR-Gamma terms (bin/slemm_gamma.py:296-325)
# ------------------------------------------------------------------------------------------
def gamma_terms(counts_a2, Py, rr, Q, mac):
    """Per SNP: x = allele-1 count (pgenlib) = 2 − count_A2; MAC filter; xy = (x−x̄)·y and
    xx = ‖(I−QQᵀ)(rr∘(x−x̄))‖² in FP32 (bin/slemm_gamma.py:306-319)."""
    f32 = np.float32
    m, n = counts_a2.shape
    y = np.asarray(Py, f32)
    rr = np.asarray(rr, f32)
    Q = np.asarray(Q, f32)
    is_one_rr = rr.min() > 0.99999 and rr.max() < 1.00001
    xy = np.empty(m, f32)
    xx = np.empty(m, f32)
    for j in range(m):
        x = (2 - counts_a2[j].astype(np.int16)).astype(f32)
        s = x.sum(dtype=f32)
        if s <= mac or (2 * n - s) <= mac:
            xy[j] = np.nan
            xx[j] = np.nan
            continue
        x = x - s / f32(n)
        xy[j] = np.dot(x, y)
        if not is_one_rr:
            x = x * rr
        if Q.shape[1]:
            x = x - Q @ (Q.T @ x)
        xx[j] = np.dot(x, x)
    return xy, xx


def gamma_stats(xy, xx, cfactor, snp_var):
    """bin/slemm_gamma.py:322-325."""
    from scipy.stats import chi2
    beta = xy / xx * np.float32(cfactor)
    serr = np.sqrt((np.float32(snp_var) * np.float32(cfactor)) / xx)
    chisq = np.square(beta / serr)
    pval = chi2.sf(chisq, 1)
    return beta, serr, chisq, pval


def mean_wo_outliers(x):
    """bin/slemm_gamma.py:90-105 — mean of values strictly inside the 1.5·IQR fences."""
    q1 = np.percentile(x, 25)
    q3 = np.percentile(x, 75)
    lower = q1 - (q3 - q1) * 1.5
    upper = q3 + (q3 - q1) * 1.5
    keep = [v for v in x if lower < v < upper]
    return sum(keep) / len(keep)


# ------------------------------------------------------------------------------------------
# dense FP64 ground truth for tiny problems (known-answer checks of the restatement)
# ------------------------------------------------------------------------------------------
def dense_reml_criterion(counts, gm, gw, rr, Q, y_proj, h2):
    """Exact FP64 REML quantities at h² for a tiny problem: with A = rr∘Z W Zᵀ∘rr and
    H = A + τI (τ = (1−h²)/h²), returns yᵀP̃y and log det(H) and log det(QᵀH⁻¹Q)."""
    Z = counts.T.astype(np.float64) - gm.astype(np.float64)
    rr = rr.astype(np.float64)
    A = (rr[:, None] * Z) @ (gw.astype(np.float64)[:, None] * (Z.T * rr[None, :]))
    tau = (1 - h2) / h2
    H = A + tau * np.eye(A.shape[0])
    Q = Q.astype(np.float64)
    P = np.eye(A.shape[0]) - Q @ Q.T
    Pt = P @ H @ P + tau * 0.0
    yp = y_proj.astype(np.float64)
    sol = np.linalg.lstsq(Pt + Q @ Q.T, yp, rcond=None)[0]
    return float(yp @ sol), float(np.linalg.slogdet(H)[1]), float(
        np.linalg.slogdet(Q.T @ np.linalg.solve(H, Q))[1])


# ------------------------------------------------------------------------------------------
# REML log-likelihood and its gradient (variance components, per-window SNP weights), FP64
# ------------------------------------------------------------------------------------------
def _grad_model(counts, rvec, X, y, persnp, window, wwin):
    """Dense pieces of Ṽ = σ_g²·Z̃WZ̃ᵀ + σ_e²·I in the rr-transformed space (rr = R^-½ in FP32
    as the reference, Z̃ = rr∘(Z − gm)), W_j = gw_j·w_{window_j} with gw from
    src/reml.cpp:613-622 (FP32) and weight 1 outside every window."""
    m, n = counts.shape
    pc = popcounts(counts)
    gm = genotype_mean(pc, n)
    gw = snp_weights(gm, np.asarray(persnp, np.float32)).astype(np.float64)
    ww = np.ones(m)
    if window is not None:
        window = np.asarray(window)
        sel = window >= 0
        ww[sel] = np.asarray(wwin, np.float64)[window[sel]]
    rr = np.ones(n) if rvec is None else (np.float32(1) / np.sqrt(np.asarray(rvec, np.float32))).astype(np.float64)
    Zt = rr[:, None] * (counts.T.astype(np.float64) - gm.astype(np.float64)[None, :])
    Xt = rr[:, None] * np.asarray(X, np.float64)
    yt = rr * np.asarray(y, np.float64)
    return Zt, Xt, yt, gw, ww


def _reml_P(Zt, Xt, W, sg2, se2):
    n = Zt.shape[0]
    V = sg2 * (Zt * W[None, :]) @ Zt.T + se2 * np.eye(n)
    Vi = np.linalg.inv(V)
    ViX = Vi @ Xt
    XVX = Xt.T @ ViX
    P = Vi - ViX @ np.linalg.solve(XVX, ViX.T)
    return V, XVX, P


def reml_loglik_dense(counts, rvec, X, y, persnp, window, wwin, sg2, se2):
    """ℓ = −½[log|Ṽ| + log|X̃ᵀṼ⁻¹X̃| + ỹᵀP̃ỹ] (the constant dropped), exact FP64 for small n."""
    Zt, Xt, yt, gw, ww = _grad_model(counts, rvec, X, y, persnp, window, wwin)
    V, XVX, P = _reml_P(Zt, Xt, gw * ww, sg2, se2)
    return -0.5 * (np.linalg.slogdet(V)[1] + np.linalg.slogdet(XVX)[1] + yt @ P @ yt)


def reml_grad_dense(counts, rvec, X, y, persnp, window, wwin, sg2, se2, probes=None):
    """∂ℓ/∂θ = −½[tr(P̃·∂Ṽ/∂θ) − ỹᵀP̃(∂Ṽ/∂θ)P̃ỹ] for θ = σ_g², σ_e², w_1 … w_K.  Traces exact, or by
    Hutchinson with the given normalised probes (n×n_V): tr(A) ≈ (n/n_V)·Σ_v vᵀAv.  Returns
    (d_sigma_g2, d_sigma_e2, d_w)."""
    Zt, Xt, yt, gw, ww = _grad_model(counts, rvec, X, y, persnp, window, wwin)
    n, m = Zt.shape
    W = gw * ww
    _, _, P = _reml_P(Zt, Xt, W, sg2, se2)
    py = P @ yt
    a = (Zt.T @ py) ** 2                               # (z̃_jᵀP̃ỹ)²
    if probes is None:
        b = np.einsum("ij,ij->j", Zt, P @ Zt)          # z̃_jᵀP̃z̃_j
        trP = np.trace(P)
    else:
        Vp = np.asarray(probes, np.float64)
        s = n / Vp.shape[1]
        b = s * np.einsum("jv,jv->j", Zt.T @ (P @ Vp), Zt.T @ Vp)
        trP = s * np.einsum("iv,iv->", Vp, P @ Vp)
    d_sg = -0.5 * (W @ b - W @ a)
    d_se = -0.5 * (trP - py @ py)
    K = 0 if wwin is None else len(wwin)
    d_w = np.zeros(K)
    if K:
        window = np.asarray(window)
        for k in range(K):
            sel = window == k
            d_w[k] = -0.5 * sg2 * (gw[sel] @ (b[sel] - a[sel]))
    return d_sg, d_se, d_w
