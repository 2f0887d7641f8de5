"""Seeded synthetic genotype/phenotype generator with the shapes of the benchmark workloads.

Per SNP j the allele-2 frequency is p_j ~ U(0.05, 0.5); genotypes are Binomial(2, p_j), or, with
``ld_rho > 0``, an AR(1) latent Gaussian along SNPs inside blocks of ``ld_block`` SNPs
thresholded at the Binomial(2, p_j) quantiles.  ``missing`` sets that fraction of calls to the
PLINK missing code 01.  The phenotype is y = Z_std·β + e with ``n_causal`` causal SNPs,
β ~ N(0, h²/n_causal) and e ~ N(0, 1 − h²).

PLINK .bed codes (SNP-major, 4 genotypes per byte, first genotype in the low bits):
allele-2 count 0 → 00, 1 → 10, 2 → 11, missing → 01.
"""
from __future__ import annotations

import os

import numpy as np

BED_MAGIC = bytes([0x6C, 0x1B, 0x01])
_CODE_OF_COUNT = np.array([0b00, 0b10, 0b11], dtype=np.uint8)


def simulate_counts(n: int, m: int, seed: int = 1, ld_rho: float = 0.0, ld_block: int = 50,
                    chunk: int = 2048):
    """Returns (counts m×n uint8 in {0,1,2}, p m float64)."""
    rng = np.random.default_rng(seed)
    p = rng.uniform(0.05, 0.5, size=m)
    counts = np.empty((m, n), dtype=np.uint8)
    if ld_rho <= 0.0:
        for j0 in range(0, m, chunk):
            j1 = min(m, j0 + chunk)
            counts[j0:j1] = rng.binomial(2, p[j0:j1, None], size=(j1 - j0, n)).astype(np.uint8)
        return counts, p
    from scipy.special import ndtr
    s = np.sqrt(1.0 - ld_rho * ld_rho)
    z = np.empty(n)
    for j in range(m):
        if j % ld_block == 0:
            z = rng.standard_normal(n)
        else:
            z = ld_rho * z + s * rng.standard_normal(n)
        u = ndtr(z)
        q0 = (1 - p[j]) ** 2
        q1 = q0 + 2 * p[j] * (1 - p[j])
        counts[j] = (u >= q0).astype(np.uint8) + (u >= q1).astype(np.uint8)
    return counts, p


def encode_bed(counts: np.ndarray, missing: float = 0.0, seed: int = 2) -> np.ndarray:
    """m×n counts → m×ceil(n/4) .bed rows; a `missing` fraction of calls become code 01."""
    m, n = counts.shape
    codes = _CODE_OF_COUNT[counts]
    if missing > 0:
        rng = np.random.default_rng(seed)
        codes = codes.copy()
        codes[rng.random((m, n)) < missing] = 0b01
    nb = (n + 3) // 4
    pad = np.zeros((m, nb * 4), dtype=np.uint8)
    pad[:, :n] = codes
    pad = pad.reshape(m, nb, 4)
    return (pad[:, :, 0] | (pad[:, :, 1] << 2) | (pad[:, :, 2] << 4) | (pad[:, :, 3] << 6)).astype(np.uint8)


def counts_of_bed(rows: np.ndarray, n: int) -> np.ndarray:
    """Vectorised decode with the missing→1 rule (bit0 + bit1 of each code)."""
    m, nb = rows.shape
    sh = np.array([0, 2, 4, 6], dtype=np.uint8)
    codes = (rows[:, :, None] >> sh) & 3
    codes = codes.reshape(m, nb * 4)[:, :n]
    return ((codes & 1) + (codes >> 1)).astype(np.uint8)


def simulate_phenotype(counts: np.ndarray, h2: float, n_causal: int = 1000, seed: int = 1):
    """y = Z_std β + e (standardised causal genotypes), returns (y float64, causal idx, β)."""
    m, n = counts.shape
    rng = np.random.default_rng(seed + 7919)
    n_causal = min(n_causal, m)
    idx = np.sort(rng.choice(m, size=n_causal, replace=False))
    beta = rng.normal(0.0, np.sqrt(h2 / n_causal), size=n_causal)
    g = np.zeros(n)
    for j, b in zip(idx, beta):
        x = counts[j].astype(np.float64)
        sd = x.std()
        if sd > 0:
            g += b * (x - x.mean()) / sd
    e = rng.normal(0.0, np.sqrt(1.0 - h2), size=n)
    return g + e, idx, beta


def write_plink(prefix: str, rows: np.ndarray, n: int, chrom=None, snp_ids=None, iids=None,
                a1="1", a2="2"):
    """Writes prefix.bed/.bim/.fam.  Allele 2 (.bim column 6) is the counted allele."""
    m = rows.shape[0]
    os.makedirs(os.path.dirname(os.path.abspath(prefix)), exist_ok=True)
    with open(prefix + ".bed", "wb") as f:
        f.write(BED_MAGIC)
        f.write(np.ascontiguousarray(rows, dtype=np.uint8).tobytes())
    snp_ids = snp_ids if snp_ids is not None else [f"snp{j + 1}" for j in range(m)]
    chrom = chrom if chrom is not None else [1 + (j * 30) // max(m, 1) for j in range(m)]
    with open(prefix + ".bim", "w") as f:
        for j in range(m):
            f.write(f"{chrom[j]}\t{snp_ids[j]}\t0\t{1000 * (j + 1)}\t{a1}\t{a2}\n")
    iids = iids if iids is not None else [f"{1000001 + i}" for i in range(n)]
    with open(prefix + ".fam", "w") as f:
        for i in range(n):
            f.write(f"0 {iids[i]} 0 0 2 -9\n")
    return snp_ids, iids


def write_csv(path: str, header, columns):
    with open(path, "w") as f:
        f.write(",".join(header) + "\n")
        for row in zip(*columns):
            f.write(",".join("" if v is None else str(v) for v in row) + "\n")


def simulate_bed_torch(n: int, m: int, seed: int = 1, h2: float = 0.4, n_causal: int = 1000,
                       missing: float = 0.0, device: str = "cuda", chunk: int = 2048,
                       ld_rho: float = 0.0, ld_block: int = 50, n_traits: int = 1,
                       rows_device: bool = False):
    """Device-side generator for benchmark-sized inputs (same model as the NumPy path, torch's
    RNG): returns (.bed rows as a pinned host uint8 tensor m×ceil(n/4), y float32 numpy).
    With ``ld_rho > 0`` the genotypes of each block of ``ld_block`` SNPs come from an AR(1)
    latent Gaussian along the SNPs, thresholded at the Binomial(2, p_j) quantiles.
    ``n_traits > 1`` draws that many phenotypes, each with its own causal SNPs and effects (y is
    then n × n_traits); ``rows_device`` keeps the rows in device memory.  With the defaults the
    random stream is that of the single-trait generator.
    Torch is used only as a random-number and memory utility here."""
    import torch
    if ld_rho > 0.0:   # whole LD blocks per chunk, ≈1 GB of latent values at a time
        chunk = ld_block * max(1, min(chunk, (1 << 28) // max(n, 1)) // ld_block)
    gen = torch.Generator(device=device)
    gen.manual_seed(seed)
    nb = (n + 3) // 4
    if rows_device:
        rows = torch.empty((m, nb), dtype=torch.uint8, device=device)
    else:
        rows = torch.empty((m, nb), dtype=torch.uint8, pin_memory=torch.cuda.is_available())
    p = torch.rand(m, generator=gen, device=device, dtype=torch.float64) * 0.45 + 0.05
    code_of = torch.tensor([0b00, 0b10, 0b11], dtype=torch.uint8, device=device)
    causal_t, beta_t = [], []
    for _ in range(max(1, n_traits)):
        causal = torch.randperm(m, generator=gen, device=device)[: min(n_causal, m)]
        causal_sorted, _ = torch.sort(causal)
        beta = torch.randn(causal_sorted.numel(), generator=gen, device=device, dtype=torch.float64) * \
            (h2 / max(causal_sorted.numel(), 1)) ** 0.5
        causal_t.append(causal_sorted)
        beta_t.append(beta)
    gt = torch.zeros((len(causal_t), n), dtype=torch.float64, device=device)
    shifts = torch.tensor([0, 2, 4, 6], dtype=torch.uint8, device=device)
    for j0 in range(0, m, chunk):
        j1 = min(m, j0 + chunk)
        pj = p[j0:j1, None]
        if ld_rho > 0.0:
            z = torch.empty((j1 - j0, n), device=device, dtype=torch.float32)
            sd = (1.0 - ld_rho * ld_rho) ** 0.5
            for r in range(j1 - j0):
                e = torch.randn(n, generator=gen, device=device, dtype=torch.float32)
                z[r] = e if (j0 + r) % ld_block == 0 else ld_rho * z[r - 1] + sd * e
            u = torch.special.ndtr(z)
            q0 = ((1.0 - pj) ** 2).float()
            q1 = (q0 + 2.0 * pj * (1.0 - pj)).float()
            cnt = (u >= q0).to(torch.uint8) + (u >= q1).to(torch.uint8)
            del z, u
        else:
            u1 = torch.rand((j1 - j0, n), generator=gen, device=device, dtype=torch.float32)
            u2 = torch.rand((j1 - j0, n), generator=gen, device=device, dtype=torch.float32)
            cnt = (u1 < pj).to(torch.uint8) + (u2 < pj).to(torch.uint8)       # Binomial(2, p)
        for t, (causal_sorted, beta) in enumerate(zip(causal_t, beta_t)):
            sel = (causal_sorted >= j0) & (causal_sorted < j1)
            if bool(sel.any()):
                idx = causal_sorted[sel] - j0
                x = cnt[idx].to(torch.float64)
                sd = x.std(dim=1, unbiased=False).clamp_min(1e-12)
                gt[t] += (beta[sel, None] * (x - x.mean(dim=1, keepdim=True)) / sd[:, None]).sum(0)
        codes = code_of[cnt.long()]
        if missing > 0:
            miss = torch.rand((j1 - j0, n), generator=gen, device=device) < missing
            codes = torch.where(miss, torch.ones_like(codes), codes)
        pad = torch.zeros((j1 - j0, nb * 4), dtype=torch.uint8, device=device)
        pad[:, :n] = codes
        packed = (pad.view(j1 - j0, nb, 4) << shifts).sum(dim=2, dtype=torch.uint8)
        rows[j0:j1].copy_(packed, non_blocking=False)
    ys = []
    for t in range(gt.shape[0]):
        e = torch.randn(n, generator=gen, device=device, dtype=torch.float64) * (1.0 - h2) ** 0.5
        ys.append((gt[t] + e).float().cpu().numpy())
    return rows, (ys[0] if n_traits <= 1 else np.stack(ys, axis=1))
