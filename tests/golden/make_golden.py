"""Generates the golden fixtures of tests/golden/ (run here, where the reference checkout and
oracle/_ref exist; the fixtures are committed and the tests read only them).

  hwe_ref.json       SNPHWE2 p-values from the reference's own src/snphwe.cpp (compiled by
                     `make -C oracle ref`) on a grid of genotype class counts, plain and mid-p.
  rng_draws.json     the first probe draws of the reference's generators (libstdc++ mt19937):
                     Rademacher (reml.cpp:597-605) and MC normals (reml.cpp:795-809).
  format.json        header lines and row layouts of the reference's example outputs
                     (examples/expected/slemm/*).
  gamma_case/        a small synthetic .bed/.bim/.fam with SLEMM step-1 style inputs and the
                     output of the reference's bin/slemm_gamma.py run on it (pgenlib replaced
                     by tests/golden/pgenlib_shim, which reads PLINK1 .bed files).
  gwa_case/          the same kind of case for the reference's bin/slemm_gwa.py (windowed
                     MLMA on chromosome 1), with step-1 files from the oracle.
Usage: python tests/golden/make_golden.py /path/to/reference/checkout [gwa]
(or with the checkout in the SLEMM_REFERENCE environment variable)
"""
import ctypes
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
REF = sys.argv[1] if len(sys.argv) > 1 and sys.argv[1] != "gwa" else os.environ.get("SLEMM_REFERENCE", "")
if not REF or not os.path.isdir(os.path.join(REF, "src")):
    sys.exit("give the reference checkout as the first argument or in SLEMM_REFERENCE")


def hwe():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "ref", f"REF={REF}"], check=True)
    lib = ctypes.CDLL(os.path.join(ROOT, "oracle", "_ref", "libslemm_ref.so"))
    lib.ref_SNPHWE2.restype = ctypes.c_double
    lib.ref_SNPHWE2.argtypes = [ctypes.c_int32, ctypes.c_int32, ctypes.c_int32, ctypes.c_uint32]
    rng = np.random.default_rng(2024)
    cases = [(0, 0, 0), (1, 0, 0), (0, 1, 0), (0, 0, 1), (2, 1, 1), (10, 20, 5), (50, 25, 25),
             (0, 50, 50), (100, 0, 0), (480, 250, 270), (1862, 7500, 638), (3000, 5000, 2000)]
    for _ in range(60):
        n = int(rng.integers(5, 20000))
        p = rng.uniform(0.01, 0.5)
        het = int(rng.binomial(n, 2 * p * (1 - p) * rng.uniform(0.7, 1.3)))
        het = min(het, n)
        h2 = int(rng.binomial(n - het, p * p / max(p * p + (1 - p) ** 2, 1e-9)))
        cases.append((het, n - het - h2, h2))
    out = []
    for het, h1, h2 in cases:
        for midp in (0, 1):
            out.append([het, h1, h2, midp, lib.ref_SNPHWE2(het, h1, h2, midp)])
    json.dump({"source": "src/snphwe.cpp SNPHWE2 (reference, compiled unmodified)",
               "cases": out}, open(os.path.join(HERE, "hwe_ref.json"), "w"), indent=0)


def rng_draws():
    from oracle import slemm_np as orc
    d = {}
    for seed in (0, 1, 42):
        V = orc.rademacher(seed, 37, 3)
        d[f"rademacher_seed{seed}_n37_nv3"] = (np.sign(V).astype(int)).T.tolist()
        u, e = orc.lmc_draws(seed, 11, 7, 2)
        d[f"lmc_seed{seed}_m11_n7_nmc2_u"] = u.T.tolist()
        d[f"lmc_seed{seed}_m11_n7_nmc2_e"] = e.T.tolist()
    json.dump(d, open(os.path.join(HERE, "rng_draws.json"), "w"))


def formats():
    exp = os.path.join(REF, "examples", "expected", "slemm")
    f = {}
    for name in ("10k.reml.py.txt", "10k.reml.snp.csv", "10k.reml.blue.csv", "10k.reml.vc.csv",
                 "10k.gstat.txt", "10k.gebv.csv", "10k.gamma.txt"):
        lines = open(os.path.join(exp, name)).read().splitlines()
        f[name] = {"header": lines[0], "row1": lines[1] if len(lines) > 1 else "",
                   "nrows": len(lines) - 1}
    f["10k.reml.vc.csv"]["all"] = open(os.path.join(exp, "10k.reml.vc.csv")).read().splitlines()
    json.dump(f, open(os.path.join(HERE, "format.json"), "w"), indent=1)


def gamma_case():
    """Runs the reference's slemm_gamma.py on a synthetic case whose step-1 files come from the
    oracle's LMC_REML restatement."""
    from oracle import slemm_np as orc
    from slemm_gb300 import synth
    d = os.path.join(HERE, "gamma_case")
    os.makedirs(d, exist_ok=True)
    n, m = 600, 400
    counts, _ = synth.simulate_counts(n, m, seed=21)
    rows = synth.encode_bed(counts, 0.0)
    y, _, _ = synth.simulate_phenotype(counts, 0.4, n_causal=50, seed=21)
    ids, iids = synth.write_plink(os.path.join(d, "geno"), rows, n)
    rng = np.random.default_rng(8)
    rvec = rng.uniform(0.8, 1.5, n).astype(np.float32)
    X = np.column_stack([np.ones(n), rng.standard_normal(n)]).astype(np.float32)
    res = orc.LMC_REML(counts, rvec, X, y.astype(np.float32), np.ones(m, np.float32), seed=3,
                       n_MC=4, dtype=np.float32)
    # step-1 outputs in the reference's formats (output.cpp:28-37, 74-82, 98-120)
    with open(os.path.join(d, "s1.reml.py.txt"), "w") as f:
        f.write("IID Py intercept x1 R\n")
        for i in range(n):
            f.write(f"{iids[i]} {res['Py'][i]:.6g} {X[i,0]:.6g} {X[i,1]:.6g} {rvec[i]:.6g}\n")
    with open(os.path.join(d, "s1.reml.vc.csv"), "w") as f:
        f.write(f"pop_size,{n}\nnum_markers,{m}\nVg,{res['vg']:.6g}\nVe,{res['ve']:.6g}\n")
    with open(os.path.join(d, "s1.gstat.txt"), "w") as f:
        f.write("variant\tChr\tPos\tMAC\tMAF\tHWEP\txPy\txPx\txBx\txSx\tWindowSize\tChiSq\tPval\n")
        g = np.random.default_rng(4)
        for j in range(30):
            xpx = g.uniform(100, 200)
            f.write(f"snp{j+1}\t1\t{1000*(j+1)}\t50\t0.1\t0.5\t1.0\t{xpx:.6g}\t1\t{xpx*g.uniform(9,11):.6g}\t20\t0.1\t0.7\n")
    env = dict(os.environ, PYTHONPATH=os.path.join(HERE, "pgenlib_shim"))
    subprocess.run([sys.executable, os.path.join(REF, "bin", "slemm_gamma.py"), "--pfile",
                    os.path.join(d, "geno"), "--slemm", os.path.join(d, "s1"), "--out",
                    os.path.join(d, "gamma.txt")], check=True, env=env, capture_output=True)


def gwa_case():
    """Runs the reference's bin/slemm_gwa.py (windowed MLMA) on a synthetic two-chromosome case.
    Step-1 files come from the oracle: MC-REML on the model SNPs (every chromosome-2 SNP and all
    chromosome-1 SNPs but every 7th), and real --lmm quadratic forms for .gstat.txt."""
    from oracle import slemm_np as orc
    from slemm_gb300 import synth
    d = os.path.join(HERE, "gwa_case")
    os.makedirs(d, exist_ok=True)
    n, m = 500, 420
    counts, _ = synth.simulate_counts(n, m, seed=33)
    rows = synth.encode_bed(counts, 0.0)
    chrom = [1] * 360 + [2] * 60
    ids, iids = synth.write_plink(os.path.join(d, "geno"), rows, n, chrom=chrom)
    y, _, _ = synth.simulate_phenotype(counts, 0.5, n_causal=40, seed=33)
    rng = np.random.default_rng(12)
    rvec = rng.uniform(0.8, 1.5, n).astype(np.float32)
    X = np.column_stack([np.ones(n), rng.standard_normal(n)]).astype(np.float32)
    model = [j for j in range(m) if chrom[j] == 2 or j % 7 != 3]
    cm = counts[model]
    res = orc.LMC_REML(cm, rvec, X, y.astype(np.float32), np.ones(len(model), np.float32), seed=5,
                       n_MC=4, dtype=np.float32)
    pc = orc.popcounts(cm)
    gm = orc.genotype_mean(pc, n)
    gw = orc.snp_weights(gm, np.ones(len(model), np.float32))
    rr = (1.0 / np.sqrt(rvec)).astype(np.float32)
    Q, _, _ = orc.qr_colpiv(rr[:, None].astype(np.float64) * X, dtype=np.float32)
    tau1 = res["ve"] / res["vg"]
    ws = 60
    qf = orc.LMM_quadforms(cm, res["Py"], rr, Q, gm, gw, tau1, num_qf=30, window_size=ws)
    with open(os.path.join(d, "s1.reml.py.txt"), "w") as f:
        f.write("IID Py intercept x1 R\n")
        for i in range(n):
            f.write(f"{iids[i]} {res['Py'][i]:.6g} {X[i,0]:.6g} {X[i,1]:.6g} {rvec[i]:.6g}\n")
    with open(os.path.join(d, "s1.reml.vc.csv"), "w") as f:
        f.write(f"pop_size,{n}\nnum_markers,{len(model)}\nVg,{res['vg']:.6g}\nVe,{res['ve']:.6g}\n")
    with open(os.path.join(d, "s1.reml.snp.csv"), "w") as f:
        f.write("SNP,Chr,Pos,Allele1,Allele2,MAF,HWE_Pval,Group,Weight,Effect\n")
        for k, j in enumerate(model):
            f.write(f"{ids[j]},{chrom[j]},{1000 * (j + 1)},2,1,0.1,0.5,NULL,1,{res['snp_blup'][k]:.6g}\n")
    with open(os.path.join(d, "s1.gstat.txt"), "w") as f:
        f.write("variant\tChr\tPos\tMAC\tMAF\tHWEP\txPy\txPx\txBx\txSx\tWindowSize\tChiSq\tPval\n")
        for k, j in enumerate(qf["variants"]):
            jj = model[j]
            f.write(f"{ids[jj]}\t{chrom[jj]}\t{1000 * (jj + 1)}\t50\t0.1\t0.5\t{qf['xPy'][k]:.6g}\t"
                    f"{qf['xPx'][k]:.6g}\t{qf['xBx'][k]:.6g}\t{qf['xSx'][k]:.6g}\t{ws}\t0.1\t0.7\n")
    env = dict(os.environ, PYTHONPATH=os.path.join(HERE, "pgenlib_shim"))
    subprocess.run([sys.executable, os.path.join(REF, "bin", "slemm_gwa.py"), "--pfile",
                    os.path.join(d, "geno"), "--slemm", os.path.join(d, "s1"), "--out",
                    os.path.join(d, "gwa.txt"), "--chr", "1"], check=True, env=env, capture_output=True)


if __name__ == "__main__":
    only = sys.argv[2] if len(sys.argv) > 2 else None
    if only == "gwa":
        gwa_case()
        sys.exit(0)
    hwe()
    rng_draws()
    formats()
    gamma_case()
    gwa_case()
    print("golden fixtures written to", HERE)
