"""GWAS step 2, GRAMMAR-Gamma score tests: the options, inputs and output file of the reference's
bin/slemm_gamma.py, with the per-variant terms computed on the GPU.

    python -m slemm_gb300.cli.slemm_gamma --pfile geno --slemm run1 --out run1.gamma.txt

Inputs (slemm_gamma.py:123-274): the genotypes (--pfile prefix, or --pgen/--psam/--pvar; PLINK 1
.bed/.fam/.bim — a PLINK 2 .pgen is reported as unsupported), and the step-1 files of the SLEMM
run named by --slemm: .reml.py.txt (Py, covariates, R), .gstat.txt (the correction factor, the
outlier-trimmed mean of xSx/xPx) and .reml.vc.csv (Vg, Ve).  For every variant --begin … --end:
x = allele-1 counts of the SLEMM samples; a variant with Σx ≤ mac or 2n − Σx ≤ mac is NaN; else
xy = (x − x̄)·Py and xx = ‖(I − QQᵀ)(rr∘(x − x̄))‖² with rr = R^−½ and Q the economic QR of the
rr-scaled covariates (:296-319), here one packed pass over all variants on the GPU
(slemm_gpu_score_terms).  Statistics (:321-325): beta = xy/xx·cf, se = √(Vg·cf/xx),
χ² = (beta/se)², p = χ²₁ survival.  Output (:328-361): the variant's .pvar/.bim line then BETA,
SE, CHISQ and P, tab-separated, under the same header.
"""
from __future__ import annotations

import sys
import time

import numpy as np

from slemm_gb300.cli import _gwas_io as io


def get_parser():
    from argparse import ArgumentDefaultsHelpFormatter, ArgumentParser
    p = ArgumentParser(description="GRAMMAR-Gamma score tests (slemm_gamma.py options) on the GPU",
                       formatter_class=ArgumentDefaultsHelpFormatter)
    p.add_argument("-p", "--pfile", dest="pfile", help="PLINK2 pfile prefix", metavar="<prefix>")
    p.add_argument("-g", "--pgen", dest="pgen", help="PLINK2 pgen file", metavar="<filename>")
    p.add_argument("-v", "--pvar", dest="pvar", help="PLINK2 pvar file", metavar="<filename>")
    p.add_argument("-s", "--psam", dest="psam", help="PLINK2 psam file", metavar="<filename>")
    p.add_argument("-b", "--slemm", required=True, dest="slemm", help="SLEMM LMM filename prefix",
                   metavar="<prefix>")
    p.add_argument("-o", "--out", required=True, dest="out", help="output filename", metavar="<filename>")
    p.add_argument("-f", "--maf", dest="maf", type=float, default=0.0, help="min minor allele frequency",
                   metavar="<freq>")
    p.add_argument("-m", "--mac", dest="mac", type=int, default=20, help="min minor allele count",
                   metavar="<count>")
    p.add_argument("-i", "--begin", dest="begin", type=int, default=0, help="begin index", metavar="<index>")
    p.add_argument("-j", "--end", dest="end", type=int, default=1000000000, help="end index", metavar="<index>")
    p.add_argument("--gpu_device", dest="gpu_device", type=int, default=0, help="CUDA device")
    return p


def mean_wo_outliers(x):
    """Mean of the values strictly inside Tukey's fences q1 − 1.5·IQR, q3 + 1.5·IQR
    (slemm_gamma.py:88-104)."""
    x = np.asarray(x, np.float64)
    q1, q3 = np.percentile(x, 25), np.percentile(x, 75)
    lo, hi = q1 - (q3 - q1) * 1.5, q3 + (q3 - q1) * 1.5
    keep = x[(x < hi) & (x > lo)]
    if keep.size < x.size:
        print(int(x.size - keep.size), "outliers identified when calculating correction factor")
        print("If not removing outliers, the correction factor is", sum(x) / len(x))
        print("Removed outliers")
    return float(sum(keep)) / keep.size


def correction_factor(gsfile):
    with open(gsfile) as fp:
        next(fp)
        r = []
        for line in fp:
            e = line.strip().split()
            r.append(float(e[9]) / float(e[7]))
    return mean_wo_outliers(r)


def variances(vcfile):
    with open(vcfile) as fp:
        fp.readline()
        fp.readline()
        snp_var = float(fp.readline().strip().split(",")[1])
        err_var = float(fp.readline().strip().split(",")[1])
    return snp_var, err_var


def stats(xy, xx, cfactor, snp_var):
    """beta, se, χ² in FP32 and p in FP64, as the script's NumPy arithmetic gives them."""
    from scipy.stats import chi2
    xy = np.asarray(xy, np.float32)
    xx = np.asarray(xx, np.float32)
    with np.errstate(invalid="ignore", divide="ignore"):
        beta = xy / xx * np.float32(cfactor)
        serr = np.sqrt(np.float32(snp_var * cfactor) / xx)
        chisq = np.square(beta / serr)
    return beta, serr, chisq, chi2.sf(chisq, 1)


def main(argv=None):
    start = time.time()
    print("*******************************************************************")
    print("* slemm_gb300 GRAMMAR-Gamma (options and output of slemm_gamma.py)")
    print("*******************************************************************")
    args = get_parser().parse_args(argv)
    args.begin = max(args.begin, 0)
    args.end = max(args.end, 0)
    pgen, psam, pvar = io.resolve_genotype_files(args)
    phenofile = io.require(args.slemm + ".reml.py.txt")
    gsfile = io.require(args.slemm + ".gstat.txt")
    vcfile = io.require(args.slemm + ".reml.vc.csv")

    cfactor = correction_factor(gsfile)
    print("Correction factor is", cfactor)
    snp_var, err_var = variances(vcfile)
    print("SNP var is", snp_var)
    print("ERR var is", err_var)

    pheno, covar, diagr, covar_ct = io.read_reml_py(phenofile)
    sample_ct = len(pheno)
    print("\nSample count in SLEMM file is", sample_ct)
    print("Number of covariates is", covar_ct)
    mac = io.mac_threshold(args.mac, args.maf, sample_ct)
    raw_ct, subset, y, cov, R = io.read_samples(psam, pheno, covar, diagr, covar_ct)
    print("Raw sample count in psam is", raw_ct)
    print("Sample count in GWA is", sample_ct)

    is_one_rr = bool(np.min(R) > 0.99999 and np.max(R) < 1.00001)
    is_const_covar = covar_ct == 1 and np.max(cov) == np.min(cov)
    rr = (1.0 / np.sqrt(R)).astype(np.float32)
    from scipy import linalg
    Q = linalg.qr(np.transpose(np.transpose(cov) * rr), mode="economic")[0]
    print("Completed QR decomposition of covariate matrix.")

    header, lines = io.read_variant_lines(pvar)
    last = min(args.end, len(lines) - 1)
    if args.begin > last:
        raise SystemExit(f"--begin {args.begin} is past the last variant ({len(lines) - 1})")
    rows = io.bed_rows(pgen, raw_ct, len(lines))[args.begin:last + 1]

    print("\nStarting assoc tests...")
    from slemm_gb300 import api
    api.init(args.gpu_device)
    with api.Genotypes(rows, raw_ct, subset) as g:
        m = rows.shape[0]
        g.set_weights(np.zeros(m, np.float32), np.zeros(m, np.float32), None if is_one_rr else rr)
        if not (is_one_rr and is_const_covar):
            g.set_projection(np.asarray(Q, np.float32))
        xy, xx = g.score_terms(y, mac=mac)
    beta, serr, chisq, pval = stats(xy, xx, cfactor, snp_var)
    print("Computed association statistics.")

    print("\nWriting stats into", args.out)
    io.write_stats(args.out, header, lines, args.begin, beta, serr, chisq, pval)
    print(int(time.time() - start), "s taken for the whole analysis.\n")


if __name__ == "__main__":
    sys.exit(main())
