"""GWAS step 2, windowed MLMA: the options, inputs and output file of the reference's
bin/slemm_gwa.py, with the block Grams, Cholesky factors and per-variant solves on the GPU.

    python -m slemm_gb300.cli.slemm_gwa --pfile geno --slemm run1 --chr 1 --out run1.chr1.gwa.txt

Inputs (slemm_gwa.py:106-285): the genotypes (--pfile prefix, or --pgen/--psam/--pvar; PLINK 1
.bed/.fam/.bim — a PLINK 2 .pgen is reported as unsupported) and the step-1 files of the SLEMM
run named by --slemm: .reml.py.txt (Py, covariates, R), .gstat.txt (the block size from its
WindowSize column and the correction factor, the mean of xBx/xPx), .reml.vc.csv (the model SNP
count, Vg, Ve) and .reml.snp.csv (the model SNPs; those on --chr).  Every variant of --chr is
tested against blocks of the chromosome's model SNPs (block_size, step block_size/2, the last
block flush with the end; a block serves the variants up to its model SNP block_size − step/2)
whose projected Gram plus model_snp_ct·tau·var is Cholesky-factored (:287-396); xx = x̃ᵀx̃ −
(Zx̃)ᵀH⁻¹(Zx̃), xy = (x − x̄)·Py, then xx/τ, beta = xy/xx·cf, se = √(Vg·cf/xx), χ², p
(:397-403) — slemm_gpu_gwa_windows.  Output (:405-434): the variant's .pvar/.bim line then
BETA, SE, CHISQ and P under the same header.
"""
from __future__ import annotations

import sys
import time

import numpy as np

from slemm_gb300.cli import _gwas_io as io


def get_parser():
    from argparse import ArgumentDefaultsHelpFormatter, ArgumentParser
    p = ArgumentParser(description="Windowed MLMA (slemm_gwa.py options) on the GPU",
                       formatter_class=ArgumentDefaultsHelpFormatter)
    p.add_argument("-p", "--pfile", dest="pfile", help="PLINK2 pfile prefix", metavar="<prefix>")
    p.add_argument("-g", "--pgen", dest="pgen", help="PLINK2 pgen file", metavar="<filename>")
    p.add_argument("-v", "--pvar", dest="pvar", help="PLINK2 pvar file", metavar="<filename>")
    p.add_argument("-s", "--psam", dest="psam", help="PLINK2 psam file", metavar="<filename>")
    p.add_argument("-b", "--slemm", required=True, dest="slemm", help="SLEMM LMM filename prefix",
                   metavar="<prefix>")
    p.add_argument("-o", "--out", required=True, dest="out", help="output filename", metavar="<filename>")
    p.add_argument("-c", "--chr", required=True, dest="chr", help="chromosome", metavar="<chr>")
    p.add_argument("-f", "--maf", dest="maf", type=float, default=0.0, help="min minor allele frequency",
                   metavar="<freq>")
    p.add_argument("-m", "--mac", dest="mac", type=int, default=20, help="min minor allele count",
                   metavar="<count>")
    p.add_argument("--gpu_device", dest="gpu_device", type=int, default=0, help="CUDA device")
    return p


def gstat(gsfile):
    """(correction factor = mean of xBx/xPx, block size = the last WindowSize) (:139-158)."""
    sum_r, num_r, block_size = 0.0, 0, None
    with open(gsfile) as fp:
        next(fp)
        for line in fp:
            e = line.strip().split()
            sum_r += float(e[8]) / float(e[7])
            num_r += 1
            block_size = int(e[10])
    if num_r == 0:
        raise SystemExit(f"{gsfile} has no variants")
    return sum_r / num_r, block_size


def vc(vcfile):
    with open(vcfile) as fp:
        fp.readline()
        model_snp_ct = int(fp.readline().strip().split(",")[1])
        snp_var = float(fp.readline().strip().split(",")[1])
        err_var = float(fp.readline().strip().split(",")[1])
    return model_snp_ct, snp_var, err_var


def model_snps(snpfile, chrom):
    with open(snpfile) as fp:
        next(fp)
        return {e[0] for e in (line.strip().split(",") for line in fp) if len(e) > 1 and e[1] == chrom}


def blocks_of(n_model, block_size):
    """Start of every block in the model-SNP list (:319-335)."""
    step = block_size // 2
    starts = [i * step for i in range((n_model - step) // step)]
    if (n_model - step) % step != 0:
        starts.append(n_model - block_size)
    return starts


def main(argv=None):
    start = time.time()
    print("*******************************************************************")
    print("* slemm_gb300 windowed MLMA (options and output of slemm_gwa.py)")
    print("*******************************************************************")
    args = get_parser().parse_args(argv)
    pgen, psam, pvar = io.resolve_genotype_files(args)
    phenofile = io.require(args.slemm + ".reml.py.txt")
    gsfile = io.require(args.slemm + ".gstat.txt")
    vcfile = io.require(args.slemm + ".reml.vc.csv")
    snpfile = io.require(args.slemm + ".reml.snp.csv")

    cfactor, block_size = gstat(gsfile)
    print("Correction factor is", cfactor)
    model_snp_ct, snp_var, err_var = vc(vcfile)
    print("Block size is", block_size)
    print("SNP var is", snp_var)
    print("ERR var is", err_var)
    tau = err_var / snp_var

    ksnp_set = model_snps(snpfile, args.chr)
    print("\nCount of model variants on Chr", args.chr, "is", len(ksnp_set))
    if not ksnp_set:
        print("Error: Is --chr", args.chr, "correctly specified?\n")
        sys.exit()

    pheno, covar, diagr, covar_ct = io.read_reml_py(phenofile)
    sample_ct = len(pheno)
    print("\nSample count in SLEMM file is", sample_ct)
    print("Number of covariates is", covar_ct)
    mac = io.mac_threshold(args.mac, args.maf, sample_ct)
    raw_ct, subset, y, cov, R = io.read_samples(psam, pheno, covar, diagr, covar_ct)
    print("Raw sample count in psam is", raw_ct)
    print("Sample count in GWA is", sample_ct)

    header, lines = io.read_variant_lines(pvar)
    id_col = 2 if (header is not None and header[1] == "C") else 1
    fields = [l.strip().split() for l in lines]
    ksnp = [j for j, f in enumerate(fields) if f[id_col] in ksnp_set]
    on_chr = [j for j, f in enumerate(fields) if f[0] == args.chr]
    if not on_chr:
        print("Error: Is --chr", args.chr, "correctly specified?\n")
        sys.exit()
    chr_start, chr_end = min(on_chr), max(on_chr)
    print("\nIdx range for variants on chr", args.chr, "is", chr_start, "-", chr_end)
    print("Count of variants to be tested is", chr_end - chr_start + 1)
    print("Count of model variants to be used is", len(ksnp))
    if len(ksnp) < 4:
        raise SystemExit("fewer than 4 model variants on the chromosome")
    if block_size > len(ksnp):
        block_size = int(len(ksnp) / 2) * 2
        print("\nWarning: Block size in SLEMM was too big and reduced to", block_size)
    starts = blocks_of(len(ksnp), block_size)
    ext = block_size // 4
    bound = np.empty((len(starts), 2), np.uint32)
    for i, s in enumerate(starts):
        bound[i, 0] = chr_start if i == 0 else bound[i - 1, 1]
        bound[i, 1] = ksnp[s + block_size - ext]
    bound[-1, 1] = chr_end + 1
    print("\nCompleted building blocks:")
    print(bound)

    rows = io.bed_rows(pgen, raw_ct, len(lines))[chr_start:chr_end + 1]
    print("\nStarting assoc tests...")
    print("There are", len(starts), "blocks.")
    from slemm_gb300 import api
    api.init(args.gpu_device)
    is_one_rr = bool(np.min(R) > 0.99999 and np.max(R) < 1.00001)
    with api.Genotypes(rows, raw_ct, subset) as g:
        beta, se, chisq, pval = g.gwa_windows(y, None if is_one_rr else R, cov,
                                              np.asarray(ksnp, np.int64) - chr_start, 0, chr_end - chr_start,
                                              block_size, tau, model_snp_ct, cfactor, snp_var, mac)
    print("Computed association statistics.")

    print("\nWriting stats into", args.out)
    io.write_stats(args.out, header, lines, chr_start, beta, se, chisq, pval)
    print(int(time.time() - start), "s taken for the whole analysis.\n")


if __name__ == "__main__":
    sys.exit(main())
