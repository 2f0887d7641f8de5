"""Inputs shared by the GWAS step-2 commands (slemm_gamma, slemm_gwa): the genotype file set, the
step-1 files of a SLEMM run, and the PLINK .bed rows.

The reference's scripts (bin/slemm_gamma.py, bin/slemm_gwa.py) read genotypes through pgenlib,
which accepts a PLINK 2 .pgen or a PLINK 1 .bed (variant-major).  This build reads .bed files only
(the packed 2-bit layout its GPU kernels consume); a .pgen is reported as unsupported.
"""
from __future__ import annotations

import os
import sys

import numpy as np

BED_MAGIC = bytes([0x6C, 0x1B, 0x01])


def resolve_genotype_files(args):
    """(genotypes, samples, variants) paths as the scripts choose them (slemm_gamma.py:123-147):
    --pfile P → P.pgen/.psam/.pvar, else P.bed/.fam/.bim; or the explicit --pgen/--psam/--pvar.
    Prints the scripts' messages and exits when the files are missing."""
    if args.pfile is not None:
        pgen, psam, pvar = args.pfile + ".pgen", args.pfile + ".psam", args.pfile + ".pvar"
        if not (os.path.isfile(pgen) and os.path.isfile(psam) and os.path.isfile(pvar)):
            print("Files do not exit:", pgen, psam, pvar)
            print("Searching for bed/bim/fam files.")
            pgen, psam, pvar = args.pfile + ".bed", args.pfile + ".fam", args.pfile + ".bim"
    elif args.pgen is not None and args.psam is not None and args.pvar is not None:
        pgen, psam, pvar = args.pgen, args.psam, args.pvar
    else:
        print("Genotype files are not specified. Use following arguments.")
        print("    --pfile <prefix>")
        print("    --pgen <filename> --pvar <filename> --psam <filename>")
        sys.exit()
    if not (os.path.isfile(pgen) and os.path.isfile(psam) and os.path.isfile(pvar)):
        print("Files do not exit:", pgen, psam, pvar)
        sys.exit()
    return pgen, psam, pvar


def require(path):
    if not os.path.isfile(path):
        print("File path {} does not exist.".format(path))
        sys.exit()
    return path


def read_reml_py(path):
    """.reml.py.txt (src/output.cpp:28-37): IID, Py, the covariates, R.  Returns dicts keyed by IID
    of the raw strings, as the scripts keep them, and the covariate count."""
    pheno, covar, diagr = {}, {}, {}
    with open(path) as fp:
        covar_ct = len(fp.readline().strip().split()) - 3
        for line in fp:
            e = line.strip().split()
            pheno[e[0]] = e[1]
            covar[e[0]] = e[2:2 + covar_ct]
            diagr[e[0]] = e[-1]
    return pheno, covar, diagr, covar_ct


def read_samples(psam, pheno, covar, diagr, covar_ct):
    """Walks the .psam/.fam (slemm_gamma.py:219-251): the IID column is the first of a .psam whose
    header starts '#I', else the second.  Returns the raw sample count, the increasing raw indices
    of the SLEMM samples (None when all are), and y, covariates and R in that order."""
    sample_ct = len(pheno)
    subset = np.empty(sample_ct, np.int64)
    y = np.empty(sample_ct, np.float32)
    cov = np.empty((sample_ct, covar_ct), np.float32)
    R = np.empty(sample_ct, np.float32)
    header, lines = None, []
    with open(psam) as fp:
        for line in fp:
            if not lines and line[0] == "#":
                header = line
                continue
            lines.append(line)
    iid_col = 0 if (header is not None and header[1] == "I") else 1
    idx = 0
    for raw, line in enumerate(lines):
        iid = line.strip().split()[iid_col]
        if iid in pheno:
            if idx >= sample_ct:
                raise SystemExit(f"sample {iid} appears twice in {psam}")
            subset[idx] = raw
            y[idx] = float(pheno[iid])
            cov[idx] = [float(v) for v in covar[iid]]
            R[idx] = float(diagr[iid])
            idx += 1
    if idx != sample_ct:
        raise SystemExit(f"{sample_ct - idx} samples of the SLEMM file are not in {psam}")
    raw_ct = len(lines)
    return raw_ct, (None if sample_ct == raw_ct else subset), y, cov, R


def read_variant_lines(pvar):
    """The .pvar/.bim: (header line or None, the variant lines)."""
    header, lines = None, []
    with open(pvar) as fp:
        for line in fp:
            if not lines and line[0] == "#":
                header = line
                continue
            if line.strip():
                lines.append(line)
    return header, lines


def bed_rows(path, raw_sample_ct, variant_ct):
    """The .bed's variant rows as a read-only memory map, variant_ct × ⌈raw_sample_ct/4⌉ bytes."""
    with open(path, "rb") as f:
        magic = f.read(3)
    if magic != BED_MAGIC:
        if magic[:2] == BED_MAGIC[:2]:
            raise SystemExit(f"{path} is a PLINK 2 .pgen (storage mode 0x{magic[2]:02x}); this build reads "
                             "PLINK 1 .bed files only (plink2 --make-bed converts it)")
        raise SystemExit(f"{path} is not a variant-major PLINK .bed file")
    rb = (raw_sample_ct + 3) // 4
    size = os.path.getsize(path) - 3
    if size < variant_ct * rb:
        raise SystemExit(f"{path} holds {size} bytes of genotypes, fewer than {variant_ct} variants x {rb}")
    return np.memmap(path, dtype=np.uint8, mode="r", offset=3, shape=(variant_ct, rb))


def output_header(header, first_line):
    """Header of the statistics file (slemm_gamma.py:333-346)."""
    if header is not None:
        return header.strip() + "\tBETA\tSE\tCHISQ\tP\n"
    if len(first_line.split()) == 6:
        return "CHR\tSNP\tCM\tBP\tA1\tA2\tBETA\tSE\tCHISQ\tP\n"
    return "CHR\tSNP\tBP\tA1\tA2\tBETA\tSE\tCHISQ\tP\n"


def write_stats(out, header, lines, first, beta, se, chisq, pval):
    """One line per variant first … first+len(beta)−1: the variant line, then BETA, SE, CHISQ, P as
    the scripts print NumPy scalars (str of float32 statistics and a float64 p)."""
    with open(out, "w") as f:
        f.write(output_header(header, lines[0]))
        for k in range(len(beta)):
            f.write(lines[first + k].strip() + "\t" + str(beta[k]) + "\t" + str(se[k]) + "\t" +
                    str(chisq[k]) + "\t" + str(pval[k]) + "\n")


def mac_threshold(mac, maf, sample_ct):
    """--maf raises --mac to the count it implies (slemm_gamma.py:208-209)."""
    if 2 * sample_ct * maf > mac:
        return int(2 * sample_ct * maf + 0.5)
    return mac
