"""The `slemm` command line (slemm_gb300/bin/slemm): the reference's options, CSV and PLINK inputs and
output files (src/option.cpp, src/input.cpp, src/output.cpp, src/pred.cpp).

CPU: argument and input-file errors are reported before any GPU work, with the reference's
messages and exit statuses.  GPU: on a synthetic PLINK set with missing phenotypes, --reml --lrt
writes .reml.{py.txt,snp.csv,blue.csv,vc.csv} in the pinned formats (tests/golden/format.json)
with h² within 1e-4 of the FP64 oracle; --prediction from that .reml.snp.csv gives the oracle's
GEBVs (FP64, rtol 1e-6 of the printed six digits); --lmm writes .gstat.txt; --wls the SNP file.
"""
import json
import os
import subprocess

import numpy as np
import pytest

from oracle import slemm_np as orc
from slemm_gb300 import synth

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SLEMM = os.path.join(ROOT, "slemm_gb300", "bin", "slemm")
GOLD = os.path.join(ROOT, "tests", "golden")


@pytest.fixture(scope="module")
def cli():
    from slemm_gb300 import build
    build.build()
    return SLEMM


def run(cli, *args, cwd=None):
    return subprocess.run([cli, *args], capture_output=True, text=True, cwd=cwd, timeout=600)


def write_plink(d, counts, rows, prefix="geno"):
    m, n = counts.shape
    with open(os.path.join(d, prefix + ".fam"), "w") as f:
        for i in range(n):
            f.write(f"F{i} I{i} 0 0 1 -9\n")
    with open(os.path.join(d, prefix + ".bim"), "w") as f:
        for j in range(m):
            f.write(f"{1 + j // 500}\tS{j}\t0\t{1000 + 37 * j}\tA\tG\n")
    with open(os.path.join(d, prefix + ".bed"), "wb") as f:
        f.write(bytes([0x6C, 0x1B, 0x01]))
        f.write(np.ascontiguousarray(rows).tobytes())


def test_cli_without_arguments_prints_help_and_exits_1(cli):
    r = run(cli)
    assert r.returncode == 1 and "documentation" in r.stdout


def test_cli_reports_missing_required_options(cli):
    r = run(cli, "--reml", "--bfile", "nothing")
    assert r.returncode == 0 and "--phenotype_file is required" in r.stderr
    r = run(cli, "--rem", "--phenotype", "p.csv", "--trait", "y")       # abbreviations as getopt_long
    assert "--snp_info_file is required" in r.stderr
    r = run(cli, "--reml", "--phenotype_file", "p.csv", "--trait_name", "y", "--snp_info_file", "s.csv",
            "--bfile", "g", "--output_file", "o", "--min_maf", "0.7")
    assert "--min_maf is out of [0, 0.5)" in r.stderr


def test_cli_input_file_errors_exit_1(cli, tmp_path):
    (tmp_path / "p.csv").write_text("IID,y,cov1\nI0,1.0,2\n")
    (tmp_path / "s.csv").write_text("SNP\nS0\n")
    r = run(cli, "--reml", "--phenotype_file", "p.csv", "--trait_name", "y", "--covariate_names", "nope",
            "--snp_info_file", "s.csv", "--bfile", "g", "--output_file", "o", cwd=tmp_path)
    assert r.returncode == 1 and "nope not in covariate file" in r.stdout
    r = run(cli, "--reml", "--phenotype_file", "p.csv", "--trait_name", "z", "--snp_info_file", "s.csv",
            "--bfile", "g", "--output_file", "o", cwd=tmp_path)
    assert r.returncode == 1 and "z not found in the header of p.csv" in r.stdout


@pytest.fixture(scope="module")
def plink_case(tmp_path_factory):
    d = tmp_path_factory.mktemp("cli")
    n_fam, m = 1200, 900
    counts, _ = synth.simulate_counts(n_fam, m, seed=91)
    rows = synth.encode_bed(counts, missing=0.01, seed=92)
    write_plink(str(d), counts, rows)
    dec = orc.bed_decode(rows, n_fam)
    y, _, _ = synth.simulate_phenotype(dec, 0.5, n_causal=120, seed=93)
    rng = np.random.default_rng(94)
    cov1 = rng.standard_normal(n_fam)
    miss = rng.random(n_fam) < 0.05                       # 5 % of the trait missing
    with open(d / "pheno.csv", "w") as f:
        f.write("IID,mu,cov1,y\n")
        for i in range(n_fam):
            f.write(f"I{i},1,{cov1[i]:.6f},{'' if miss[i] else f'{y[i]:.6f}'}\n")
    with open(d / "snps.csv", "w") as f:
        f.write("SNP\n" + "".join(f"S{j}\n" for j in range(m)))
    keep = np.nonzero(~miss)[0]
    X = np.column_stack([np.ones(keep.size), np.float32(np.round(cov1[keep], 6))]).astype(np.float32)
    yk = np.array([float(f"{v:.6f}") for v in y[keep]], np.float32)
    return dict(d=d, dec=dec, keep=keep, X=X, y=yk, n_fam=n_fam, m=m)


def read_vc(path):
    return {k: float(v) for k, v in (l.split(",") for l in open(path).read().split())}


@pytest.mark.gpu
def test_cli_reml_lrt_prediction_lmm_wls(cli, plink_case):
    c = plink_case
    d = str(c["d"])
    fmt = json.load(open(os.path.join(GOLD, "format.json")))
    common = ["--phenotype_file", "pheno.csv", "--trait_name", "y", "--covariate_names", "mu,cov1", "--bfile", "geno",
              "--snp_info_file", "snps.csv", "--num_random_vectors", "12", "--seed", "3"]
    r = run(cli, "--reml", "--lrt", *common, "--output_file", "out", cwd=d)
    assert r.returncode == 0 and r.stderr.strip() == "", r.stderr
    ct = np.ascontiguousarray(c["dec"][:, c["keep"]])
    r64 = orc.SLDF_REML(ct, None, c["X"], c["y"], np.ones(c["m"], np.float32), seed=3, n_V=12, dtype=np.float64)
    vc = read_vc(os.path.join(d, "out.reml.vc.csv"))
    assert vc["pop_size"] == c["keep"].size and vc["num_markers"] == c["m"]
    assert abs(vc["h2"] - r64["h2"]) <= 1e-4
    assert [l.split(",")[0] for l in open(os.path.join(d, "out.reml.vc.csv")).read().split()] == \
        [l.split(",")[0] for l in fmt["10k.reml.vc.csv"]["all"]]
    snp = open(os.path.join(d, "out.reml.snp.csv")).read().splitlines()
    assert snp[0] == fmt["10k.reml.snp.csv"]["header"] and len(snp) == 1 + c["m"]
    eff = np.array([float(l.split(",")[9]) for l in snp[1:]])
    assert np.corrcoef(eff, r64["snp_blup"])[0, 1] >= 0.99999
    py = open(os.path.join(d, "out.reml.py.txt")).read().splitlines()
    assert py[0] == "IID Py mu cov1 R" and len(py) == 1 + c["keep"].size
    blue = open(os.path.join(d, "out.reml.blue.csv")).read().splitlines()
    assert blue[0] == "covar,blue,se,pval,mu,cov1" and len(blue) == 3
    # GEBV from the written SNP effects (src/pred.cpp): every .fam individual
    r = run(cli, "--prediction", "--bfile", "geno", "--snp_estimate_file", "out.reml.snp.csv",
            "--output_file", "out.gebv.csv", cwd=d)
    assert r.returncode == 0 and r.stderr.strip() == "", r.stderr
    gebv = open(os.path.join(d, "out.gebv.csv")).read().splitlines()
    assert gebv[0] == fmt["10k.gebv.csv"]["header"] and len(gebv) == 1 + c["n_fam"]
    got = np.array([float(l.split(",")[1]) for l in gebv[1:]])
    want = orc.gebv(c["dec"], eff)
    assert np.allclose(got, want, rtol=1e-5, atol=1e-5 * np.max(np.abs(want)))
    # --lmm: the MC-REML fit and the .gstat.txt quadratic forms
    r = run(cli, "--lmm", *common, "--window_size", "100", "--num_qf_markers", "10", "--output_file", "lmm", cwd=d)
    assert r.returncode == 0 and r.stderr.strip() == "", r.stderr
    gs = open(os.path.join(d, "lmm.gstat.txt")).read().splitlines()
    assert gs[0] == fmt["10k.gstat.txt"]["header"] and len(gs) == 11
    assert all(l.split("\t")[10] == "100" for l in gs[1:])
    assert open(os.path.join(d, "lmm.reml.blue.csv")).read().splitlines()[0] == "covar,blue"
    # --wls
    r = run(cli, "--wls", *common, "--output_file", "wls", cwd=d)
    assert r.returncode == 0 and r.stderr.strip() == "", r.stderr
    w = open(os.path.join(d, "wls.reml.snp.csv")).read().splitlines()
    assert len(w) == 1 + c["m"]
    ref = orc.WLS(ct, None, c["X"], c["y"])
    got = np.array([float(l.split(",")[9]) for l in w[1:]])
    assert np.linalg.norm(got - ref) / np.linalg.norm(ref) <= 1e-3
