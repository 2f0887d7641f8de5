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


def test_cli_gpu_options_parse(cli):
    """The options beyond the reference's are parsed (and echoed like the reference's own) before
    the input checks: --gpu_device, --gpu_precision, --gpu_autotune, --gpu_lanczos_reorth."""
    r = run(cli, "--reml", "--gpu_device", "0", "--gpu_precision", "bf16x2", "--gpu_autotune", "--gpu_lanczos_reorth",
            "--bfile", "nothing")
    assert "OPTION gpu_autotune initialized" in r.stdout and "OPTION gpu_lanczos_reorth initialized" in r.stdout
    assert "OPTION gpu_precision with ARG bf16x2" in r.stdout
    assert "--phenotype_file is required" in r.stderr


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


# ---- GWAS step 2: slemm_gamma / slemm_gwa (bin/slemm_gamma.py, bin/slemm_gwa.py) ------------------
import shutil
import sys


def run_py(module, *args, cwd=None):
    env = dict(os.environ, PYTHONPATH=ROOT + os.pathsep + os.environ.get("PYTHONPATH", ""))
    return subprocess.run([sys.executable, "-m", module, *args], capture_output=True, text=True, cwd=cwd,
                          env=env, timeout=600)


def test_gwas_commands_report_missing_files(tmp_path):
    for mod in ("slemm_gb300.cli.slemm_gamma", "slemm_gb300.cli.slemm_gwa"):
        extra = ["--chr", "1"] if mod.endswith("gwa") else []
        r = run_py(mod, "--pfile", str(tmp_path / "nothing"), "--slemm", "s1", "--out", "o.txt", *extra)
        assert r.returncode == 0 and "Files do not exit:" in r.stdout and "Searching for bed/bim/fam" in r.stdout
        r = run_py(mod, "--slemm", "s1", "--out", "o.txt", *extra)
        assert r.returncode == 0 and "Genotype files are not specified" in r.stdout
    r = run_py("slemm_gb300.cli.slemm_gamma", "--slemm", "s1")
    assert r.returncode == 2 and "--out" in r.stderr                      # argparse: required option


def test_gwas_commands_reject_pgen(tmp_path):
    """A PLINK 2 .pgen (magic 6c 1b, storage mode ≠ 01) is reported as unsupported before any GPU
    work; the step-1 files and the sample/variant files are read first, as the scripts do."""
    src = os.path.join(GOLD, "gamma_case")
    for f in ("s1.gstat.txt", "s1.reml.py.txt", "s1.reml.vc.csv"):
        shutil.copy(os.path.join(src, f), tmp_path / f)
    shutil.copy(os.path.join(src, "geno.fam"), tmp_path / "geno.psam")
    shutil.copy(os.path.join(src, "geno.bim"), tmp_path / "geno.pvar")
    (tmp_path / "geno.pgen").write_bytes(bytes([0x6C, 0x1B, 0x10]) + bytes(64))
    r = run_py("slemm_gb300.cli.slemm_gamma", "--pfile", "geno", "--slemm", "s1", "--out", "o.txt", cwd=tmp_path)
    assert r.returncode == 1 and "PLINK 2 .pgen (storage mode 0x10)" in r.stderr, r.stderr
    assert "Correction factor is" in r.stdout and not (tmp_path / "o.txt").exists()


def _stats_file(path):
    rows = [l.split("\t") for l in open(path).read().splitlines()]
    return rows[0], [r[:-4] for r in rows[1:]], np.array([[float(v) for v in r[-4:]] for r in rows[1:]])


def _compare_stats(got_path, want_path):
    h1, v1, s1 = _stats_file(got_path)
    h2, v2, s2 = _stats_file(want_path)
    assert h1 == h2 and v1 == v2                                 # header and variant columns identical
    ok = np.isfinite(s2[:, 3])
    assert np.array_equal(ok, np.isfinite(s1[:, 3]))             # same filtered variants
    assert np.allclose(s1[ok, 0], s2[ok, 0], rtol=1e-3, atol=1e-5)   # beta
    assert np.allclose(s1[ok, 1], s2[ok, 1], rtol=1e-3)              # se
    assert np.max(np.abs(np.log10(s1[ok, 3]) - np.log10(s2[ok, 3]))) <= 1e-3


@pytest.mark.gpu
def test_gamma_command_matches_reference_script_output(tmp_path):
    """slemm_gamma on the golden case against the output of the reference's own script."""
    src = os.path.join(GOLD, "gamma_case")
    r = run_py("slemm_gb300.cli.slemm_gamma", "--pfile", os.path.join(src, "geno"), "--slemm",
               os.path.join(src, "s1"), "--out", str(tmp_path / "gamma.txt"))
    assert r.returncode == 0, r.stderr
    _compare_stats(tmp_path / "gamma.txt", os.path.join(src, "gamma.txt"))
    # --begin/--end select a variant range: the same lines of the full output
    r = run_py("slemm_gb300.cli.slemm_gamma", "--pfile", os.path.join(src, "geno"), "--slemm",
               os.path.join(src, "s1"), "--out", str(tmp_path / "part.txt"), "--begin", "5", "--end", "20")
    assert r.returncode == 0, r.stderr
    full = open(tmp_path / "gamma.txt").read().splitlines()
    part = open(tmp_path / "part.txt").read().splitlines()
    assert part[0] == full[0] and len(part) == 17
    assert [l.split("\t")[:6] for l in part[1:]] == [l.split("\t")[:6] for l in full[6:22]]


@pytest.mark.gpu
def test_gwa_command_matches_reference_script_output(tmp_path):
    """slemm_gwa --chr 1 on the golden two-chromosome case against the reference script's output."""
    src = os.path.join(GOLD, "gwa_case")
    r = run_py("slemm_gb300.cli.slemm_gwa", "--pfile", os.path.join(src, "geno"), "--slemm", os.path.join(src, "s1"),
               "--out", str(tmp_path / "gwa.txt"), "--chr", "1")
    assert r.returncode == 0, r.stderr
    assert "Completed building blocks:" in r.stdout
    _compare_stats(tmp_path / "gwa.txt", os.path.join(src, "gwa.txt"))


def test_gwas_io_helpers(tmp_path):
    """The step-2 commands' readers and writers, as bin/slemm_gamma.py / slemm_gwa.py parse and
    print: .psam IID column ('#IID' header → first column, .fam → second), the SLEMM sample
    subset in .psam order, output headers, NumPy-style value printing, --maf raising --mac."""
    from slemm_gb300.cli import _gwas_io as io
    pheno = {"b": "1.5", "d": "-2"}
    covar = {"b": ["1", "0.5"], "d": ["1", "-0.25"]}
    diagr = {"b": "1", "d": "2"}
    (tmp_path / "x.psam").write_text("#IID\tSEX\na\t1\nb\t2\nc\t1\nd\t2\n")
    raw, subset, y, cov, R = io.read_samples(str(tmp_path / "x.psam"), pheno, covar, diagr, 2)
    assert raw == 4 and list(subset) == [1, 3] and list(y) == [1.5, -2.0]
    assert cov.tolist() == [[1.0, 0.5], [1.0, -0.25]] and list(R) == [1.0, 2.0]
    (tmp_path / "x.fam").write_text("F b 0 0 1 -9\nF d 0 0 2 -9\n")
    raw, subset, y, _, _ = io.read_samples(str(tmp_path / "x.fam"), pheno, covar, diagr, 2)
    assert raw == 2 and subset is None and list(y) == [1.5, -2.0]
    with pytest.raises(SystemExit):   # a SLEMM sample missing from the sample file
        io.read_samples(str(tmp_path / "x.fam"), dict(pheno, e="0"), dict(covar, e=["1", "0"]),
                        dict(diagr, e="1"), 2)
    assert io.output_header("#CHROM\tPOS\tID\tREF\tALT\n", "1\t5\ts\tA\tG") == \
        "#CHROM\tPOS\tID\tREF\tALT\tBETA\tSE\tCHISQ\tP\n"
    assert io.output_header(None, "1 s 0 5 A G").startswith("CHR\tSNP\tCM\tBP\tA1\tA2\t")
    assert io.output_header(None, "1 s 5 A G").startswith("CHR\tSNP\tBP\tA1\tA2\t")
    io.write_stats(str(tmp_path / "o.txt"), None, ["1 s1 0 5 A G\n", "1 s2 0 9 A G\n"], 1,
                   np.array([0.25], np.float32), np.array([0.1], np.float32), np.array([6.25], np.float32),
                   np.array([0.0124193], np.float64))
    assert open(tmp_path / "o.txt").read().splitlines() == [
        "CHR\tSNP\tCM\tBP\tA1\tA2\tBETA\tSE\tCHISQ\tP", "1 s2 0 9 A G\t0.25\t0.1\t6.25\t0.0124193"]
    assert io.mac_threshold(20, 0.0, 1000) == 20 and io.mac_threshold(20, 0.05, 1000) == 100
    (tmp_path / "p.bed").write_bytes(bytes([0x6C, 0x1B, 0x01, 0xFF, 0x00]))
    assert io.bed_rows(str(tmp_path / "p.bed"), 4, 2).tolist() == [[0xFF], [0x00]]
    with pytest.raises(SystemExit):
        io.bed_rows(str(tmp_path / "p.bed"), 4, 3)                       # fewer rows than variants
    (tmp_path / "q.bed").write_bytes(bytes([0x6C, 0x1B, 0x00, 0x00]))  # individual-major PLINK 1
    with pytest.raises(SystemExit):
        io.bed_rows(str(tmp_path / "q.bed"), 4, 1)


def test_gamma_statistics_and_correction_factor():
    """beta = xy/xx·cf, se = √(Vg·cf/xx), χ² = (beta/se)², p = χ²₁ survival in the script's dtypes
    (FP32 statistics, FP64 p), NaN where filtered; the correction factor is the mean inside
    Tukey's fences (bin/slemm_gamma.py:88-104, 321-325)."""
    from scipy.stats import chi2
    from slemm_gb300.cli import slemm_gamma as sg
    xy = np.array([2.0, np.nan, -1.0], np.float32)
    xx = np.array([4.0, np.nan, 8.0], np.float32)
    beta, se, chisq, p = sg.stats(xy, xx, 1.1, 0.3)
    assert beta.dtype == np.float32 and se.dtype == np.float32 and p.dtype == np.float64
    assert np.isnan(beta[1]) and np.isnan(p[1])
    assert beta[0] == np.float32(2.0) / np.float32(4.0) * np.float32(1.1)
    assert np.isclose(se[2], np.sqrt(0.3 * 1.1 / 8.0), rtol=1e-6)
    assert np.isclose(p[0], chi2.sf(float(chisq[0]), 1), rtol=1e-12)
    x = [1.0, 1.1, 0.9, 1.05, 0.95, 10.0]                 # 10 is outside the fences
    assert np.isclose(sg.mean_wo_outliers(x), np.mean(x[:5]))
