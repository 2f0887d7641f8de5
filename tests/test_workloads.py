"""Host-side inputs of the benchmark workloads, checked on CPU: the per-trait individual sets of
the multi-trait workload, the windows of the gradient workload and the synthetic generator's
multi-trait option (whose single-trait random stream must stay that of the other workloads)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import bench  # noqa: E402
from slemm_gb300 import synth  # noqa: E402


def test_trait_individual_sets():
    cfg = dict(bench.CONFIGS[5], n=20000)
    keeps, frac = bench.trait_keeps(cfg)
    assert len(keeps) == cfg["traits"] == len(frac)
    assert frac[0] == pytest.approx(cfg["miss_lo"]) and frac[-1] == pytest.approx(cfg["miss_hi"])
    for k, f in zip(keeps, frac):
        assert k.dtype == np.int64
        assert k.size == cfg["n"] - int(round(f * cfg["n"]))
        assert np.all(np.diff(k) > 0)                 # sorted, no repeats
        assert k[0] >= 0 and k[-1] < cfg["n"]
    again, _ = bench.trait_keeps(cfg)                 # seeded: every run analyses the same sets
    assert all(np.array_equal(a, b) for a, b in zip(keeps, again))


def test_gradient_windows():
    cfg = bench.CONFIGS[4]
    window, wwin = bench.grad_inputs(cfg)
    assert window.shape == (cfg["m"],) and window.dtype == np.int32
    assert window.min() == 0 and window.max() == cfg["grad_windows"] - 1
    assert np.all(np.diff(window) >= 0)
    assert np.all(np.bincount(window) == cfg["m"] // cfg["grad_windows"])   # 50 SNPs each
    assert wwin.shape == (cfg["grad_windows"],)
    assert np.all(wwin > 0) and np.all(wwin <= 2)


@pytest.mark.parametrize("kw", [dict(), dict(missing=0.02), dict(ld_rho=0.6, ld_block=25)])
def test_generator_traits_option(kw):
    torch = pytest.importorskip("torch")
    rows1, y1 = synth.simulate_bed_torch(600, 140, seed=5, device="cpu", chunk=64, **kw)
    rowsT, yT = synth.simulate_bed_torch(600, 140, seed=5, device="cpu", chunk=64, n_traits=3,
                                         rows_device=True, **kw)
    assert y1.shape == (600,) and yT.shape == (600, 3)
    assert isinstance(rowsT, torch.Tensor) and rowsT.shape == rows1.shape
    # each trait has its own causal SNPs: the phenotypes are far from collinear
    c = np.corrcoef(yT.T)
    assert np.all(np.abs(c[np.triu_indices(3, 1)]) < 0.5)
    # the .bed rows decode to valid codes only (no 01 unless missing calls were asked for)
    codes = np.unpackbits(rowsT.numpy()[:, :, None], axis=2, bitorder="little").reshape(140, -1, 2)
    codes = codes[:, :600]
    if not kw.get("missing"):
        assert not np.any((codes[..., 0] == 1) & (codes[..., 1] == 0))


def test_generator_single_trait_stream_is_stable():
    """n_traits = 1 is the default call: the same draws in the same order, so the single-trait
    workloads keep their genotypes and phenotypes."""
    pytest.importorskip("torch")
    rows, y = synth.simulate_bed_torch(300, 90, seed=3, device="cpu", chunk=32)
    rows2, y2 = synth.simulate_bed_torch(300, 90, seed=3, device="cpu", chunk=32, n_traits=1)
    assert np.array_equal(rows.numpy(), rows2.numpy()) and np.array_equal(y, y2)


def test_roofline_object_arithmetic():
    """The bench's roofline object for one packed-product launch shape: algorithmic FLOPs per
    launch over the measured launch time, against the measured BF16 peak (and the hi+lo ceiling,
    half of it), and the per-launch DRAM traffic scaled from the committed ncu summary."""
    n, m = 100000, 50000
    prof = [{"tc": 1, "N": 144, "k": 66, "pieces": 2, "dir": 2, "splits": 3, "plan": 0, "launches": 10, "ms": 7.2},
            {"tc": 1, "N": 16, "k": 1, "pieces": 2, "dir": 1, "splits": 5, "plan": 0, "launches": 1, "ms": 0.58}]
    roof, gbs = bench.roofline(prof, n, m, "fp16x2")
    pk = bench.peaks()
    t = 7.2e-3 / 10
    flops = 2.0 * n * m * 66
    assert roof["bound"] == "tensor" and roof["unit"] == "TFLOP/s"
    assert roof["achieved"] == pytest.approx(flops / t / 1e12)
    assert roof["peak"] == pytest.approx(pk["bf16"])
    assert roof["frac"] == pytest.approx(roof["achieved"] / pk["bf16"])
    assert roof["frac_eff"] == pytest.approx(2 * roof["frac"])
    assert roof["executed_tflops"] == pytest.approx(2.0 * n * m * 144 / t / 1e12)
    assert gbs == pytest.approx(m * ((n + 3) // 4) / t / 1e9)
    # traffic: the committed capture's reads scaled by the packed bytes, its writes by the
    # split-K partial bytes of this launch (3 splits x kp 72 x M_pad 100,096 x 4 B)
    import json
    with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
        c = json.load(f)["fp16x2_tc1_N144_dir2"]
    want = c["read"] * (m * 25000) / c["packed"] + c["write"] * (3 * 72 * 100096 * 4) / c["partials"]
    assert roof["traffic"] == pytest.approx(want)
    assert bench.roofline(prof, n, m, "bf16x2")[0]["traffic"] is None   # no capture of that kernel
    assert bench.roofline([], n, m, "fp16x2") == (None, None)


def test_reference_arm_application_model():
    """The reference arm's whole-fit model: every Lanczos step of a seed runs the reference's whole
    subset loop on that seed's block (src/reml.cpp:293-322); the window-weighted workload adds the
    MC-REML first stage.  Seconds = Σ count·(m/1000)·(a + passes·b·k)."""
    cfg = bench.CONFIGS[3]
    st = bench.REF_STEPS[3]
    apps = bench.reference_applications(cfg, st)
    by = {w: (p, k, c) for w, p, k, c in apps}
    assert by["DF-REML L_Seed ldet V"] == (2, cfg["probes"], st["iters_V"])
    assert by["DF-REML L_Seed quadform y"] == (2, 1, st["iters_y"])
    assert by["MC-REML L_Seed quadform [y|Zu|e]"] == (2, 1 + 2 * st["n_mc"], st["first_iters_V"])
    a, b = 0.07, 0.001
    want = sum(c * (cfg["m"] / 1000) * (a + p * b * k) for _, p, k, c in apps)
    assert bench.reference_seconds(a, b, cfg["m"], apps) == pytest.approx(want)
    # DF-REML alone for the workload without windows
    assert all(not w.startswith("MC-REML") for w, *_ in bench.reference_applications(bench.CONFIGS[2],
                                                                                      bench.REF_STEPS[2]))
    # the counts a GPU fit reports map onto the same model
    res = {"iters": [287, 2, 331], "fixed": [], "first_stage": {"iters_V": 15, "n_criterion": 4}}
    st2 = bench.fit_counts(cfg, res)
    assert st2 == dict(iters_y=287, iters_Q=2, iters_V=331, c=1, first_iters_V=15, first_n_criterion=4,
                       n_mc=bench.mc_samples(cfg["n"]))


def test_both_arms_print_the_same_config():
    """The GPU and reference arms share one config object per workload (their arithmetic is each
    line's own precision key), and the L2 note states the packed bytes each pass streams."""
    cfg = bench.CONFIGS[3]
    c = bench.gpu_config(cfg)
    assert c == bench.gpu_config(dict(cfg))
    assert "precision" not in c and c["n"] == 500000 and c["m"] == 60000
    assert "7.50 GB packed" in c["l2"]
