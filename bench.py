"""Benchmark of the GB300 engine on SLEMM's REML + SNP-BLUP path.

Default workload (the metric's own configuration): n = 500,000 individuals, m = 60,000 SNPs in a
packed PLINK .bed with block LD (AR(1) latent correlation 0.6 within 50-SNP blocks, thresholded to
0/1/2), h² = 0.3, one trait, intercept only; `slemm --reml --lrt --iter_weighting
--window_size 50` with 64 Rademacher probes: an MC-REML equal-weight stage, window weights from
its SNP-BLUP (1,200 windows), fixed-effect SNPs by clumping, then the window-weighted DF-REML
(Lanczos seeds for y, Q and the probe block, golden-section search on h²), BLUP and BLUE.
Synthetic data, seed 1.  `--config N` selects the other workloads (see CONFIGS).

One step = one whole fit through the C ABI.
  value  — device-timed (CUDA events on the library stream) wall time of one fit with the
           packed genotypes already resident in HBM (each packed pass streams Z from HBM: the
           packed matrix is far larger than the 129 MB L2);
  e2e    — the same fit through the reference-facing calls with HOST buffers: genotype upload
           from pinned staging + fit + results back to the host, timed on the host;
  fp32_* — the plain FP32 GPU path (CUDA-core FP32 products, per vector by default) on the same
           fit: its time (the speed-up) and its h² (dh2_vs_fp32, the metric's precision bar);
  roofline — the dominant packed-product kernel, measured per launch with CUDA events during
           the timed steps;
  cpu_baseline — the reference's operator loop restated on this host's cores (threaded C
           decode of each 1000-SNP subset + OpenBLAS SGEMMs) timed at full n on a bounded sample
           of subsets, times this fit's operator applications.
  integer_stages — decode, popcounts and class counts: the GPU pack from rows in HBM vs the C
           restatement on this host's cores (bounded sample, scaled).
`--impl reference` times that CPU loop on the same workload on this host's cores, with the step
counts of the FP32 GPU fit (REF_STEPS).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "REML wall time + genotype-matvec GB/s, mixed-prec vs FP32 on GB300 at dh2<=1e-4"
CONFIGS = {
    1: dict(n=2000, m=10000, probes=30, h2=0.5, missing=0.01,
            name="n=2000 m=10000, 1% missing, 30 Rademacher probes, DF-REML + BLUP"),
    2: dict(n=100000, m=50000, probes=64, h2=0.4, missing=0.0,
            name="n=100000 m=50000, 64 Rademacher probes in one block, DF-REML + BLUP"),
    3: dict(n=500000, m=60000, probes=64, h2=0.3, missing=0.0, ld_rho=0.6, ld_block=50, window=50,
            name="n=500000 m=60000, block LD (AR(1) latent rho=0.6 in 50-SNP blocks), --iter_weighting "
                 "with 1,200 windows of 50 SNPs, 64 Rademacher probes, DF-REML + BLUP"),
    4: dict(n=200000, m=100000, probes=64, h2=0.4, missing=0.0, grad_windows=2000, sigma_g2=0.4, sigma_e2=0.6,
            name="n=200000 m=100000, REML log-likelihood gradient for (sigma_g2, sigma_e2) and 2,000 per-window "
                 "SNP weights in (0, 2] (windows of 50 SNPs), 64 Rademacher probes"),
    5: dict(n=1000000, m=50000, probes=64, h2=0.4, missing=0.0, traits=16, miss_lo=0.05, miss_hi=0.40,
            gwas_m=200000,
            name="n=1000000 m=50000, 16 traits with 5-40% of individuals missing per trait (the .bed rows held "
                 "in HBM packed once per step, each trait a view of its individuals over the shared packed copies), "
                 "DF-REML + BLUP with 64 probes each; GWAS score terms over a 1000000 x 200000 .bed for the first "
                 "trait's individuals"),
}


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return dict(hbm=float(p["hbm_gbs"]), bf16=float(p["bf16_tflops"]),
                    bf16_sus=float(p["bf16_tflops_sustained"]), src="measured")
    except Exception:
        return dict(hbm=6800.0, bf16=1900.0, bf16_sus=1700.0, src="fallback")


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append((time.perf_counter(), line.strip()))

    def window(self, t0, t1):
        """Keeps the lines read between host times t0 and t1 (plus one sampling period)."""
        self.lines = [x for x in self.lines if t0 <= x[0] <= t1 + 0.25]

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for _, ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = max(mx, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


class NvmlSampler:
    """SM clock, power and clock-event reasons read through NVML (libnvidia-ml, ctypes) every
    10 ms while running: the timed fits last ~0.1 s, too short for nvidia-smi's 200 ms loop."""
    BITS = {"sw_power_cap": 0x4, "hw_slowdown": 0x8 | 0x80, "sw_thermal_slowdown": 0x20,
            "hw_thermal_slowdown": 0x40}

    def __init__(self, cuda_index=0, interval=None):
        if interval is None:
            interval = float(os.environ.get("SLEMM_BENCH_NVML_MS", "10")) / 1000.0
        self.cuda_index, self.interval = cuda_index, interval
        self.samples, self.max_mhz, self.ok = [], 0.0, False
        self._stop = threading.Event()

    def _handle(self, nv):
        import ctypes
        h = ctypes.c_void_p()
        try:
            import torch
            pr = torch.cuda.get_device_properties(self.cuda_index)
            bus = "%08X:%02X:%02X.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
            if nv.nvmlDeviceGetHandleByPciBusId_v2(bus.encode(), ctypes.byref(h)) == 0:
                return h
        except Exception:
            pass
        vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
        idx = self.cuda_index
        if vis:
            try:
                idx = int(vis.split(",")[self.cuda_index])
            except ValueError:
                return None
        return h if nv.nvmlDeviceGetHandleByIndex_v2(idx, ctypes.byref(h)) == 0 else None

    def __enter__(self):
        import ctypes
        if self.interval <= 0:
            return self
        try:
            nv = ctypes.CDLL("libnvidia-ml.so.1")
            if nv.nvmlInit_v2() != 0:
                return self
            h = self._handle(nv)
            if h is None:
                return self
            mx = ctypes.c_uint()
            if nv.nvmlDeviceGetMaxClockInfo(h, 1, ctypes.byref(mx)) == 0:   # NVML_CLOCK_SM
                self.max_mhz = float(mx.value)
            reasons_fn = getattr(nv, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
                nv.nvmlDeviceGetCurrentClocksThrottleReasons
            self.nv, self.h, self.reasons_fn, self.ok = nv, h, reasons_fn, True
            self.t = threading.Thread(target=self._loop, daemon=True)
            self.t.start()
        except Exception:
            self.ok = False
        return self

    def _loop(self):
        import ctypes
        clk, rs, pw = ctypes.c_uint(), ctypes.c_ulonglong(), ctypes.c_uint()
        while not self._stop.is_set():
            if self.nv.nvmlDeviceGetClockInfo(self.h, 1, ctypes.byref(clk)) == 0 and \
                    self.reasons_fn(self.h, ctypes.byref(rs)) == 0:
                p = pw.value / 1000.0 if self.nv.nvmlDeviceGetPowerUsage(self.h, ctypes.byref(pw)) == 0 else None
                self.samples.append((float(clk.value), int(rs.value), p, time.perf_counter()))
            time.sleep(self.interval)

    def __exit__(self, *a):
        self._stop.set()
        if self.ok:
            self.t.join(timeout=2)

    def window(self, t0, t1):
        """Keeps the samples taken between host times t0 and t1 (the timed fits): the sampler is
        started before the warm-up so that NVML's own start-up does not fall into the timed steps."""
        self.samples = [x for x in self.samples if t0 <= x[3] <= t1]

    def summary(self):
        if not self.samples:
            return None
        reasons = sorted(k for k, b in self.BITS.items() if any(x[1] & b for x in self.samples))
        pw = [x[2] for x in self.samples if x[2] is not None]
        return {"sm_mhz": statistics.median(x[0] for x in self.samples), "sm_max_mhz": self.max_mhz,
                "reasons": reasons, "samples": len(self.samples), "power_w_median": statistics.median(pw) if pw else None,
                "source": f"NVML every {self.interval * 1e3:.0f} ms during the timed fits"}


def max_over_ranks(x, dist=None, device="cuda"):
    """The largest of the ranks' values (every rank gets it): replicas run side by side, so a
    step lasts as long as the slowest rank's.  x is None on no rank or on all of them."""
    if dist is None or x is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def pinned_copy(rows):
    """The .bed rows as a NumPy view of page-locked host memory (copied once, outside any timed
    region): the end-to-end steps upload a step's inputs from pinned host memory."""
    import torch
    t = rows if isinstance(rows, torch.Tensor) else torch.from_numpy(rows)
    return t.pin_memory().numpy()


def make_inputs(cfg, device="cuda"):
    from slemm_gb300 import synth
    rows, y = synth.simulate_bed_torch(cfg["n"], cfg["m"], seed=1, h2=cfg["h2"], missing=cfg["missing"],
                                       device=device, ld_rho=cfg.get("ld_rho", 0.0),
                                       ld_block=cfg.get("ld_block", 50))
    n, m = cfg["n"], cfg["m"]
    X = np.ones((n, 1), np.float32)
    persnp = np.ones(m, np.float32)
    return rows, y.astype(np.float32), X, persnp


# ------------------------------------------------------------------------------------------------
# CPU path (oracle port): the reference's subset loop timed at full n, one cost model for both the
# reference arm and the GPU arm's cpu_baseline
# ------------------------------------------------------------------------------------------------
SUBSET = 1000   # the reference's SNP subset size (--subset_size default, src/option.cpp:53-78)

# Lanczos step counts and criterion evaluations of the plain FP32 path (CUDA-core FP32 products,
# the reference's arithmetic) on each workload, as the GPU arm's `fp32_*.counts` reports them: the
# reference arm multiplies its measured per-application times by these.
REF_STEPS = {
    2: dict(iters_y=14, iters_Q=1, iters_V=14, c=1,
            source="FP32 per-vector GPU fit of the n=100000 m=50000 workload (fp32_per_vector.counts)"),
    3: dict(iters_y=297, iters_Q=2, iters_V=303, c=1, first_iters_V=15, first_n_criterion=4, n_mc=3,
            source="FP32 per-vector GPU fit of the n=500000 m=60000 window-weighted workload (fp32_per_vector.counts)"),
}


def cpu_app_model(rows_np, n, probes, subsets, start=0, threads=None):
    """Per-subset cost of the reference's operator loop (src/reml.cpp:28-47: decode 1000 SNPs of
    kmat into a centred FP32 block, then SGEMMs) at full n, measured on `subsets` consecutive
    subsets of 1000 packed .bed rows from subset `start`: H0_ldet_mv on 1 + probes columns and
    H0_quadform_mv on one column, fitted as t = a + passes·b·k per subset (a: the decode, b: SGEMM
    time per column and pass).  Returns (a, b, measured seconds, description)."""
    from oracle import slemm_np as orc
    threads = threads or os.cpu_count() or 1
    nsub = max(1, rows_np.shape[0] // SUBSET)
    subsets = max(1, min(subsets, nsub))
    s0 = start % (nsub - subsets + 1)
    rows_s = rows_np[s0 * SUBSET:(s0 + subsets) * SUBSET]   # a view: consecutive rows
    rng = np.random.default_rng(0)
    ms = rows_s.shape[0]
    gm = rng.uniform(0.1, 0.9, ms).astype(np.float32)        # values do not change the timing
    w = np.full(ms, 1.0 / ms, np.float32)
    Q = np.full((n, 1), 1.0 / np.sqrt(n), np.float32)
    ops = orc.PackedOperators(rows_s, n, gm, w, None, Q, subset_size=SUBSET, dtype=np.float32, threads=threads)
    V = rng.standard_normal((n, 1 + probes)).astype(np.float32)
    t0 = time.perf_counter()
    ops.H0_ldet_mv(0.4285714, V)
    t_wide = time.perf_counter() - t0
    t0 = time.perf_counter()
    ops.H0_quadform_mv(0.4285714, V[:, :1].copy())
    t_one = time.perf_counter() - t0
    b = max((t_wide - t_one) / subsets / (2.0 * probes), 0.0)
    a = max(t_one / subsets - 2.0 * b, 0.0)
    info = (f"subsets {s0}..{s0 + subsets - 1} of {SUBSET} SNPs x {n} individuals on {threads} threads: H0_ldet_mv "
            f"on {1 + probes} columns {t_wide:.2f} s, H0_quadform_mv on 1 column {t_one:.2f} s; per subset "
            f"a={a:.4f} s (decode) + passes*k*{b:.6f} s (SGEMM)")
    return a, b, t_wide + t_one, info


def mc_samples(n):
    """MC samples of an MC-REML first stage: max(min(4e9/n², 30), 3) (src/option.cpp:445)."""
    return max(min(int(4e9 / n / n), 30), 3)


def reference_applications(cfg, st):
    """(what, passes, columns, count) of the operator applications the reference's algorithm makes
    in one fit of the workload, from the step counts `st`: each Lanczos step of a seed applies its
    operator to the seed's block (src/reml.cpp:293-322) and each application runs the whole subset
    loop (quadform and ldet: decode once, two SGEMMs; matvec and rmatvec: one)."""
    probes, c = cfg["probes"], st["c"]
    apps = []
    if cfg.get("window"):   # --iter_weighting, n ≥ 5000: MC-REML first stage (src/option.cpp:437-470)
        k = st["n_mc"]
        apps += [("MC-REML matvec of the MC draws", 1, k, 1),
                 ("MC-REML L_Seed quadform [y|Zu|e]", 2, 1 + 2 * k, st["first_iters_V"]),
                 ("MC-REML first-order rmatvec", 1, 1 + k, st["first_n_criterion"]),
                 ("MC-REML SNP-BLUP + BLUE", 1, 1, 2)]
    apps += [("DF-REML L_Seed quadform y", 2, 1, st["iters_y"]),
             ("DF-REML L_Seed ldet Q", 2, c, st["iters_Q"]),
             ("DF-REML L_Seed ldet V", 2, probes, st["iters_V"]),
             ("DF-REML SNP-BLUP + BLUE", 1, 1, 2)]
    return apps


def reference_seconds(a, b, m, apps):
    """Whole-fit seconds of the reference's loop: Σ count · (m/1000) · (a + passes·b·k)."""
    return sum(cnt * (m / SUBSET) * (a + p * b * k) for _, p, k, cnt in apps)


def fit_counts(cfg, res):
    """Step counts of a GPU fit in the form reference_applications takes."""
    st = dict(iters_y=int(res["iters"][0]), iters_Q=int(res["iters"][1]), iters_V=int(res["iters"][2]),
              c=1 + len(res.get("fixed", [])))
    if cfg.get("window"):
        st.update(first_iters_V=int(res["first_stage"]["iters_V"]),
                  first_n_criterion=int(res["first_stage"]["n_criterion"]), n_mc=mc_samples(cfg["n"]))
    return st


def cpu_operator_sample(rows_np, n, m, probes, subsets=4):
    """Seconds of one full-m H0_ldet_mv on 1 + probes columns and one H0_quadform_mv on a column,
    from cpu_app_model on `subsets` subsets.  Returns (s_ldet, s_quad, info)."""
    a, b, _, info = cpu_app_model(rows_np, n, probes, subsets)
    return (m / SUBSET) * (a + 2 * b * (1 + probes)), (m / SUBSET) * (a + 2 * b), info


def cpu_integer_sample(rows_np, n, m, threads, rows_max=4000):
    """The integer stages (src/input.cpp:343-386 decode, src/reml.cpp:613-621 popcounts,
    src/input.cpp:10-22 class counts) through the oracle's C restatement, on `rows_max` SNP rows
    split over `threads` host threads (ctypes releases the GIL), scaled to all m rows."""
    from concurrent.futures import ThreadPoolExecutor
    from oracle import slemm_np as orc
    rows_s = np.ascontiguousarray(rows_np[:min(m, rows_max)])
    parts = [c for c in np.array_split(np.arange(rows_s.shape[0]), threads) if c.size]

    def work(ix):
        dec = orc.bed_decode(rows_s[ix[0]:ix[-1] + 1], n)
        orc.popcounts(dec)
        orc.hwe_counts(dec)

    with ThreadPoolExecutor(len(parts)) as ex:
        t0 = time.perf_counter()
        list(ex.map(work, parts))
        dt = time.perf_counter() - t0
    return dt * m / rows_s.shape[0], f"{rows_s.shape[0]} SNP rows × {n} individuals on {len(parts)} threads, scaled ×{m / rows_s.shape[0]:.1f}"


def cpu_threads():
    return os.cpu_count() or 1


def l2_note(n, m):
    """How the timed passes relate to the 129 MB L2: every packed pass streams Z from HBM."""
    return (f"inputs larger than L2: each packed pass streams Z ({m * ((n + 3) // 4) / 1e9:.2f} GB packed) "
            f"from HBM, 129 MB L2")


def gpu_config(cfg):
    """The `config` object both arms print for the workload (the arithmetic each arm runs in is
    its line's own `precision` key)."""
    n, m = cfg["n"], cfg["m"]
    out = {"workload": cfg["name"], "n": n, "m": m, "probes": cfg["probes"], "h2_sim": cfg["h2"]}
    if cfg.get("window"):
        out.update(ld_rho=cfg["ld_rho"], ld_block=cfg["ld_block"], window_size=cfg["window"])
    out.update(l2=l2_note(n, m), parallelism="replicas")
    return out


def run_reference(args, cfg):
    """CPU reference arm: the oracle port of the reference's operator loop (threaded C decode of
    each 1000-SNP subset + OpenBLAS SGEMMs, the structure of src/reml.cpp:28-47) timed at full n on
    this host's cores.  Each timed step measures the loop on a block of consecutive subsets (the
    blocks rotate over the whole .bed across the steps) and turns it into the whole fit's seconds
    with the workload's application counts (reference_applications, REF_STEPS)."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    n, m, probes = cfg["n"], cfg["m"], cfg["probes"]
    st = REF_STEPS.get(args.config)
    if st is None:
        print(json.dumps({"impl": "reference", "unavailable": "no FP32 step counts recorded for this workload"}),
              flush=True)
        return
    apps = reference_applications(cfg, st)
    rng = np.random.default_rng(1)
    rows_np = rng.integers(0, 256, size=(m, (n + 3) // 4), dtype=np.uint8)   # timing only
    nsub = m // SUBSET
    spent = 1.0
    for _ in range(args.warmup):   # warm-up: one subset
        _, _, spent, _ = cpu_app_model(rows_np, n, probes, 1)
    # size each timed step so that the K steps take about args.ref_budget seconds of CPU work
    S = int(max(1, min(nsub, args.ref_budget / max(args.steps, 1) / max(spent, 1e-3))))
    vals, walls, infos = [], [], []
    for s in range(args.steps):
        t0 = time.perf_counter()
        a, b, _, info = cpu_app_model(rows_np, n, probes, S, start=s * S)
        walls.append(time.perf_counter() - t0)
        vals.append(reference_seconds(a, b, m, apps))
        infos.append(info)
    value = statistics.mean(vals)
    covered = min(nsub, S * args.steps)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": statistics.mean(walls) * 1e3,
        "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (random packed bytes of the workload's shape: the loop's time does not depend on the values)",
        "config": gpu_config(cfg), "precision": "FP32 (the reference's float arithmetic)",
        "steps_are": f"each timed step runs the reference's full-n subset loop on {S} of the {nsub} subsets "
                     f"({covered} subsets covered over the {args.steps} steps) and converts it to one whole fit; "
                     f"ms_per_step is that step's measured wall time",
        "applications": [{"what": w, "passes": p, "columns": k, "count": c} for w, p, k, c in apps],
        "step_counts": st,
        "cpu_baseline": {"value": value, "unit": "s", "cores": cpu_threads(), "kind": "port",
                         "sample": infos[-1] + "; whole fit = sum over the applications of count*(m/1000)*(a+passes*b*k)"},
        "e2e": {"value": value, "unit": "s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------------------------------------------
# GPU arm
# ------------------------------------------------------------------------------------------------
PRECISIONS = {
    "fp16x2": ("FP16 hi+lo pieces of each dense column scaled by a power of two (integer hi piece, exact FP32 "
               "accumulation of count*hi), tcgen05 MMA with FP32 accumulation, FP64 Lanczos scalars"),
    "bf16x2": "BF16 hi+lo products, FP32 accumulation, FP64 Lanczos scalars",
    "bf16x3": "BF16 hi+mid+lo products, FP32 accumulation, FP64 Lanczos scalars",
    "fp32": "CUDA-core FP32 products on exact integer counts, FP64 Lanczos scalars",
}


def prec_code(name):
    from slemm_gb300 import _lib
    return {"fp16x2": _lib.PREC_FP16X2, "bf16x2": _lib.PREC_BF16X2, "bf16x3": _lib.PREC_BF16X3,
            "fp32": _lib.PREC_FP32}[name]


def run_gpu(args, cfg):
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from slemm_gb300 import api, _lib
    api.init(local)
    n, m, probes = cfg["n"], cfg["m"], cfg["probes"]
    rows, y, X, persnp = make_inputs(cfg)
    rows_np = rows.numpy()
    opts = dict(seed=0, n_V=probes)
    prec = prec_code(args.prec)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    window = cfg.get("window")

    def fit(gh):
        """One REML + BLUP through the reference-facing calls: DF-REML, or for the windowed
        workload `--iter_weighting` (MAF from the handle, MC-REML equal-weight stage, window
        weights, window-weighted DF-REML)."""
        if window:
            maf = gh.marker_qc()[0]
            return gh.REML_iter_weighting(None, X, y, persnp, maf, lrt=True, window_size=window, **opts)
        return gh.SLDF_REML(None, X, y, persnp, **opts)

    g = api.Genotypes(rows_np, n)
    stream = torch.cuda.ExternalStream(g.stream())
    g.set_precision(prec)
    g.set_autotune(not args.no_autotune)   # shapes are tuned during the warm-up fits
    # clock samplers start before the warm-up (their start-up stays out of the timed steps) and
    # keep only the samples of the timed window
    nvml = NvmlSampler(local).__enter__()
    clocks = ClockSampler(local).__enter__()
    for _ in range(args.warmup):
        fit(g)
    # ---- timed: REML + BLUP with genotypes resident ----
    launches0 = api.launch_count()
    _prof(g, 1)
    times, res = [], None
    barrier()
    t_timed0 = time.perf_counter()
    for _ in range(args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        res = fit(g)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    barrier()
    t_timed1 = time.perf_counter()
    time.sleep(0.25)   # the nvidia-smi line of the last period
    for smp in (nvml, clocks):
        smp.__exit__(None, None, None)
        smp.window(t_timed0, t_timed1)
    launches = api.launch_count() - launches0
    prof = _prof(g, 0)
    mean_step = max_over_ranks(statistics.mean(times), dist)
    # ---- e2e: host buffers through the reference-facing calls (the first call grows the pool) ----
    e2e_times = []
    rows_pinned = pinned_copy(rows) if not args.skip_e2e else None   # the user's .bed rows in pinned host memory
    for _ in range(0 if args.skip_e2e else args.e2e_steps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with api.Genotypes(rows_pinned, n) as g2:
            g2.set_precision(prec)
            g2.set_autotune(not args.no_autotune)
            fit(g2)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    e2e = statistics.mean(e2e_times[1:]) if len(e2e_times) > 1 else None
    e2e = max_over_ranks(e2e, dist)
    h2d = rows_np.nbytes + y.nbytes + X.nbytes + persnp.nbytes
    d2h = (n + m + 1 + 1) * 4 + (4 * m if window else 0)
    # ---- plain FP32 GPU path (the comparison the metric names), one fit ----
    fp32 = None
    if args.fp32 != "skip":
        g.set_precision(_lib.PREC_FP32)
        g.set_per_vector(args.fp32 == "per_vector")
        _prof(g, 1)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rf = fit(g)
        torch.cuda.synchronize()
        t_fp32 = time.perf_counter() - t0
        pf = _prof(g, 0)
        packed = m * ((n + 3) // 4)
        one = [s_ for s_ in pf if s_["k"] == 1]
        passes = sum(s_["launches"] for s_ in one)
        avg = sum(s_["ms"] for s_ in one) / max(passes, 1) / 1e3
        fp32 = {"mode": args.fp32, "s": t_fp32, "h2": rf["h2"], "iters": list(rf["iters"]),
                "counts": fit_counts(cfg, rf),
                "k1_pass": {"launches": passes, "avg_ms": avg * 1e3,
                            "packed_gbs": packed / avg / 1e9 if passes else None,
                            "frac_hbm": packed / avg / 1e9 / peaks()["hbm"] if passes else None}}
        g.set_per_vector(False)
        g.set_precision(prec)
    # ---- the opt-in reorthogonalised Lanczos on the same fit (one fit, outside the timed steps) ----
    reorth = None
    if not args.skip_reorth:
        g.set_lanczos(reorth=True)
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        rr_ = fit(g)
        e1.record(stream)
        e1.synchronize()
        g.set_lanczos(reorth=False)
        reorth = {"s": e0.elapsed_time(e1) / 1e3, "h2": rr_["h2"], "iters": list(rr_["iters"]),
                  "counts": fit_counts(cfg, rr_), "dh2_vs_plain": abs(rr_["h2"] - res["h2"])}
        if fp32:
            reorth["dh2_vs_fp32"] = abs(rr_["h2"] - fp32["h2"])
    # ---- roofline of the dominant packed-product launch shape ----
    roof, matvec_gbs = roofline(prof, n, m, args.prec, sustained=min(times) > 1.0)
    # ---- CPU baseline (oracle port, this fit's step counts), rank 0, N = 1 only ----
    cpu = None
    counts = fit_counts(cfg, res)
    if rank == 0 and world == 1 and not args.skip_cpu:
        a, b, spent, info = cpu_app_model(rows_np, n, probes, args.cpu_subsets)
        apps = reference_applications(cfg, counts)
        cpu = {"value": reference_seconds(a, b, m, apps), "unit": "s", "cores": cpu_threads(), "kind": "port",
               "sample": f"{info} ({spent:.1f} s of CPU work); whole fit = sum over the reference's operator "
                         f"applications (this fit's Lanczos steps) of count*(m/1000)*(a+passes*b*k)",
               "applications": [{"what": w, "passes": p, "columns": k, "count": c} for w, p, k, c in apps]}
    # ---- integer stages (decode, popcounts, class counts): GPU pack from HBM vs the C oracle ----
    integer = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        rows_dev = torch.from_numpy(rows_np).to("cuda")
        tg = []
        for _ in range(3):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            with api.Genotypes(rows_dev, n) as g3:
                g3.counts()
            torch.cuda.synchronize()
            tg.append(time.perf_counter() - t0)
        del rows_dev
        thr = os.cpu_count() or 1
        s_int, info_int = cpu_integer_sample(rows_np, n, m, thr)
        integer = {"gpu_s": min(tg), "cpu_s": s_int, "cores": thr, "kind": "port",
                   "gpu": "genotype_create from .bed rows already in HBM (both tiled copies and the "
                          "per-SNP class counts) + counts to the host",
                   "cpu_sample": info_int}
    line = {
        "metric": METRIC, "value": mean_step, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mean_step * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": args.prec,
        "data": "synthetic (seeded, generated on the GPU)",
        "config": gpu_config(cfg), "precision": PRECISIONS[args.prec],
        "h2": res["h2"], "vg": res["vg"], "ve": res["ve"], "lrt": res["lrt"],
        "lanczos_steps": {"y": res["iters"][0], "Q": res["iters"][1], "V": res["iters"][2]},
        "counts": counts,
        "phases_s": res.get("phases"),
        "step_ms": [round(t * 1e3, 3) for t in times],
        "matvec_gbs": matvec_gbs,
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "step_ms": [round(t * 1e3, 3) for t in e2e_times],
                "note": "host .bed rows (pinned) uploaded and packed + fit + results to the host, timed on the host; "
                        "mean of the steps after the first (the first grows the device memory pool)"},
        "gpu_launches": int(launches),
        "gpu_launches_per_step": int(launches / max(args.steps, 1)),
        "roofline": roof,
        "autotune": None if args.no_autotune else api.autotune_table(),
        "cpu_baseline": cpu,
        "integer_stages": integer,
        "clocks": nvml.summary() or clocks.summary(),
        "clocks_nvidia_smi": clocks.summary(),
    }
    if window:
        line["fixed_snps"] = len(res.get("fixed", []))
    if reorth:
        line["reorthogonalised"] = reorth
    if fp32:
        line["fp32_" + args.fp32] = fp32
        line["speedup_vs_fp32_" + args.fp32] = fp32["s"] / mean_step
        line["dh2_vs_fp32"] = abs(fp32["h2"] - res["h2"])
    g.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def roofline(prof, n, m, prec, sustained=False):
    """Roofline object of the dominant packed-product launch shape (most device time in the
    timed region) and the packed bytes per second it streamed.  sustained: the launches run
    inside a fit of seconds, so the measured sustained BF16 figure is the peak (else the burst)."""
    pk = peaks()
    dom = max(prof, key=lambda r: r["ms"]) if prof else None
    if not dom:
        return None, None
    k = dom["k"]
    t_launch = dom["ms"] / dom["launches"] / 1e3
    packed = m * ((n + 3) // 4)
    bytes_alg = packed + 4 * n * k + 4 * m * k
    flops_alg = 2.0 * n * m * k
    ach_tf = flops_alg / t_launch / 1e12
    exe_tf = 2.0 * n * m * dom["N"] / t_launch / 1e12 if dom["tc"] else ach_tf
    gbs = bytes_alg / t_launch / 1e9
    # wide tensor-core shapes are tensor-bound; the narrow shape (N = 16, one to seven columns) is
    # bound by its count decode and reported against HBM, like the CUDA-core kernel
    tensor = dom["tc"] == 1 and dom["N"] > 16
    tc_peak = pk["bf16_sus"] if sustained else pk["bf16"]
    roof = {
        "bound": "tensor" if tensor else "hbm",
        "achieved": ach_tf if tensor else gbs,
        "peak": tc_peak if tensor else pk["hbm"],
        "unit": "TFLOP/s" if tensor else "GB/s",
        "frac": (ach_tf / tc_peak) if tensor else gbs / pk["hbm"],
        "peak_source": (("measured " + ("sustained" if sustained else "burst") + " cuBLAS BF16 (MEASURED_PEAKS.json)")
                        if tensor else "measured HBM copy (MEASURED_PEAKS.json)") if pk["src"] == "measured"
        else "fallback",
        # a split into P 16-bit pieces executes P products per algorithmic one, so the algorithmic
        # ceiling of this kernel is the 16-bit peak over P
        "tc_peak_eff": tc_peak / dom["pieces"] if dom["tc"] else None,
        "frac_eff": ach_tf / (tc_peak / dom["pieces"]) if dom["tc"] else None,
        "traffic": _traffic(dom, n, m, prec),
        "kernel": "gemm_tc_kernel" if dom["tc"] else "gemm_simt_kernel",
        "launch": {"N": dom["N"], "k": k, "pieces": dom["pieces"],
                   "direction": "Z^T U (M=SNPs)" if dom["dir"] == 1 else "Z V (M=individuals)",
                   "avg_ms": t_launch * 1e3, "launches": dom["launches"],
                   "algorithmic_flops": flops_alg, "algorithmic_bytes": bytes_alg},
        "executed_tflops": exe_tf, "frac_executed": exe_tf / tc_peak,
        "algorithmic_gbs": gbs, "frac_hbm": gbs / pk["hbm"],
        "shapes": prof,
    }
    return roof, packed / t_launch / 1e9


def grad_inputs(cfg):
    """Window index per SNP (consecutive windows of m / K SNPs) and K weights in (0, 2]."""
    m, K = cfg["m"], cfg["grad_windows"]
    window = np.minimum(np.arange(m) // (m // K), K - 1).astype(np.int32)
    wwin = (2.0 - np.random.default_rng(7).uniform(0.0, 2.0, K)).astype(np.float32)
    return window, wwin


def run_grad(args, cfg):
    """Gradient workload: one step = ∂ℓ/∂(σ_g², σ_e², w_1..w_K) of the REML log-likelihood through
    the reference-facing call (projected Lanczos seed/solve of [ỹ | probes], one packed product
    Z̃ᵀ[P_Hỹ | P_HV | V], per-window reductions)."""
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from slemm_gb300 import api, _lib
    api.init(local)
    n, m, probes = cfg["n"], cfg["m"], cfg["probes"]
    rows, y, X, persnp = make_inputs(cfg)
    rows_np = rows.numpy()
    window, wwin = grad_inputs(cfg)
    sg2, se2 = cfg["sigma_g2"], cfg["sigma_e2"]

    def step(gh):
        return gh.REML_grad(None, X, y, persnp, window, wwin, sg2, se2, n_V=probes, seed=0, tol=1e-6)

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    g = api.Genotypes(rows_np, n)
    stream = torch.cuda.ExternalStream(g.stream())
    g.set_precision(prec_code(args.prec))
    nvml = NvmlSampler(local).__enter__()
    clocks = ClockSampler(local).__enter__()
    for _ in range(args.warmup):
        r = step(g)
    launches0 = api.launch_count()
    _prof(g, 1)
    times = []
    barrier()
    t_timed0 = time.perf_counter()
    for _ in range(args.steps):
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        r = step(g)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1) / 1e3)
    barrier()
    t_timed1 = time.perf_counter()
    time.sleep(0.25)
    for smp in (nvml, clocks):
        smp.__exit__(None, None, None)
        smp.window(t_timed0, t_timed1)
    launches = api.launch_count() - launches0
    prof = _prof(g, 0)
    mean_step = max_over_ranks(statistics.mean(times), dist)
    e2e_times = []
    rows_pinned = pinned_copy(rows) if not args.skip_e2e else None   # the user's .bed rows in pinned host memory
    for _ in range(0 if args.skip_e2e else max(5, args.steps)):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with api.Genotypes(rows_pinned, n) as g2:
            g2.set_precision(prec_code(args.prec))
            step(g2)
        torch.cuda.synchronize()
        e2e_times.append(time.perf_counter() - t0)
    e2e = (statistics.mean(e2e_times[1:]) if len(e2e_times) > 1 else e2e_times[0]) if e2e_times else None
    e2e = max_over_ranks(e2e, dist)
    h2d = rows_np.nbytes + y.nbytes + X.nbytes + persnp.nbytes + window.nbytes + wwin.nbytes
    d2h = 8 * (2 + wwin.size)
    # the same gradient with FP32 products throughout the Lanczos solves
    fp32 = None
    if args.fp32 != "skip":
        g.set_precision(_lib.PREC_FP32)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rf = step(g)
        torch.cuda.synchronize()
        dw = np.max(np.abs(rf["d_w"] - r["d_w"])) / np.max(np.abs(rf["d_w"]))
        fp32 = {"s": time.perf_counter() - t0,
                "rel_diff": {"d_sigma_g2": abs(rf["d_sigma_g2"] - r["d_sigma_g2"]) / abs(rf["d_sigma_g2"]),
                             "d_sigma_e2": abs(rf["d_sigma_e2"] - r["d_sigma_e2"]) / abs(rf["d_sigma_e2"]),
                             "d_w_max_over_max": float(dw)}}
        g.set_precision(prec_code(args.prec))
    roof, matvec_gbs = roofline(prof, n, m, args.prec)
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        s_ldet, _, info = cpu_operator_sample(rows_np, n, m, probes, subsets=args.cpu_subsets)
        t = 1 + probes
        # Lanczos steps: Zᵀ passes of the solve block, each weighted by its width against 1 + probes;
        # the closing Z̃ᵀ[P_Hỹ | P_HV | V] pass counts as one more block application
        # (the closing pass is the one at hi+mid+lo)
        zt = [s for s in prof if s["dir"] == 1 and s["pieces"] != 3]
        eq = sum(s["launches"] * s["k"] / t for s in zt) / max(args.steps, 1) + 1.0
        cpu = {"value": eq * s_ldet, "unit": "s", "cores": cpu_threads(), "kind": "port",
               "sample": f"{info}; gradient time = {eq:.1f} block applications of H0_ldet_mv on "
                         f"{t} columns (this run's Lanczos steps + the closing Z^T pass)"}
    h = {"d_sigma_g2": r["d_sigma_g2"], "d_sigma_e2": r["d_sigma_e2"],
         "d_w_head": [float(v) for v in r["d_w"][:4]],
         "homogeneity_residual": abs(sg2 * r["d_sigma_g2"] - float(np.dot(wwin.astype(np.float64), r["d_w"])))
                                 / abs(sg2 * r["d_sigma_g2"])}
    line = {
        "metric": "REML log-likelihood gradient wall time", "value": mean_step, "unit": "s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": mean_step * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": args.prec,
        "data": "synthetic (seeded, generated on the GPU)",
        "config": {"workload": cfg["name"], "n": n, "m": m, "probes": probes, "windows": int(wwin.size),
                   "sigma_g2": sg2, "sigma_e2": se2, "l2": l2_note(n, m), "parallelism": "replicas"},
        "precision": PRECISIONS[args.prec] + " in the Lanczos solves; column-scaled FP16 hi+lo in "
                     "the closing Z^T pass; FP64 reductions",
        "gradient": h,
        "step_ms": [round(t * 1e3, 3) for t in times],
        "matvec_gbs": matvec_gbs,
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "step_ms": [round(t * 1e3, 3) for t in e2e_times],
                "median_s": statistics.median(e2e_times[1:]) if len(e2e_times) > 1 else None,
                "note": "mean of the steps after the first (the first grows the device memory pool)"},
        "gpu_launches": int(launches),
        "gpu_launches_per_step": int(launches / max(args.steps, 1)),
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": nvml.summary() or clocks.summary(),
        "clocks_nvidia_smi": clocks.summary(),
    }
    if fp32:
        line["fp32"] = fp32
    g.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def trait_keeps(cfg):
    """Per trait the kept individuals (sorted .fam indices): trait t misses a fraction of the
    individuals that runs evenly from miss_lo to miss_hi over the traits, drawn at random."""
    n, T = cfg["n"], cfg["traits"]
    rng = np.random.default_rng(11)
    frac = np.linspace(cfg["miss_lo"], cfg["miss_hi"], T)
    return [np.sort(rng.choice(n, size=n - int(round(f * n)), replace=False)).astype(np.int64) for f in frac], frac


def _mem_available_gb():
    try:
        with open("/proc/meminfo") as f:
            for ln in f:
                if ln.startswith("MemAvailable:"):
                    return int(ln.split()[1]) / 1e6
    except OSError:
        pass
    return 0.0


def run_multi(args, cfg):
    """Multi-trait workload: one step = DF-REML + BLUP for every trait on its own individuals —
    the .bed rows held in HBM packed once (both tiled copies), every trait a view of its
    individuals over those copies (its own counts, frequencies, centring and fit, as the reference
    analyses each trait on its own individual set) — then the GWAS score terms of the first trait
    over a 10⁶-row, 2·10⁵-SNP .bed (resident handle of that trait's individuals)."""
    import torch
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from slemm_gb300 import api, _lib, synth
    api.init(local)
    n, m, probes, T, m2 = cfg["n"], cfg["m"], cfg["probes"], cfg["traits"], cfg["gwas_m"]
    rows_dev, Y = synth.simulate_bed_torch(n, m, seed=1, h2=cfg["h2"], n_traits=T, rows_device=True)
    Y = Y.astype(np.float32)
    keeps, frac = trait_keeps(cfg)
    persnp = np.ones(m, np.float32)
    Xs = [np.ones((k.size, 1), np.float32) for k in keeps]
    ys = [np.ascontiguousarray(Y[k, t]) for t, k in enumerate(keeps)]
    # GWAS .bed: rows generated in HBM, packed for trait 0's individuals, rows then released
    grows, _ = synth.simulate_bed_torch(n, m2, seed=7, h2=cfg["h2"], rows_device=True)
    torch.cuda.empty_cache()   # the generator's temporaries
    gw = api.Genotypes(grows, n, keep_idx=keeps[0])
    keep_gw_host = None
    if not args.skip_e2e and _mem_available_gb() > 2.0 * (grows.numel() + rows_dev.numel()) / 1e9:
        keep_gw_host = grows.cpu().pin_memory().numpy()   # pinned host copy for the end-to-end leg
    del grows
    torch.cuda.empty_cache()
    n0 = keeps[0].size
    Q0 = np.full((n0, 1), 1.0 / np.sqrt(n0), np.float32)
    ones0 = np.ones(n0, np.float32)
    zeros2 = np.zeros(m2, np.float32)

    def gwas(gh, Py):
        gh.set_weights(zeros2, zeros2, ones0)
        gh.set_projection(Q0)
        return gh.score_terms(Py, mac=20)

    def step(rows, gwas_handle=None, gwas_rows=None):
        """One pack of the .bed rows for all individuals, then every trait's fit on a view of it."""
        res = []
        with api.Genotypes(rows, n) as parent:
            for t in range(T):
                with api.Genotypes.view(parent, keeps[t]) as gt:
                    gt.set_precision(prec_code(args.prec))
                    gt.set_autotune(not args.no_autotune)
                    res.append(gt.SLDF_REML(None, Xs[t], ys[t], persnp, seed=0, n_V=probes))
        if gwas_handle is not None:
            sc = gwas(gwas_handle, res[0]["Py"])
        else:
            with api.Genotypes(gwas_rows, n, keep_idx=keeps[0]) as g2:
                sc = gwas(g2, res[0]["Py"])
        return res, sc

    def barrier():
        torch.cuda.synchronize()
        if dist is not None:
            dist.barrier()

    nvml = NvmlSampler(local).__enter__()
    clocks = ClockSampler(local).__enter__()
    for _ in range(args.warmup):
        step(rows_dev, gw)
    launches0 = api.launch_count()
    times = []
    barrier()
    t_timed0 = time.perf_counter()
    for _ in range(args.steps):
        # the per-trait handles run on their own streams: time on the host around a device sync
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        res, sc = step(rows_dev, gw)
        torch.cuda.synchronize()
        times.append(time.perf_counter() - t0)
    barrier()
    t_timed1 = time.perf_counter()
    time.sleep(0.25)
    for smp in (nvml, clocks):
        smp.__exit__(None, None, None)
        smp.window(t_timed0, t_timed1)
    launches = api.launch_count() - launches0
    mean_step = max_over_ranks(statistics.mean(times), dist)
    # per-phase split of one step: trait handles (pack), fits, GWAS score pass
    # (the first trait's fit also gives the packed-product launch shapes for the roofline)
    ph = {"pack_s": 0.0, "views_s": 0.0, "fit_s": 0.0}
    prof = None
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    parent = api.Genotypes(rows_dev, n)
    torch.cuda.synchronize()
    ph["pack_s"] = time.perf_counter() - t0
    for t in range(T):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gt = api.Genotypes.view(parent, keeps[t])
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        gt.set_precision(prec_code(args.prec))
        gt.set_autotune(not args.no_autotune)
        if t == 0:
            _prof(gt, 1)
        gt.SLDF_REML(None, Xs[t], ys[t], persnp, seed=0, n_V=probes)
        torch.cuda.synchronize()
        if t == 0:
            prof = _prof(gt, 0)
        ph["views_s"] += t1 - t0
        ph["fit_s"] += time.perf_counter() - t1
        gt.close()
    parent.close()
    roof, matvec_gbs = roofline(prof, int(keeps[0].size), m, args.prec, sustained=mean_step > 1.0)
    t0 = time.perf_counter()
    gwas(gw, res[0]["Py"])
    torch.cuda.synchronize()
    ph["gwas_score_s"] = time.perf_counter() - t0
    # ---- e2e: .bed rows from host memory through the reference-facing calls ----
    e2e, e2e_times, h2d, e2e_note = None, [], 0, None
    if not args.skip_e2e:
        rows_host = rows_dev.cpu().pin_memory()
        for _ in range(2):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            # the .bed rows cross the link once, through genotype_create's upload pipeline
            if keep_gw_host is not None:
                step(rows_host.numpy(), gwas_rows=keep_gw_host)
            else:
                step(rows_host.numpy(), gw)
            torch.cuda.synchronize()
            e2e_times.append(time.perf_counter() - t0)
        e2e = max_over_ranks(statistics.mean(e2e_times), dist)
        h2d = rows_host.numel() + sum(y.nbytes + x.nbytes for y, x in zip(ys, Xs)) + T * persnp.nbytes
        if keep_gw_host is not None:
            h2d += keep_gw_host.nbytes
            e2e_note = ("the REML .bed rows uploaded from pinned host memory once per step, packed once in HBM, every trait "
                        "a view of its individuals; the GWAS .bed uploaded from host memory through genotype_create")
        else:
            e2e_note = ("the REML .bed rows uploaded from pinned host memory once per step, packed once in HBM, every trait "
                        "a view of its individuals; the GWAS handle stays resident (too little free host memory "
                        "for a host copy of its 50 GB of rows)")
        del rows_host
    d2h = sum((k.size + m + 1 + 1) * 4 for k in keeps) + 2 * 4 * m2
    # plain FP32 per-vector fit of the first trait (the comparison the metric names)
    fp32 = None
    if args.fp32 != "skip":
        with api.Genotypes(rows_dev, n, keep_idx=keeps[0]) as gt:
            gt.set_precision(_lib.PREC_FP32)
            gt.set_per_vector(True)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            rf = gt.SLDF_REML(None, Xs[0], ys[0], persnp, seed=0, n_V=probes)
            torch.cuda.synchronize()
            fp32 = {"trait": 0, "s": time.perf_counter() - t0, "h2": rf["h2"], "dh2": abs(rf["h2"] - res[0]["h2"])}
    # CPU baseline: the oracle's operators on a bounded SNP sample at full n, scaled per trait
    cpu = None
    if rank == 0 and world == 1 and not args.skip_cpu:
        rows_s = rows_dev[:4000].cpu().numpy()
        s_ldet, s_quad, info = cpu_operator_sample(rows_s, n, 4000, probes, subsets=max(1, args.cpu_subsets - 1))
        s_ldet *= m / 4000
        s_quad *= m / 4000
        est = 0.0
        for r, k in zip(res, keeps):
            it_y, it_q, it_v = r["iters"]
            est += (max(it_q, it_v) * s_ldet + it_y * s_quad) * k.size / n
        from oracle import slemm_np as orc
        sel = np.arange(0, m2, m2 // 64)[:64]
        mask = np.zeros(n, np.uint8)
        mask[keeps[0]] = 1
        t0 = time.perf_counter()
        grows_s = keep_gw_host[sel] if keep_gw_host is not None else None
        if grows_s is not None:
            dec = orc.bed_decode(grows_s, n, mask)
            orc.gamma_terms(dec, res[0]["Py"], ones0, Q0.astype(np.float64), 20)
            s_gw = (time.perf_counter() - t0) * m2 / sel.size
            est += s_gw
            info += f"; GWAS score terms: {sel.size} SNPs decoded and scored by the oracle, scaled ×{m2 / sel.size:.0f}"
        cpu = {"value": est, "unit": "s", "cores": cpu_threads(), "kind": "port",
               "sample": f"{info} (4000 SNP rows of the REML .bed); per trait Lanczos steps × t(ldet, 65 cols) "
                         f"+ steps × t(quadform), scaled by the trait's share of individuals"}
    line = {
        "metric": METRIC, "value": mean_step, "unit": "s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": mean_step * 1e3, "higher_is_better": False,
        "scaling": "weak", "vs_baseline": None, "dtype": args.prec,
        "data": "synthetic (seeded, generated on the GPU)",
        "config": {"workload": cfg["name"], "n": n, "m": m, "probes": probes, "traits": T,
                   "missing_fraction": [round(float(f), 4) for f in frac], "gwas_m": m2,
                   "l2": l2_note(n, m), "parallelism": "replicas",
                   "timing": "host clock around a device synchronisation (each trait handle has its own stream)"},
        "precision": PRECISIONS[args.prec] + "; GWAS score pass at column-scaled FP16 hi+lo",
        "per_trait": [{"n": int(k.size), "h2": r["h2"], "iters": list(r["iters"])} for r, k in zip(res, keeps)],
        "phases_s": ph,
        "gwas": {"tested": int(np.isfinite(sc[0]).sum())},
        "step_ms": [round(t * 1e3, 3) for t in times],
        "e2e": {"value": e2e, "unit": "s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "step_ms": [round(t * 1e3, 3) for t in e2e_times], "note": e2e_note},
        "gpu_launches": int(launches),
        "gpu_launches_per_step": int(launches / max(args.steps, 1)),
        "roofline": roof,
        "matvec_gbs_trait0": matvec_gbs,
        "cpu_baseline": cpu,
        "clocks": nvml.summary() or clocks.summary(),
        "clocks_nvidia_smi": clocks.summary(),
    }
    if fp32:
        line["fp32_per_vector_trait0"] = fp32
    gw.close()
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist is not None:
        dist.destroy_process_group()


def _prof(g, enable):
    import ctypes
    from slemm_gb300 import _lib
    lib = _lib.load()
    rows = ctypes.c_int(0)
    info = (ctypes.c_int32 * (7 * 64))()
    la = (ctypes.c_int64 * 64)()
    ms = (ctypes.c_double * 64)()
    _lib.check(lib.slemm_gpu_profile(g.h, enable, 64, ctypes.byref(rows), info, la, ms))
    out = []
    for r in range(min(rows.value, 64)):
        out.append({"tc": info[7 * r], "N": info[7 * r + 1], "k": info[7 * r + 2],
                    "pieces": info[7 * r + 3], "dir": info[7 * r + 4], "splits": info[7 * r + 5],
                    "plan": info[7 * r + 6], "launches": int(la[r]), "ms": float(ms[r])})
    return out


def _traffic(dom, n, m, prec):
    """DRAM bytes per launch of the dominant kernel from the committed ncu summary (captured on a
    small case, n = 40,000, m = 20,000), carried to this launch: the reads (packed matrix once plus
    the dense operand) grow with the packed bytes, the writes with the split-K partial bytes
    (splits x kp x M_pad x 4, kp = k rounded up to 8, M_pad = m or n rounded up to 256)."""
    p = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(p) as f:
            t = json.load(f)
        c = t.get(f"{prec}_tc{dom['tc']}_N{dom['N']}_dir{dom['dir']}")
        if c is None or not dom.get("splits"):
            return None
        M_pad = -(-(m if dom["dir"] == 1 else n) // 256) * 256
        partials = dom["splits"] * (-(-dom["k"] // 8) * 8) * M_pad * 4
        packed = m * ((n + 3) // 4)
        return c["read"] * packed / c["packed"] + c["write"] * partials / c["partials"]
    except (OSError, ValueError, KeyError):
        return None


def run_kernel_case(args):
    """Small profiling case for ncu: n = 40,000, m = 20,000 (each packed copy 200 MB, above the
    129 MB L2), H0_ldet_mv on a block of --kernel-k columns (65: the wide kernel at N = 144;
    1: the narrow one at N = 16): 3 warm-up applications, then 2 timed (each is one Zᵀ and one Z
    pass, i.e. 2 gemm_tc_kernel launches)."""
    import torch
    from slemm_gb300 import api, _lib, synth
    torch.cuda.set_device(0)
    api.init(0)
    n, m, k = 40000, 20000, args.kernel_k
    rows, _ = synth.simulate_bed_torch(n, m, seed=3)
    rows_np = rows.numpy()
    g = api.Genotypes(rows_np, n)
    gm = np.full(m, 0.55, np.float32)
    w = np.full(m, 1.0 / m, np.float32)
    g.set_weights(gm, w)
    g.set_precision(prec_code(args.prec))
    v = torch.randn(k, n, device="cuda")
    out = torch.empty(k, n, device="cuda")
    for _ in range(3):
        g.op_device(_lib.OP_LDET, v, out, 0.4285714)
    stream = torch.cuda.ExternalStream(g.stream())
    _prof(g, 1)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(2):
        g.op_device(_lib.OP_LDET, v, out, 0.4285714)
    e1.record(stream)
    e1.synchronize()
    prof = _prof(g, 0)
    print(json.dumps({"case": "kernel", "n": n, "m": m, "k": k, "op_ms": e0.elapsed_time(e1) / 2,
                      "shapes": prof}), flush=True)
    g.close()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--kernel-case", action="store_true", help="small operator case for ncu captures")
    ap.add_argument("--kernel-k", type=int, default=65, help="columns of the kernel case's block")
    ap.add_argument("--skip-e2e", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=2, help="end-to-end fits timed after one pool-growing fit")
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=3, choices=sorted(CONFIGS))
    ap.add_argument("--prec", default="fp16x2", choices=sorted(PRECISIONS),
                    help="product precision of the timed fits (and of the kernel case)")
    ap.add_argument("--fp32", default="per_vector", choices=["per_vector", "batched", "skip"],
                    help="the plain FP32 GPU fit the metric compares with")
    ap.add_argument("--skip-fp32", action="store_true", help="same as --fp32 skip")
    ap.add_argument("--no-autotune", action="store_true",
                    help="fixed split-K rule instead of the autotuner's timed choice")
    ap.add_argument("--skip-reorth", action="store_true",
                    help="leave out the one reorthogonalised fit reported beside the timed ones")
    ap.add_argument("--skip-cpu", action="store_true")
    ap.add_argument("--cpu-subsets", type=int, default=4)
    ap.add_argument("--ref-budget", type=float, default=120.0,
                    help="seconds of CPU work the reference arm's timed steps aim at in total")
    args = ap.parse_args()
    if args.skip_fp32:
        args.fp32 = "skip"
    cfg = CONFIGS[args.config]
    if args.kernel_case:
        from slemm_gb300 import build
        build.build()
        run_kernel_case(args)
        return
    if args.impl == "reference":
        if cfg.get("grad_windows"):
            if int(os.environ.get("RANK", "0")) == 0:
                print(json.dumps({"impl": "reference", "unavailable": "the reference computes no REML gradient; "
                                  "the gb300 line's cpu_baseline times the same operator work on the host"}),
                      flush=True)
            return
        run_reference(args, cfg)
    else:
        from slemm_gb300 import build
        build.build()
        (run_grad if cfg.get("grad_windows") else run_multi if cfg.get("traits") else run_gpu)(args, cfg)


if __name__ == "__main__":
    main()
