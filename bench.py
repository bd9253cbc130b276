"""Benchmark: batched lnL + gradient of 1024 MBHB samples on one GB300.

Workload (the adjoint configuration): one LISA-like heliocentric detector
(L = 2.5e9 m, trailing 20 deg), first-generation ("1.5") TDI A/E/T,
T = 2^22 s, dt = 8 s, dense grid 1e-4..0.03 Hz (125 410 bins x 3 channels),
data = IMRPhenomD injection (m1 = 1e6, m2 = 5e5 Msun, chi = 0.5/-0.3,
10 Gpc, ...) + seeded noise; 1024 prior samples (seed 2026 + rank) with the
per-sample cutoff 1.2 f_RD; lnL and its gradient w.r.t. the 11 parameters
(ln Mc, q, chi1, chi2, ln D_L, cos i, lambda, sin beta, psi, phi_c, t_c).

One step = one call of the batched lnL+gradient over the 1024 samples.
`value` times steps with inputs resident in HBM (CUDA events around each
step; the L2 is flushed between steps by writing a 512 MB buffer outside the
timed events); `e2e` times the same call through the public API with the
parameters copied from pinned host memory and lnL/gradient copied back.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--precision mixed|fp64]
    python bench.py --impl reference   # the reference's CPU path (oracle port)
    python bench.py --workload ref-shape   # the reference's published benchmark shape
    python bench.py --workload td-tdi      # time-domain TDI combination (own metric)
    python bench.py --workload network-hm  # the higher-mode network configuration alone

The default run also times the higher-mode network configuration (IMRPhenomHM,
LISA + Taiji + TianQin, T = 2^25 s, 4096 samples, lnL through one CUDA graph)
and reports it under "network_hm" (N = 1 only; --no-network-hm skips it).

Multi-GPU (torchrun): replicas; every rank evaluates its own 1024 samples
(weak scaling); rank 0 prints the line with the max-over-ranks step time.
"""

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# (T, dt, f_min, f_max, TDI generation, description)
WORKLOADS = {
    "adjoint": (2.0 ** 22, 8.0, 1e-4, 0.03, "1.5",
                "adjoint: 1024-sample prior batch, LISA TDI1.5 AET, T=2^22 s, dt=8 s, 125410 bins, cutoff 1.2 f_RD"),
    # the shape of the reference's own published timings (65 471 bins x 3, TDI 2.0),
    # with IMRPhenomD in place of the reference's IMRPhenomXAS
    "ref-shape": (655360.0, 5.0, 1e-4, 0.1, "2.0",
                  "ref-shape: 1024-sample prior batch, LISA TDI2.0 AET, T=655360 s, dt=5 s, 65471 bins, "
                  "cutoff 1.2 f_RD, IMRPhenomD"),
    # the network geometry of the higher-mode configuration with the (2,2)-mode IMRPhenomD
    "network-d": (2.0 ** 25, 4.0, 3e-5, 0.1, "1.5",
                  "network-d: prior batch, LISA + Taiji + TianQin TDI1.5 AET, T=2^25 s, dt=4 s, 3354437 bins "
                  "per channel (9 channels), 2048 sparse nodes, cutoff 1.2 f_RD, IMRPhenomD (2,2)"),
    # the higher-mode configuration: IMRPhenomHM on the three-detector network, lnL only,
    # 4096 samples through one CUDA graph
    "network-hm": (2.0 ** 25, 4.0, 3e-5, 0.1, "1.5",
                   "network-hm: 4096-sample prior batch, IMRPhenomHM (6 modes), LISA + Taiji + TianQin TDI1.5 AET, "
                   "T=2^25 s, dt=4 s, 3354437 bins per channel (9 channels), 2048 sparse nodes per mode, "
                   "cutoff 1.2 f_RD of the highest mode, mixed precision, CUDA graph"),
    # SMC-style sweep: half IMRPhenomD particles on LISA (lnL, gradient, Fisher), half
    # IMRPhenomHM particles on the three-detector network (lnL)
    "smc-sweep": (2.0 ** 22, 8.0, 1e-4, 0.03, "1.5",
                  "smc-sweep: 16384 particles, 8192 IMRPhenomD on LISA (T=2^22 s, 125410 bins; lnL, gradient and "
                  "11x11 Fisher) + 8192 IMRPhenomHM on LISA + Taiji + TianQin (T=2^25 s, 3354437 bins; lnL), mixed"),
    # time-domain TDI combination of six single-link series (no likelihood): its own metric
    "td-tdi": (2.0 ** 25, 4.0, None, None, "2.0",
               "td-tdi: LISA TDI2.0 AET from six single-link time series, T=2^25 s, dt=4 s, 8388609 samples"),
}
N_SPARSE = {"network-d": 2048, "network-hm": 2048}
HM_METRIC = "lnL evals/s, 4096 MBHB samples, IMRPhenomHM 3-detector network, 1 GB300 (mixed, CUDA graph)"
SMC_METRIC = "particles/s, 16384-particle sweep (8192 IMRPhenomD lnL+grad+Fisher, 8192 IMRPhenomHM lnL), 1 GB300"
TD_METRIC = "TD TDI output samples/s (A/E/T from six single-link series), 1 GB300"
LISA_ARM_M = 2.5e9
C_SI = 299792458.0
DUR, DT, FMIN, FMAX, GEN, WORKLOAD = WORKLOADS["adjoint"]
BATCH = 1024
METRIC = "lnL+grad evals/s, 1024 MBHB samples, 1 GB300: mixed vs FP64, |dlnL|<=1e-2"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="native", choices=["native", "reference"])
    ap.add_argument("--precision", default=os.environ.get("PES_BENCH_PRECISION", "mixed"),
                    choices=["mixed", "fp64"])
    ap.add_argument("--batch", type=int, default=BATCH)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-network-hm", action="store_true", help="skip the higher-mode network leg")
    ap.add_argument("--workload", default="adjoint", choices=sorted(WORKLOADS))
    ap.add_argument("--n-sparse", type=int, default=None, help="sparse nodes of the mixed plan (default per workload)")
    args = ap.parse_args()
    global DUR, DT, FMIN, FMAX, GEN, WORKLOAD
    DUR, DT, FMIN, FMAX, GEN, WORKLOAD = WORKLOADS[args.workload]
    return args


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("WORLD_SIZE", 1)), int(os.environ.get("LOCAL_RANK", 0))


class ClockSampler:
    """nvidia-smi clocks/throttle reasons sampled every 200 ms while running."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.idx = device_index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.idx}", f"--query-gpu={self.QUERY}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except FileNotFoundError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
            except (ValueError, IndexError):
                continue
            for n, v in zip(names, r[5:9]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f)
    return None


def gemm_peak_tflops(torch, dtype):
    """Pipe throughput denominator: cuBLAS GEMM 8192^3 in `dtype` (best of 5; TF32 off for FP32)."""
    tf32 = torch.backends.cuda.matmul.allow_tf32
    torch.backends.cuda.matmul.allow_tf32 = False
    a = torch.randn(8192, 8192, dtype=dtype, device="cuda")
    b = torch.randn(8192, 8192, dtype=dtype, device="cuda")
    for _ in range(2):
        torch.matmul(a, b)
    torch.cuda.synchronize()
    best = math.inf
    for _ in range(5):
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        torch.matmul(a, b)
        e.record()
        e.synchronize()
        best = min(best, s.elapsed_time(e) / 1e3)
    del a, b
    torch.backends.cuda.matmul.allow_tf32 = tf32
    return 2 * 8192 ** 3 / best / 1e12


def stratified(B, n):
    """Indices of n samples spread evenly over a batch of B (the CPU arms' subsets)."""
    return np.unique(np.linspace(0, B - 1, max(1, min(n, B))).round().astype(int))


def workload_config(B, world):
    """The `config` of both arms' lines: the workload and its sizes."""
    g_nbins = int(np.count_nonzero((np.fft.rfftfreq(int(DUR // DT + 1), DT) >= FMIN) *
                                   (np.fft.rfftfreq(int(DUR // DT + 1), DT) <= FMAX)))
    return {"workload": WORKLOAD, "global_batch": B * world, "per_gpu_batch": B, "nbins": g_nbins}


def td_config():
    """The `config` of both arms' time-domain TDI lines."""
    arm = LISA_ARM_M / C_SI
    n = int(DUR // DT + 1)
    return {"workload": WORKLOAD, "samples": n, "link_samples": n + int(7 * arm // DT + 1), "batch": 1,
            "generation": GEN}


def cpu_baseline_run(n_samples, threads, precision_note, grad=True, batch=None):
    """The reference's CPU path (oracle port, FP64 dense, OpenMP over samples) on
    n_samples of the GPU arm's seeded batch of `batch` samples, spread evenly
    over it (rank 0's batch)."""
    from oracle import fdpath as oracle
    from pespace_gb300.replicas import rank_theta
    from pespace_gb300.workloads import config0_theta

    oracle.build()
    g = oracle.grid(DUR, DT, FMIN, FMAX)
    th0 = config0_theta(DUR - 86400.0)
    # the workload's detectors: LISA, or LISA + Taiji + TianQin for the network
    # workloads (seeded noise per detector); IMRPhenomHM for network-hm
    approx = "IMRPhenomHM" if WORKLOAD.startswith("network-hm") else "IMRPhenomD"
    specs = [(oracle.heliocentric(2.5e9, 0.0, -math.pi / 9), "LISA_SciRDv1")]
    if WORKLOAD.startswith("network"):
        specs += [(oracle.heliocentric(3.0e9, 0.0, math.pi / 9), "Taiji_TDC"),
                  (oracle.geocentric(math.sqrt(3.0) * 1e8), "Tianqin_GWSpace")]
    dets = []
    for k, (orb, model) in enumerate(specs):
        psd = oracle.psd(g["freqs"], "AET", False, GEN, **oracle.PSD_PRESETS[model])
        noise = oracle.noise_realization(g, psd, "AET", 2026 + k)
        dets.append((orb, GEN, np.stack([noise[c] for c in "AET"]), np.stack([psd[c] for c in "AET"])))
    plan = oracle.Plan(g, dets, 1e-4, cut_factor=1.2, approximant=approx)
    dets = [(orb, gen, data + plan.model_tdi(k, th0), psd_arr) for k, (orb, gen, data, psd_arr) in enumerate(dets)]
    plan = oracle.Plan(g, dets, 1e-4, cut_factor=1.2, approximant=approx)
    batch = BATCH if batch is None else batch
    if approx == "IMRPhenomHM":  # the GPU leg's batch (its own seed)
        from pespace_gb300.workloads import prior_samples

        thetas = prior_samples(np.random.default_rng(2027), batch, th0[10])[stratified(batch, n_samples)]
    else:
        thetas = rank_theta(0, batch, th0[10])[stratified(batch, n_samples)]
    t0 = time.perf_counter()
    plan.lnl(thetas, grad=grad, nthreads=threads)
    dt = time.perf_counter() - t0
    return len(thetas) / dt, dt


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    if args.workload == "td-tdi":
        arm = LISA_ARM_M / C_SI
        rates = []
        for _ in range(args.warmup):
            td_cpu_baseline(arm, 0.5)
        for _ in range(args.steps):
            rates.append(td_cpu_baseline(arm, 1.0)[0])
        v = float(np.mean(rates))
        line = {"impl": "reference", "metric": TD_METRIC, "value": v, "unit": "samples/s", "n_gpus": 0,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * (1 << 20) / v,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
                "data": "synthetic", "config": td_config(),
                "cpu_baseline": {"value": v, "unit": "samples/s", "cores": 1, "kind": "port",
                                 "sample": "2^20-sample blocks for 1 s per step (numpy); taichi absent on this host"},
                "e2e": {"value": v, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    threads = os.cpu_count() or 1
    B = args.batch
    if args.workload == "smc-sweep":
        print(json.dumps({"impl": "reference", "unavailable": "a 16384-particle sweep with Fisher matrices is hours "
                          "of the CPU port; its halves are timed by --workload adjoint and --workload network-hm"}),
              flush=True)
        return
    if args.workload == "network-hm":
        # lnL only (as the GPU leg), a few samples of its 4096 spread over the batch:
        # each is about a minute of FP64 work per core over 3 x 3.35 M bins x 6 modes
        B, n = 4096, max(2, threads // 4)
        rates = []
        for _ in range(args.warmup):
            cpu_baseline_run(n, threads, "", grad=False, batch=B)
        for _ in range(args.steps):
            rates.append(cpu_baseline_run(n, threads, "", grad=False, batch=B)[0])
        v = float(np.mean(rates))
        line = {"impl": "reference", "metric": HM_METRIC, "value": v, "unit": "lnL evals/s", "n_gpus": 0,
                "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n / v, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
                "config": {"workload": WORKLOAD, "batch": B},
                "cpu_baseline": {"value": v, "unit": "lnL evals/s", "cores": threads, "kind": "port",
                                 "sample": f"{n} of the {B} seeded samples per step (evenly spread over the batch), "
                                           "full grid, FP64 dense IMRPhenomHM, OpenMP over samples"},
                "e2e": {"value": v, "unit": "lnL evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line), flush=True)
        return
    # a bounded sample of the GPU arm's seeded batch, spread evenly over it:
    # 64 of the 1024 samples (every 16th); network-d (three detectors, 3.35 M
    # bins each, about 9 s of FP64 work per sample and core) a quarter of the cores
    n = max(4, threads // 4) if WORKLOAD.startswith("network-d") else 64
    n = len(stratified(B, n))
    rates = []
    for _ in range(args.warmup):
        cpu_baseline_run(n, threads, "", batch=B)
    for _ in range(args.steps):
        r, _ = cpu_baseline_run(n, threads, "", batch=B)
        rates.append(r)
    v = float(np.mean(rates))
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": "lnL+grad evals/s", "n_gpus": 0,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * n / v, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": workload_config(B, world),
        "cpu_baseline": {"value": v, "unit": "lnL+grad evals/s", "cores": threads, "kind": "port",
                         "sample": f"{n} of the {B} seeded samples per step (evenly spread over the batch), "
                                   "full grid, FP64 dense with forward-mode gradient, OpenMP over samples; "
                                   "taichi/jax absent on this host"},
        "e2e": {"value": v, "unit": "lnL+grad evals/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def td_cpu_baseline(arm, budget_s=10.0):
    """Oracle (numpy, one core) on 2^20-sample blocks of the TD TDI workload until budget_s elapses."""
    from oracle import td_tdi

    n = 1 << 20
    added = td_tdi.layout(arm, DT, GEN)[0]
    links = np.random.default_rng(2026).standard_normal((6, n + added))
    done, t0 = 0, time.perf_counter()
    while time.perf_counter() - t0 < budget_s:
        td_tdi.combine(links, n, arm, DT, GEN, True)
        done += n
    dt = time.perf_counter() - t0
    return done / dt, done, dt


def run_td_tdi(args):
    """One step = one pes_td_tdi_combination call over the whole series (HBM-bound)."""
    import torch

    from pespace_gb300 import _lib, replicas

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    arm = LISA_ARM_M / C_SI
    n = int(DUR // DT + 1)
    added = int(7 * arm // DT + 1)
    n_ext, B = n + added, 1
    gen = torch.Generator(device="cuda").manual_seed(2026 + rank)
    links = torch.randn((B, 6, n_ext), dtype=torch.float64, device="cuda", generator=gen)
    out = torch.empty((B, 3, n), dtype=torch.float64, device="cuda")
    lib = _lib.load()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def call(x, y):
        _lib.check(lib.pes_td_tdi_combination(_lib.ptr(x), B, n_ext, n, arm, DT, 20, 1, _lib.ptr(y),
                                              _lib.stream_handle()))

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    for _ in range(max(3, args.warmup)):
        call(links, out)
    clocks = ClockSampler(local)
    ev = []
    with clocks:
        barrier()
        for _ in range(args.steps):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            call(links, out)
            e.record()
            ev.append((s, e))
        barrier()
    mean_ms = replicas.reduce_max(float(np.mean([s.elapsed_time(e) for s, e in ev])), "cuda")
    value = world * B * n / (mean_ms / 1e3)
    alg_bytes = B * (6 * n_ext + 3 * n) * 8

    # the float-float entry point on the same series, against the exact result
    out_ff = torch.empty_like(out)

    def call_ff(x, y):
        _lib.check(lib.pes_td_tdi_combination_mixed(_lib.ptr(x), B, n_ext, n, arm, DT, 20, 1, _lib.ptr(y),
                                                    _lib.stream_handle()))

    for _ in range(max(3, args.warmup)):
        call_ff(links, out_ff)
    ev_ff = []
    barrier()
    for _ in range(args.steps):
        flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        call_ff(links, out_ff)
        e.record()
        ev_ff.append((s, e))
    barrier()
    ff_ms = replicas.reduce_max(float(np.mean([s.elapsed_time(e) for s, e in ev_ff])), "cuda")
    ff_err = float(((out_ff - out).abs().max() / links.abs().max()).item())

    # e2e: links from pinned host memory, channels back to pinned host memory
    links_host = links.cpu().pin_memory()
    out_host = torch.empty((B, 3, n), dtype=torch.float64).pin_memory()
    links_dev = torch.empty_like(links)
    e2e = []
    barrier()
    for _ in range(args.steps):
        flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        links_dev.copy_(links_host, non_blocking=True)
        call(links_dev, out)
        out_host.copy_(out, non_blocking=True)
        e.record()
        e.synchronize()
        e2e.append(s.elapsed_time(e))
    e2e_ms = replicas.reduce_max(float(np.mean(e2e)), "cuda")
    if rank != 0:
        return
    from pespace_gb300 import census

    peaks = measured_peaks() or {}
    hbm_peak = peaks.get("hbm_gbs")
    hbm_achieved = alg_bytes / (mean_ms / 1e3) / 1e9
    # the reference's operation order leaves every FP64 operation unfused: the FP64 pipe binds
    ops = census.td_tdi_fp64_ops_per_sample(7) * B * n
    dgemm = gemm_peak_tflops(torch, torch.float64)
    op_peak = dgemm * 1e3 / 2.0  # G instructions/s: one DFMA instruction is 2 flops
    op_achieved = ops / (mean_ms / 1e3) / 1e9
    line = {
        "metric": TD_METRIC, "value": value, "unit": "samples/s", "n_gpus": world, "steps": args.steps,
        "warmup": max(3, args.warmup), "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded normal link series)",
        "config": td_config(), "l2": "flushed between steps (512 MB write outside the timed events); inputs 403 MB",
        "parallelism": f"replicas x{world}",
        "e2e": {"value": world * B * n / (e2e_ms / 1e3), "unit": "samples/s",
                "h2d_bytes_per_step": int(B * 6 * n_ext * 8), "d2h_bytes_per_step": int(B * 3 * n * 8)},
        "gpu_launches": args.steps,
        "roofline": {"kernel": "k_td_tdi<7, staged>", "bound": "fp64", "unit": "G FP64 op/s",
                     "achieved": op_achieved, "peak": op_peak,
                     "peak_source": "measured cuBLAS DGEMM 8192^3 in bench.py, flops / 2 (one DFMA = 2 flops)",
                     "frac": op_achieved / op_peak,
                     "traffic": census.TD_TDI_DRAM_BYTES_PER_SAMPLE * B * n,
                     "units_per_launch": {"samples": B * n, "algorithmic_bytes": alg_bytes, "fp64_ops": ops},
                     "hbm": {"achieved_gbs": hbm_achieved, "peak_gbs": hbm_peak,
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs (copy, burst)",
                             "frac": hbm_achieved / hbm_peak if hbm_peak else None}},
        "clocks": clocks.summary(),
        "float_float": {"entry": "pes_td_tdi_combination_mixed", "value": world * B * n / (ff_ms / 1e3),
                        "unit": "samples/s", "ms_per_step": ff_ms,
                        "hbm": {"achieved_gbs": alg_bytes / (ff_ms / 1e3) / 1e9, "peak_gbs": hbm_peak,
                                "frac": alg_bytes / (ff_ms / 1e3) / 1e9 / hbm_peak if hbm_peak else None},
                        "max_abs_err_over_max_link": ff_err},
    }
    if not args.no_cpu_baseline:
        v, done, dt = td_cpu_baseline(arm)
        line["cpu_baseline"] = {"value": v, "unit": "samples/s", "cores": 1, "kind": "port",
                                "sample": f"{done} output samples in 2^20-sample blocks ({dt:.1f} s, numpy)"}
    print(json.dumps(line), flush=True)


def network_hm_leg(steps, warmup, batch=4096, max_batch=512, check=16):
    """The higher-mode network configuration on this GPU: the mixed IMRPhenomHM
    plan over ``batch`` prior samples (chunks of ``max_batch``) captured in one
    CUDA graph; lnL only.  Returns the measurements as a dict."""
    import torch

    from pespace_gb300 import _lib
    from pespace_gb300.inference import CapturedStep, WhittleLikelihood
    from pespace_gb300.workloads import config0_theta, network_dataset, prior_samples

    T, dt, fmin, fmax, gen, desc = WORKLOADS["network-hm"]
    th0 = config0_theta(T - 86400.0)
    dets = network_dataset(T, dt, fmin, fmax, th0, gen, seed=2026, approximant="IMRPhenomHM")
    eng = WhittleLikelihood(dets, precision="mixed", approximant="IMRPhenomHM", reference_frequency=1e-4,
                            cut_factor=1.2, max_batch=max_batch, n_sparse=N_SPARSE["network-hm"])
    theta_host = torch.as_tensor(prior_samples(np.random.default_rng(2027), batch, th0[10])).pin_memory()
    theta = theta_host.to("cuda")
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    lib = _lib.load()
    # one profiled (uncaptured) pass: launches and device time per kernel class, work units
    eng.log_likelihood_batch(theta)
    torch.cuda.synchronize()
    n_cls = _lib.KERNEL_CLASSES
    import ctypes

    launches, dev_ms = (ctypes.c_int64 * n_cls)(), (ctypes.c_double * n_cls)()
    lib.pes_plan_profile(eng._plan, 1)
    lib.pes_plan_stats(eng._plan, launches, dev_ms)
    work = {"dense_bins": 0, "fp64_bins": 0, "sparse_nodes": 0, "samples": 0, "refined_ff": 0, "refined_exact": 0}
    for lo in range(0, batch, max_batch):
        eng.log_likelihood_batch(theta[lo:lo + max_batch])
        for k, v in eng.last_work(min(max_batch, batch - lo)).items():
            work[k] += v
    torch.cuda.synchronize()
    lib.pes_plan_stats(eng._plan, launches, dev_ms)
    lib.pes_plan_profile(eng._plan, 0)
    kern = {lib.pes_kernel_class_name(k).decode(): {"launches": int(launches[k]), "ms": float(dev_ms[k])}
            for k in range(n_cls) if launches[k]}
    step = CapturedStep(eng, batch, grad=False)
    for _ in range(max(3, warmup)):
        step(theta)
    torch.cuda.synchronize()
    clocks = ClockSampler(torch.cuda.current_device())
    ms = []
    with clocks:
        for _ in range(steps):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            step.graph.replay()
            e.record()
            e.synchronize()
            ms.append(s.elapsed_time(e))
    mean_ms = float(np.mean(ms))
    # end to end: parameters from pinned host memory, lnL back to the host
    lnl_host = torch.empty(batch, dtype=torch.float64).pin_memory()
    e2e = []
    for _ in range(steps):
        flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        step.theta.copy_(theta_host, non_blocking=True)
        step.graph.replay()
        lnl_host.copy_(step.lnl, non_blocking=True)
        e.record()
        e.synchronize()
        e2e.append(s.elapsed_time(e))
    got = step.lnl.clone()
    ok = int((step.status == 0).sum().item())
    del step, flush
    # accuracy and speed of the FP64 plan on an evenly spread subset
    idx = torch.as_tensor(stratified(batch, check), device="cuda")
    ref = WhittleLikelihood(dets, precision="fp64", approximant="IMRPhenomHM", reference_frequency=1e-4,
                            cut_factor=1.2, max_batch=len(idx))
    sub = theta[idx]
    want = ref.log_likelihood_batch(sub)
    torch.cuda.synchronize()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    s.record()
    ref.log_likelihood_batch(sub)
    e.record()
    e.synchronize()
    ms64 = s.elapsed_time(e)
    d = (got[idx] - want).abs()
    return {"metric": HM_METRIC, "value": batch / (mean_ms / 1e3), "unit": "lnL evals/s", "steps": steps,
            "warmup": max(3, warmup), "ms_per_step": mean_ms, "dtype": "f32+f64",
            "config": {"workload": desc, "batch": batch, "max_batch": max_batch, "nbins": int(eng.desc.nbins),
                       "detectors": 3, "modes": 6},
            "l2": "flushed between steps (512 MB write outside the timed events)",
            "e2e": {"value": batch / (float(np.mean(e2e)) / 1e3), "unit": "lnL evals/s",
                    "h2d_bytes_per_step": batch * 11 * 8, "d2h_bytes_per_step": batch * 8},
            "samples_ok": ok, "kernels": kern, "work_per_step": work,
            "dense_bins_per_s": (work["dense_bins"] + work["fp64_bins"]) / (mean_ms / 1e3),
            "fp64_gpu": {"value": len(idx) / (ms64 / 1e3), "unit": "lnL evals/s", "samples": len(idx),
                         "ms": ms64},
            "vs_fp64": (batch / (mean_ms / 1e3)) / (len(idx) / (ms64 / 1e3)),
            "dlnl_vs_fp64": {"samples": len(idx), "max_abs": float(d.max().item()),
                             "n_within_1e-2": int((d <= 1e-2).sum().item())},
            "clocks": clocks.summary()}


def smc_sweep_leg(steps, warmup, n_half=8192, check=64):
    """One SMC-style sweep per step over 2 n_half particles: the IMRPhenomD half
    (LISA, config of the default workload) gets lnL, gradient and the 11x11
    Fisher matrix from the mixed plan; the IMRPhenomHM half (three-detector
    network) gets lnL from the mixed plan (its gradient and Fisher matrix are
    the FP64 plan's, too slow for a sweep of this size: not timed here).
    Accuracy on evenly spread subsets against the FP64 plans."""
    import torch

    from pespace_gb300.inference import WhittleLikelihood
    from pespace_gb300.workloads import config0_theta, lisa_dataset, network_dataset, prior_samples

    T1, dt1, f1, F1, g1, _ = WORKLOADS["adjoint"]
    th1 = config0_theta(T1 - 86400.0)
    det1 = lisa_dataset(T1, dt1, f1, F1, th1, g1, seed=2026)
    T3, dt3, f3, F3, g3, _ = WORKLOADS["network-hm"]
    th3 = config0_theta(T3 - 86400.0)
    det3 = network_dataset(T3, dt3, f3, F3, th3, g3, seed=2026, approximant="IMRPhenomHM")
    eng_d = WhittleLikelihood(det1, precision="mixed", reference_frequency=1e-4, cut_factor=1.2, max_batch=1024)
    eng_h = WhittleLikelihood(det3, precision="mixed", approximant="IMRPhenomHM", reference_frequency=1e-4,
                              cut_factor=1.2, max_batch=512, n_sparse=N_SPARSE["network-hm"])
    rng = np.random.default_rng(2028)
    th_d = torch.as_tensor(prior_samples(rng, n_half, th1[10]), device="cuda")
    th_h = torch.as_tensor(prior_samples(rng, n_half, th3[10]), device="cuda")
    out = {}

    def sweep():
        out["lnl_d"], out["grad_d"] = eng_d.log_likelihood_and_grad(th_d)
        out["fisher_d"] = eng_d.fisher_matrix(th_d)
        out["lnl_h"] = eng_h.log_likelihood_batch(th_h)

    for _ in range(max(1, warmup)):
        sweep()
    torch.cuda.synchronize()
    ms, parts = [], {"phenomd_lnl_grad": [], "phenomd_fisher": [], "phenomhm_lnl": []}
    for _ in range(steps):
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        ev[0].record()
        out["lnl_d"], out["grad_d"] = eng_d.log_likelihood_and_grad(th_d)
        ev[1].record()
        out["fisher_d"] = eng_d.fisher_matrix(th_d)
        ev[2].record()
        out["lnl_h"] = eng_h.log_likelihood_batch(th_h)
        ev[3].record()
        ev[3].synchronize()
        ms.append(ev[0].elapsed_time(ev[3]))
        for k, (a, b) in zip(parts, ((0, 1), (1, 2), (2, 3))):
            parts[k].append(ev[a].elapsed_time(ev[b]))
    mean_ms = float(np.mean(ms))
    # accuracy against the FP64 plans on evenly spread subsets
    idx = torch.as_tensor(stratified(n_half, check), device="cuda")
    ref_d = WhittleLikelihood(det1, precision="fp64", reference_frequency=1e-4, cut_factor=1.2, max_batch=len(idx))
    d_lnl = (out["lnl_d"][idx] - ref_d.log_likelihood_batch(th_d[idx])).abs()
    Fw = ref_d.fisher_matrix(th_d[idx])
    sd = torch.sqrt(torch.diagonal(Fw, dim1=1, dim2=2).abs())
    f_err = ((out["fisher_d"][idx] - Fw).abs() / (sd[:, :, None] * sd[:, None, :])).amax()
    del ref_d
    idx_h = idx[: check // 4]
    ref_h = WhittleLikelihood(det3, precision="fp64", approximant="IMRPhenomHM", reference_frequency=1e-4,
                              cut_factor=1.2, max_batch=len(idx_h))
    d_h = (out["lnl_h"][idx_h] - ref_h.log_likelihood_batch(th_h[idx_h])).abs()
    # what the IMRPhenomHM half's gradient and Fisher matrices cost from the
    # FP64 plan (the only plan that gives the six-mode gradient), on a few
    # particles: the reason they are not in the timed sweep
    few = th_h[idx_h[:4]]
    ref_h.log_likelihood_and_grad(few[:1])
    ref_h.fisher_matrix(few[:1])
    torch.cuda.synchronize()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    ev[0].record()
    ref_h.log_likelihood_and_grad(few)
    ev[1].record()
    ref_h.fisher_matrix(few)
    ev[2].record()
    ev[2].synchronize()
    g_ms, f_ms = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    hm_fp64 = {"particles": len(few), "lnl_grad_ms": g_ms, "fisher_ms": f_ms,
               "sweep_half_s_at_this_rate": n_half * (g_ms + f_ms) / len(few) / 1e3}
    return {"metric": SMC_METRIC, "value": 2 * n_half / (mean_ms / 1e3), "unit": "particles/s", "steps": steps,
            "warmup": max(1, warmup), "ms_per_step": mean_ms, "dtype": "f32+f64",
            "config": {"workload": WORKLOADS["smc-sweep"][5], "particles": 2 * n_half},
            "ms_per_part": {k: float(np.mean(v)) for k, v in parts.items()},
            "not_timed": "IMRPhenomHM gradient and Fisher: FP64 plan only (no mixed multi-mode adjoint)",
            "phenomhm_grad_fisher_fp64": hm_fp64,
            "accuracy": {"phenomd_samples": len(idx), "phenomd_max_abs_dlnl": float(d_lnl.max().item()),
                         "phenomd_n_within_1e-2": int((d_lnl <= 1e-2).sum().item()),
                         "phenomd_fisher_max_rel": float(f_err.item()),
                         "phenomhm_samples": len(idx_h), "phenomhm_max_abs_dlnl": float(d_h.max().item()),
                         "phenomhm_n_within_1e-2": int((d_h <= 1e-2).sum().item())}}


def run_smc_sweep(args):
    line = smc_sweep_leg(args.steps, args.warmup)
    line.update({"n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                 "data": "synthetic"})
    print(json.dumps(line), flush=True)


def run_network_hm(args):
    line = network_hm_leg(args.steps, args.warmup)
    line.update({"n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                 "data": "synthetic", "gpu_launches": sum(v["launches"] for v in line["kernels"].values())})
    print(json.dumps(line), flush=True)


def run_native(args):
    import torch

    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from pespace_gb300 import _lib
    from pespace_gb300.inference import WhittleLikelihood
    from pespace_gb300 import replicas
    from pespace_gb300.workloads import config0_theta, lisa_dataset, network_dataset

    B = args.batch
    th0 = config0_theta(DUR - 86400.0)
    if args.workload == "network-d":
        det = network_dataset(DUR, DT, FMIN, FMAX, th0, GEN, seed=2026)
    else:
        det = lisa_dataset(DUR, DT, FMIN, FMAX, th0, GEN, seed=2026)
    eng = WhittleLikelihood(det, precision=args.precision, reference_frequency=1e-4, cut_factor=1.2, max_batch=B,
                            n_sparse=args.n_sparse or N_SPARSE.get(args.workload, 1024))
    theta_host = torch.as_tensor(replicas.rank_theta(rank, B, th0[10])).pin_memory()
    theta = theta_host.to("cuda")
    lib = _lib.load()
    flush = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step_device():
        return eng.log_likelihood_and_grad(theta)

    for _ in range(max(3, args.warmup)):
        step_device()
    torch.cuda.synchronize()
    lib.pes_plan_profile(eng._plan, 1)
    n_cls = _lib.KERNEL_CLASSES
    launches = (ctypes_i64 := __import__("ctypes").c_int64 * n_cls)()
    dev_ms = (__import__("ctypes").c_double * n_cls)()
    lib.pes_plan_stats(eng._plan, launches, dev_ms)  # reset

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    clocks = ClockSampler(local)
    step_ms = []
    with clocks:
        barrier()
        for _ in range(args.steps):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            step_device()
            e.record()
            step_ms.append((s, e))
        barrier()
    times = [s.elapsed_time(e) for s, e in step_ms]
    work = eng.last_work(B)
    lib.pes_plan_stats(eng._plan, launches, dev_ms)
    lib.pes_plan_profile(eng._plan, 0)
    kern = {lib.pes_kernel_class_name(k).decode(): (int(launches[k]), float(dev_ms[k])) for k in range(n_cls)
            if launches[k]}
    gpu_launches = sum(v[0] for v in kern.values())
    mean_ms = replicas.reduce_max(float(np.mean(times)), "cuda")
    value = replicas.job_rate(world, B, mean_ms)

    # ---------------- e2e through host buffers
    lnl_host = torch.empty(B, dtype=torch.float64).pin_memory()
    grad_host = torch.empty((B, 11), dtype=torch.float64).pin_memory()
    e2e_ms = []
    barrier()
    for _ in range(args.steps):
        flush.zero_()
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record()
        th_dev = theta_host.to("cuda", non_blocking=True)
        lnl, grad = eng.log_likelihood_and_grad(th_dev)
        lnl_host.copy_(lnl, non_blocking=True)
        grad_host.copy_(grad, non_blocking=True)
        e.record()
        e.synchronize()
        e2e_ms.append(s.elapsed_time(e))
    e2e_value = replicas.job_rate(world, B, replicas.reduce_max(float(np.mean(e2e_ms)), "cuda"))

    # ---------------- lnL-only calls and CUDA-graph replays of the lnL+gradient call
    from pespace_gb300.inference import CapturedStep

    def timed(fn, n):
        ms = []
        for _ in range(n):
            flush.zero_()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            fn()
            e.record()
            e.synchronize()
            ms.append(s.elapsed_time(e))
        return float(np.mean(ms))

    for _ in range(max(3, args.warmup)):
        eng.log_likelihood_batch(theta)
    lnl_ms = replicas.reduce_max(timed(lambda: eng.log_likelihood_batch(theta), args.steps), "cuda")
    graph_step = CapturedStep(eng, B)
    for _ in range(max(3, args.warmup)):
        graph_step(theta)
    graph_ms = replicas.reduce_max(timed(lambda: graph_step(theta), args.steps), "cuda")
    del graph_step

    # ---------------- accuracy against the FP64 path on this workload
    err = err_split = fp64_gpu = None
    err_samples = B if args.workload != "network-d" else min(B, 128)  # FP64 over 10 M bins x 3: a subset
    if args.precision == "mixed":
        ref = WhittleLikelihood(det, precision="fp64", reference_frequency=1e-4, cut_factor=1.2, max_batch=B)
        a, _ = eng.log_likelihood_and_grad(theta)
        b = ref.log_likelihood_batch(theta[:err_samples])
        d = (a[:err_samples] - b).abs()
        err = float(d.max().item())
        # the FP32 floor scales with |lnL|: report it apart for templates far below the posterior
        quiet = b.abs() <= 1e6
        err_split = {"max_abs_lnl_le_1e6": float(d[quiet].max().item()) if bool(quiet.any()) else None,
                     "n_lnl_le_1e6": int(quiet.sum().item()),
                     "n_within_1e-2": int((d <= 1e-2).sum().item()),
                     "max_rel": float((d / b.abs().clamp_min(1.0)).max().item())}
        # the templates a sampler visits: draws from the Fisher approximation of the posterior
        # about the injection (covariance F^-1 of the FP64 plan's Fisher matrix)
        from pespace_gb300.inference.fisher import sample_from_fisher

        try:
            F = ref.fisher_matrix(torch.as_tensor(th0[None], dtype=torch.float64, device="cuda"))[0]
            n_post = min(B, 256)
            post = torch.as_tensor(th0[None] + sample_from_fisher(F, n_post, 2026), device="cuda")
            bp = ref.log_likelihood_batch(post)
            dp = (eng.log_likelihood_batch(post) - bp).abs()
            err_split.update(posterior_draws=n_post, max_abs_posterior=float(dp.max().item()),
                             median_abs_posterior=float(dp.median().item()),
                             lnl_range_posterior=[float(bp.min().item()), float(bp.max().item())])
        except np.linalg.LinAlgError:
            err_split.update(posterior_draws=0)
        # the plain FP64 GPU path timed on the same batch: the metric's comparison
        fp64_n = err_samples
        th64 = theta[:fp64_n]
        ref.log_likelihood_and_grad(th64)
        ms64 = replicas.reduce_max(timed(lambda: ref.log_likelihood_and_grad(th64), 2), "cuda")
        fp64_gpu = {"value": replicas.job_rate(world, fp64_n, ms64), "unit": "lnL+grad evals/s",
                    "ms_per_step": ms64, "steps": 2, "warmup": 1, "samples": fp64_n,
                    "path": "FP64 plan: dense FP64 evaluation of every live bin, forward-mode gradient"}
        del ref

    # ---------------- roofline of the dominant kernel (the dense stage)
    roofline = None
    if rank == 0:
        from pespace_gb300 import census

        dom = "dense_mixed" if args.precision == "mixed" else "dense_fp64"
        roofline = census.roofline(dom, kern[dom], args.steps, work, True, gemm_peak_tflops(torch, torch.float32))
        roofline["fp64_peak_tflops"] = gemm_peak_tflops(torch, torch.float64)

    config = workload_config(B, world)
    assert config["nbins"] == int(eng.desc.nbins), (config, eng.desc.nbins)
    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "lnL+grad evals/s", "n_gpus": world, "steps": args.steps,
            "warmup": max(3, args.warmup), "ms_per_step": mean_ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32+f64" if args.precision == "mixed" else "f64", "data": "synthetic",
            "config": config, "precision": args.precision,
            "l2": "flushed between steps (512 MB write outside the timed events)",
            "parallelism": f"replicas x{world}",
            "e2e": {"value": e2e_value, "unit": "lnL+grad evals/s", "h2d_bytes_per_step": int(B * 11 * 8),
                    "d2h_bytes_per_step": int(B * 12 * 8)},
            "gpu_launches": int(gpu_launches),
            "kernels": {k: {"launches": v[0], "ms": v[1]} for k, v in kern.items()},
            "work_per_step": work,
            "dense_bins_per_s": world * (work["dense_bins"] + work["fp64_bins"]) / (mean_ms / 1e3),
            "lnl_only": {"value": replicas.job_rate(world, B, lnl_ms), "unit": "lnL evals/s", "ms_per_step": lnl_ms},
            "cuda_graph": {"value": replicas.job_rate(world, B, graph_ms), "unit": "lnL+grad evals/s",
                           "ms_per_step": graph_ms},
            "roofline": roofline,
            "clocks": clocks.summary(),
        }
        if fp64_gpu is not None:
            line["fp64_gpu"] = fp64_gpu
            line["vs_fp64"] = value / fp64_gpu["value"]
        if err is not None:
            line["max_abs_dlnl_vs_fp64"] = err
            line["dlnl_samples"] = err_samples
            line["dlnl_vs_fp64"] = err_split
        if not args.no_cpu_baseline and args.workload != "network-d":
            threads = os.cpu_count() or 1
            n = min(B, 20 * threads)  # about 10 s of the 16-core host
            v, dt = cpu_baseline_run(n, threads, "", batch=B)
            line["cpu_baseline"] = {"value": v, "unit": "lnL+grad evals/s", "cores": threads, "kind": "port",
                                    "sample": f"{n} of the {B} samples (evenly spread over the batch), full grid, "
                                              f"FP64 dense + forward-mode gradient ({dt:.1f} s)"}
            # lnL only on one core: the setting of the reference's published single-core figure
            n1 = 32
            v1, dt1 = cpu_baseline_run(n1, 1, "", grad=False, batch=B)
            line["cpu_baseline_1core_lnl"] = {"value": v1, "unit": "lnL evals/s", "cores": 1, "kind": "port",
                                              "sample": f"{n1} of the {B} samples, full grid, FP64 dense "
                                                        f"({dt1:.1f} s)"}
        if world == 1 and not args.no_network_hm and args.workload == "adjoint":
            del eng
            torch.cuda.empty_cache()
            line["network_hm"] = network_hm_leg(3, 3)
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "td-tdi":
        run_td_tdi(args)
    elif args.workload == "network-hm":
        run_network_hm(args)
    elif args.workload == "smc-sweep":
        run_smc_sweep(args)
    else:
        run_native(args)


if __name__ == "__main__":
    main()
