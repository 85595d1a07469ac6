"""Benchmark of the matched-filter hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--workload config4|config1|config2|config0|config3|variable|variable_full]
                    [--precision ...] [--templates T] [--samples N] [--no-frontend]

One *step* is one complete search of the workload (every template against
every channel and output index: preprocessing kernels + correlation
kernel).  Metric: template*lag*channel multiply-accumulates per second
(T * n_corr * S * C * L per step, TMAC/s).

  value     device-resident inputs, K steps timed with CUDA events on the
            launching stream, barrier + synchronize on both sides, max over
            ranks; inputs (1 GB of data for the full-day search) exceed L2.
  e2e       the same search through the C ABI (fmf_matched_filter_ex) with
            pinned host buffers: H2D of every input and D2H of the whole
            output inside each timed step.
  roofline  the correlation kernel, event-timed inside the timed region.
  frontend_numpy  the drop-in Python call on the workload's
            numpy arrays (pageable host memory), wall clock per call.
  cpu_baseline  the oracle's C port of the reference CPU algorithm (OpenMP,
            all host cores) on a bounded sample of the same workload.

Workloads: config4 the full-day search (default); config1 a continuous record;
config2 DC offsets with 'full' normalisation and step 2; config0 the small case;
config3 64 uneven searches in one batched launch; variable / variable_full
per-channel template lengths with the Fisher-z network sum.

--impl reference times that CPU algorithm alone (rank 0; other ranks exit).
Under torchrun each rank searches its own template set against the same
data (weak scaling); the only collectives are the barrier and the max of
the per-rank times.
"""
import argparse
import contextlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

METRIC = "template*lag*channel TMAC/s"
UNIT = "TMAC/s"
PEAKS_FILE = os.path.join(HERE, "MEASURED_PEAKS.json")
FALLBACK_PEAKS = {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
                  "sm_max_mhz": 2070.0}
N_SM = 152


def parse_args(argv=None):
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=5)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="ours", choices=["ours", "reference"])
    p.add_argument("--workload", default="config4")
    p.add_argument("--precision", default="auto")
    p.add_argument("--no-e2e", action="store_true")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-compare", action="store_true",
                   help="skip the plain FP32 comparison run")
    p.add_argument("--no-precision-report", action="store_true",
                   help="skip the FP64 error report on a subset")
    p.add_argument("--no-detect", action="store_true",
                   help="skip the detection leg (threshold + peaks on the search output)")
    p.add_argument("--no-frontend", action="store_true",
                   help="skip timing the drop-in Python call on numpy (pageable) arrays")
    p.add_argument("--templates", type=int, default=0, help="override T (smaller runs)")
    p.add_argument("--samples", type=int, default=0, help="override N (smaller runs)")
    return p.parse_args(argv)


def load_peaks():
    try:
        with open(PEAKS_FILE) as f:
            pk = json.load(f)
        return pk, "measured"
    except (OSError, ValueError):
        return dict(FALLBACK_PEAKS), "fallback"


# ---------------------------------------------------------------- workload
def make_workload(name, rank=0, templates=0, samples=0):
    from fast_matched_filter_gb300 import synthetic
    kw = {}
    if templates:
        kw["n_templates"] = templates
    if samples:
        kw["n_samples"] = samples
    gen = {"config0": synthetic.config0, "config1": synthetic.config1,
           "config2": synthetic.config2, "config4": synthetic.config4,
           "variable": synthetic.variable, "variable_full": synthetic.variable}[name]
    if name == "variable_full":
        kw["normalize"] = "full"
    if name == "config0":
        cfg = gen(seed=100 + 1000 * rank)
    else:
        cfg = gen(seed={"config1": 101, "config2": 102, "config4": 104, "variable": 105,
                        "variable_full": 105}[name] + 1000 * rank, **kw)
    tp = cfg["templates"]
    cfg["sst"] = np.sum(tp ** 2, axis=-1).astype(np.float32)
    cfg["macs"] = synthetic.macs(tp.shape, cfg["data"].shape[-1], cfg["step"])
    if "n_samples_template" in cfg:
        cfg["macs"] = synthetic.variable_macs(cfg["n_samples_template"], cfg["data"].shape[-1],
                                              cfg["step"])
    cfg["n_corr"] = (cfg["data"].shape[-1] - tp.shape[-1]) // cfg["step"] + 1
    return cfg


def describe(cfg, extra=None):
    T, S, C, L = cfg["templates"].shape
    d = {"workload": cfg["name"], "templates": T, "stations": S, "components": C,
         "template_length": L, "samples": int(cfg["data"].shape[-1]), "step": cfg["step"],
         "normalize": cfg["normalize"], "network_sum": cfg["network_sum"],
         "n_corr": int(cfg["n_corr"]),
         "l2": "inputs larger than L2 (data %.2f GB > 129 MB); no flush"
               % (cfg["data"].nbytes / 1e9)}
    if extra:
        d.update(extra)
    return d


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi sampling of SM clock and throttle reasons while running."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index):
        self.dev = device_index
        self.proc = None
        self.off = device_index < 0
        self.path = os.path.join(tempfile.gettempdir(),
                                 "fmf_bench_clocks_%d_%d.csv" % (os.getpid(), device_index))

    def __enter__(self):
        if self.off:
            return self
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None:
            return None
        rows = []
        with open(self.path) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) < 9:
                    continue
                try:
                    rows.append((float(parts[1]), float(parts[2]), float(parts[3]), parts[5:9]))
                except ValueError:
                    continue
        with contextlib.suppress(OSError):
            os.remove(self.path)
        if not rows:
            return None
        loaded = [r for r in rows if r[2] > 200.0] or rows
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in loaded for i, v in enumerate(r[3]) if v == "Active"})
        return {"sm_mhz": statistics.median(r[0] for r in loaded),
                "sm_max_mhz": max(r[1] for r in rows), "reasons": reasons,
                "samples": len(loaded), "power_w_max": max(r[2] for r in rows)}


# ---------------------------------------------------------------- distributed
def dist_info():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def dist_max(value, world):
    """Max of a float over ranks (the only cross-rank reduction of the bench)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([value], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


# ---------------------------------------------------------------- CPU baseline
CPU_SAMPLE_MACS = 4e11  # about 15 s of the CPU algorithm on 16 cores


def cpu_sample(cfg, n_templates=None):
    """Bounded sample of the workload for the CPU algorithm: the first
    template(s) against the whole trace -- as many as fit about 15 s of CPU
    work (all of them for the small workloads)."""
    if n_templates is None:
        T = cfg["templates"].shape[0]
        per = cfg["macs"] / T
        n_templates = int(max(1, min(T, CPU_SAMPLE_MACS // max(per, 1.0))))
    sub = dict(cfg)
    sub["templates"] = cfg["templates"][:n_templates]
    sub["moveouts"] = cfg["moveouts"][:n_templates]
    sub["weights"] = cfg["weights"][:n_templates]
    from fast_matched_filter_gb300 import synthetic
    sub["macs"] = synthetic.macs(sub["templates"].shape, cfg["data"].shape[-1], cfg["step"])
    if "n_samples_template" in cfg:
        nt = cfg["n_samples_template"][:n_templates]
        sub["n_samples_template"] = nt
        # the sample keeps the full template axis, so its lag range is the search's
        n_corr = cfg["n_corr"]
        sub["macs"] = int(n_corr) * int(nt.astype(np.int64).sum())
    return sub


def run_cpu_once(sub, threads):
    from oracle import cpu
    arch = "cpu" if sub["normalize"] == "short" else "precise"
    t0 = time.perf_counter()
    if "n_samples_template" in sub:
        cpu.run_oracle_variable(sub["templates"], sub["n_samples_template"], sub["moveouts"],
                                sub["weights"], sub["data"], sub["step"], sub["normalize"],
                                n_threads=threads)
    else:
        cpu.run_oracle(sub["templates"], sub["moveouts"], sub["weights"], sub["data"],
                       sub["step"], arch, sub["normalize"], sub["network_sum"], n_threads=threads)
    return time.perf_counter() - t0


def cpu_baseline(cfg, reps=1):
    """The CPU algorithm on a bounded sample: the reference library compiled
    from its own source (oracle/_ref) where it exists, else the oracle port."""
    from oracle import cpu
    if not os.path.exists(cpu.ORACLE_SO):
        cpu.build()
    threads = os.cpu_count() or 1
    sub = cpu_sample(cfg)
    kind = "reference" if cpu.reference_available() else "port"
    if "n_samples_template" in sub:
        kind = "port"  # the timed run below uses the oracle for this arch too
    if kind == "reference":
        os.environ["OMP_NUM_THREADS"] = str(threads)
        arch = "cpu" if sub["normalize"] == "short" else "precise"
        t0 = time.perf_counter()
        cpu.run_reference(sub["templates"], sub["moveouts"], sub["weights"], sub["data"],
                          sub["step"], arch, sub["normalize"], sub["network_sum"])
        secs = time.perf_counter() - t0
    else:
        secs = min(run_cpu_once(sub, threads) for _ in range(reps))
    what = ("reference CPU library compiled from its source" if kind == "reference"
            else "oracle C port of the reference CPU algorithm")
    return {"value": sub["macs"] / secs / 1e12, "unit": UNIT, "cores": threads, "kind": kind,
            "sample": "%d of %d templates x full trace (%d samples), %.3g MAC in %.2f s; "
                      "%s (OpenMP %d threads)"
                      % (sub["templates"].shape[0], cfg["templates"].shape[0],
                         cfg["data"].shape[-1], sub["macs"], secs, what, threads),
            "seconds": secs}


def run_reference_arm(args):
    world, rank, local = dist_info()
    if rank != 0:
        return 0
    cfg = make_workload(args.workload, 0, args.templates, args.samples)
    from oracle import cpu
    cpu.build()
    threads = os.cpu_count() or 1
    sub = cpu_sample(cfg)
    for _ in range(args.warmup):
        run_cpu_once(sub, threads)
    times = [run_cpu_once(sub, threads) for _ in range(args.steps)]
    tot = sum(times)
    value = sub["macs"] * args.steps / tot / 1e12
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic", "impl": "reference",
            "config": describe(cfg, {"sample": "first %d template(s) x full trace per step"
                                               % sub["templates"].shape[0]}),
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": "port",
                             "sample": "%d of %d templates x full trace, %.3g MAC per step"
                                       % (sub["templates"].shape[0], cfg["templates"].shape[0],
                                          sub["macs"])},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ---------------------------------------------------------------- our arm
def run_ours(args):
    import torch

    world, rank, local = dist_info()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", init_method="env://")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    import fast_matched_filter_gb300 as fmf
    from fast_matched_filter_gb300 import _lib
    lib = _lib.load()

    cfg = make_workload(args.workload, rank, args.templates, args.samples)
    requested = args.precision  # 'auto': the library picks the form whose error bound holds 1e-5
    T, S, C, L = cfg["templates"].shape
    n_corr = cfg["n_corr"]
    out_shape = (T, n_corr) if cfg["network_sum"] else (T, n_corr, S, C)

    g = {k: torch.from_numpy(np.ascontiguousarray(cfg[k])).to(dev)
         for k in ("templates", "sst", "moveouts", "weights", "data")}
    out = torch.empty(out_shape, dtype=torch.float32, device=dev)
    stream = torch.cuda.current_stream()

    def timed(prec, steps, warmup, sample_clocks):
        def step():
            return fmf.matched_filter_device(g["templates"], g["sst"], g["moveouts"],
                                             g["weights"], g["data"], cfg["step"], out,
                                             cfg["normalize"], cfg["network_sum"], prec, stream)

        for _ in range(max(warmup, 0)):
            step()
        torch.cuda.synchronize()
        barrier(world)
        torch.cuda.synchronize()
        launches = 0
        import ctypes as ct
        with ClockSampler(local if sample_clocks else -1) as clocks:
            lib.fmf_timing_begin()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                launches += step()
            e1.record(stream)
            torch.cuda.synchronize()
            prep_ms, kern_ms, ncalls = ct.c_double(), ct.c_double(), ct.c_int()
            lib.fmf_timing_end(ct.byref(prep_ms), ct.byref(kern_ms), ct.byref(ncalls))
        _lib.check(lib.fmf_device_errors(), lib)
        barrier(world)
        torch.cuda.synchronize()
        t_max = dist_max(e0.elapsed_time(e1), world)
        return {"value": cfg["macs"] * steps * world / (t_max / 1e3) / 1e12,
                "ms_per_step": t_max / steps, "launches": launches,
                "kernel_ms_avg": kern_ms.value / max(ncalls.value, 1),
                "prep_ms_avg": prep_ms.value / max(ncalls.value, 1),
                "clocks": clocks.summary() if sample_clocks else None}

    main = timed(requested, args.steps, args.warmup, True)
    precision = _lib.PRECISION_NAMES[lib.fmf_last_precision()]  # the form that ran
    value = main["value"]
    roof = roofline(cfg, precision, main["kernel_ms_avg"], main["prep_ms_avg"],
                    measured_fp32_tflops(lib) if precision == "fp32" else None)
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": main["ms_per_step"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp32": "f32", "split_bf16": "bf16x3", "bf16": "bf16"}[precision],
            "data": "synthetic",
            "config": describe(cfg, {"precision": precision, "precision_requested": requested,
                                     "parallelism": "template sets per rank" if world > 1
                                     else "single GPU"}),
            "roofline": roof, "gpu_launches": main["launches"], "clocks": main["clocks"]}
    if precision != "fp32" and not args.no_compare:
        plain = timed("fp32", max(1, min(args.steps, 2)), 1, False)
        line["plain_fp32"] = {"value": plain["value"], "unit": UNIT,
                              "ms_per_step": plain["ms_per_step"],
                              "kernel_ms_avg": plain["kernel_ms_avg"],
                              "speedup_of_headline": value / plain["value"],
                              "roofline": roofline(cfg, "fp32", plain["kernel_ms_avg"],
                                                   plain["prep_ms_avg"],
                                                   fp32_measured=measured_fp32_tflops(lib))}

    if rank == 0 and not args.no_precision_report:
        line["precision_vs_fp64"] = precision_report(cfg)
    if cfg["network_sum"] and not args.no_detect:
        # the search output of the last timed step is still in `out`
        line["detection"] = run_detection(cfg, out, world)
    # end to end through the C ABI with pinned host buffers
    del g
    if not args.no_e2e:
        line["e2e"] = run_e2e(cfg, out, requested, args, world, lib)
        if cfg["network_sum"] and not args.no_detect:
            line["e2e_search_detect"] = run_e2e_detect(cfg, requested, args, world, lib)
    del out
    torch.cuda.empty_cache()
    if not args.no_frontend and world == 1:
        line["frontend_numpy"] = run_frontend(cfg, requested, args)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(cfg)
    if rank == 0:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


def tc_executed_macs(cfg, nb=None):
    """Multiply-accumulates the tensor-core kernel issues for one search
    (one product; x3 for split-BF16): per busy tile, template, channel and
    phase, K steps of 16 x 128 phases x NB lag blocks.  Mirrors the K range
    of fmf_tc.cu (s = phase moveout mod 128, K = s + L_phi + 127 rounded to
    16 from s rounded down to 16)."""
    Q = 128
    tp = cfg["templates"]
    T, S, C, L = tp.shape
    step = cfg["step"]
    N = cfg["data"].shape[-1]
    n_corr = cfg["n_corr"]
    if nb is None:
        nb = 128
        lphi = -(-L // step)
        for cand in (128, 64, 32):
            k_span = ((2 * Q - 2 + lphi) + 15) & ~15
            R = cand + (k_span - 1) // Q + 1
            NW = k_span // 8 + 16
            stage = 2 * (16 * R * 16 + NW * 128)
            stage = (stage + 1023) & ~1023
            if 2 * stage + 128 <= 227 * 1024:
                nb = cand
                break
    mo = cfg["moveouts"].reshape(T, S * C).astype(np.int64)
    w = cfg["weights"].reshape(T, S * C)
    tile = Q * nb
    n_tiles = -(-n_corr // tile)
    total = 0
    for t in range(T):
        lo, hi = min(0, mo[t].min()), max(0, mo[t].max())
        klo = -(-(-lo) // step) if lo < 0 else 0
        last = N - L - hi
        khi = min(n_corr, last // step + 1) if last >= 0 else 0
        if khi <= klo:
            continue
        busy = sum(1 for i in range(n_tiles) if i * tile < khi and (i + 1) * tile > klo)
        ksteps = 0
        own = cfg.get("n_samples_template")
        own = None if own is None else np.asarray(own).reshape(T, S * C)
        for ch in range(S * C):
            if w[t, ch] == 0:
                continue
            for phi in range(step):
                mu = (mo[t, ch] + phi) // step
                s = mu % Q
                lphi = (L - phi + step - 1) // step
                if own is not None:  # the issuers stop at the channel's own length
                    n = int(own[t, ch])
                    lphi = min(lphi, (n - phi + step - 1) // step if n > phi else 0)
                ksteps += (((s + lphi + Q - 1 + 15) & ~15) - (s & ~15)) // 16
        total += busy * ksteps * 16 * Q * nb
    return total, nb


def profiled_traffic(kernel_prefix, cfg):
    """DRAM bytes per launch for this workload, scaled from the committed ncu
    summary of the kernel (profiles/<kernel>_*.md, line
    'traffic_bytes_per_template_lag: X'): X * templates * lags, or None."""
    import glob
    for path in sorted(glob.glob(os.path.join(HERE, "profiles", kernel_prefix + "_*.md"))):
        for line in open(path):
            if line.startswith("traffic_bytes_per_template_lag:"):
                per = float(line.split(":")[1])
                return per * cfg["templates"].shape[0] * cfg["n_corr"], os.path.basename(path)
    return None, None


def measured_fp32_tflops(lib):
    """The FP32 FMA rate measured in this run (fmf_measure_fp32_fma: independent
    FMA chains on every SM), in TFLOP/s, or None."""
    import ctypes as ct
    v = ct.c_double()
    return v.value if lib.fmf_measure_fp32_fma(ct.byref(v)) == 0 and v.value > 0 else None


def fp32_peak(measured):
    """(peak, nominal, source) of the FP32 FMA roofline: the rate measured in this run
    when there is one, else the nominal 152 SMs x 128 lanes x max SM clock."""
    peaks, src = load_peaks()
    mhz = float(peaks.get("sm_max_mhz", 2070.0))
    nominal = N_SM * 128 * 2 * mhz * 1e6 / 1e12
    if measured:
        return measured, nominal, ("measured in this run: FP32 FMA kernel of independent chains on "
                                   "every SM (fmf_measure_fp32_fma)")
    return nominal, nominal, ("nominal FP32 FMA rate: 152 SMs x 128 lanes x %.0f MHz (%s max SM "
                              "clock)" % (mhz, src))


def roofline(cfg, precision, kern_ms, prep_ms, fp32_measured=None):
    peaks, src = load_peaks()
    algo_tflops = 2.0 * cfg["macs"] / (kern_ms / 1e3) / 1e12
    if precision == "fp32":
        peak, nominal, psrc = fp32_peak(fp32_measured)
        roof = {"bound": "fp32_fma", "achieved": algo_tflops, "peak": peak, "unit": "TFLOP/s",
                "frac": algo_tflops / peak, "nominal_peak": nominal, "nominal_frac": algo_tflops / nominal,
                "traffic": None, "kernel": "plain_kernel", "peak_source": psrc}
    else:
        bf16 = float(peaks.get("bf16_tflops_sustained", peaks["bf16_tflops"]))
        products = 3 if precision == "split_bf16" else 1
        # the bound in algorithmic FLOP/s: each multiply-accumulate costs `products`
        # bf16 tensor-core products
        peak = bf16 / products
        ex, nb = tc_executed_macs(cfg)
        executed = 2.0 * ex * products / (kern_ms / 1e3) / 1e12
        traffic, tsrc = profiled_traffic("tc_persistent", cfg)
        roof = {"bound": "tensor", "achieved": algo_tflops, "peak": peak, "unit": "TFLOP/s",
                "frac": algo_tflops / peak, "traffic": traffic, "traffic_source": tsrc,
                "kernel": "tc_persistent (nb=%d)" % nb,
                "peak_source": "%s bf16_tflops_sustained (cuBLAS bf16 GEMM, seconds-long loop) "
                               "/ %d bf16 products per multiply-accumulate" % (src, products),
                "bf16_peak": bf16,
                "executed_tflops": executed, "executed_frac": executed / bf16,
                "executed_over_algorithmic": ex * products / cfg["macs"]}
    roof["kernel_ms_avg"] = kern_ms
    roof["prep_ms_avg"] = prep_ms
    return roof


def precision_report(cfg, n_templates=2, n_lags=50000):
    """max and p99.9 |cc - FP64| of every form on a bounded subset (the first
    templates, a window of output indices in the middle of the trace), plus the
    reference CPU algorithm's own error on the same subset."""
    import torch

    import fast_matched_filter_gb300 as fmf
    from oracle import cpu, fp64
    tp = cfg["templates"][:n_templates]
    mo, w = cfg["moveouts"][:n_templates], cfg["weights"][:n_templates]
    d, step = cfg["data"], cfg["step"]
    L = tp.shape[-1]
    n_corr = cfg["n_corr"]
    k0 = max(0, n_corr // 2 - n_lags // 2)
    k1 = min(n_corr, k0 + n_lags)
    # data window that outputs [k0, k1) read, re-indexed from 0
    lo = int(k0 * step + min(0, mo.min()))
    hi = int((k1 - 1) * step + max(0, mo.max()) + L)
    lo -= lo % step
    win = np.ascontiguousarray(d[:, :, lo:hi])
    ref = fp64.fp64_matched_filter(tp, mo, w, win, step, cfg["normalize"], True)
    out = {}
    for prec in ("fp32", "split_bf16", "bf16"):
        got = fmf.matched_filter(tp, mo, w, win, step, check_zeros=False,
                                 normalize=cfg["normalize"], precision=prec)
        err = np.abs(got.astype(np.float64) - ref)
        out[prec] = {"max": float(err.max()), "p99.9": float(np.quantile(err, 0.999))}
    arch = "cpu" if cfg["normalize"] == "short" else "precise"
    r = cpu.run_oracle(tp, mo, w, win, step, arch, cfg["normalize"], True)
    err = np.abs(r.astype(np.float64) - ref)
    out["reference_cpu_" + arch] = {"max": float(err.max()), "p99.9": float(np.quantile(err, 0.999))}
    out["subset"] = "templates 0-%d, %d outputs around the middle of the trace" % (n_templates - 1,
                                                                                   ref.shape[1])
    torch.cuda.synchronize()
    return out


def run_frontend(cfg, precision, args):
    """The drop-in call as a user of the reference makes it: fmf.matched_filter
    on the workload's numpy arrays (pageable host memory, a fresh numpy output
    per call, check_zeros='first' as the reference's default), wall clock per
    call after one untimed call."""
    import ctypes as ct
    import torch
    import fast_matched_filter_gb300 as fmf
    from fast_matched_filter_gb300 import _lib
    lib = _lib.load()
    secs, got = [], None
    ms = (ct.c_double * 5)()
    for i in range(1 + args.steps):
        got = None  # free the previous output first
        torch.cuda.synchronize()
        if i == 1:
            lib.fmf_timing_begin()
        t = time.perf_counter()
        got = fmf.matched_filter(cfg["templates"], cfg["moveouts"], cfg["weights"], cfg["data"],
                                 cfg["step"], arch="gpu", check_zeros="first",
                                 normalize=cfg["normalize"], network_sum=cfg["network_sum"],
                                 precision=precision)
        secs.append(time.perf_counter() - t)
    lib.fmf_timing_end_ex(ms, 5, None)
    med = float(np.median(secs[1:]))
    n = max(1, args.steps)
    parts = {k: ms[i] / n for i, k in enumerate(("preprocessing_ms", "kernel_ms", "input_copies_ms",
                                                 "output_copies_ms", "output_tail_ms"))}
    return {"value": cfg["macs"] / med / 1e12, "unit": UNIT, "seconds": secs[1:],
            "first_call_s": secs[0], "output_shape": list(got.shape),
            "breakdown_per_call": parts,
            "api": "fmf.matched_filter(..., arch='gpu') on numpy arrays (pageable host memory)"}


def run_e2e(cfg, dev_out, precision, args, world, lib):
    import torch
    from fast_matched_filter_gb300 import _lib
    pinned = {k: torch.from_numpy(np.ascontiguousarray(cfg[k])).pin_memory()
              for k in ("templates", "sst", "moveouts", "weights", "data")}
    host_out = torch.empty(tuple(dev_out.shape), dtype=torch.float32).pin_memory()
    T, S, C, L = cfg["templates"].shape
    N = cfg["data"].shape[-1]
    prec = _lib.PRECISIONS[precision]

    def call():
        st = lib.fmf_matched_filter_ex(
            pinned["templates"].data_ptr(), pinned["sst"].data_ptr(),
            pinned["moveouts"].data_ptr(), pinned["data"].data_ptr(),
            pinned["weights"].data_ptr(), cfg["step"], L, N, T, S, C, cfg["n_corr"],
            host_out.data_ptr(), 1 if cfg["normalize"] == "full" else 0,
            int(cfg["network_sum"]), prec, 0, None)
        _lib.check(st, lib)

    import ctypes as ct
    for _ in range(2):  # warm-up (pool growth)
        call()
    barrier(world)
    n = max(5, args.steps)
    per_step, step_parts = [], []
    ms = (ct.c_double * 5)()
    for _ in range(n):  # each step is one call; its copy/kernel spans are read after it
        lib.fmf_timing_begin()
        t = time.perf_counter()
        call()
        per_step.append(time.perf_counter() - t)
        lib.fmf_timing_end_ex(ms, 5, None)
        step_parts.append(list(ms))
    secs = dist_max(sum(per_step), world)
    h2d = sum(int(v.numel() * v.element_size()) for v in pinned.values())
    d2h = int(host_out.numel() * 4)
    wall_ms = 1e3 * secs / n
    parts = {k: sum(p[i] for p in step_parts) / n
             for i, k in enumerate(("preprocessing_ms", "kernel_ms", "input_copies_ms",
                                    "output_copies_ms", "output_tail_ms"))}
    parts["host_and_other_ms"] = wall_ms - (parts["input_copies_ms"] + parts["preprocessing_ms"]
                                            + parts["kernel_ms"] + parts["output_tail_ms"])
    return {"value": cfg["macs"] * n * world / secs / 1e12, "unit": UNIT,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": n,
            "ms_per_step": wall_ms, "step_ms": [round(1e3 * x, 2) for x in per_step],
            "step_input_copies_ms": [round(p[2], 2) for p in step_parts],
            "breakdown_per_step": parts,
            "h2d_gbs": h2d / (parts["input_copies_ms"] / 1e3) / 1e9 if parts["input_copies_ms"] else None,
            "d2h_window_gbs": d2h / (parts["output_copies_ms"] / 1e3) / 1e9
            if parts["output_copies_ms"] else None,
            "api": "fmf_matched_filter_ex (C ABI, host pointers, pinned)"}


DETECT_KW = dict(n_mad=8.0, min_separation=100, max_detections=64)


def run_detection(cfg, dev_out, world, steps=3, warmup=1):
    """fmf_detect on the device-resident search output (every template's
    valid lag window): robust threshold + peaks.  HBM-bound; the algorithmic
    bytes are one read of the rows (4 B per template*lag)."""
    import torch
    import fast_matched_filter_gb300 as fmf
    from fast_matched_filter_gb300 import _lib
    lib = _lib.load()
    T, S, C, L = cfg["templates"].shape
    N = cfg["data"].shape[-1]
    b, e = fmf.valid_lag_range(cfg["moveouts"], cfg["step"], L, N, cfg["n_corr"])
    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        fmf.detect(dev_out, lag_begin=b, lag_end=e, stream=stream, **DETECT_KW)
    torch.cuda.synchronize()
    barrier(world)
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    launches = 0
    e0.record(stream)
    for _ in range(steps):
        det = fmf.detect(dev_out, lag_begin=b, lag_end=e, stream=stream, **DETECT_KW)
        launches += lib.fmf_last_launch_count()
    e1.record(stream)
    torch.cuda.synchronize()
    ms = dist_max(e0.elapsed_time(e1), world) / steps
    rows = int(np.sum(e.astype(np.int64) - b))
    peaks, peak_kind = load_peaks()
    gbs = rows * 4 / (ms / 1e3) / 1e9
    counts = det.count.cpu().numpy()
    return {"ms_per_call": ms, "rows": T, "lags": rows, "launches_per_call": launches // steps,
            "detections": int(counts[counts > 0].sum()), "settings": DETECT_KW,
            "roofline": {"bound": "hbm", "achieved": gbs, "peak": peaks["hbm_gbs"],
                         "unit": "GB/s", "frac": gbs / peaks["hbm_gbs"],
                         "traffic": profiled_detect_traffic(rows),
                         "traffic_source": "fmf_detect_500rows_day.md: DRAM bytes of one call's "
                                           "launches per row byte, scaled to these rows",
                         "peak_source": "%s hbm_gbs (copy)" % peak_kind,
                         "kernel": "fmf_detect (det_sample x2, det_count x2: one read of each "
                                   "row; det_hist x6 over the candidates, det_resolve x6, "
                                   "det_select)"}}


def profiled_detect_traffic(lags):
    """DRAM bytes of one detection call over `lags` row values, from the
    committed launch-list profile (bytes per row byte, which stays constant
    as the rows grow: every pass reads each row once)."""
    path = os.path.join(HERE, "profiles", "fmf_detect_500rows_day.md")
    try:
        with open(path) as f:
            for line in f:
                if line.startswith("dram_bytes_per_row_byte:"):
                    return float(line.split(":")[1]) * lags * 4
    except OSError:
        pass
    return None


def run_e2e_detect(cfg, precision, args, world, lib):
    """Search + detection through fmf_matched_filter_detect with pinned host
    inputs: H2D of every input inside each step, only the detections come
    back (the (T, n_corr) rows stay in device memory)."""
    import torch
    from fast_matched_filter_gb300 import _lib
    pinned = {k: torch.from_numpy(np.ascontiguousarray(cfg[k])).pin_memory()
              for k in ("templates", "sst", "moveouts", "weights", "data")}
    T, S, C, L = cfg["templates"].shape
    N = cfg["data"].shape[-1]
    m = DETECT_KW["max_detections"]
    outs = [torch.empty(T, dtype=torch.float32).pin_memory() for _ in range(3)] + [
        torch.empty(T, dtype=torch.int32).pin_memory(),
        torch.empty((T, m), dtype=torch.int32).pin_memory(),
        torch.empty((T, m), dtype=torch.float32).pin_memory()]

    def call():
        st = lib.fmf_matched_filter_detect(
            pinned["templates"].data_ptr(), pinned["sst"].data_ptr(),
            pinned["moveouts"].data_ptr(), pinned["data"].data_ptr(),
            pinned["weights"].data_ptr(), cfg["step"], L, N, T, S, C, cfg["n_corr"],
            1 if cfg["normalize"] == "full" else 0, _lib.PRECISIONS[precision],
            DETECT_KW["n_mad"], DETECT_KW["min_separation"], m,
            *[o.data_ptr() for o in outs], 0, None)
        _lib.check(st, lib)

    call()
    barrier(world)
    n = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(n):
        call()
    secs = dist_max(time.perf_counter() - t0, world)
    h2d = sum(int(v.numel() * v.element_size()) for v in pinned.values())
    d2h = sum(int(o.numel() * o.element_size()) for o in outs)
    return {"value": cfg["macs"] * n * world / secs / 1e12, "unit": UNIT,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "steps": n,
            "detections_per_step": int(outs[3].numpy().clip(min=0).sum()),
            "api": "fmf_matched_filter_detect (C ABI, host pointers, pinned; search + "
                   "threshold + peaks, rows kept on the device)"}


def run_variable(args):
    """Per-channel template lengths (Fisher-z network sum) through
    fmf_matched_filter_variable_ex: device-resident inputs (value) and host
    inputs (e2e).  MACs count each channel's own length.  --precision auto
    runs the tensor-core numerators (split bf16), with the plain FP32 form
    timed beside them."""
    import torch
    from fast_matched_filter_gb300 import _lib
    torch.cuda.set_device(0)
    lib = _lib.load()
    precision = "split_bf16" if args.precision == "auto" else args.precision
    cfg = make_workload(args.workload, 0, args.templates, args.samples)
    nz = 1 if cfg["normalize"] == "full" else 0
    T, S, C, L = cfg["templates"].shape
    N = cfg["data"].shape[-1]
    n_corr = cfg["n_corr"]
    nt = np.ascontiguousarray(cfg["n_samples_template"], dtype=np.int32)
    host = {k: np.ascontiguousarray(cfg[k]) for k in ("templates", "sst", "moveouts", "weights",
                                                      "data")}
    dev = {k: torch.from_numpy(v).cuda() for k, v in host.items()}
    dnt = torch.from_numpy(nt).cuda()
    out = torch.empty((T, n_corr), dtype=torch.float32, device="cuda")
    stream = torch.cuda.current_stream()

    def timed(prec, steps, warmup, sample_clocks):
        flags = _lib.FLAG_DEVICE_POINTERS | _lib.flag_precision(prec)

        def call():
            st = lib.fmf_matched_filter_variable_ex(
                dev["templates"].data_ptr(), dev["sst"].data_ptr(), dev["moveouts"].data_ptr(),
                dev["data"].data_ptr(), dev["weights"].data_ptr(), cfg["step"], dnt.data_ptr(), N,
                T, S, C, n_corr, out.data_ptr(), nz, flags, stream.cuda_stream)
            _lib.check(st, lib)
            return lib.fmf_last_launch_count()

        for _ in range(max(warmup, 0)):
            call()
        torch.cuda.synchronize()
        launches = 0
        sampler = ClockSampler(0) if sample_clocks else contextlib.nullcontext()
        with sampler as clocks:
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(steps):
                launches += call()
            e1.record(stream)
            torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / steps
        _lib.check(lib.fmf_device_errors(), lib)
        return ms, launches, (clocks.summary() if sample_clocks else None)

    peaks, kind = load_peaks()
    fma_peak, fma_nominal, fma_src = fp32_peak(measured_fp32_tflops(lib))  # TFLOP/s

    def plain_roofline(ms):
        # the kernel runs each channel over its own taps rounded up to its 20-tap unroll
        executed = int(n_corr) * int(((nt.astype(np.int64) + 19) // 20 * 20).sum())
        achieved = 2 * cfg["macs"] / (ms / 1e3) / 1e12
        return {"bound": "fp32_fma", "achieved": achieved, "peak": fma_peak, "unit": "TFLOP/s",
                "frac": achieved / fma_peak, "nominal_peak": fma_nominal,
                "nominal_frac": achieved / fma_nominal,
                "executed_frac": 2 * executed / (ms / 1e3) / 1e12 / fma_peak,
                "traffic": None, "kernel": "plain_kernel (per-channel lengths)",
                "peak_source": fma_src}

    def tc_roofline(ms):
        bf16 = peaks.get("bf16_tflops_sustained", FALLBACK_PEAKS["bf16_tflops_sustained"])
        achieved = 2 * cfg["macs"] / (ms / 1e3) / 1e12
        executed, nb = tc_executed_macs(cfg)
        n_prod = 3 if precision == "split_bf16" else 1
        peak = bf16 / n_prod  # algorithmic FLOP/s bound: n_prod bf16 products per MAC
        ex = 2 * executed * n_prod / (ms / 1e3) / 1e12
        return {"bound": "tensor", "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
                "frac": achieved / peak, "traffic": None,
                "kernel": "tc_persistent (nb=%d, per-channel K ranges)" % nb,
                "peak_source": "%s bf16_tflops_sustained (cuBLAS bf16 GEMM, seconds-long loop) "
                               "/ %d bf16 products per multiply-accumulate" % (kind, n_prod),
                "bf16_peak": bf16, "executed_tflops": ex, "executed_frac": ex / bf16,
                "executed_over_algorithmic": executed * n_prod / cfg["macs"]}

    ms, launches, clocks = timed(precision, args.steps, args.warmup, True)
    value = cfg["macs"] / (ms / 1e3) / 1e12
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": {"fp32": "f32", "split_bf16": "bf16x3", "bf16": "bf16"}[precision],
            "data": "synthetic",
            "config": describe(cfg, {"precision": precision,
                                     "template_lengths": "400-800 per channel",
                                     "parallelism": "single GPU"}),
            "roofline": plain_roofline(ms) if precision == "fp32" else tc_roofline(ms),
            "gpu_launches": launches, "clocks": clocks}
    if precision != "fp32" and not args.no_compare:
        pms, _, _ = timed("fp32", max(1, min(args.steps, 2)), 1, False)
        pv = cfg["macs"] / (pms / 1e3) / 1e12
        line["plain_fp32"] = {"value": pv, "unit": UNIT, "ms_per_step": pms,
                              "speedup_of_headline": value / pv, "roofline": plain_roofline(pms)}
    # end to end: host inputs, synchronous entry point (inputs copied in, cc copied out)
    cc = np.zeros((T, n_corr), dtype=np.float32)

    def call_host():
        st = lib.fmf_matched_filter_variable_ex(
            host["templates"].ctypes.data, host["sst"].ctypes.data, host["moveouts"].ctypes.data,
            host["data"].ctypes.data, host["weights"].ctypes.data, cfg["step"], nt.ctypes.data, N,
            T, S, C, n_corr, cc.ctypes.data, nz, _lib.flag_precision(precision), None)
        _lib.check(st, lib)

    call_host()
    n = max(1, min(args.steps, 3))
    t0 = time.perf_counter()
    for _ in range(n):
        call_host()
    secs = (time.perf_counter() - t0) / n
    line["e2e"] = {"value": cfg["macs"] / secs / 1e12, "unit": UNIT,
                   "h2d_bytes_per_step": int(sum(v.nbytes for v in host.values()) + nt.nbytes),
                   "d2h_bytes_per_step": int(cc.nbytes), "steps": n,
                   "api": "fmf_matched_filter_variable_ex (C ABI, host pointers)"}
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(cfg)
    print(json.dumps(line))
    return 0


def run_batch(args):
    """Batched uneven searches: one graph (preprocessing + persistent tile-queue
    launch) vs the same searches as sequential plain FP32 calls and as
    sequential tensor-core calls."""
    import torch

    import fast_matched_filter_gb300 as fmf
    from fast_matched_filter_gb300 import synthetic
    torch.cuda.set_device(0)
    shapes = synthetic.config3_shapes(max_templates=args.templates or 500,
                                      max_samples=args.samples or 4320000)
    probs, total_macs = [], 0
    for sh in shapes:
        cfg = synthetic.config3_problem(sh)
        tp = cfg["templates"]
        n_corr = (sh["N"] - sh["L"]) // sh["step"] + 1
        g = [torch.from_numpy(np.ascontiguousarray(x)).cuda() for x in
             (tp, np.sum(tp ** 2, axis=-1).astype(np.float32), cfg["moveouts"], cfg["weights"],
              cfg["data"])]
        out = torch.empty((sh["T"], n_corr), dtype=torch.float32, device="cuda")
        probs.append((sh, g, out))
        total_macs += synthetic.macs(tp.shape, sh["N"], sh["step"])
    batch = fmf.Batch("split_bf16")
    for sh, g, out in probs:
        batch.add(*g, sh["step"], out, sh["normalize"], True)
    stream = torch.cuda.current_stream()

    def timeit(fn, steps, warmup):
        for _ in range(warmup):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    def sequential(prec):
        for sh, g, out in probs:
            fmf.matched_filter_device(*g, sh["step"], out, sh["normalize"], True, prec, stream)

    with ClockSampler(0) as clocks:
        ms_batch = timeit(batch.run, args.steps, max(args.warmup, 1))
    launches = batch.run()
    ms_seq_tc = timeit(lambda: sequential("split_bf16"), max(1, args.steps // 2), 1)
    ms_seq_plain = timeit(lambda: sequential("fp32"), max(1, args.steps // 2), 1)
    lib = fmf.fast_matched_filter._require_lib()
    from fast_matched_filter_gb300 import _lib
    _lib.check(lib.fmf_device_errors(), lib)
    v = total_macs / (ms_batch / 1e3) / 1e12
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": 1, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_batch, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "bf16x3", "data": "synthetic",
            "config": {"workload": "config3_64_uneven_searches", "searches": len(shapes),
                       "templates_max": args.templates or 500,
                       "samples_max": args.samples or 4320000,
                       "total_macs": total_macs, "shapes_seed": 103,
                       "form": "one CUDA graph: per-search preprocessing + persistent "
                               "tile-queue tensor-core launch"},
            "gpu_launches": launches * args.steps, "clocks": clocks.summary(),
            "sequential_split_bf16": {"value": total_macs / (ms_seq_tc / 1e3) / 1e12,
                                      "ms_per_step": ms_seq_tc},
            "sequential_plain_fp32": {"value": total_macs / (ms_seq_plain / 1e3) / 1e12,
                                      "ms_per_step": ms_seq_plain,
                                      "batched_speedup": ms_seq_plain / ms_batch}}
    batch.close()
    print(json.dumps(line))
    return 0


def main(argv=None):
    args = parse_args(argv)
    if args.impl == "reference":
        return run_reference_arm(args)
    if args.workload == "config3":
        return run_batch(args)
    if args.workload in ("variable", "variable_full"):
        return run_variable(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
