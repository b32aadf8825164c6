"""Benchmark of the GB300 RRTMG clear-sky LW+SW radiation step.

Workload: MiMA's radiation call on the T85 Gaussian grid (256 x 128 = 32768
columns, 40 layers; seeded synthetic atmospheres, synthetic LW
k-distribution, real AER SW tables).  One step = one LW + one SW call.

Default arm: the sm_103a path through the C-ABI.
  value       FP32-split columns/s with inputs resident in HBM, the LW+SW step
              captured once in a CUDA graph and replayed (device entry points)
  fp64        the same for the FP64 path (the ratio split/fp64 is the metric's
              "FP32-split vs FP64")
  e2e         FP32-split columns/s through the host-array entry points
              (rrtmg_lw_c / rrtmg_sw_c) from pinned host memory: H2D copies,
              kernels, D2H copies of all outputs in every step
  error       FP32-split vs FP64 heating-rate / OLR / surface-flux differences
              on the timed workload
  cpu_baseline the FP64 CPU oracle (C++ restatement of the reference) on the
              host cores, bounded sample
  kernels_ms  CUDA-event duration of each kernel of the split and FP64 steps;
              the roofline object is for the dominant one
  adjoint     one vector-Jacobian product against the forward it differentiates
              (FP64, and FP32/FP64-split), full Jacobians of the 256-column
              adjoint configuration
--config 2: T170 x 60 (131072 columns); --config 4: the 1,048,576 x 60 stress
ensemble (forward, forward + adjoint, memory footprint, subset errors).
--impl reference: the CPU restatement alone, all host threads, same workload.

L2 (126 MB) is flushed before every timed step by writing a 256 MB buffer on
the same stream, outside the CUDA-event interval of the step.
Multi-GPU (torchrun): each rank runs its own T85 ensemble member (weak
scaling, no collective on the data path); barrier + max over ranks.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "RRTMG LW+SW columns/s at T85×40L: FP32-split vs FP64 on GB300 at ≤0.05 K/day"
UNIT = "columns/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", type=int, default=1, help="workload configuration index (1 = T85x40)")
    ap.add_argument("--cpu-sample", type=int, default=2048, help="columns per CPU baseline step")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the adjoint cost measurement")
    ap.add_argument("--no-driver", action="store_true", help="skip the run_rrtmg (GCM slab) measurement")
    ap.add_argument("--no-clouds", action="store_true", help="skip the cloudy-step measurement")
    ap.add_argument("--members", type=int, default=32, help="stress configuration (4): ensemble members")
    ap.add_argument("--stress-adjoint", default="split", choices=["split", "fp64"],
                    help="stress configuration (4): precision of the adjoint")
    return ap.parse_args()


class ClockSampler:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.dev}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for n, v in zip(names, p[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)), "reasons": sorted(reasons),
                "samples": len(sm)}


def dominant_traffic(kernel, ncol):
    """DRAM bytes per launch of the kernel from the committed ncu summary
    (profiles/dram_traffic.json: bytes per column from one capture), scaled to
    ncol columns; None when the kernel has no entry."""
    p = ROOT / "profiles" / "dram_traffic.json"
    if not p.exists():
        return None
    t = json.loads(p.read_text()).get(kernel)
    return None if t is None else float(t["dram_bytes_per_column"]) * ncol


def executed_flops(kernel, ncol):
    """Executed FP32 operations per launch of the kernel from the committed
    ncu capture (profiles/dram_traffic.json), scaled to ncol columns."""
    p = ROOT / "profiles" / "dram_traffic.json"
    if not p.exists():
        return None
    t = json.loads(p.read_text()).get(kernel) or {}
    f = t.get("executed_fp32_flops_per_column")
    return None if f is None else float(f) * ncol


# Algorithmic FLOPs per column of the reference's clear-sky arithmetic (one
# two-stream pass, analytic exp, every operation 1), counted by the oracle's
# FLOP-count build at 20/40/60/80 layers and checked by tests/test_opcount.py.
# They are the whole LW / SW path's; the share of inatm + setcoef, which the
# prep kernels do, is 2.9 % (LW) and 0.3 % (SW) at 40 layers, the rest is the
# g-point kernels' taumol and solver.
ALG_FLOPS_LAYERS = (20, 40, 60, 80)
ALG_FLOPS_PER_COLUMN = {"lw_gpoint": (143454, 285492, 418424, 556934),
                        "sw_gpoint": (405562, 811754, 1209065, 1612670)}
ALG_FLOPS_FIT = {"lw_gpoint": (6866.845, 7733.75), "sw_gpoint": (20093.184, 5103.625)}


def algorithmic_flops(kernel, nlay):
    """Counted algorithmic FLOPs per column of the LW or SW path at nlay layers:
    interpolated between the counted layer counts, the least-squares line
    (slope, intercept) outside them."""
    Ls, ys = ALG_FLOPS_LAYERS, ALG_FLOPS_PER_COLUMN[kernel]
    if Ls[0] <= nlay <= Ls[-1]:
        return float(np.interp(nlay, Ls, ys))
    a, b = ALG_FLOPS_FIT[kernel]
    return a * nlay + b


# FP32 (non-tensor) peak of the GB300 at its 2070 MHz maximum SM clock:
# 152 SMs x 128 FP32 lanes x 2 operations per FMA.
FP32_PEAK_TFLOPS = 152 * 128 * 2 * 2.070e9 / 1e12


def measure_fp32_peak(device: int):
    """FP32 FMA rate of the device, measured (mima_gb300/csrc/fp32_peak.cu:
    8 independent FMA chains per thread, 2048 threads per SM, CUDA events):
    the best of five launches, TFLOP/s; None if the library is missing."""
    import ctypes as C
    lib_path = ROOT / "mima_gb300" / "lib" / "libfp32peak.so"
    if not lib_path.exists():
        return None
    lib = C.CDLL(str(lib_path))
    lib.fp32_peak_measure.argtypes = [C.c_int, C.POINTER(C.c_double), C.POINTER(C.c_double)]
    best = None
    for _ in range(5):
        tf, ms = C.c_double(), C.c_double()
        if lib.fp32_peak_measure(device, C.byref(tf), C.byref(ms)) != 0:
            return None
        best = tf.value if best is None else max(best, tf.value)
    return best


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text()), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "fallback"


def algorithmic_bytes(atm, lw_in, sw_in):
    """Bytes one LW+SW step must move at minimum: every input array read once,
    every output array written once (FP64)."""
    n = atm.ncol
    L = atm.nlay
    nin = sum(v.numel() for v in lw_in.values()) + sum(v.numel() for k, v in sw_in.items() if k not in lw_in)
    nout = n * (8 * (L + 1) + 4 * L)
    return 8 * (nin + nout)


def cpu_baseline(atm_full, sample, steps=1):
    """FP64 oracle (C++ restatement of the reference) on the host cores."""
    from mima_gb300 import tables
    from oracle import oracle as orc
    orc.load(tables.ensure_blob())
    orc.set_table_mode(True)
    idx = np.linspace(0, atm_full.ncol - 1, min(sample, atm_full.ncol)).astype(int)
    sub = atm_full.subset(idx)
    threads = orc.max_threads()
    orc.rrtmg_lw(sub.subset(np.arange(min(64, sub.ncol))))  # warm
    times = []
    for _ in range(steps):
        t0 = time.perf_counter()
        orc.rrtmg_lw(sub, nthreads=threads)
        orc.rrtmg_sw(sub, nthreads=threads)
        times.append(time.perf_counter() - t0)
    return sub.ncol / float(np.median(times)), threads, sub.ncol, times


def cpu_model() -> str:
    """The host CPU's model name (lscpu), else the machine type."""
    import platform
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                return ln.split(":", 1)[1].strip()
    except Exception:
        pass
    return platform.machine() or "unknown"


def run_reference(args):
    from mima_gb300 import atmosphere
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    atm = atmosphere.config_atmosphere(args.config)
    warm = max(1, min(args.warmup, 3))
    cpu_baseline(atm, min(args.cpu_sample, 256), steps=warm)
    value, threads, nsample, times = cpu_baseline(atm, args.cpu_sample, steps=args.steps)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * float(np.median(times)),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded atmospheres of the configured grid; synthetic LW k-distribution, AER SW tables)",
        "config": {"workload": workload_name(args.config, atm), "per_gpu_columns": atm.ncol,
                   "sample": f"{nsample} of the {atm.ncol} columns per step"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "model": cpu_model(), "kind": "port",
                         "sample": f"{nsample} of {atm.ncol} columns, LW+SW, FP64 lookup-table path"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference Fortran not buildable here (no Fortran compiler); C++ FP64 restatement timed",
    }
    print(json.dumps(line), flush=True)
    return 0


def graph_step(torch, r, stream, atm, d, olw, osw, precision):
    """Capture one LW+SW step in a CUDA graph through the fused entry point
    rrtmg_step_dev, which runs the SW call on a second stream of the handle
    so that the two independent calls overlap on the GPU."""
    r.set_precision(precision)

    def call():
        r.rrtmg_step_dev(stream.cuda_stream, atm.ncol, atm.nlay, d, olw, osw, atm.adjes, atm.dyofyr, atm.scon)
    with torch.cuda.stream(stream):
        call()  # first call outside capture (workspace already reserved)
    stream.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=stream):
        call()
    return g


def time_graph(torch, g, stream, flush, steps, warmup):
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            g.replay()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for e0, e1 in evs:
        with torch.cuda.stream(stream):
            flush.add_(1.0)  # 256 MB write: evicts L2 between timed steps
            e0.record(stream)
            g.replay()
            e1.record(stream)
    torch.cuda.synchronize()
    return [e0.elapsed_time(e1) for e0, e1 in evs]


def workload_name(config, atm):
    grid = {0: "T42", 1: "T85", 2: "T170", 3: "T42", 4: "T170"}[config]
    return f"{grid}x{atm.nlay} ({atm.ncol} columns, {atm.nlay} layers) LW+SW clear sky per GPU"


def kernel_bytes(name, ncol, nlay):
    """Algorithmic bytes of one launch of an FP32-split g-point kernel: the
    per-layer inputs it needs, read once in the float layout the prep kernel
    writes, and the FP64 band partials it writes once."""
    L = nlay
    if name == "lw_gpoint":
        rd = 4 * L + 4 * 25 * L + 4 * 16 * L + 4 * 16 * (L + 1) + 4 * 16 * 2 + 4 + 8 * 16
        wr = 8 * 2 * 16 * (L + 1)
    elif name == "sw_gpoint":
        rd = 4 * L + 4 * 14 * L + 4 + 4 * 14 + 8 * 5
        wr = 8 * 2 * 14 * (L + 1)
    else:
        return None
    return ncol * (rd + wr)


def dev_step(r, stream, atm, d, olw, osw):
    r.rrtmg_lw_dev(stream.cuda_stream, atm.ncol, atm.nlay, 0, 0, d, olw)
    r.rrtmg_sw_dev(stream.cuda_stream, atm.ncol, atm.nlay, 0, 0, d, osw, atm.adjes, atm.dyofyr, atm.scon)


def profile_kernels(torch, r, stream, atm, d, olw, osw, precision, flush, n):
    """Median CUDA-event duration of each kernel of the step, L2 flushed
    before each of the LW and SW calls (non-graph launches)."""
    r.set_precision(precision)
    r.set_profiling(True)
    runs = []
    try:
        for _ in range(n):
            with torch.cuda.stream(stream):
                flush.add_(1.0)
                r.rrtmg_lw_dev(stream.cuda_stream, atm.ncol, atm.nlay, 0, 0, d, olw)
                flush.add_(1.0)
                r.rrtmg_sw_dev(stream.cuda_stream, atm.ncol, atm.nlay, 0, 0, d, osw, atm.adjes, atm.dyofyr,
                               atm.scon)
            runs.append(r.profile())
    finally:
        r.set_profiling(False)
    return {k: float(np.median([x[k] for x in runs])) for k in runs[0]}


def time_calls(torch, stream, flush, fn, steps, warmup):
    """Mean CUDA-event time (ms) of fn() on stream, L2 flushed before each call."""
    with torch.cuda.stream(stream):
        for _ in range(warmup):
            fn()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    for e0, e1 in evs:
        with torch.cuda.stream(stream):
            flush.add_(1.0)
            e0.record(stream)
            fn()
            e1.record(stream)
    torch.cuda.synchronize()
    return float(np.mean([e0.elapsed_time(e1) for e0, e1 in evs]))


def measure_adjoint(torch, rrtmg, atmosphere, r, stream, atm, d, olw, osw, flush, steps, warmup):
    """Cost of the adjoint against the forward it differentiates (FP64,
    analytic transcendentals): one vector-Jacobian product over the whole
    workload, and full Jacobians of the 256-column adjoint configuration."""
    dev = d["tlay"].device
    nx, ny = rrtmg.adjoint_shape(atm.nlay)
    cot = torch.randn(ny, atm.ncol, dtype=torch.float64, device=dev)
    grad = torch.empty(nx, atm.ncol, dtype=torch.float64, device=dev)
    r.set_precision("fp64")
    r.set_transcendentals("analytic")
    try:
        fwd = lambda: dev_step(r, stream, atm, d, olw, osw)
        vjp = lambda: r.vjp_dev(stream.cuda_stream, atm.ncol, atm.nlay, d, cot, grad, atm.adjes, atm.dyofyr,
                                atm.scon)
        ms_f = time_calls(torch, stream, flush, fwd, steps, warmup)
        ms_v = time_calls(torch, stream, flush, vjp, steps, warmup)
        # FP32/FP64-split adjoint against the split forward it pairs with
        r.set_precision("split")
        ms_fs = time_calls(torch, stream, flush, fwd, steps, warmup)
        ms_vs = time_calls(torch, stream, flush, vjp, steps, warmup)
        r.set_precision("fp64")
        a3 = atmosphere.config_atmosphere(3)
        d3 = rrtmg.atm_device_inputs(a3, dev)
        nx3, ny3 = rrtmg.adjoint_shape(a3.nlay)
        jac = torch.empty(nx3, ny3, a3.ncol, dtype=torch.float64, device=dev)
        o3lw, o3sw = rrtmg.device_outputs(a3.ncol, a3.nlay, dev)
        jfn = lambda: r.jacobian_dev(stream.cuda_stream, a3.ncol, a3.nlay, d3, jac, a3.adjes, a3.dyofyr, a3.scon)
        ms_j = time_calls(torch, stream, flush, jfn, steps, warmup)
        ms_f3 = time_calls(torch, stream, flush, lambda: dev_step(r, stream, a3, d3, o3lw, o3sw), steps, warmup)
    finally:
        r.set_transcendentals("table")
    return {"precision": "fp64 (analytic transcendentals)", "forward_ms": ms_f, "vjp_ms": ms_v,
            "forward_plus_vjp_over_forward": (ms_f + ms_v) / ms_f,
            "vjp_columns_per_s": atm.ncol / (ms_v * 1e-3),
            "split": {"forward_ms": ms_fs, "vjp_ms": ms_vs, "forward_plus_vjp_over_forward": (ms_fs + ms_vs) / ms_fs,
                      "note": "FP32 dual numbers and reverse sweeps, FP64-accurate g-point sums, FP64 band sums; analytic forward"},
            "jacobian": {"workload": f"T42x40 adjoint configuration, {a3.ncol} columns", "ms": ms_j,
                         "forward_ms": ms_f3, "rows": ny3, "inputs": nx3,
                         "forward_plus_jacobian_over_forward": (ms_f3 + ms_j) / ms_f3}}


def measure_clouds(torch, rrtmg, atmosphere, r, stream, atm, d, flush, steps, warmup, dev):
    """The cloudy step on the same columns: seeded overcast clouds with the
    cloud physics (LW maximum/random overlap, cldprop inflag 2 with Fu ice and
    Hu-Stamnes liquid; SW cldprop_sw inflag 2, the same parameterisations),
    LW then SW on one stream (no graph), FP32-split and FP64, L2 flushed
    before each step; beside it the clear-sky step timed the same way.  The
    split outputs' error against the FP64 ones."""
    cl = atmosphere.cloud_physics_fields(atm, seed=2024)
    dc = {k: torch.from_numpy(np.ascontiguousarray(v)).to(dev) for k, v in cl.items()}
    flags = dict(inflag=2, iceflag=3, liqflag=1)
    dl = dict(d, **dc)
    outs = {pr: rrtmg.device_outputs(atm.ncol, atm.nlay, dev) for pr in ("split", "fp64")}

    def cloudy(pr):
        olw, osw = outs[pr]
        r.rrtmg_lw_dev(stream.cuda_stream, atm.ncol, atm.nlay, 2, 0, dl, olw, inflglw=2, iceflglw=3, liqflglw=1)
        r.rrtmg_sw_dev(stream.cuda_stream, atm.ncol, atm.nlay, 1, 0, d, osw, atm.adjes, atm.dyofyr, atm.scon,
                       cloud=dict(dc, **flags))

    res = {}
    try:
        for pr in ("split", "fp64"):
            r.set_precision(pr)
            n = steps if pr == "split" else max(2, steps // 4)
            res[pr] = time_calls(torch, stream, flush, lambda: cloudy(pr), n, warmup)
            if r.sync_status(stream.cuda_stream) != 0:
                return {"status": "error", "message": r.last_error()}
        r.set_precision("split")
        olw, osw = outs["split"]
        clear_ms = time_calls(torch, stream, flush, lambda: dev_step(r, stream, atm, d, olw, osw), steps, warmup)
        cloudy("split")
        torch.cuda.synchronize()
    finally:
        r.set_precision("split")
    (l32, s32), (l64, s64) = outs["split"], outs["fp64"]
    hr = float((l32["hr"] - l64["hr"]).abs().max())
    shr = float((s32["swhr"] - s64["swhr"]).abs().max())
    olr = float((l32["uflx"][-1] - l64["uflx"][-1]).abs().max())
    sfc = max(float((l32[k][0] - l64[k][0]).abs().max()) for k in ("uflx", "dflx"))
    sfc = max(sfc, max(float((s32[k][0] - s64[k][0]).abs().max()) for k in ("swuflx", "swdflx")))
    return {"workload": (f"{atm.ncol} columns x {atm.nlay} layers, {100 * float(cl['cldfr'].mean()):.1f} % of the "
                         "layers overcast; LW icld 2 inflglw 2 (iceflglw 3, liqflglw 1), SW icld 1 inflgsw 2 "
                         "(iceflgsw 3, liqflgsw 1)"),
            "split_ms": res["split"], "columns_per_s": atm.ncol / (res["split"] * 1e-3),
            "fp64_ms": res["fp64"], "split_over_fp64": res["fp64"] / res["split"],
            "clear_sky_same_calls_ms": clear_ms,
            "error_vs_fp64": {"lw_hr_max_kday": hr, "sw_hr_max_kday": shr, "olr_max_wm2": olr,
                              "sfc_flux_max_wm2": sfc},
            "timing": "LW then SW device calls on one stream, CUDA events, L2 flushed before each step"}


def measure_driver(torch, rrtmg, atmosphere, r, stream, dev, flush, steps, warmup, lw_sw_ms):
    """MiMA's whole radiation step (run_rrtmg with interp_temp and the zenith
    angle) on a T85 GCM slab of 256 x 128 points x 40 levels, FP32-split:
    through rrtmg_run_dev on device arrays, and end to end through
    rrtmg_run_c on page-locked host arrays."""
    slab = atmosphere.gcm_slab(256, 128, 40, seed=12346)
    prm = rrtmg.run_params()
    r.set_precision("split")
    d = {k: torch.from_numpy(np.ascontiguousarray(getattr(slab, k))).to(dev) for k in rrtmg.RUN_IN
         if getattr(slab, k) is not None}
    shp3, shp2 = (slab.sk, slab.sj, slab.si), (slab.sj, slab.si)
    out = {"tdt": torch.from_numpy(slab.tdt.copy()).to(dev),
           "coszen": torch.empty(shp2, dtype=torch.float64, device=dev),
           "flux_sw": torch.empty(shp2, dtype=torch.float64, device=dev),
           "flux_lw": torch.empty(shp2, dtype=torch.float64, device=dev)}
    call = lambda: r.run_rrtmg_dev(stream.cuda_stream, prm, slab.si, slab.sj, slab.sk, 43200, 100, 365, d, out)
    t = time_calls(torch, stream, flush, call, steps, warmup)
    ms = float(np.mean(t))
    status = r.sync_status(stream.cuda_stream)
    # host arrays: inputs in, tdt in and out, coszen and surface fluxes out
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy() if a is not None else None
    hslab = atmosphere.GcmSlab(**{k: (pin(v) if isinstance(v, np.ndarray) else v) for k, v in vars(slab).items()})
    h2d = sum(getattr(hslab, k).nbytes for k in rrtmg.RUN_IN if getattr(hslab, k) is not None) + slab.tdt.nbytes
    d2h = slab.tdt.nbytes + 3 * slab.lat.nbytes
    # page-locked outputs; tdt is updated in place step after step, as the
    # model's tendency array is
    hout = {"tdt": pin(slab.tdt), "coszen": pin(np.zeros(shp2)), "flux_sw": pin(np.zeros(shp2)),
            "flux_lw": pin(np.zeros(shp2))}
    for _ in range(max(2, min(warmup, 3))):
        r.run_rrtmg(prm, hslab, 43200, 100, out=hout)
    ts = []
    for _ in range(max(3, steps // 4)):
        t0 = time.perf_counter()
        r.run_rrtmg(prm, hslab, 43200, 100, out=hout)
        ts.append(time.perf_counter() - t0)
    host_ms = float(np.mean(ts)) * 1e3
    ncol = slab.si * slab.sj
    return {"workload": "run_rrtmg on a T85 GCM slab 256x128x40 (lonstep 1, daily-mean zenith), FP32-split",
            "device_ms": ms, "device_columns_per_s": ncol / (ms * 1e-3),
            "lw_sw_graph_ms": lw_sw_ms, "driver_overhead_ms": None if lw_sw_ms is None else ms - lw_sw_ms,
            "host_e2e_ms": host_ms, "host_e2e_columns_per_s": ncol / (host_ms * 1e-3),
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "status": status,
            "api": "rrtmg_run_dev (device arrays) / rrtmg_run_c (page-locked host arrays)"}


def run_stress(args):
    """1,048,576 x 60 stress configuration: a seeded ensemble of 32 members of
    32768 T170-like columns (60 layers, top 0.01 hPa, Ts noise 3 K), all
    resident in HBM; one launch sequence runs the FP32-split forward of every
    member, a second one the forward plus the adjoint (one vector-Jacobian
    product per member, analytic transcendentals; FP32/FP64-split by default).
    Reports columns/s of both, their cost ratio, the peak device-memory
    footprint and the FP32-split errors against FP64 (forward and adjoint) on a
    4096-column subset."""
    import torch
    from mima_gb300 import atmosphere, rrtmg
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(0)
    free0, total = torch.cuda.mem_get_info()
    r = rrtmg.RRTMG(device=0)
    members = []
    for m in range(args.members):
        a = atmosphere.config_atmosphere(4, member=m)
        members.append((a, rrtmg.atm_device_inputs(a, dev)))
    a0 = members[0][0]
    L, n = a0.nlay, a0.ncol
    nx, ny = rrtmg.adjoint_shape(L)
    olw, osw = rrtmg.device_outputs(n, L, dev)
    cot = torch.randn(ny, n, dtype=torch.float64, device=dev)
    grad = torch.empty(nx, n, dtype=torch.float64, device=dev)
    stream = torch.cuda.Stream(device=dev)
    r.reserve(n, L)

    def forward(a, d):
        r.set_precision("split")
        r.set_transcendentals("table")
        dev_step(r, stream, a, d, olw, osw)

    def adjoint(a, d):
        r.set_precision(args.stress_adjoint)
        r.set_transcendentals("analytic")
        r.vjp_dev(stream.cuda_stream, a.ncol, a.nlay, d, cot, grad, a.adjes, a.dyofyr, a.scon)

    def sequence(with_adjoint):
        for a, d in members:
            forward(a, d)
            if with_adjoint:
                adjoint(a, d)

    with torch.cuda.stream(stream):
        forward(*members[0])
        adjoint(*members[0])
    torch.cuda.synchronize()
    peak_used = total - torch.cuda.mem_get_info()[0]
    times = {}
    with ClockSampler(0) as clk:
        for key, adj, reps in (("forward", False, 3), ("forward_adjoint", True, 1)):
            ts = []
            for it in range(1 + reps):
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                with torch.cuda.stream(stream):
                    e0.record(stream)
                    sequence(adj)
                    e1.record(stream)
                torch.cuda.synchronize()
                if it >= 1:
                    ts.append(e0.elapsed_time(e1))
            times[key] = float(np.mean(ts))
    r.set_transcendentals("table")
    peak_used = max(peak_used, total - torch.cuda.mem_get_info()[0])
    # FP32-split error against FP64 on a 4096-column subset of the first member
    sub = a0.subset(np.linspace(0, n - 1, 4096).astype(int))
    r.set_precision("fp64")
    lw64, sw64 = r.lw(sub), r.sw(sub)
    r.set_precision("split")
    lw32, sw32 = r.lw(sub), r.sw(sub)
    err = {"lw_hr_max_kday": float(np.abs(lw32["hr"] - lw64["hr"]).max()),
           "sw_hr_max_kday": float(np.abs(sw32["swhr"] - sw64["swhr"]).max()),
           "olr_max_wm2": float(np.abs(lw32["uflx"][-1] - lw64["uflx"][-1]).max()),
           "sfc_flux_max_wm2": float(max(np.abs(lw32[k][0] - lw64[k][0]).max() for k in ("uflx", "dflx")))}
    # adjoint: split VJP against FP64 VJP on the same subset and cotangents
    rng = np.random.default_rng(7)
    csub = rng.standard_normal((ny, sub.ncol))
    r.set_transcendentals("analytic")
    r.set_precision("fp64")
    g64 = r.vjp(sub, csub)
    r.set_precision("split")
    g32 = r.vjp(sub, csub)
    r.set_transcendentals("table")
    scale = np.maximum(np.abs(g64), 1e-3 * np.abs(g64).max(axis=1, keepdims=True)) + 1e-300
    rel = np.abs(g32 - g64) / scale
    err["vjp_split_vs_fp64_rel_max"] = float(rel.max())
    err["vjp_split_vs_fp64_rel_p99"] = float(np.quantile(rel, 0.99))
    ncols = n * len(members)
    line = {
        "metric": METRIC, "value": ncols / (times["forward"] * 1e-3), "unit": UNIT, "n_gpus": 1,
        "steps": 3, "warmup": 1, "ms_per_step": times["forward"],
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64 (FP32-split)",
        "data": "synthetic (seeded T170-like ensemble; synthetic LW k-distribution, AER SW tables)",
        "config": {"workload": f"stress: {len(members)} members x {n} columns x {L} layers = {ncols} columns",
                   "l2": "inputs (GBs) far larger than L2"},
        "stress": {"forward_columns_per_s": ncols / (times["forward"] * 1e-3),
                   "forward_adjoint_columns_per_s": ncols / (times["forward_adjoint"] * 1e-3),
                   "forward_adjoint_over_forward": times["forward_adjoint"] / times["forward"],
                   "adjoint": (f"{'FP32/FP64-split' if args.stress_adjoint == 'split' else 'FP64'} "
                               "vector-Jacobian product per member (analytic transcendentals)"),
                   "peak_device_bytes": int(peak_used), "device_bytes_before": int(total - free0),
                   "error_vs_fp64_4096_subset": err},
        "gpu_launches": 8 * len(members) * 3,
        "clocks": clk.summary(),
    }
    print(json.dumps(line), flush=True)
    return 0


def run_ours(args):
    import torch
    from mima_gb300 import atmosphere, rrtmg
    from mima_gb300.shard import env_rank_world

    rank, world, local = env_rank_world()
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    atm = atmosphere.config_atmosphere(args.config, member=rank)
    r = rrtmg.RRTMG(device=local)
    r.reserve(atm.ncol, atm.nlay)
    d = rrtmg.atm_device_inputs(atm, dev)
    lw_keys = ("play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr",
               "cfc11vmr", "cfc12vmr", "cfc22vmr", "ccl4vmr", "emis")
    sw_keys = ("play", "plev", "tlay", "tlev", "tsfc", "h2ovmr", "o3vmr", "co2vmr", "ch4vmr", "n2ovmr", "o2vmr",
               "asdir", "asdif", "aldir", "aldif", "coszen")
    nbytes = algorithmic_bytes(atm, {k: d[k] for k in lw_keys}, {k: d[k] for k in sw_keys})
    olw64, osw64 = rrtmg.device_outputs(atm.ncol, atm.nlay, dev)
    olw32, osw32 = rrtmg.device_outputs(atm.ncol, atm.nlay, dev)
    stream = torch.cuda.Stream(device=dev)
    flush = torch.zeros(32 * 1024 * 1024, dtype=torch.float64, device=dev)
    g64 = graph_step(torch, r, stream, atm, d, olw64, osw64, "fp64")
    g32 = graph_step(torch, r, stream, atm, d, olw32, osw32, "split")

    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    launches0 = r.launch_count()
    with ClockSampler(local) as clk:
        t32 = time_graph(torch, g32, stream, flush, args.steps, args.warmup)
        t64 = time_graph(torch, g64, stream, flush, max(3, args.steps // 4), min(args.warmup, 3))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    # graph replays re-run the captured kernels: 8 launches of ours per step
    launches = 8 * args.steps
    ms32 = float(np.mean(t32))
    ms64 = float(np.mean(t64))
    if dist:
        m = torch.tensor([ms32, ms64], device=dev)
        dist.all_reduce(m, op=dist.ReduceOp.MAX)
        ms32, ms64 = m.tolist()

    # FP32-split error against FP64 on the timed workload
    hr = (olw32["hr"] - olw64["hr"]).abs()
    shr = (osw32["swhr"] - osw64["swhr"]).abs()
    olr = (olw32["uflx"][-1] - olw64["uflx"][-1]).abs()
    sfc = max(float((olw32[k][0] - olw64[k][0]).abs().max()) for k in ("uflx", "dflx"))
    sfc = max(sfc, max(float((osw32[k][0] - osw64[k][0]).abs().max()) for k in ("swuflx", "swdflx")))
    err = {"lw_hr_max_kday": float(hr.max()), "lw_hr_rms_kday": float(hr.pow(2).mean().sqrt()),
           "sw_hr_max_kday": float(shr.max()), "sw_hr_rms_kday": float(shr.pow(2).mean().sqrt()),
           "olr_max_wm2": float(olr.max()), "sfc_flux_max_wm2": sfc}

    ncol_total = atm.ncol * world
    value = ncol_total / (ms32 * 1e-3)
    fp64_value = ncol_total / (ms64 * 1e-3)

    # per-kernel durations (CUDA events around each launch on the launching stream)
    nprof = max(3, args.steps // 4)
    kms32 = profile_kernels(torch, r, stream, atm, d, olw32, osw32, "split", flush, nprof)
    kms64 = profile_kernels(torch, r, stream, atm, d, olw64, osw64, "fp64", flush, max(3, nprof // 2))
    adjoint = None
    if not args.no_adjoint:
        adjoint = measure_adjoint(torch, rrtmg, atmosphere, r, stream, atm, d, olw64, osw64, flush,
                                  max(3, args.steps // 4), min(args.warmup, 3))

    clouds = None
    if not args.no_clouds:
        clouds = measure_clouds(torch, rrtmg, atmosphere, r, stream, atm, d, flush, max(3, args.steps // 4),
                                min(args.warmup, 3), dev)

    driver = None
    if not args.no_driver:
        # the driver slab is the T85 x 40 grid: its LW + SW step is this run's
        # only for that workload
        driver = measure_driver(torch, rrtmg, atmosphere, r, stream, dev, flush, max(3, args.steps // 4),
                                min(args.warmup, 3), ms32 if args.config == 1 else None)

    # end to end through the host-array entry points, pinned host memory
    e2e = None
    if not args.no_e2e:
        r.set_precision("split")
        pin = {}
        for k, v in d.items():
            pin[k] = v.cpu().pin_memory()
        hp = lambda k: pin[k].numpy()
        # the two calls copy their own inputs: the arrays both take move twice
        h2d = sum(pin[k].numel() * 8 for k in lw_keys) + sum(pin[k].numel() * 8 for k in sw_keys)
        d2h = 8 * atm.ncol * (8 * (atm.nlay + 1) + 4 * atm.nlay)
        # page-locked output arrays, as for the inputs
        pout = lambda rows: torch.empty((rows, atm.ncol), dtype=torch.float64).pin_memory().numpy()
        L = atm.nlay
        lw_out = {k: pout(L + 1) for k in ("uflx", "dflx", "uflxc", "dflxc")}
        lw_out.update(hr=pout(L), hrc=pout(L))
        sw_out = {k: pout(L + 1) for k in ("swuflx", "swdflx", "swuflxc", "swdflxc")}
        sw_out.update(swhr=pout(L), swhrc=pout(L))
        def host_step():
            r.rrtmg_lw(atm.ncol, atm.nlay, 0, 0, *[hp(k) for k in lw_keys], out=lw_out)
            r.rrtmg_sw(atm.ncol, atm.nlay, 0, 0, *[hp(k) for k in sw_keys], atm.adjes, atm.dyofyr, atm.scon,
                       out=sw_out)
        for _ in range(max(2, min(args.warmup, 3))):
            host_step()
        ts = []
        for _ in range(max(3, args.steps // 4)):
            t0 = time.perf_counter()
            host_step()
            ts.append(time.perf_counter() - t0)
        e2e = {"value": atm.ncol * world / float(np.mean(ts)), "unit": UNIT, "h2d_bytes_per_step": h2d,
               "d2h_bytes_per_step": d2h, "api": "rrtmg_lw_c + rrtmg_sw_c (host arrays), FP32-split"}

    if rank != 0:
        if dist:
            dist.destroy_process_group()
        return 0
    cpu_value, threads, nsample, _ = cpu_baseline(atm, min(args.cpu_sample, 2048), steps=1)
    peaks, src = measured_peaks()
    dom = max(("lw_gpoint", "sw_gpoint"), key=lambda k: kms32[k])
    dom_bytes = kernel_bytes(dom, atm.ncol, atm.nlay)
    achieved = dom_bytes / (kms32[dom] * 1e-3) / 1e9
    traffic = dominant_traffic(dom, atm.ncol)
    flops = executed_flops(dom, atm.ncol)
    compute = None
    fp32_peak = measure_fp32_peak(local)
    peak32 = fp32_peak or FP32_PEAK_TFLOPS
    if flops:
        tf = flops / (kms32[dom] * 1e-3) / 1e12
        compute = {"bound": "fp32 pipe", "achieved": tf, "peak": peak32, "unit": "TFLOP/s",
                   "frac": tf / peak32, "executed_flops_per_launch": flops,
                   "peak_source": ("measured: FFMA-chain microkernel, best of 5 launches (CUDA events)"
                                   if fp32_peak else "nominal (microkernel library missing)"),
                   "peak_nominal": FP32_PEAK_TFLOPS,
                   "note": "executed FP32 operations (ncu, FMA = 2) / CUDA-event kernel time; nominal peak "
                           "152 SMs x 128 lanes x 2 x 2.07 GHz"}
        alg = algorithmic_flops(dom, atm.nlay) * atm.ncol
        atf = alg / (kms32[dom] * 1e-3) / 1e12
        compute.update({"algorithmic_flops_per_launch": alg, "algorithmic_achieved": atf,
                        "algorithmic_frac": atf / peak32})
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64 (FP32-split)",
        "data": "synthetic (seeded atmospheres of the configured grid; synthetic LW k-distribution, AER SW tables)",
        "config": {"workload": workload_name(args.config, atm),
                   "per_gpu_columns": atm.ncol, "l2": "flushed (256 MB write) before every timed step",
                   "graph": "LW+SW step captured in one CUDA graph", "parallelism": f"columns x{world}"},
        "fp64": {"value": fp64_value, "unit": UNIT, "ms_per_step": ms64},
        "split_over_fp64": fp64_value and value / fp64_value,
        "error_vs_fp64": err,
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": traffic, "kernel": f"{dom} (FP32-split)",
                     "algorithmic_bytes_per_launch": dom_bytes, "kernel_ms": kms32[dom],
                     "note": (f"peak {src}; the g-point solvers are latency/FP-pipe bound, not HBM bound: "
                              f"step algorithmic bytes {nbytes}"),
                     "compute": compute},
        "kernels_ms": {"split": kms32, "fp64": kms64},
        "cpu_baseline": {"value": cpu_value, "unit": UNIT, "cores": threads, "model": cpu_model(), "kind": "port",
                         "sample": f"{nsample} of {atm.ncol} columns, LW+SW FP64 C++ restatement"},
    }
    if e2e:
        line["e2e"] = e2e
    if adjoint:
        line["adjoint"] = adjoint
    if driver:
        line["driver"] = driver
    if clouds:
        line["clouds"] = clouds
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.config == 4:
        return run_stress(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
