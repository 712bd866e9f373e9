"""Benchmark of the spatial-convolution hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision bf16|fp32] [--no-secondary]

Headline (`value`): af_convolve2_nn forward + data gradient + filter
gradient TFLOP/s on the 128x128x64x32 signal / 3x3x64x128 filter workload
(stride 1, padding 1, dilation 1; 3 x 77.31 GFLOP per step), inputs resident
in HBM, each step one pass of forward and both gradients.  Inputs are
seeded synthetic N(0,1) / He-normal arrays (no dataset).  Timing: CUDA events
on the launching stream around each step; between steps a 512 MB buffer is
written to flush the 126 MB L2.

`secondary` reports the bandwidth-bound direct convolutions (64 images of
2048x2048 with the 15-tap separable filter in f32 and u8, 64 distinct 7x7
filters in SAME batch mode, a 256^3 volume with a 3x3x3 filter) as HBM GB/s
against the measured copy bandwidth.

`e2e` is the same headline metric through the C ABI with host buffers:
af_create_array from pinned host memory, the three calls, af_get_data_ptr
back to host, all inside the timed region.

`--impl reference` times the reference's CPU algorithm for the same metric
(the oracle's C restatement of unwrap/wrap plus the BLAS sgemm bundled with
numpy, as the reference CPU backend's unwrap + CBLAS path) on a bounded
sample, with all host threads the BLAS can use.

Multi-GPU: the path does not shard (replicas only): each rank runs the same
workload on its own GPU; `value` sums the ranks' work over the slowest rank's
time.
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

METRIC = ("conv2_nn fwd+bwd TFLOP/s BF16-TC vs FP32 (rel err≤2e-2); convolve2 HBM GB/s")
NN_SHAPE = dict(W=128, H=128, C=64, N=32, fw=3, fh=3, K=128, stride=(1, 1), pad=(1, 1), dil=(1, 1))
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of each
# tensor-core kernel on NN_SHAPE, from one ncu capture of `bench.py --only
# fwd|dgrad|wgrad` (ncu cannot run inside the timed bench)
NCU_TRAFFIC = {"tc_fwd_kernel": 67.30e6 + 212.86e6, "tc_dgrad_kernel": 134.60e6 + 90.88e6,
               "tc_wgrad_kernel": 206.02e6 + 18.06e6}


def nn_flops(s=NN_SHAPE) -> float:
    Wo = 1 + (s["W"] + 2 * s["pad"][0] - ((s["fw"] - 1) * s["dil"][0] + 1)) // s["stride"][0]
    Ho = 1 + (s["H"] + 2 * s["pad"][1] - ((s["fh"] - 1) * s["dil"][1] + 1)) // s["stride"][1]
    return 2.0 * Wo * Ho * s["N"] * s["K"] * s["fw"] * s["fh"] * s["C"]


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", d["bf16_tflops"]),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "source": "fallback"}


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "20"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except FileNotFoundError:
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# our implementation
# ---------------------------------------------------------------------------
def _timed_steps(step_fn, steps: int, warmup: int, flush) -> tuple[float, list[float]]:
    import torch

    for _ in range(warmup):
        step_fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        flush()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        step_fn()
        b.record()
        b.synchronize()
        times.append(a.elapsed_time(b))
    return sum(times), times


def run_ours(args, peaks, rank: int, world: int) -> dict:
    import torch

    import arrayfire_gb300 as af

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    af.set_stream(torch.cuda.current_stream())
    L = af.lib()
    s = NN_SHAPE
    g = np.random.Generator(np.random.Philox(1234 + rank))
    X = np.asfortranarray(g.standard_normal((s["W"], s["H"], s["C"], s["N"]), dtype=np.float32))
    std = np.sqrt(2.0 / (s["fw"] * s["fh"] * s["C"]))
    Wt = np.asfortranarray((g.standard_normal((s["fw"], s["fh"], s["C"], s["K"])) * std
                            ).astype(np.float32))
    Xa, Wa = af.Array.from_numpy(X), af.Array.from_numpy(Wt)
    st, pd, dl = s["stride"], s["pad"], s["dil"]
    prec = args.precision
    try:
        Y = af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec)
    except af.AfError as e:
        if prec == "fp32" or e.code != af.AF_ERR_NOT_SUPPORTED:
            raise
        prec = "fp32"
        Y = af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec)
    Gd = np.asfortranarray(g.standard_normal(Y.dims, dtype=np.float32))
    Ga = af.Array.from_numpy(Gd)
    flush_buf = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def flush():
        flush_buf.zero_()

    def step():
        # forward, then both input gradients in one call (one shared bf16
        # copy of the incoming gradient)
        y = af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec)
        dx, dw, _ = af.convolve2_gradients_nn(Ga, Xa, Wa, st, pd, dl, precision=prec)
        return y, dx, dw

    # parity of this exact workload against FP64 on sampled points
    y, dx, dw = step()
    import oracle.oracle as O  # checker only

    idx = g.integers(0, int(np.prod(Y.dims)), 256)
    ref = O.nn_forward_points_f64(X, Wt, st, pd, dl, idx)
    got = y.to_numpy().ravel(order="F")[idx].astype(np.float64)
    rel_fwd = float(np.linalg.norm(got - ref) / np.linalg.norm(ref))
    maxabs_fwd = float(np.abs(got - ref).max())
    idx2 = g.integers(0, X.size, 128)
    ref2 = O.nn_data_grad_points_f64(Gd, list(X.shape), Wt, st, pd, dl, idx2)
    got2 = dx.to_numpy().ravel(order="F")[idx2].astype(np.float64)
    rel_dx = float(np.linalg.norm(got2 - ref2) / np.linalg.norm(ref2))
    idx3 = g.integers(0, Wt.size, 64)
    ref3 = O.nn_filter_grad_points_f64(Gd, X, list(Wt.shape), st, pd, dl, idx3)
    got3 = dw.to_numpy().ravel(order="F")[idx3].astype(np.float64)
    rel_dw = float(np.linalg.norm(got3 - ref3) / np.linalg.norm(ref3))
    del y, dx, dw

    L.afgb_kernel_timing(1)
    launches0 = af.launch_count()
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    torch.cuda.synchronize()
    clock = ClockSampler(dev)
    clock.start()
    total_ms, times = _timed_steps(step, args.steps, args.warmup, flush)
    clocks = clock.stop()
    launches = af.launch_count() - launches0
    torch.cuda.synchronize()

    # dominant kernel timing (events around each launch, same stream)
    import ctypes

    kt = {}
    for name in ("simt_fwd_kernel", "simt_dgrad_kernel", "simt_wgrad_kernel", "tc_fwd_kernel",
                 "tc_dgrad_kernel", "tc_wgrad_kernel", "tc_convert_kernel", "wgrad_reduce_kernel"):
        c = ctypes.c_ulonglong()
        ms = ctypes.c_double()
        L.afgb_kernel_time(name.encode(), ctypes.byref(c), ctypes.byref(ms))
        if c.value:
            kt[name] = (c.value, ms.value)
    L.afgb_kernel_timing(0)
    flops = nn_flops()
    steps_total = args.warmup + args.steps
    value = 3 * flops * args.steps / (total_ms / 1e3) / 1e12

    mains = {k: v for k, v in kt.items() if k.endswith(("fwd_kernel", "dgrad_kernel", "wgrad_kernel"))}
    dom = max(mains.items(), key=lambda kv: kv[1][1]) if mains else None
    roofline = None
    if dom:
        name, (cnt, ms) = dom
        avg_s = ms / cnt / 1e3
        achieved = flops / avg_s / 1e12
        peak = peaks["bf16_tflops"]
        roofline = {"bound": "tensor", "kernel": name, "achieved": round(achieved, 2),
                    "peak": peak, "unit": "TFLOP/s", "frac": round(achieved / peak, 4),
                    "peak_source": peaks["source"] + " bf16 dense",
                    "traffic": NCU_TRAFFIC.get(name) if prec == "bf16" else None,
                    "traffic_source": "ncu capture, one launch (bytes)",
                    "launches": cnt, "avg_ms": round(ms / cnt, 4)}

    # e2e through the C ABI with pinned host buffers
    e2e = run_e2e(af, X, Wt, Gd, prec, args)

    # the plain FP32 CUDA-core path on the same workload (the >= 5x target's
    # denominator), fewer steps
    fp32 = None
    if prec != "fp32":
        def step32():
            y = af.convolve2_nn(Xa, Wa, st, pd, dl)
            dx, dw, _ = af.convolve2_gradients_nn(Ga, Xa, Wa, st, pd, dl)
            return y, dx, dw
        k32 = max(3, min(args.steps, 5))
        t32, _ = _timed_steps(step32, k32, 3, flush)
        v32 = 3 * flops * k32 / (t32 / 1e3) / 1e12
        fp32 = {"value": v32, "ms_per_step": t32 / k32, "unit": "TFLOP/s",
                "speedup_of_" + prec: value / v32}

    res = {
        "value": value, "ms_per_step": total_ms / args.steps, "precision": prec,
        "errors_vs_fp64": {"fwd_rel": rel_fwd, "fwd_maxabs": maxabs_fwd, "dgrad_rel": rel_dx,
                           "wgrad_rel": rel_dw, "points": [256, 128, 64]},
        "kernel_times_ms": {k: round(v[1] / v[0], 4) for k, v in kt.items()},
        "roofline": roofline, "clocks": clocks, "e2e": e2e, "fp32_path": fp32,
        "gpu_launches": int(launches), "step_times_ms": [round(t, 4) for t in times],
    }
    if not args.no_secondary:
        res["secondary"] = run_direct_workloads(af, peaks, args)
        res["cnn4"] = run_cnn(af, args)
    return res


def run_e2e(af, X, Wt, Gd, prec, args) -> dict:
    import ctypes

    import torch

    L = af.lib()
    s = NN_SHAPE
    st, pd, dl = s["stride"], s["pad"], s["dil"]
    pin = {k: torch.from_numpy(np.ascontiguousarray(v.ravel(order="F"))).pin_memory()
           for k, v in (("x", X), ("w", Wt), ("g", Gd))}
    Wo, Ho = X.shape[0], X.shape[1]
    y_host = torch.empty(Wo * Ho * s["K"] * s["N"], dtype=torch.float32).pin_memory()
    dx_host = torch.empty(X.size, dtype=torch.float32).pin_memory()
    dw_host = torch.empty(Wt.size, dtype=torch.float32).pin_memory()

    def mk(t, dims):
        out = ctypes.c_void_p()
        d = (ctypes.c_longlong * 4)(*dims)
        af._check(L.af_create_array(ctypes.byref(out), ctypes.c_void_p(t.data_ptr()), 4, d, af.f32))
        return af.Array(out.value)

    def step():
        Xa = mk(pin["x"], X.shape)
        Wa = mk(pin["w"], Wt.shape)
        Ga = mk(pin["g"], Gd.shape)
        y = af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec)
        dx, dw, _ = af.convolve2_gradients_nn(Ga, Xa, Wa, st, pd, dl, precision=prec)
        af._check(L.af_get_data_ptr(ctypes.c_void_p(y_host.data_ptr()), y.handle))
        af._check(L.af_get_data_ptr(ctypes.c_void_p(dx_host.data_ptr()), dx.handle))
        af._check(L.af_get_data_ptr(ctypes.c_void_p(dw_host.data_ptr()), dw.handle))

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    h2d = (X.size + Wt.size + Gd.size) * 4
    d2h = (y_host.numel() + dx_host.numel() + dw_host.numel()) * 4
    return {"value": 3 * nn_flops() * args.steps / dt / 1e12, "unit": "TFLOP/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": dt * 1e3 / args.steps}


CNN_CHANNELS = [(3, 32), (32, 64), (64, 128), (128, 128)]
CNN_GEOMS = [((2, 2), (1, 1), (1, 1)), ((2, 2), (1, 1), (1, 1)), ((1, 1), (1, 1), (1, 1)),
             ((1, 1), (2, 2), (2, 2))]


def _nn_out_hw(h, w, k, s, p, d):
    return (1 + (h + 2 * p[1] - ((k - 1) * d[1] + 1)) // s[1],
            1 + (w + 2 * p[0] - ((k - 1) * d[0] + 1)) // s[0])


def run_cnn(af, args) -> dict:
    """Four conv2_nn + ReLU layers on 224x224x3x64 (loss = sum of squares of
    the output), forward + backward with activation recomputation, BF16 and
    the plain FP32 path: step time, useful TFLOP/s, peak device memory and
    the error of each filter gradient against the same network in FP64."""
    import torch
    import torch.nn.functional as F

    from arrayfire_gb300.autograd import cnn_step
    from arrayfire_gb300.autograd import nn_flops as layer_flops

    gen = torch.Generator(device="cuda").manual_seed(5)
    n = 64
    x0 = torch.rand((n, 3, 224, 224), device="cuda", generator=gen) * 2 - 1
    ws = [torch.randn((k, c, 3, 3), device="cuda", generator=gen) * (2.0 / (9 * c)) ** 0.5
          for c, k in CNN_CHANNELS]
    # useful work: every layer's forward and filter gradient, data gradients of layers 2-4
    shape, fl, patch = tuple(x0.shape), [], []
    for (c, k), (st, pd, dl) in zip(CNN_CHANNELS, CNN_GEOMS):
        fl.append(layer_flops(shape, (k, c, 3, 3), st, pd, dl))
        ho, wo = _nn_out_hw(shape[2], shape[3], 3, st, pd, dl)
        patch.append(wo * ho * 9 * c * n * 4)  # the reference's unwrap buffer of this layer
        shape = (n, k, ho, wo)
    useful = 2 * sum(fl) + sum(fl[1:])

    # FP64 reference gradients (torch float64 on the flipped filters)
    wl = [w.double().requires_grad_() for w in ws]
    h = x0.double()
    for w, (st, pd, dl) in zip(wl, CNN_GEOMS):
        h = torch.relu(F.conv2d(h, w.flip([2, 3]), stride=(st[1], st[0]), padding=(pd[1], pd[0]),
                                dilation=(dl[1], dl[0])))
    (h ** 2).sum().backward()
    ref = [w.grad for w in wl]
    del wl, h
    torch.cuda.empty_cache()

    out = {"workload": "4 x (conv2_nn + ReLU), input 224x224x3x64 U[-1,1), 3->32 s2, 32->64 s2, "
                       "64->128, 128->128 d2 p2; loss = sum(out^2)",
           "useful_gflop_per_step": round(useful / 1e9, 2),
           "reference_unwrap_bytes": {"largest_layer": int(max(patch)), "all_layers": int(sum(patch))}}
    for prec in ("bf16", "fp32"):
        for _ in range(2):
            loss, grads, rfl = cnn_step(x0, ws, CNN_GEOMS, precision=prec, recompute=True)
        del grads
        torch.cuda.synchronize()
        af.device_mem_peak(reset=True)
        base = torch.cuda.memory_allocated()
        torch.cuda.reset_peak_memory_stats()
        loss, grads, rfl = cnn_step(x0, ws, CNN_GEOMS, precision=prec, recompute=True)
        torch.cuda.synchronize()
        lib_peak = af.device_mem_peak()
        torch_peak = torch.cuda.max_memory_allocated() - base
        errs = [float(torch.linalg.vector_norm(g.double() - r) / torch.linalg.vector_norm(r))
                for g, r in zip(grads, ref)]
        del grads
        k = 5
        tot = 0.0
        for _ in range(k):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            loss, grads, rfl = cnn_step(x0, ws, CNN_GEOMS, precision=prec, recompute=True)
            b.record()
            b.synchronize()
            tot += a.elapsed_time(b)
            del grads
        ms = tot / k
        out[prec] = {"ms_per_step": round(ms, 3), "TFLOP/s": round(useful / (ms / 1e3) / 1e12, 2),
                     "recompute_gflop": round(rfl / 1e9, 2),
                     "peak_library_bytes": int(lib_peak), "peak_torch_harness_bytes": int(torch_peak),
                     "filter_grad_rel_err_vs_fp64": [float(f"{e:.3e}") for e in errs]}
    out["bf16_speedup_over_fp32"] = round(out["fp32"]["ms_per_step"] / out["bf16"]["ms_per_step"], 2)
    return out


def run_direct_workloads(af, peaks, args) -> dict:
    """Bandwidth-bound direct convolutions (64 x 2048^2 separable and 7x7,
    256^3 volume) and the patch / FFT lines, GB/s of
    algorithmic traffic (each input and output counted once)."""
    import ctypes

    import torch

    L = af.lib()
    g = np.random.Generator(np.random.Philox(77))
    flush_buf = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    out = {}

    def measure(name, fn, nbytes, kernel):
        for _ in range(3):
            r = fn()
        del r
        torch.cuda.synchronize()
        L.afgb_kernel_timing(1)
        tot = 0.0
        steps = max(3, min(args.steps, 10))
        for _ in range(steps):
            flush_buf.zero_()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record()
            r = fn()
            b.record()
            b.synchronize()
            tot += a.elapsed_time(b)
            del r
        c = ctypes.c_ulonglong()
        ms = ctypes.c_double()
        for cand in kernel:  # the first candidate that ran is the one reported
            L.afgb_kernel_time(cand.encode(), ctypes.byref(c), ctypes.byref(ms))
            if c.value:
                kernel = cand
                break
        else:
            kernel = kernel[0]
        L.afgb_kernel_timing(0)
        call_ms = tot / steps
        k_ms = ms.value / c.value if c.value else None
        gbs = nbytes / (call_ms / 1e3) / 1e9
        kgbs = nbytes / (k_ms / 1e3) / 1e9 if k_ms else None
        out[name] = {"ms": round(call_ms, 4), "GB/s": round(gbs, 1),
                     "kernel": kernel, "kernel_ms": round(k_ms, 4) if k_ms else None,
                     "kernel_GB/s": round(kgbs, 1) if kgbs else None,
                     "frac_of_hbm": round((kgbs or gbs) / peaks["hbm_gbs"], 4),
                     "bytes": int(nbytes)}

    # 64 x 2048 x 2048 separable 15-tap, f32 and u8, LHS batch
    t = g.standard_normal(15)
    cf = (t / t.sum()).astype(np.float32)
    t = g.standard_normal(15)
    rf = (t / t.sum()).astype(np.float32)
    CF, RF = af.Array.from_numpy(cf), af.Array.from_numpy(rf)
    xs = torch.rand(64, 2048, 2048, device="cuda")
    S = af.Array.view_torch(xs)
    n = xs.numel()
    measure("sep15_f32_64x2048x2048", lambda: af.convolve2_separable(CF, RF, S), n * 8 + 120,
            ("sep_tma_kernel", "sep_fused_kernel"))
    xu = torch.randint(0, 256, (64, 2048, 2048), dtype=torch.uint8, device="cuda")
    SU = af.Array.view_torch(xu)
    measure("sep15_u8_64x2048x2048", lambda: af.convolve2_separable(CF, RF, SU), n * 2 + 120,
            ("sep_tma_kernel", "sep_fused_kernel"))
    del SU, xu
    # SAME batch, 64 distinct 7x7 filters (AF_CONV_SPATIAL: AUTO would pick FFT)
    f7 = g.standard_normal((7, 7, 64))
    f7 = (f7 / f7.sum(axis=(0, 1), keepdims=True)).astype(np.float32)
    F7 = af.Array.from_numpy(np.asfortranarray(f7))
    measure("same7x7_f32_64x2048x2048",
            lambda: af.convolve2(S, F7, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL),
            n * 8 + f7.size * 4, ("conv2_tma_kernel", "conv2_tile_kernel"))
    # a 31x31 filter: AUTO takes the frequency-domain route (the whole
    # pipeline is timed: pads, cuFFT transforms, spectrum product, crop)
    f31 = g.standard_normal((31, 31))
    F31 = af.Array.from_numpy(np.asfortranarray((f31 / f31.sum()).astype(np.float32)))
    measure("fft31x31_f32_64x2048x2048",
            lambda: af.convolve2(S, F31, af.AF_CONV_DEFAULT, af.AF_CONV_AUTO),
            n * 8 + 31 * 31 * 4, ("fft_pipeline",))
    # several transform passes over 2304x2187 padded slices: its GB/s above
    # counts input + output once; the direct-convolution work it replaces is
    # 2*31*31 flops per output
    e = out["fft31x31_f32_64x2048x2048"]
    e["equivalent_direct_TFLOP/s"] = round(2 * 31 * 31 * n / (e["ms"] / 1e3) / 1e12, 1)
    e["bound"] = "cuFFT transforms (multi-pass), not one HBM pass"
    del S, xs
    # 256^3 volume, 3x3x3
    v = torch.rand(256, 256, 256, device="cuda")
    V = af.Array.view_torch(v)
    k3 = g.standard_normal((3, 3, 3))
    F3 = af.Array.from_numpy(np.asfortranarray((k3 / k3.sum()).astype(np.float32)))
    measure("conv3_3x3x3_f32_256^3_default",
            lambda: af.convolve3(V, F3, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL),
            v.numel() * 8 + 108, ("conv3_tma_kernel", "conv3_tile_kernel", "conv_generic_kernel"))
    measure("conv3_3x3x3_f32_256^3_expand",
            lambda: af.convolve3(V, F3, af.AF_CONV_EXPAND, af.AF_CONV_SPATIAL),
            v.numel() * 4 + 258 ** 3 * 4 + 108, ("conv3_tma_kernel", "conv3_tile_kernel", "conv_generic_kernel"))
    del V, v
    # 1-D: 64 signals of 2^20 samples, a 31-tap filter (LHS batch)
    s1 = torch.rand(64, 1 << 20, device="cuda")
    S1 = af.Array.view_torch(s1)
    k1 = g.standard_normal(31)
    F1 = af.Array.from_numpy((k1 / k1.sum()).astype(np.float32))
    measure("conv1_31tap_f32_64x1M", lambda: af.convolve1(S1, F1, af.AF_CONV_DEFAULT,
                                                          af.AF_CONV_SPATIAL),
            s1.numel() * 8 + 124, ("conv1_tile_kernel", "conv_generic_kernel"))
    del S1, s1
    # af_unwrap / af_wrap of the NN image (128x128x64x32 f32, 3x3 windows,
    # stride 1, padding 1): the 9x larger patch matrix is written / read once
    xi = torch.rand(32, 64, 128, 128, device="cuda")
    XI = af.Array.view_torch(xi)
    ni = xi.numel()
    measure("unwrap_3x3_f32_128x128x64x32", lambda: af.unwrap(XI, 3, 3, 1, 1, 1, 1),
            ni * 4 * 10, ("unwrap_rows_kernel", "unwrap_kernel"))
    U = af.unwrap(XI, 3, 3, 1, 1, 1, 1)
    measure("wrap_3x3_f32_128x128x64x32", lambda: af.wrap(U, 128, 128, 3, 3, 1, 1, 1, 1),
            ni * 4 * 10, ("wrap_tiled_kernel", "wrap_kernel"))
    del U
    # the same with is_column = false (patch elements along dim 1)
    measure("unwrap_rows_3x3_f32_128x128x64x32",
            lambda: af.unwrap(XI, 3, 3, 1, 1, 1, 1, False), ni * 4 * 10,
            ("unwrap_rows_kernel", "unwrap_kernel"))
    R = af.unwrap(XI, 3, 3, 1, 1, 1, 1, False)
    measure("wrap_rows_3x3_f32_128x128x64x32",
            lambda: af.wrap(R, 128, 128, 3, 3, 1, 1, 1, 1, False), ni * 4 * 10,
            ("wrap_rows_kernel", "wrap_kernel"))
    return out


# ---------------------------------------------------------------------------
# CPU baseline: the reference's algorithm on the host cores
# ---------------------------------------------------------------------------
def cpu_nn_sample(seconds_budget: float = 20.0) -> dict:
    """Forward + both gradients of the headline workload for a subset of the
    batch (images of the same 128x128x64 shape), timed on the host:
    oracle unwrap/wrap (C restatement of the reference CPU kernels) + numpy's
    BLAS sgemm in place of CBLAS (src/backend/cpu/convolve.cpp:123-243)."""
    import oracle.oracle as O

    s = NN_SHAPE
    st, pd, dl = s["stride"], s["pad"], s["dil"]
    g = np.random.Generator(np.random.Philox(99))
    nimg = 1
    X = np.asfortranarray(g.standard_normal((s["W"], s["H"], s["C"], nimg), dtype=np.float32))
    Wt = np.asfortranarray((g.standard_normal((s["fw"], s["fh"], s["C"], s["K"])) * 0.06
                            ).astype(np.float32))
    Gd = np.asfortranarray(g.standard_normal((s["W"], s["H"], s["K"], nimg), dtype=np.float32))
    fd = Wt.shape
    wsz = fd[0] * fd[1]

    def one():
        y = O.nn_forward_unwrap_gemm_f32(X, Wt, st, pd, dl)
        cols = O.unwrap(X, fd[0], fd[1], st[0], st[1], pd[0], pd[1], dl[0], dl[1])
        npix = cols.shape[1]
        A = np.ascontiguousarray(cols.transpose(1, 3, 2, 0)).reshape(npix * nimg, s["C"] * wsz)
        G2 = np.asfortranarray(Gd).reshape(npix, s["K"], nimg, order="F").transpose(2, 0, 1
                                                                                     ).reshape(-1, s["K"])
        wflip = Wt[::-1, ::-1, :, :]
        B = np.ascontiguousarray(wflip.reshape(wsz, s["C"], s["K"], order="F").transpose(1, 0, 2)
                                 ).reshape(s["C"] * wsz, s["K"])
        dw = A.T @ G2
        colsg = (G2 @ B.T).reshape(nimg, npix, s["C"], wsz).transpose(3, 1, 2, 0)
        dx = O.wrap_dilated(np.asfortranarray(colsg), list(X.shape), fd[0], fd[1], st[0], st[1],
                            pd[0], pd[1], dl[0], dl[1])
        return y, dx, dw

    one()
    t0 = time.perf_counter()
    reps = 0
    while True:
        one()
        reps += 1
        if time.perf_counter() - t0 > seconds_budget or reps >= 20:
            break
    dt = (time.perf_counter() - t0) / reps
    flops = 3 * nn_flops() * nimg / s["N"]
    return {"value": flops / dt / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(),
            "kind": "port",
            "sample": f"{nimg} of {s['N']} images per step (fwd+dgrad+wgrad), {reps} reps; "
                      "oracle unwrap/wrap + numpy BLAS sgemm",
            "seconds_per_step": dt}


def run_only(args) -> None:
    """One operation of the bench workload, same shapes and inputs."""
    import torch

    import arrayfire_gb300 as af

    torch.cuda.set_device(0)
    af.set_stream(torch.cuda.current_stream())
    s = NN_SHAPE
    st, pd, dl = s["stride"], s["pad"], s["dil"]
    g = np.random.Generator(np.random.Philox(1234))
    if args.only == "cnn":
        from arrayfire_gb300.autograd import cnn_step

        gen = torch.Generator(device="cuda").manual_seed(5)
        x0 = torch.rand((64, 3, 224, 224), device="cuda", generator=gen) * 2 - 1
        ws = [torch.randn((k, c, 3, 3), device="cuda", generator=gen) * (2.0 / (9 * c)) ** 0.5
              for c, k in CNN_CHANNELS]
        prec = "fp32" if args.precision == "fp32" else "bf16"
        fn = lambda: cnn_step(x0, ws, CNN_GEOMS, precision=prec, recompute=True)  # noqa: E731
    elif args.only in ("fwd", "dgrad", "wgrad"):
        X = np.asfortranarray(g.standard_normal((s["W"], s["H"], s["C"], s["N"]), dtype=np.float32))
        Wt = np.asfortranarray((g.standard_normal((s["fw"], s["fh"], s["C"], s["K"])) * 0.06
                                ).astype(np.float32))
        Xa, Wa = af.Array.from_numpy(X), af.Array.from_numpy(Wt)
        Y = af.convolve2_nn(Xa, Wa, st, pd, dl)
        Ga = af.Array.from_numpy(np.asfortranarray(g.standard_normal(Y.dims, dtype=np.float32)))
        prec = args.precision
        fn = {"fwd": lambda: af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec),
              "dgrad": lambda: af.convolve2_gradient_nn(Ga, Xa, Wa, Y, st, pd, dl,
                                                        af.AF_CONV_GRADIENT_DATA, precision=prec),
              "wgrad": lambda: af.convolve2_gradient_nn(Ga, Xa, Wa, Y, st, pd, dl,
                                                        af.AF_CONV_GRADIENT_FILTER, precision=prec)
              }[args.only]
    else:
        t = g.standard_normal(15)
        CF = af.Array.from_numpy((t / t.sum()).astype(np.float32))
        RF = af.Array.from_numpy((t[::-1] / t.sum()).astype(np.float32))
        if args.only in ("unwrap", "wrap", "unwrap_rows", "wrap_rows"):
            xi = torch.rand(32, 64, 128, 128, device="cuda")
            XI = af.Array.view_torch(xi)
            col = not args.only.endswith("_rows")
            U = af.unwrap(XI, 3, 3, 1, 1, 1, 1, col)
            fn = ((lambda: af.unwrap(XI, 3, 3, 1, 1, 1, 1, col)) if args.only.startswith("unwrap")
                  else (lambda: af.wrap(U, 128, 128, 3, 3, 1, 1, 1, 1, col)))
        elif args.only == "conv3":
            v = torch.rand(256, 256, 256, device="cuda")
            V = af.Array.view_torch(v)
            k3 = g.standard_normal((3, 3, 3))
            F3 = af.Array.from_numpy(np.asfortranarray((k3 / k3.sum()).astype(np.float32)))
            fn = lambda: af.convolve3(V, F3, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)  # noqa: E731
        elif args.only == "sep_u8":
            xu = torch.randint(0, 256, (64, 2048, 2048), dtype=torch.uint8, device="cuda")
            S = af.Array.view_torch(xu)
            fn = lambda: af.convolve2_separable(CF, RF, S)  # noqa: E731
        else:
            xs = torch.rand(64, 2048, 2048, device="cuda")
            S = af.Array.view_torch(xs)
            if args.only == "sep_f32":
                fn = lambda: af.convolve2_separable(CF, RF, S)  # noqa: E731
            else:
                f7 = g.standard_normal((7, 7, 64))
                F7 = af.Array.from_numpy(np.asfortranarray(
                    (f7 / f7.sum(axis=(0, 1), keepdims=True)).astype(np.float32)))
                fn = lambda: af.convolve2(S, F7, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)  # noqa: E731
    for _ in range(args.warmup):
        r = fn()
    del r
    torch.cuda.synchronize()
    times = []
    for _ in range(args.steps):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        r = fn()
        b.record()
        b.synchronize()
        times.append(a.elapsed_time(b))
        del r
    print(json.dumps({"only": args.only, "precision": args.precision, "ms": times}))


# ---------------------------------------------------------------------------
def replica_reduce(ms: float, world: int) -> float:
    """The slowest rank's time per step: a MAX all-reduce over the replicas
    (NCCL with a device tensor, gloo with a host tensor)."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms], device=dev, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(ms: float, world: int) -> float:
    """Whole-job TFLOP/s of `world` replicas of the headline step that each
    took `ms` (the slowest rank's time) per step."""
    return 3 * nn_flops() * world / (ms / 1e3) / 1e12


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="bf16", choices=["bf16", "fp32", "fp8"])
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--only", default=None,
                    choices=["fwd", "dgrad", "wgrad", "sep_f32", "sep_u8", "same7", "conv3", "cnn",
                             "unwrap", "wrap", "unwrap_rows", "wrap_rows"],
                    help="run one operation of the workload --steps times after --warmup "
                         "(for profiler captures); prints its timing, not the bench line")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)

    rank = int(os.environ.get("RANK", 0))
    world = int(os.environ.get("WORLD_SIZE", 1))
    peaks = load_peaks()
    if args.only:
        run_only(args)
        return
    config = {"workload": "conv2_nn fwd+dgrad+wgrad, signal 128x128x64x32 (W,H,C,N), filter "
                          "3x3x64x128, stride 1, pad 1, dilation 1 (afgb_convolve2_nn_ex + "
                          "afgb_convolve2_gradients_nn per step)",
              "global_batch": NN_SHAPE["N"] * world, "flops_per_step": 3 * nn_flops() * world,
              "l2": "flushed between timed steps (512 MB write)", "parallelism": "replicas"}

    if args.impl == "reference":
        if rank != 0:
            return
        cpu = cpu_nn_sample(args.cpu_seconds)
        line = {"impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": "TFLOP/s",
                "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": cpu["seconds_per_step"] * 1e3 * NN_SHAPE["N"],
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic", "config": config,
                "cpu_baseline": {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")},
                "e2e": {"value": cpu["value"], "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    res = run_ours(args, peaks, rank, world)
    value = res["value"]
    ms = res["ms_per_step"]
    if world > 1:
        ms = replica_reduce(ms, world)
        value = replica_value(ms, world)
    if rank != 0:
        return
    cpu = cpu_nn_sample(args.cpu_seconds)
    line = {
        "metric": METRIC, "value": value, "unit": "TFLOP/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16" if res["precision"] == "bf16" else
        ("fp8_e4m3" if res["precision"] == "fp8" else "f32"),
        "data": "synthetic (seeded Philox N(0,1) signal, He-normal filter)", "config": config,
        "roofline": res["roofline"], "cpu_baseline": {k: cpu[k] for k in
                                                      ("value", "unit", "cores", "kind", "sample")},
        "e2e": res["e2e"], "clocks": res["clocks"], "gpu_launches": res["gpu_launches"],
        "errors_vs_fp64": res["errors_vs_fp64"], "kernel_times_ms": res["kernel_times_ms"],
        "fp32_path": res["fp32_path"],
        "secondary": res.get("secondary"), "cnn4": res.get("cnn4"), "peaks": peaks,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
