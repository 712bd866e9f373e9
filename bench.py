"""Benchmark of the spatial-convolution hot path on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--precision bf16|fp32|fp8] [--no-secondary]

Headline (`value`): af_convolve2_nn forward + data gradient + filter
gradient TFLOP/s on the 128x128x64x32 signal / 3x3x64x128 filter workload
(stride 1, padding 1, dilation 1; 3 x 77.31 GFLOP per step), inputs resident
in HBM, each step one pass of forward and both gradients.  Inputs are
seeded synthetic N(0,1) / He-normal arrays (no dataset).  Timing: CUDA events
on the launching stream around each step, with the library's per-kernel
timers off; between steps a 512 MB buffer is written to flush the 126 MB L2.
Per-kernel times (the roofline) come from a separate pass with the kernel
timers on.

`e2e` is the same headline metric through the C ABI with host buffers:
af_create_array from pinned host memory, the three calls, af_get_data_ptr
back to host, all inside the timed region.

`cudnn` times cuDNN (through torch) on the same shapes, in BF16 and in FP32
with TF32 off: the reference's CUDA backend calls cuDNN for this operation.
`nn_workloads` adds the 56x56x256x64 1x1 workload, the FP8-E4M3 forward and
the strided / dilated backward shapes, each with errors against FP64.
`secondary` reports the bandwidth-bound direct convolutions and the patch /
FFT lines as HBM GB/s against the measured copy bandwidth, each with its
error against the oracle on a sampled slice and the reference CPU kernel's
single-thread rate on a bounded sample of the same workload.

`--impl reference` times the reference's CPU algorithm for the headline
metric on full 32-image steps (the oracle's C restatement of unwrap/wrap plus
the BLAS sgemm bundled with numpy, as the reference CPU backend's unwrap +
CBLAS path), with all host threads the BLAS can use.

Multi-GPU: the path does not shard (replicas only): each rank runs the same
workload on its own GPU; `value` sums the ranks' work over the slowest rank's
time.
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
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
# the other NN workloads: (W, H, C, N), (fw, fh, C, K), stride, padding, dilation
NN_OTHER = {
    "56x56x256x64_1x1x256x512": ((56, 56, 256, 64), (1, 1, 256, 512), (1, 1), (0, 0), (1, 1)),
    "64x64x128x16_3x3x128x256_s2p1": ((64, 64, 128, 16), (3, 3, 128, 256), (2, 2), (1, 1),
                                      (1, 1)),
    "64x64x128x16_5x5x128x256_s2p4d2": ((64, 64, 128, 16), (5, 5, 128, 256), (2, 2), (4, 4),
                                        (2, 2)),
}
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) per launch of each
# tensor-core kernel on NN_SHAPE, from one ncu capture of `bench.py --only
# fwd|dgrad|wgrad` (ncu cannot run inside the timed bench)
NCU_TRAFFIC = {"tc_fwd_kernel": 69.68e6 + 207.37e6, "tc_dgrad_kernel": 143.89e6 + 85.84e6,
               "tc_wgrad_kernel": 206.27e6 + 18.41e6}
MAIN_KERNELS = ("simt_fwd_kernel", "simt_dgrad_kernel", "simt_wgrad_kernel", "tc_fwd_kernel",
                "tc_fwd_fp8_kernel", "tc_dgrad_kernel", "tc_wgrad_kernel", "tc_convert_kernel",
                "wgrad_reduce_kernel")


def shape_dict(sd, fd, st, pd, dl) -> dict:
    return dict(W=sd[0], H=sd[1], C=sd[2], N=sd[3], fw=fd[0], fh=fd[1], K=fd[3], stride=st,
                pad=pd, dil=dl)


def nn_out_hw(s) -> tuple[int, int]:
    Wo = 1 + (s["W"] + 2 * s["pad"][0] - ((s["fw"] - 1) * s["dil"][0] + 1)) // s["stride"][0]
    Ho = 1 + (s["H"] + 2 * s["pad"][1] - ((s["fh"] - 1) * s["dil"][1] + 1)) // s["stride"][1]
    return Wo, Ho


def nn_flops(s=NN_SHAPE) -> float:
    Wo, Ho = nn_out_hw(s)
    return 2.0 * Wo * Ho * s["N"] * s["K"] * s["fw"] * s["fh"] * s["C"]


def nn_kernel_bytes(name: str, s=NN_SHAPE) -> float:
    """Algorithmic HBM bytes of one launch of a BF16 NN kernel: its bf16 operand
    image(s) read once, its f32 result written once, the weights once."""
    Wo, Ho = nn_out_hw(s)
    x = s["N"] * s["H"] * s["W"] * s["C"]
    g = s["N"] * Ho * Wo * s["K"]
    w = s["fw"] * s["fh"] * s["C"] * s["K"]
    if name.endswith("wgrad_kernel"):
        return 2.0 * (x + g) + 4.0 * w
    if name.endswith("dgrad_kernel"):
        return 2.0 * g + 4.0 * x + 2.0 * w
    return 2.0 * x + 4.0 * g + 2.0 * w


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"],
                "bf16_tflops_sustained": d.get("bf16_tflops_sustained", d["bf16_tflops"]),
                "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0,
            "source": "fallback"}


def cpu_model() -> str:
    try:
        for ln in Path("/proc/cpuinfo").read_text().splitlines():
            if ln.lower().startswith(("model name", "cpu part")):
                return ln.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.machine()


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
# timing helpers
# ---------------------------------------------------------------------------
def _timed(fn, steps: int, warmup: int, flush) -> list[float]:
    """CUDA-event milliseconds of `steps` calls of fn after `warmup` calls,
    with `flush` (an L2-sized write) before each timed call."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    times = []
    for _ in range(steps):
        flush()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        times.append(a.elapsed_time(b))
    return times


def _kernel_times(af, fn, reps: int, flush) -> dict:
    """Average device ms per launch of the library's main kernels over `reps`
    calls of fn, with the kernel timers on (a pass apart from the timed one)."""
    import ctypes

    import torch

    L = af.lib()
    fn()
    torch.cuda.synchronize()
    L.afgb_kernel_timing(1)
    for _ in range(reps):
        flush()
        fn()
    torch.cuda.synchronize()
    kt = {}
    for name in MAIN_KERNELS:
        c = ctypes.c_ulonglong()
        ms = ctypes.c_double()
        L.afgb_kernel_time(name.encode(), ctypes.byref(c), ctypes.byref(ms))
        if c.value:
            kt[name] = {"launches": int(c.value), "avg_ms": ms.value / c.value,
                        "per_call": c.value / reps}
    L.afgb_kernel_timing(0)
    return kt


def _err(got, ref) -> dict:
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    return {"rel": float(np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300)),
            "maxabs": float(np.abs(got - ref).max()),
            "maxabs_over_max_ref": float(np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300))}


def make_flush():
    import torch

    buf = torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    return lambda: buf.zero_()


# ---------------------------------------------------------------------------
# NN workloads
# ---------------------------------------------------------------------------
def nn_inputs(s, seed):
    g = np.random.Generator(np.random.Philox(seed))
    X = np.asfortranarray(g.standard_normal((s["W"], s["H"], s["C"], s["N"]), dtype=np.float32))
    std = np.sqrt(2.0 / (s["fw"] * s["fh"] * s["C"]))
    Wt = np.asfortranarray((g.standard_normal((s["fw"], s["fh"], s["C"], s["K"])) * std
                            ).astype(np.float32))
    Wo, Ho = nn_out_hw(s)
    Gd = np.asfortranarray(g.standard_normal((Wo, Ho, s["K"], s["N"]), dtype=np.float32))
    return X, Wt, Gd, g


def nn_errors(af, O, s, X, Wt, Gd, prec, g, grads=True) -> dict:
    """Errors of one forward (and gradient) call against FP64 on sampled points."""
    st, pd, dl = s["stride"], s["pad"], s["dil"]
    Xa, Wa, Ga = af.Array.from_numpy(X), af.Array.from_numpy(Wt), af.Array.from_numpy(Gd)
    y = af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec).to_numpy().ravel(order="F")
    idx = g.integers(0, y.size, 256)
    out = {"fwd": _err(y[idx], O.nn_forward_points_f64(X, Wt, st, pd, dl, idx))}
    if grads:
        dx, dw, _ = af.convolve2_gradients_nn(Ga, Xa, Wa, st, pd, dl, precision=prec)
        dxn = dx.to_numpy().ravel(order="F")
        i2 = g.integers(0, X.size, 128)
        out["dgrad"] = _err(dxn[i2], O.nn_data_grad_points_f64(Gd, list(X.shape), Wt, st, pd, dl,
                                                                i2))
        dwn = dw.to_numpy().ravel(order="F")
        i3 = g.integers(0, Wt.size, 64)
        out["wgrad"] = _err(dwn[i3], O.nn_filter_grad_points_f64(Gd, X, list(Wt.shape), st, pd, dl,
                                                                  i3))
    out["points"] = [256, 128, 64] if grads else [256]
    return out


def nn_workload(af, O, s, prec, steps, flush, seed, grads=True) -> dict:
    """Device time of forward (+ both gradients) per step on one NN shape,
    per-kernel times from a separate pass, and errors against FP64."""
    X, Wt, Gd, g = nn_inputs(s, seed)
    st, pd, dl = s["stride"], s["pad"], s["dil"]
    Xa, Wa, Ga = af.Array.from_numpy(X), af.Array.from_numpy(Wt), af.Array.from_numpy(Gd)

    def step():
        Xa.device_ptr()  # a new signal each step (drops the converted copy)
        af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec)
        if grads:
            af.convolve2_gradients_nn(Ga, Xa, Wa, st, pd, dl, precision=prec)

    times = _timed(step, steps, 3, flush)
    ms = float(np.median(times))
    fl = nn_flops(s) * (3 if grads else 1)
    kt = _kernel_times(af, step, 3, flush)
    errs = nn_errors(af, O, s, X, Wt, Gd, prec, g, grads)
    return {"precision": prec, "ops": "fwd+dgrad+wgrad" if grads else "fwd",
            "gflop_per_step": round(fl / 1e9, 2), "ms_per_step": round(ms, 4),
            "TFLOP/s": round(fl / (ms / 1e3) / 1e12, 1),
            "kernel_ms": {k: round(v["avg_ms"], 4) for k, v in kt.items()},
            "errors_vs_fp64": errs}


def cudnn_bar(s, steps, flush) -> dict:
    """cuDNN through torch on one NN shape: forward (conv2d with the filter
    flipped, since af_convolve2_nn is a true convolution) and the backward of
    data and filter (aten.convolution_backward), BF16 and FP32 with TF32 off,
    in NCHW and channels-last; the faster layout is kept per precision.
    Inputs are already in the timed precision and layout (the library's own
    times include its f32 -> bf16 conversions)."""
    import torch
    import torch.nn.functional as F

    torch.backends.cudnn.benchmark = True
    torch.backends.cudnn.allow_tf32 = False
    torch.backends.cuda.matmul.allow_tf32 = False
    gen = torch.Generator(device="cuda").manual_seed(3)
    Wo, Ho = nn_out_hw(s)
    x0 = torch.randn((s["N"], s["C"], s["H"], s["W"]), device="cuda", generator=gen)
    w0 = torch.randn((s["K"], s["C"], s["fh"], s["fw"]), device="cuda", generator=gen) * 0.05
    g0 = torch.randn((s["N"], s["K"], Ho, Wo), device="cuda", generator=gen)
    stv = (s["stride"][1], s["stride"][0])
    pdv = (s["pad"][1], s["pad"][0])
    dlv = (s["dil"][1], s["dil"][0])
    fl = nn_flops(s)
    res = {}
    for name, dt in (("bf16", torch.bfloat16), ("fp32_no_tf32", torch.float32)):
        best = None
        for layout in ("nchw", "channels_last"):
            mf = torch.channels_last if layout == "channels_last" else torch.contiguous_format
            x = x0.to(dt).contiguous(memory_format=mf)
            w = w0.flip([2, 3]).to(dt).contiguous(memory_format=mf)
            gg = g0.to(dt).contiguous(memory_format=mf)

            def fwd():
                return F.conv2d(x, w, None, stv, pdv, dlv)

            def bwd():
                return torch.ops.aten.convolution_backward(gg, x, w, None, stv, pdv, dlv, False,
                                                           [0, 0], 1, [True, True, False])

            def dgr():
                return torch.ops.aten.convolution_backward(gg, x, w, None, stv, pdv, dlv, False,
                                                           [0, 0], 1, [True, False, False])

            def wgr():
                return torch.ops.aten.convolution_backward(gg, x, w, None, stv, pdv, dlv, False,
                                                           [0, 0], 1, [False, True, False])

            def step():
                fwd()
                bwd()

            t = {k: float(np.median(_timed(f, steps, 3, flush)))
                 for k, f in (("fwd", fwd), ("dgrad", dgr), ("wgrad", wgr), ("bwd", bwd),
                              ("step", step))}
            rec = {"layout": layout, **{k + "_ms": round(v, 4) for k, v in t.items()},
                   "step_TFLOP/s": round(3 * fl / (t["step"] / 1e3) / 1e12, 1)}
            if best is None or t["step"] < best["step_ms"]:
                best = rec
        res[name] = best
    # the reference's own call: f32 NCHW arrays, cuDNN's default math type
    # (src/backend/cuda/convolveNN.cpp sets none), which lets FP32
    # convolutions run on TF32 tensor cores
    torch.backends.cudnn.allow_tf32 = True
    x, w, gg = x0.contiguous(), w0.flip([2, 3]).contiguous(), g0.contiguous()

    def step_ref():
        F.conv2d(x, w, None, stv, pdv, dlv)
        torch.ops.aten.convolution_backward(gg, x, w, None, stv, pdv, dlv, False, [0, 0], 1,
                                            [True, True, False])
    t = float(np.median(_timed(step_ref, steps, 3, flush)))
    res["fp32_default_math_nchw"] = {"layout": "nchw", "step_ms": round(t, 4),
                                     "step_TFLOP/s": round(3 * fl / (t / 1e3) / 1e12, 1),
                                     "note": "TF32 tensor cores allowed, as in the reference"}
    torch.backends.cudnn.allow_tf32 = False
    # BF16 cuDNN for a caller holding f32 NCHW arrays (this library's
    # interface): casts to bf16 channels-last in, f32 NCHW out, inside the step
    cl = torch.channels_last

    def step_cast():
        xb = x0.to(torch.bfloat16).contiguous(memory_format=cl)
        wb = w0.flip([2, 3]).to(torch.bfloat16).contiguous(memory_format=cl)
        gb = g0.to(torch.bfloat16).contiguous(memory_format=cl)
        y = F.conv2d(xb, wb, None, stv, pdv, dlv)
        y.float().contiguous()
        dx, dw, _ = torch.ops.aten.convolution_backward(gb, xb, wb, None, stv, pdv, dlv, False,
                                                        [0, 0], 1, [True, True, False])
        dx.float().contiguous()
        dw.float().contiguous()
    t = float(np.median(_timed(step_cast, steps, 3, flush)))
    res["bf16_from_f32_arrays"] = {"layout": "channels_last", "step_ms": round(t, 4),
                                   "step_TFLOP/s": round(3 * fl / (t / 1e3) / 1e12, 1),
                                   "note": "casts of signal, filter and incoming gradient to bf16 "
                                           "channels-last and of the three results to f32 NCHW "
                                           "inside the step"}
    torch.backends.cudnn.benchmark = False
    return res


def ours_split(af, s, prec, steps, flush, seed) -> dict:
    """The library's forward call and gradients call timed apart (same events
    and flush as the cuDNN bar)."""
    X, Wt, Gd, _ = nn_inputs(s, seed)
    st, pd, dl = s["stride"], s["pad"], s["dil"]
    Xa, Wa, Ga = af.Array.from_numpy(X), af.Array.from_numpy(Wt), af.Array.from_numpy(Gd)
    def fwd():
        Xa.device_ptr()  # a new signal each call (drops the converted copy)
        af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec)

    def step():
        fwd()
        af.convolve2_gradients_nn(Ga, Xa, Wa, st, pd, dl, precision=prec)

    t = {k: float(np.median(_timed(f, steps, 3, flush))) for k, f in (("fwd", fwd), ("step", step))}
    t["bwd"] = t["step"] - t["fwd"]  # the gradients after a forward of the same signal
    fl = nn_flops(s)
    return {**{k + "_ms": round(v, 4) for k, v in t.items()},
            "step_TFLOP/s": round(3 * fl / (t["step"] / 1e3) / 1e12, 1)}


# ---------------------------------------------------------------------------
# our implementation
# ---------------------------------------------------------------------------
def bind_to_gpu_numa(dev: int) -> dict:
    """Runs this process on the host CPUs attached to the GPU (read from the
    PCI device's local_cpulist), so the pinned host buffers the e2e leg
    allocates afterwards are placed on the GPU's side of the host link.  A
    process-local affinity only; nothing on the machine is changed."""
    import torch

    try:
        pr = torch.cuda.get_device_properties(dev)
        bus = "%04x:%02x:%02x.0" % (pr.pci_domain_id, pr.pci_bus_id, pr.pci_device_id)
        text = open(f"/sys/bus/pci/devices/{bus}/local_cpulist").read().strip()
        cpus = set()
        for part in text.split(","):
            if "-" in part:
                a, b = part.split("-")
                cpus.update(range(int(a), int(b) + 1))
            elif part:
                cpus.add(int(part))
        allowed = os.sched_getaffinity(0)
        use = cpus & allowed
        if use and use != allowed:
            os.sched_setaffinity(0, use)
        return {"pci": bus, "local_cpus": text, "cpus_used": len(use or allowed)}
    except Exception as e:  # no sysfs entry (or no affinity support): leave it
        return {"unbound": str(e)[:120]}


def link_bandwidth(nbytes: int) -> dict:
    """One pinned host->device and one device->host copy of nbytes (GB/s)."""
    import torch

    h = torch.empty(nbytes // 4, dtype=torch.float32).pin_memory()
    d = torch.empty(nbytes // 4, dtype=torch.float32, device="cuda")
    out = {}
    for name, fn in (("h2d", lambda: d.copy_(h, non_blocking=True)),
                     ("d2h", lambda: h.copy_(d, non_blocking=True))):
        fn()
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        fn()
        b.record()
        b.synchronize()
        out[name + "_GBs"] = round(nbytes / (a.elapsed_time(b) / 1e3) / 1e9, 1)
    return out


def run_ours(args, peaks, rank: int, world: int) -> dict:
    import torch

    import arrayfire_gb300 as af

    dev = int(os.environ.get("LOCAL_RANK", 0))
    torch.cuda.set_device(dev)
    numa = bind_to_gpu_numa(dev)
    af.set_stream(torch.cuda.current_stream())
    L = af.lib()
    L.afgb_kernel_timing(0)
    s = NN_SHAPE
    X, Wt, Gd, g = nn_inputs(s, 1234 + rank)
    Xa, Wa = af.Array.from_numpy(X), af.Array.from_numpy(Wt)
    st, pd, dl = s["stride"], s["pad"], s["dil"]
    prec = args.precision
    try:
        af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec)
    except af.AfError as e:
        if prec == "fp32" or e.code != af.AF_ERR_NOT_SUPPORTED:
            raise
        prec = "fp32"
    Ga = af.Array.from_numpy(Gd)
    flush = make_flush()
    grads = prec != "fp8"  # FP8 is provided for the forward only

    def step():
        # a new signal each step, as in training: handing the buffer out for
        # writing (af_get_device_ptr) drops the library's bf16 copy of the
        # previous signal, so the forward converts it again.  The forward,
        # then both input gradients in one call (one shared bf16 copy of the
        # incoming gradient; the signal's copy from the forward reused)
        Xa.device_ptr()
        y = af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec)
        if grads:
            af.convolve2_gradients_nn(Ga, Xa, Wa, st, pd, dl, precision=prec)
        return y

    import oracle.oracle as O  # checker only

    errs = nn_errors(af, O, s, X, Wt, Gd, prec, g, grads)

    launches0 = af.launch_count()
    if world > 1:
        import torch.distributed as dist

        dist.barrier()
    torch.cuda.synchronize()
    clock = ClockSampler(dev)
    clock.start()
    times = _timed(step, args.steps, args.warmup, flush)
    clocks = clock.stop()
    torch.cuda.synchronize()
    launches = (af.launch_count() - launches0) * args.steps // (args.steps + args.warmup)
    total_ms = sum(times)
    flops = nn_flops() * (3 if grads else 1)
    value = flops * args.steps / (total_ms / 1e3) / 1e12

    # per-kernel device times: a separate pass with the kernel timers on
    kt = _kernel_times(af, step, 5, flush)
    mains = {k: v for k, v in kt.items() if k.endswith(("fwd_kernel", "fwd_fp8_kernel",
                                                       "dgrad_kernel", "wgrad_kernel"))}
    dom = max(mains.items(), key=lambda kv: kv[1]["avg_ms"]) if mains else None
    roofline = None
    if dom:
        # the dominant kernel against the roof that bounds it: the longer of its
        # tensor floor (FLOPs / bf16 peak) and its HBM floor (bytes / copy bandwidth)
        name, v = dom
        sec = v["avg_ms"] / 1e3
        nbytes = nn_kernel_bytes(name)
        tflops, gbs = nn_flops() / sec / 1e12, nbytes / sec / 1e9
        t_frac, h_frac = tflops / peaks["bf16_tflops"], gbs / peaks["hbm_gbs"]
        hbm_bound = nbytes / peaks["hbm_gbs"] > nn_flops() / 1e3 / peaks["bf16_tflops"]
        roofline = {"bound": "hbm" if hbm_bound else "tensor", "kernel": name,
                    "achieved": round(gbs if hbm_bound else tflops, 2),
                    "peak": peaks["hbm_gbs"] if hbm_bound else peaks["bf16_tflops"],
                    "unit": "GB/s" if hbm_bound else "TFLOP/s",
                    "frac": round(h_frac if hbm_bound else t_frac, 4),
                    "peak_source": peaks["source"] + (" copy bandwidth" if hbm_bound
                                                      else " bf16 dense (burst)"),
                    "traffic": NCU_TRAFFIC.get(name) if prec == "bf16" else None,
                    "traffic_source": "ncu capture, one launch (bytes)",
                    "avg_ms": round(v["avg_ms"], 4),
                    "algorithmic_gflop_per_launch": round(nn_flops() / 1e9, 2),
                    "algorithmic_mb_per_launch": round(nbytes / 1e6, 1),
                    "tensor_frac": round(t_frac, 4), "hbm_frac": round(h_frac, 4)}

    # e2e through the C ABI with pinned host buffers
    e2e = run_e2e(af, X, Wt, Gd, prec, args)
    e2e["host"] = {**numa, **link_bandwidth(e2e["h2d_bytes_per_step"])}

    # the plain FP32 CUDA-core path on the same workload (the >= 5x target's
    # denominator), fewer steps
    fp32 = None
    if prec == "bf16":
        def step32():
            af.convolve2_nn(Xa, Wa, st, pd, dl)
            af.convolve2_gradients_nn(Ga, Xa, Wa, st, pd, dl)
        k32 = max(3, min(args.steps, 5))
        t32 = sum(_timed(step32, k32, 3, flush))
        v32 = 3 * nn_flops() * k32 / (t32 / 1e3) / 1e12
        fp32 = {"value": v32, "ms_per_step": t32 / k32, "unit": "TFLOP/s",
                "speedup_of_" + prec: value / v32}

    res = {
        "value": value, "ms_per_step": total_ms / args.steps, "precision": prec,
        "errors_vs_fp64": errs,
        "kernel_times_ms": {k: round(v["avg_ms"], 4) for k, v in kt.items()},
        "kernel_launches_per_step": {k: v["per_call"] for k, v in kt.items()},
        "roofline": roofline, "clocks": clocks, "e2e": e2e, "fp32_path": fp32,
        "gpu_launches": int(launches), "step_times_ms": [round(t, 4) for t in times],
    }
    del Xa, Wa, Ga
    if not args.no_secondary and prec == "bf16":
        res["cudnn"] = run_cudnn_comparison(af, args, flush)
        res["nn_workloads"] = run_nn_workloads(af, O, args, flush)
    if not args.no_secondary:
        res["secondary"] = run_direct_workloads(af, O, peaks, args)
        res["image_callers"] = run_image_callers(af, O, args)
        res["cnn4"] = run_cnn(af, args)
    return res


def run_cudnn_comparison(af, args, flush) -> dict:
    steps = max(5, min(args.steps, 10))
    out = {"note": "cuDNN via torch " + __import__("torch").__version__ + ", cudnn.benchmark on; "
                   "inputs pre-converted to the timed precision/layout (ours: f32 arrays in, "
                   "conversions inside the timed calls)"}
    for key, shp in (("128x128x64x32_3x3x64x128", NN_SHAPE),
                     ("56x56x256x64_1x1x256x512", shape_dict(*NN_OTHER["56x56x256x64_1x1x256x512"]))):
        c = cudnn_bar(shp, steps, flush)
        o = ours_split(af, shp, "bf16", steps, flush, 21)
        o32 = ours_split(af, shp, "fp32", 3, flush, 21)
        out[key] = {"cudnn": c, "ours_bf16": o, "ours_fp32": o32,
                    "ours_bf16_speedup_over_cudnn_bf16": {
                        "fwd": round(c["bf16"]["fwd_ms"] / o["fwd_ms"], 3),
                        "bwd": round(c["bf16"]["bwd_ms"] / o["bwd_ms"], 3),
                        "step": round(c["bf16"]["step_ms"] / o["step_ms"], 3)},
                    "ours_bf16_speedup_over_cudnn_bf16_from_f32_arrays": round(
                        c["bf16_from_f32_arrays"]["step_ms"] / o["step_ms"], 3),
                    "ours_bf16_speedup_over_reference_cudnn_call": round(
                        c["fp32_default_math_nchw"]["step_ms"] / o["step_ms"], 3),
                    "ours_fp32_speedup_over_cudnn_fp32": round(
                        c["fp32_no_tf32"]["step_ms"] / o32["step_ms"], 3)}
    return out


def run_nn_workloads(af, O, args, flush) -> dict:
    steps = max(5, min(args.steps, 10))
    out = {}
    s3b = shape_dict(*NN_OTHER["56x56x256x64_1x1x256x512"])
    out["56x56x256x64_1x1x256x512_bf16"] = nn_workload(af, O, s3b, "bf16", steps, flush, 31)
    out["56x56x256x64_1x1x256x512_fp32"] = nn_workload(af, O, s3b, "fp32", 3, flush, 31)
    out["128x128x64x32_3x3x64x128_fp8_fwd"] = nn_workload(af, O, NN_SHAPE, "fp8", steps, flush, 32,
                                                           grads=False)
    out["56x56x256x64_1x1x256x512_fp8_fwd"] = nn_workload(af, O, s3b, "fp8", steps, flush, 33,
                                                          grads=False)
    out["128x128x64x32_3x3x64x128_bf16_fwd"] = nn_workload(af, O, NN_SHAPE, "bf16", steps, flush,
                                                           32, grads=False)
    for key in ("64x64x128x16_3x3x128x256_s2p1", "64x64x128x16_5x5x128x256_s2p4d2"):
        sh = shape_dict(*NN_OTHER[key])
        out[key + "_bf16"] = nn_workload(af, O, sh, "bf16", steps, flush, 41)
        out[key + "_fp32"] = nn_workload(af, O, sh, "fp32", 3, flush, 41)
    return out


def run_e2e(af, X, Wt, Gd, prec, args) -> dict:
    import ctypes

    import torch

    L = af.lib()
    s = NN_SHAPE
    st, pd, dl = s["stride"], s["pad"], s["dil"]
    grads = prec != "fp8"
    pin = {k: torch.from_numpy(np.ascontiguousarray(v.ravel(order="F"))).pin_memory()
           for k, v in (("x", X), ("w", Wt), ("g", Gd))}
    Wo, Ho = nn_out_hw(s)
    y_host = torch.empty(Wo * Ho * s["K"] * s["N"], dtype=torch.float32).pin_memory()
    dx_host = torch.empty(X.size, dtype=torch.float32).pin_memory()
    dw_host = torch.empty(Wt.size, dtype=torch.float32).pin_memory()

    def mk(t, dims):
        out = ctypes.c_void_p()
        d = (ctypes.c_longlong * 4)(*dims)
        af._check(L.af_create_array(ctypes.byref(out), ctypes.c_void_p(t.data_ptr()), 4, d, af.f32))
        return af.Array(out.value)

    calls = {}  # host time per call (each call blocks: the copies and the work it waits for)

    def tick(name, t0):
        t1 = time.perf_counter()
        calls[name] = calls.get(name, 0.0) + (t1 - t0) * 1e3
        return t1

    def step():
        t = time.perf_counter()
        Xa = mk(pin["x"], X.shape)
        t = tick("create_signal", t)
        Wa = mk(pin["w"], Wt.shape)
        t = tick("create_filter", t)
        y = af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec)
        t = tick("forward_call", t)
        af._check(L.af_get_data_ptr(ctypes.c_void_p(y_host.data_ptr()), y.handle))
        t = tick("get_output", t)
        if grads:
            Ga = mk(pin["g"], Gd.shape)
            t = tick("create_incoming_gradient", t)
            dx, dw, _ = af.convolve2_gradients_nn(Ga, Xa, Wa, st, pd, dl, precision=prec)
            t = tick("gradients_call", t)
            af._check(L.af_get_data_ptr(ctypes.c_void_p(dx_host.data_ptr()), dx.handle))
            t = tick("get_data_gradient", t)
            af._check(L.af_get_data_ptr(ctypes.c_void_p(dw_host.data_ptr()), dw.handle))
            tick("get_filter_gradient", t)

    for _ in range(max(1, args.warmup)):
        step()
    torch.cuda.synchronize()
    calls.clear()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    dt = time.perf_counter() - t0
    h2d = (X.size + Wt.size + (Gd.size if grads else 0)) * 4
    d2h = (y_host.numel() + ((dx_host.numel() + dw_host.numel()) if grads else 0)) * 4
    return {"value": (3 if grads else 1) * nn_flops() * args.steps / dt / 1e12, "unit": "TFLOP/s",
            "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
            "ms_per_step": dt * 1e3 / args.steps,
            "host_ms_per_call": {k: round(v / args.steps, 3) for k, v in calls.items()}}


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
        breakdown = af.device_mem_peak_breakdown()
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
                     "peak_library_bytes": int(lib_peak),
                     "peak_library_breakdown": breakdown,
                     "peak_torch_harness_bytes": int(torch_peak),
                     "filter_grad_rel_err_vs_fp64": [float(f"{e:.3e}") for e in errs]}
    out["bf16_speedup_over_fp32"] = round(out["fp32"]["ms_per_step"] / out["bf16"]["ms_per_step"], 2)
    return out


# ---------------------------------------------------------------------------
# bandwidth-bound lines: GPU GB/s, error on a sampled slice, CPU baseline
# ---------------------------------------------------------------------------
def cpu_direct_baseline(slice_fn, slices, bytes_per_slice, par_slices=None) -> dict:
    """The reference CPU kernel (the oracle's C restatement of
    src/backend/cpu/kernel/convolve.hpp, bit-identical to it) on a bounded
    sample: `slices` run one after another on one thread, as libafcpu runs
    each call on its one worker thread (src/backend/cpu/queue.hpp:79-118);
    then, informational and not the reference's behaviour, `par_slices`
    slices at once on all host threads.  Returns the first slice's output."""
    t0 = time.perf_counter()
    first = None
    for b in slices:
        r = slice_fn(b)
        if first is None:
            first = r
    dt = time.perf_counter() - t0
    out = {"value": round(bytes_per_slice * len(slices) / dt / 1e9, 3), "unit": "GB/s", "cores": 1,
           "kind": "port", "sample": f"{len(slices)} slice(s), {bytes_per_slice} bytes each, "
                                     "oracle C kernel on one thread"}
    if par_slices:
        n = len(par_slices)
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            t0 = time.perf_counter()
            list(ex.map(slice_fn, par_slices))
            dt = time.perf_counter() - t0
        out["all_threads_informational"] = {
            "value": round(bytes_per_slice * n / dt / 1e9, 3), "threads": n,
            "note": "slices in parallel; libafcpu itself runs one call on one thread"}
    return out, first


def run_direct_workloads(af, O, peaks, args) -> dict:
    """Bandwidth-bound direct convolutions (64 x 2048^2 separable and 7x7,
    256^3 volume, 64 x 2^20 1-D, the two small image workloads) and the
    patch / FFT lines: GB/s of algorithmic traffic (each input and output
    counted once), kernel time, error against the oracle on a sampled slice
    of the same output, and the CPU baseline."""
    import ctypes

    import torch

    L = af.lib()
    g = np.random.Generator(np.random.Philox(77))
    flush = make_flush()
    nthreads = min(16, os.cpu_count() or 1)
    out = {}

    def measure(name, fn, nbytes, kernel, check=None):
        for _ in range(3):
            r = fn()
        del r
        torch.cuda.synchronize()
        steps = max(3, min(args.steps, 10))
        times = _timed(fn, steps, 0, flush)
        L.afgb_kernel_timing(1)
        for _ in range(3):
            flush()
            fn()
        torch.cuda.synchronize()
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
        call_ms = float(np.median(times))
        k_ms = ms.value / c.value if c.value else None
        gbs = nbytes / (call_ms / 1e3) / 1e9
        kgbs = nbytes / (k_ms / 1e3) / 1e9 if k_ms else None
        out[name] = {"ms": round(call_ms, 4), "GB/s": round(gbs, 1),
                     "kernel": kernel, "kernel_ms": round(k_ms, 4) if k_ms else None,
                     "kernel_GB/s": round(kgbs, 1) if kgbs else None,
                     "frac_of_hbm": round((kgbs or gbs) / peaks["hbm_gbs"], 4),
                     "bytes": int(nbytes)}
        if check is not None:
            res = fn()
            torch.cuda.synchronize()
            out[name].update(check(res))

    def err_vs(got, ref):
        got = np.asarray(got).ravel(order="F")
        ref = np.asarray(ref).ravel(order="F")
        assert got.size == ref.size, (got.size, ref.size)
        e = _err(got, ref)
        return {"max_err_vs_oracle": {"maxabs": e["maxabs"], "maxabs_over_max_ref":
                                      e["maxabs_over_max_ref"],
                                      "bit_exact": bool(np.asarray(got).tobytes() ==
                                                        np.asarray(ref).tobytes())}}

    def slice2(t, b):  # torch (B, H, W) slice b -> AF (W, H) Fortran
        return np.asfortranarray(t[b].cpu().numpy().T)

    # ---- the two small image workloads (fit in L2: flushed between calls)
    sig1a = np.asfortranarray(np.random.Generator(np.random.Philox(0)).random((512, 512),
                                                                             dtype=np.float32))
    xg = np.arange(5) - 2
    k1a = np.exp(-0.5 * (xg[:, None] ** 2 + xg[None, :] ** 2))
    k1a = np.asfortranarray((k1a / k1a.sum()).astype(np.float32))
    sig1b = np.asfortranarray((np.random.Generator(np.random.Philox(1)).random((1024, 1024)) < 0.5)
                              .astype(np.float32))
    k1b = np.ones((3, 3), np.float32)
    k1b[1, 1] = 0
    for name, sg, kk in (("gauss5x5_f32_512x512", sig1a, k1a),
                         ("neighbour3x3_f32_1024x1024", sig1b, np.asfortranarray(k1b))):
        S, F = af.Array.from_numpy(sg), af.Array.from_numpy(kk)

        def chk(res, sg=sg, kk=kk):
            cpu, ref = cpu_direct_baseline(lambda b: O.convolve(sg, kk, O.F32, 2, False), range(20),
                                           sg.nbytes * 2 + kk.nbytes)
            return {**err_vs(res.to_numpy(), ref), "cpu_baseline": cpu}
        measure(name, lambda: af.convolve2(S, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL),
                sg.nbytes * 2 + kk.nbytes, ("conv2_tma_kernel", "conv2_tile_kernel"), chk)

    # ---- 64 x 2048 x 2048 separable 15-tap, f32 and u8, LHS batch
    t = g.standard_normal(15)
    cf_ = (t / t.sum()).astype(np.float32)
    t = g.standard_normal(15)
    rf_ = (t / t.sum()).astype(np.float32)
    CF, RF = af.Array.from_numpy(cf_), af.Array.from_numpy(rf_)
    xs = torch.rand(64, 2048, 2048, device="cuda")
    S = af.Array.view_torch(xs)
    n = xs.numel()
    slice_bytes_f32 = 2048 * 2048 * 8

    def chk_sep(res, x=xs, dt=O.F32, bpp=8):
        o = res.to_torch().reshape(64, 2048, 2048)
        cpu, ref = cpu_direct_baseline(
            lambda b: O.convolve2_sep(slice2(x, b), cf_, rf_, dt, False), range(3),
            2048 * 2048 * bpp, par_slices=list(range(nthreads)))
        return {**err_vs(slice2(o, 0), ref), "cpu_baseline": cpu}
    measure("sep15_f32_64x2048x2048", lambda: af.convolve2_separable(CF, RF, S), n * 8 + 120,
            ("sep_tma_kernel", "sep_fused_kernel"), chk_sep)
    xu = torch.randint(0, 256, (64, 2048, 2048), dtype=torch.uint8, device="cuda")
    SU = af.Array.view_torch(xu)
    measure("sep15_u8_64x2048x2048", lambda: af.convolve2_separable(CF, RF, SU), n * 2 + 120,
            ("sep_tma_kernel", "sep_fused_kernel"),
            lambda r: chk_sep(r, xu, O.U8, 2))
    del SU, xu
    # ---- SAME batch, 64 distinct 7x7 filters (AF_CONV_SPATIAL: AUTO would pick FFT)
    f7 = g.standard_normal((7, 7, 64))
    f7 = np.asfortranarray((f7 / f7.sum(axis=(0, 1), keepdims=True)).astype(np.float32))
    F7 = af.Array.from_numpy(f7)

    def chk7(res):
        o = res.to_torch().reshape(64, 2048, 2048)
        cpu, ref = cpu_direct_baseline(
            lambda b: O.convolve(slice2(xs, b), np.asfortranarray(f7[:, :, b]), O.F32, 2, False),
            range(2), slice_bytes_f32 + 196, par_slices=list(range(nthreads)))
        return {**err_vs(slice2(o, 0), ref), "cpu_baseline": cpu}
    measure("same7x7_f32_64x2048x2048",
            lambda: af.convolve2(S, F7, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL),
            n * 8 + f7.size * 4, ("conv2_tma_kernel", "conv2_tile_kernel"), chk7)
    # ---- a 31x31 filter: AUTO takes the frequency-domain route (the whole
    # pipeline is timed: pads, the library's transforms, spectrum product, crop)
    f31 = g.standard_normal((31, 31))
    f31 = np.asfortranarray((f31 / f31.sum()).astype(np.float32))
    F31 = af.Array.from_numpy(f31)

    def chk31(res):
        o = res.to_torch().reshape(64, 2048, 2048)
        cpu, ref = cpu_direct_baseline(
            lambda b: O.fft_convolve(slice2(xs, b), f31, O.F32, 2, False), range(2),
            slice_bytes_f32 + f31.nbytes)
        cpu["sample"] += " (numpy pocketfft in FP64 standing in for FFTW)"
        return {**err_vs(slice2(o, 0), ref), "cpu_baseline": cpu}
    measure("fft31x31_f32_64x2048x2048",
            lambda: af.convolve2(S, F31, af.AF_CONV_DEFAULT, af.AF_CONV_AUTO),
            n * 8 + 31 * 31 * 4, ("fft_pipeline",), chk31)
    # several transform passes over 2304x2187 padded slices: its GB/s above
    # counts input + output once; the direct-convolution work it replaces is
    # 2*31*31 flops per output
    e = out["fft31x31_f32_64x2048x2048"]
    e["equivalent_direct_TFLOP/s"] = round(2 * 31 * 31 * n / (e["ms"] / 1e3) / 1e12, 1)
    e["bound"] = "the library's mixed-radix transforms (multi-pass), not one HBM pass"
    del S, xs
    # ---- 256^3 volume, 3x3x3
    v = torch.rand(256, 256, 256, device="cuda")
    V = af.Array.view_torch(v)
    k3 = g.standard_normal((3, 3, 3))
    F3 = af.Array.from_numpy(np.asfortranarray((k3 / k3.sum()).astype(np.float32)))
    vh = np.asfortranarray(v.cpu().numpy().transpose(2, 1, 0))
    k3f = np.asfortranarray((k3 / k3.sum()).astype(np.float32))
    for expand in (False, True):
        def chk3(res, expand=expand):
            cpu, ref = cpu_direct_baseline(lambda b: O.convolve(vh, k3f, O.F32, 3, expand), range(1),
                                           v.numel() * 4 + (258 ** 3 if expand else v.numel()) * 4)
            return {**err_vs(res.to_numpy(), ref), "cpu_baseline": cpu}
        measure("conv3_3x3x3_f32_256^3_" + ("expand" if expand else "default"),
                lambda expand=expand: af.convolve3(V, F3, af.AF_CONV_EXPAND if expand else
                                                   af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL),
                v.numel() * 4 + (258 ** 3 if expand else v.numel()) * 4 + 108,
                ("conv3_tma_kernel", "conv3_tile_kernel", "conv_generic_kernel"), chk3)
    del V, v, vh
    # ---- 1-D: 64 signals of 2^20 samples, a 31-tap filter (LHS batch)
    s1 = torch.rand(64, 1 << 20, device="cuda")
    S1 = af.Array.view_torch(s1)
    k1 = g.standard_normal(31)
    k1 = (k1 / k1.sum()).astype(np.float32)
    F1 = af.Array.from_numpy(k1)

    def chk1(res):
        o = res.to_torch().reshape(64, -1)
        cpu, ref = cpu_direct_baseline(
            lambda b: O.convolve(s1[b].cpu().numpy(), k1, O.F32, 1, False), range(4),
            (1 << 20) * 8, par_slices=list(range(nthreads)))
        return {**err_vs(o[0].cpu().numpy(), ref), "cpu_baseline": cpu}
    measure("conv1_31tap_f32_64x1M", lambda: af.convolve1(S1, F1, af.AF_CONV_DEFAULT,
                                                          af.AF_CONV_SPATIAL),
            s1.numel() * 8 + 124, ("conv1_pipe_kernel", "conv1_tile_kernel", "conv_generic_kernel"), chk1)
    del S1, s1
    # ---- af_unwrap / af_wrap of the NN image (128x128x64x32 f32, 3x3
    # windows, stride 1, padding 1): the 9x larger patch matrix is written /
    # read once
    xi = torch.rand(32, 64, 128, 128, device="cuda")
    XI = af.Array.view_torch(xi)
    ni = xi.numel()
    img0 = np.asfortranarray(xi[0].cpu().numpy().transpose(2, 1, 0))[..., None]  # (W,H,C,1)
    img_bytes = 128 * 128 * 64 * 4 * 10

    def chk_unwrap(res, col=True):
        o = res.to_numpy()
        cpu, ref = cpu_direct_baseline(lambda b: O.unwrap(img0, 3, 3, 1, 1, 1, 1, 1, 1), range(2),
                                       img_bytes, par_slices=list(range(nthreads)))
        got = o[..., 0:1] if col else np.asfortranarray(o[..., 0:1].transpose(1, 0, 2, 3))
        return {**err_vs(got, ref), "cpu_baseline": cpu}
    measure("unwrap_3x3_f32_128x128x64x32", lambda: af.unwrap(XI, 3, 3, 1, 1, 1, 1),
            ni * 4 * 10, ("unwrap_rows_kernel", "unwrap_kernel"), chk_unwrap)
    U = af.unwrap(XI, 3, 3, 1, 1, 1, 1)
    u0 = np.asfortranarray(U.to_numpy()[..., 0:1])

    def chk_wrap(res):
        cpu, ref = cpu_direct_baseline(
            lambda b: O.wrap_dilated(u0, [128, 128, 64, 1], 3, 3, 1, 1, 1, 1, 1, 1), range(2),
            img_bytes, par_slices=list(range(nthreads)))
        return {**err_vs(res.to_numpy()[..., 0:1], ref), "cpu_baseline": cpu}
    measure("wrap_3x3_f32_128x128x64x32", lambda: af.wrap(U, 128, 128, 3, 3, 1, 1, 1, 1),
            ni * 4 * 10, ("wrap_s1_kernel", "wrap_tiled_kernel", "wrap_kernel"), chk_wrap)
    del U, u0
    # the same with is_column = false (patch elements along dim 1)
    measure("unwrap_rows_3x3_f32_128x128x64x32",
            lambda: af.unwrap(XI, 3, 3, 1, 1, 1, 1, False), ni * 4 * 10,
            ("unwrap_rows_kernel", "unwrap_kernel"), lambda r: chk_unwrap(r, False))
    R = af.unwrap(XI, 3, 3, 1, 1, 1, 1, False)
    r0 = np.asfortranarray(R.to_numpy()[..., 0:1].transpose(1, 0, 2, 3))

    def chk_wrap_rows(res):
        cpu, ref = cpu_direct_baseline(
            lambda b: O.wrap_dilated(r0, [128, 128, 64, 1], 3, 3, 1, 1, 1, 1, 1, 1), range(2),
            img_bytes)
        return {**err_vs(res.to_numpy()[..., 0:1], ref), "cpu_baseline": cpu}
    measure("wrap_rows_3x3_f32_128x128x64x32",
            lambda: af.wrap(R, 128, 128, 3, 3, 1, 1, 1, 1, False), ni * 4 * 10,
            ("wrap_s1_kernel", "wrap_rows_kernel", "wrap_kernel"), chk_wrap_rows)
    return out


# ---------------------------------------------------------------------------
# CPU baseline: the reference's algorithm on the host cores
# ---------------------------------------------------------------------------
def _blocks_image(shape, seed, dtype=np.float32) -> np.ndarray:
    """Bright rectangles on a dark ground plus faint noise, in [0, ~255]."""
    g = np.random.Generator(np.random.Philox(seed))
    d0, d1 = shape
    a = np.zeros((d0, d1), np.float32)
    for _ in range(400):
        cy, cx = g.uniform(0, d0), g.uniform(0, d1)
        w = g.uniform(4, 40)
        a[max(0, int(cy - w)):int(cy + w), max(0, int(cx - 1.3 * w)):int(cx + 1.3 * w)] += \
            np.float32(g.uniform(0.3, 1.0))
    a = a * 200.0 + 5.0 * g.standard_normal((d0, d1), dtype=np.float32)
    if dtype == np.uint8:
        a = np.clip(a, 0, 255)
    return np.asfortranarray(a.astype(dtype))


def run_image_callers(af, O, args) -> dict:
    """af_harris and af_canny on 2048 x 2048 images through the C ABI: ms per
    call with the image resident on the device (each call reads its corner
    count or gradient range back to the host, as the reference does),
    megapixels per second, the result checked bit for bit against the oracle,
    and the oracle port's time on the same image on one host thread."""
    import torch

    flush = make_flush()
    steps = max(3, min(args.steps, 10))
    out = {}
    cases = [
        ("harris_2048x2048_f32_max500", np.float32, O.F32,
         lambda A: af.harris(A, 500, 1e5, 1.0, 0, 0.04),
         lambda img: O.harris(img, O.F32, 500, 1e5, 1.0, 0, 0.04)),
        ("harris_2048x2048_f32_minresp", np.float32, O.F32,
         lambda A: af.harris(A, 0, 1e6, 1.0, 0, 0.04),
         lambda img: O.harris(img, O.F32, 0, 1e6, 1.0, 0, 0.04)),
        ("canny_2048x2048_f32_manual", np.float32, O.F32,
         lambda A: af.canny(A, 0, 0.1, 0.3, 3, False),
         lambda img: O.canny(img, O.F32, False, 0.1, 0.3, False)),
        ("canny_2048x2048_u8_otsu", np.uint8, O.U8,
         lambda A: af.canny(A, 1, 0.4, 0.0, 3, False),
         lambda img: O.canny(img, O.U8, True, 0.4, 0.0, False)),
    ]
    for name, npt, dt, call, oracle_call in cases:
        img = _blocks_image((2048, 2048), 61, npt)
        A = af.Array.from_numpy(img)
        times = _timed(lambda: call(A), steps, 3, flush)
        ms = float(np.median(times))
        res = call(A)
        t0 = time.perf_counter()
        want = oracle_call(img)
        cpu_s = time.perf_counter() - t0
        if name.startswith("harris"):
            got = (res.x(), res.y(), res.score())
            same = all(a.tobytes() == b.tobytes() for a, b in zip(got, want))
            extra = {"corners": int(got[0].size)}
        else:
            got = res.to_numpy().reshape(img.shape, order="F").astype(np.int8)
            same = got.tobytes(order="F") == np.asarray(want)[:, :, 0].tobytes(order="F")
            extra = {"edge_pixels": int(got.sum())}
        mpx = img.size / 1e6
        out[name] = {"ms": round(ms, 4), "Mpixel/s": round(mpx / (ms / 1e3), 1),
                     "bit_exact_vs_oracle": bool(same), **extra,
                     "cpu_baseline": {"value": round(mpx / cpu_s, 2), "unit": "Mpixel/s",
                                      "cores": 1, "kind": "port",
                                      "sample": "the same 2048x2048 image, oracle port (numpy "
                                                "and the C separable port)"}}
        del res, A
        torch.cuda.synchronize()
    return out


def cpu_nn_steps(steps: int, warmup: int, seconds_budget: float) -> dict:
    """Forward + both gradients of the headline workload, full 32-image
    steps, timed on the host: oracle unwrap/wrap (C restatement of the
    reference CPU kernels) + numpy's BLAS sgemm in place of CBLAS
    (src/backend/cpu/convolve.cpp:123-243: unwrap of the whole batch, one
    GEMM per operation, wrap_dilated for the data gradient).  Runs `warmup`
    untimed and up to `steps` timed steps; stops early (at least one timed
    step) when the next step would exceed `seconds_budget`, and reports the
    counts it ran."""
    import oracle.oracle as O

    s = NN_SHAPE
    st, pd, dl = s["stride"], s["pad"], s["dil"]
    X, Wt, Gd, _ = nn_inputs(s, 99)
    fd = Wt.shape
    wsz = fd[0] * fd[1]
    nimg = s["N"]

    def one():
        y = O.nn_forward_unwrap_gemm_f32(X, Wt, st, pd, dl)
        cols = O.unwrap(X, fd[0], fd[1], st[0], st[1], pd[0], pd[1], dl[0], dl[1])
        npix = cols.shape[1]
        A = np.ascontiguousarray(cols.transpose(1, 3, 2, 0)).reshape(npix * nimg, s["C"] * wsz)
        G2 = np.asfortranarray(Gd).reshape(npix, s["K"], nimg, order="F").transpose(
            2, 0, 1).reshape(-1, s["K"])
        wflip = Wt[::-1, ::-1, :, :]
        B = np.ascontiguousarray(wflip.reshape(wsz, s["C"], s["K"], order="F").transpose(1, 0, 2)
                                 ).reshape(s["C"] * wsz, s["K"])
        dw = A.T @ G2
        colsg = (G2 @ B.T).reshape(nimg, npix, s["C"], wsz).transpose(3, 1, 2, 0)
        dx = O.wrap_dilated(np.asfortranarray(colsg), list(X.shape), fd[0], fd[1], st[0], st[1],
                            pd[0], pd[1], dl[0], dl[1])
        return y, dx, dw

    t_start = time.perf_counter()
    w_run = 0
    for _ in range(max(1, warmup)):
        one()
        w_run += 1
        if time.perf_counter() - t_start > seconds_budget / 3:
            break
    per = (time.perf_counter() - t_start) / w_run
    times = []
    for _ in range(max(1, steps)):
        if times and time.perf_counter() - t_start + per > seconds_budget:
            break
        t0 = time.perf_counter()
        one()
        times.append(time.perf_counter() - t0)
        per = float(np.mean(times))
    dt = float(np.mean(times))
    flops = 3 * nn_flops()
    return {"value": flops / dt / 1e12, "unit": "TFLOP/s", "cores": os.cpu_count(),
            "kind": "port", "steps": len(times), "warmup": w_run,
            "sample": f"full {nimg}-image steps (fwd+dgrad+wgrad): {w_run} warm-up + {len(times)} "
                      f"timed; oracle unwrap/wrap (1 thread) + numpy BLAS sgemm (all threads); "
                      f"host CPU {cpu_model()}",
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
    if args.only == "image_callers":
        import oracle as O

        print(json.dumps(run_image_callers(af, O, args)))
        return
    if args.only == "cnn":
        from arrayfire_gb300.autograd import cnn_step

        gen = torch.Generator(device="cuda").manual_seed(5)
        x0 = torch.rand((64, 3, 224, 224), device="cuda", generator=gen) * 2 - 1
        ws = [torch.randn((k, c, 3, 3), device="cuda", generator=gen) * (2.0 / (9 * c)) ** 0.5
              for c, k in CNN_CHANNELS]
        prec = "fp32" if args.precision == "fp32" else "bf16"
        fn = lambda: cnn_step(x0, ws, CNN_GEOMS, precision=prec, recompute=True)  # noqa: E731
    elif args.only in ("fwd", "dgrad", "wgrad", "step"):
        X = np.asfortranarray(g.standard_normal((s["W"], s["H"], s["C"], s["N"]), dtype=np.float32))
        Wt = np.asfortranarray((g.standard_normal((s["fw"], s["fh"], s["C"], s["K"])) * 0.06
                                ).astype(np.float32))
        Xa, Wa = af.Array.from_numpy(X), af.Array.from_numpy(Wt)
        Y = af.convolve2_nn(Xa, Wa, st, pd, dl)
        Ga = af.Array.from_numpy(np.asfortranarray(g.standard_normal(Y.dims, dtype=np.float32)))
        prec = args.precision

        def step():
            af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec)
            af.convolve2_gradients_nn(Ga, Xa, Wa, st, pd, dl, precision=prec)
        fn = {"fwd": lambda: af.convolve2_nn(Xa, Wa, st, pd, dl, precision=prec),
              "dgrad": lambda: af.convolve2_gradient_nn(Ga, Xa, Wa, Y, st, pd, dl,
                                                        af.AF_CONV_GRADIENT_DATA, precision=prec),
              "wgrad": lambda: af.convolve2_gradient_nn(Ga, Xa, Wa, Y, st, pd, dl,
                                                        af.AF_CONV_GRADIENT_FILTER, precision=prec),
              "step": step}[args.only]
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
        elif args.only in ("conv3", "conv3_expand"):
            v = torch.rand(256, 256, 256, device="cuda")
            V = af.Array.view_torch(v)
            k3 = g.standard_normal((3, 3, 3))
            F3 = af.Array.from_numpy(np.asfortranarray((k3 / k3.sum()).astype(np.float32)))
            mode = af.AF_CONV_EXPAND if args.only == "conv3_expand" else af.AF_CONV_DEFAULT
            fn = lambda: af.convolve3(V, F3, mode, af.AF_CONV_SPATIAL)  # noqa: E731
        elif args.only == "conv1":
            s1 = torch.rand(64, 1 << 20, device="cuda")
            S1 = af.Array.view_torch(s1)
            k1 = g.standard_normal(31)
            F1 = af.Array.from_numpy((k1 / k1.sum()).astype(np.float32))
            fn = lambda: af.convolve1(S1, F1, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)  # noqa: E731
        elif args.only == "fft31":
            xs = torch.rand(64, 2048, 2048, device="cuda")
            S = af.Array.view_torch(xs)
            k31 = g.standard_normal((31, 31))
            F31 = af.Array.from_numpy(np.asfortranarray((k31 / k31.sum()).astype(np.float32)))
            fn = lambda: af.convolve2(S, F31, af.AF_CONV_DEFAULT, af.AF_CONV_AUTO)  # noqa: E731
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
    ap.add_argument("--cpu-seconds", type=float, default=150.0,
                    help="time budget of the reference arm's full-batch CPU steps")
    ap.add_argument("--only", default=None,
                    choices=["fwd", "dgrad", "wgrad", "step", "sep_f32", "sep_u8", "same7", "fft31", "conv3",
                             "conv3_expand", "conv1", "cnn", "unwrap", "wrap", "unwrap_rows",
                             "wrap_rows", "image_callers"],
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
        cpu = cpu_nn_steps(args.steps, args.warmup, args.cpu_seconds)
        line = {"impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": "TFLOP/s",
                "n_gpus": args.gpus, "steps": cpu["steps"], "warmup": cpu["warmup"],
                "ms_per_step": cpu["seconds_per_step"] * 1e3,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                "dtype": "f32", "data": "synthetic", "config": config,
                "steps_requested": args.steps, "warmup_requested": args.warmup,
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
    cpu = cpu_nn_steps(2, 1, 30.0)
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
        "kernel_launches_per_step": res["kernel_launches_per_step"],
        "fp32_path": res["fp32_path"], "cudnn": res.get("cudnn"),
        "nn_workloads": res.get("nn_workloads"),
        "secondary": res.get("secondary"), "image_callers": res.get("image_callers"),
        "cnn4": res.get("cnn4"), "peaks": peaks,
    }
    print(json.dumps(line))


if __name__ == "__main__":
    main()
