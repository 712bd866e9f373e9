"""GPU parity at the benchmarked sizes, through the C ABI.

The bench times the direct kernels and the NN kernels on large workloads;
some code paths run only at those sizes (a 1-D signal crossing many
4096-sample tiles, persistent TMA CTAs walking several tiles through their
stage rings, split-K at full batch).  Each case here asserts which kernel
ran (the library's kernel timer) and compares with the oracle:

* direct convolutions in the exact mode: bit-exact on sampled slices
  (every slice where the oracle finishes in seconds); the default fused
  mode: |gpu - ref| <= 1e-6 * sum|s*f| per output;
* NN forward and gradients against FP64 on sampled points: FP32 max-abs
  <= 1e-5 * max|ref|; BF16 norm-wise relative <= 2e-2; FP8-E4M3 forward
  norm-wise relative <= 8e-2.
"""
import ctypes

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu


def _ran(af, name, fn):
    """Runs fn with the kernel timer on; returns (launches of `name`, fn())."""
    L = af.lib()
    L.afgb_kernel_timing(1)
    try:
        r = fn()
        af.sync()
        c = ctypes.c_ulonglong()
        ms = ctypes.c_double()
        L.afgb_kernel_time(name.encode(), ctypes.byref(c), ctypes.byref(ms))
    finally:
        L.afgb_kernel_timing(0)
    return c.value, r


def _exact(af, fn):
    af.set_exact_fp(True)
    try:
        return fn()
    finally:
        af.set_exact_fp(False)


def assert_same(got, ref, what=""):
    """Bit-for-bit equality of two float arrays of the same size, reported
    as the number of differing elements and the first few (a plain
    `assert a.tobytes() == b.tobytes()` makes pytest diff megabytes)."""
    g = np.ascontiguousarray(np.asarray(got)).ravel(order="K").view(np.uint32)
    r = np.ascontiguousarray(np.asarray(ref)).ravel(order="K").view(np.uint32)
    assert g.size == r.size, f"{what}: {g.size} vs {r.size} elements"
    bad = np.nonzero(g != r)[0]
    if bad.size:
        gf, rf = g.view(np.float32), r.view(np.float32)
        first = [(int(i), float(gf[i]), float(rf[i])) for i in bad[:6]]
        raise AssertionError(f"{what}: {bad.size} of {g.size} differ; first (index, got, ref): {first}")


def _fused_ok(oracle, out, s, f, rank, expand):
    """max over outputs of |out - ref| / sum|s*f| (all flattened in the
    same column-major order, so no broadcasting between shapes)."""
    ref = oracle.convolve(s, f, C.F32, rank, expand).ravel(order="F")
    bound = oracle.convolve(np.abs(s.astype(np.float64)), np.abs(f.astype(np.float64)), C.F64,
                            rank, expand).ravel(order="F")
    out = np.asarray(out).ravel(order="F")
    assert out.size == ref.size
    err = np.abs(out.astype(np.float64) - ref)
    return float((err / (bound + 1e-30)).max())


# ---------------------------------------------------------------------------
# 1-D: tiles of 4096 outputs
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("taps", [31, 129])
@pytest.mark.parametrize("expand", [False, True], ids=["default", "expand"])
def test_conv1_64x1M(af, oracle, taps, expand):
    """64 signals of 2^20 samples (256 tiles each; EXPAND's 2^20 + taps - 1
    outputs leave a ragged last tile); three slices compared bit for bit."""
    import torch

    gen = torch.Generator(device="cuda").manual_seed(100 + taps)
    s = torch.rand(64, 1 << 20, device="cuda", generator=gen)
    g = C.rng(taps)
    k = g.standard_normal(taps)
    f = (k / k.sum()).astype(np.float32)
    S, F = af.Array.view_torch(s), af.Array.from_numpy(f)
    mode = af.AF_CONV_EXPAND if expand else af.AF_CONV_DEFAULT
    n, out = _exact(af, lambda: _ran(af, "conv1_pipe_kernel",
                                     lambda: af.convolve1(S, F, mode, af.AF_CONV_SPATIAL)))
    assert n == 1
    assert out.dims == [(1 << 20) + (taps - 1 if expand else 0), 64, 1, 1]
    o = out.to_torch().reshape(64, -1)
    for b in (0, 29, 63):
        sb = s[b].cpu().numpy()
        ref = oracle.convolve(sb, f, C.F32, 1, expand)
        assert_same(o[b].cpu().numpy(), ref, f"slice {b}")
    fused = af.convolve1(S, F, mode, af.AF_CONV_SPATIAL).to_torch().reshape(64, -1)
    sb = s[17].cpu().numpy()
    assert _fused_ok(oracle, fused[17].cpu().numpy(), sb, f, 1, expand) <= 1e-6


@pytest.mark.parametrize("taps", [31, 129, 30])
@pytest.mark.parametrize("expand", [False, True], ids=["default", "expand"])
def test_conv1_ragged_many_tiles(af, oracle, taps, expand):
    """400 signals of 12345 samples: four tiles per signal, the last ragged,
    1600 tiles over a grid of at most 8 blocks per SM, so blocks loop over
    several tiles; every output compared bit for bit."""
    g = C.rng(500 + taps)
    s = np.asfortranarray(g.random((12345, 400), dtype=np.float32))
    k = g.standard_normal(taps)
    f = (k / k.sum()).astype(np.float32)
    S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
    mode = af.AF_CONV_EXPAND if expand else af.AF_CONV_DEFAULT
    n, out = _exact(af, lambda: _ran(af, "conv1_pipe_kernel",
                                     lambda: af.convolve1(S, F, mode, af.AF_CONV_SPATIAL)))
    assert n == 1
    ref = oracle.convolve(s, f, C.F32, 1, expand)
    assert_same(out.to_numpy(), ref)


def test_conv1_many2one_filter_batch(af, oracle):
    """One 50000-sample signal, 12 filters of 31 taps (RHS batch): 13 tiles
    per filter, each reading the same signal."""
    g = C.rng(808)
    s = g.random(50000, dtype=np.float32)
    f = np.asfortranarray(g.standard_normal((31, 12)).astype(np.float32))
    S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
    n, out = _exact(af, lambda: _ran(af, "conv1_pipe_kernel",
                                     lambda: af.convolve1(S, F, af.AF_CONV_DEFAULT,
                                                          af.AF_CONV_SPATIAL)))
    assert n == 1
    assert_same(out.to_numpy(), oracle.convolve(s, f, C.F32, 1, False))


def test_conv1_strided_signal_takes_tile_kernel(af, oracle):
    """A signal read with a stride (every other sample of a torch tensor)
    runs the shared-memory tile kernel; bit for bit in the exact mode."""
    import torch

    base = torch.rand(3, 2 * 9000, device="cuda")
    view = af.Array.view_device(base.data_ptr(), [9000, 3], af.f32, strides=[2, 18000], keep=base)
    f = C.rng(5).standard_normal(31).astype(np.float32)
    F = af.Array.from_numpy(f)
    n, out = _exact(af, lambda: _ran(af, "conv1_tile_kernel",
                                     lambda: af.convolve1(view, F, af.AF_CONV_EXPAND,
                                                          af.AF_CONV_SPATIAL)))
    assert n == 1
    dense = np.asfortranarray(base.cpu().numpy()[:, ::2].T)
    assert_same(out.to_numpy(), oracle.convolve(dense, f, C.F32, 1, True))


# ---------------------------------------------------------------------------
# 2-D persistent TMA kernels
# ---------------------------------------------------------------------------
def test_same7x7_64x2048sq(af, oracle):
    """64 images of 2048x2048, 64 distinct 7x7 filters (SAME batch,
    AF_CONV_SPATIAL): 65536 tiles over the persistent grid; three slices
    bit for bit in the exact mode, one in the fused mode."""
    import torch

    gen = torch.Generator(device="cuda").manual_seed(7)
    x = torch.rand(64, 2048, 2048, device="cuda", generator=gen)
    g = C.rng(77)
    f7 = g.standard_normal((7, 7, 64))
    f7 = np.asfortranarray((f7 / f7.sum(axis=(0, 1), keepdims=True)).astype(np.float32))
    S, F = af.Array.view_torch(x), af.Array.from_numpy(f7)
    run = lambda: af.convolve2(S, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)  # noqa: E731
    n, out = _exact(af, lambda: _ran(af, "conv2_tma_kernel", run))
    assert n == 1
    o = out.to_torch().reshape(64, 2048, 2048)
    for b in (0, 40, 63):
        sb = np.asfortranarray(x[b].cpu().numpy().T)
        ref = oracle.convolve(sb, f7[:, :, b], C.F32, 2, False)
        assert_same(np.asfortranarray(o[b].cpu().numpy().T).ravel(order="F"), ref.ravel(order="F"),
                    f"slice {b}")
    fused = run().to_torch().reshape(64, 2048, 2048)
    sb = np.asfortranarray(x[5].cpu().numpy().T)
    got = np.asfortranarray(fused[5].cpu().numpy().T)
    assert _fused_ok(oracle, got, sb, f7[:, :, 5], 2, False) <= 1e-6


@pytest.mark.parametrize("fsz,expand,kind", [(7, False, "lhs"), (5, True, "same"),
                                             (3, False, "rhs")])
def test_conv2_tma_many_tiles_per_cta(af, oracle, fsz, expand, kind):
    """More tiles than resident CTAs (2048-4096 tiles of 64x64 over at most
    two CTAs per SM), so each CTA wraps its three-stage ring several times;
    every output bit for bit in the exact mode."""
    g = C.rng(900 + fsz)
    if kind == "rhs":
        s = np.asfortranarray(g.random((1024, 1024), dtype=np.float32))
        f = np.asfortranarray(g.standard_normal((fsz, fsz, 4)).astype(np.float32))
    else:
        s = np.asfortranarray(g.random((512, 512, 32), dtype=np.float32))
        fs = (fsz, fsz) if kind == "lhs" else (fsz, fsz, 32)
        f = np.asfortranarray(g.standard_normal(fs).astype(np.float32))
    S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
    mode = af.AF_CONV_EXPAND if expand else af.AF_CONV_DEFAULT
    n, out = _exact(af, lambda: _ran(af, "conv2_tma_kernel",
                                     lambda: af.convolve2(S, F, mode, af.AF_CONV_SPATIAL)))
    assert n == 1
    assert_same(out.to_numpy(), oracle.convolve(s, f, C.F32, 2, expand))


RUN_CHILD = r"""
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests/golden")
import torch
import arrayfire_gb300 as af
import oracle as O
import cases as C
O.build_port()
af.lib(); torch.cuda.init(); af.set_stream(torch.cuda.current_stream())
res = {}
for i, (name, fsz, kind, expand, dt) in enumerate(json.loads(sys.argv[2])):
    code = C.U8 if dt == "u8" else C.F32
    nb = 12
    s = C.make_signal(code, (520, 200, nb), 910 + i)
    f = C.make_filter(code, (fsz, fsz) + ((nb,) if kind == "same" else ()), 930 + i, 2)
    S = af.Array.from_numpy(s, code)
    F = af.Array.from_numpy(f)
    mode = af.AF_CONV_EXPAND if expand else af.AF_CONV_DEFAULT
    af.set_exact_fp(True)
    out = af.convolve2(S, F, mode, af.AF_CONV_SPATIAL).to_numpy()
    af.set_exact_fp(False)
    ref = O.convolve(s, f, code, 2, expand)
    res[name] = bool(out.tobytes() == ref.tobytes())
print(json.dumps(res))
"""


@pytest.mark.parametrize("run_len", [3, 8])
def test_conv2_tma_tile_runs_in_child_process(run_len):
    """The 2-D kernel's tile order with a forced run length (AFGB_TILE_RUN, in
    a child process): each CTA takes `run_len` consecutive tiles per round,
    so runs cross image boundaries (a filter change inside a run, SAME batch
    of 12 distinct filters), the last round is partial and most CTAs get no
    tile of it.  Every output bit for bit in the exact mode, f32 and u8,
    for the 128-wide (7x7) and 64-wide (3x3, 5x5) tiles."""
    import json
    import os
    import subprocess
    import sys
    from pathlib import Path

    root = Path(__file__).resolve().parents[1]
    cases = [["f32_7x7_same", 7, "same", False, "f32"], ["f32_7x7_lhs_expand", 7, "lhs", True, "f32"],
             ["f32_5x5_same_expand", 5, "same", True, "f32"], ["f32_3x3_same", 3, "same", False, "f32"],
             ["u8_7x7_same", 7, "same", False, "u8"], ["u8_3x3_lhs", 3, "lhs", False, "u8"]]
    env = dict(os.environ, AFGB_TILE_RUN=str(run_len))
    r = subprocess.run([sys.executable, "-c", RUN_CHILD, str(root), json.dumps(cases)],
                       capture_output=True, text=True, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert res == {c[0]: True for c in cases}, res


def test_sep15_f32_64x2048sq(af, oracle):
    """The fused separable kernel on 64 images of 2048x2048 (15 + 15 taps):
    three slices bit for bit in the exact mode, one in the fused mode."""
    import torch

    gen = torch.Generator(device="cuda").manual_seed(15)
    x = torch.rand(64, 2048, 2048, device="cuda", generator=gen)
    g = C.rng(1515)
    t = g.standard_normal(15)
    cf = (t / t.sum()).astype(np.float32)
    t = g.standard_normal(15)
    rf = (t / t.sum()).astype(np.float32)
    S = af.Array.view_torch(x)
    CF, RF = af.Array.from_numpy(cf), af.Array.from_numpy(rf)
    n, out = _exact(af, lambda: _ran(af, "sep_tma_kernel",
                                     lambda: af.convolve2_separable(CF, RF, S)))
    assert n == 1
    o = out.to_torch().reshape(64, 2048, 2048)
    for b in (0, 33, 63):
        sb = np.asfortranarray(x[b].cpu().numpy().T)
        ref = oracle.convolve2_sep(sb, cf, rf, C.F32, False)
        assert_same(np.asfortranarray(o[b].cpu().numpy().T).ravel(order="F"), ref.ravel(order="F"),
                    f"slice {b}")
    fused = af.convolve2_separable(CF, RF, S).to_torch().reshape(64, 2048, 2048)
    sb = np.asfortranarray(x[9].cpu().numpy().T)
    ref = oracle.convolve2_sep(sb, cf, rf, C.F32, False)
    # |sep - ref| <= 1e-6 * (|cf| (x) |rf|) * |s|, the separable sum of |terms|
    bound = oracle.convolve2_sep(np.abs(sb.astype(np.float64)), np.abs(cf.astype(np.float64)),
                                 np.abs(rf.astype(np.float64)), C.F64, False)
    got = np.asfortranarray(fused[9].cpu().numpy().T).ravel(order="F")
    ref, bound = ref.ravel(order="F"), bound.ravel(order="F")
    assert float((np.abs(got - ref) / (bound + 1e-30)).max()) <= 1e-6


@pytest.mark.parametrize("expand", [False, True], ids=["default", "expand"])
def test_sep_tma_many_tiles_per_cta(af, oracle, expand):
    """32 images of 512x512 with 15 + 15 taps (7 + 7 in EXPAND mode; the TMA
    kernel takes equal lengths): 2048 tiles over the two-stage ring of each
    CTA; every output bit for bit."""
    g = C.rng(2222)
    s = np.asfortranarray(g.random((512, 512, 32), dtype=np.float32))
    taps = 7 if expand else 15
    cf = g.standard_normal(taps).astype(np.float32)
    rf = g.standard_normal(taps).astype(np.float32)
    S = af.Array.from_numpy(s)
    CF, RF = af.Array.from_numpy(cf), af.Array.from_numpy(rf)
    mode = af.AF_CONV_EXPAND if expand else af.AF_CONV_DEFAULT
    n, out = _exact(af, lambda: _ran(af, "sep_tma_kernel",
                                     lambda: af.convolve2_separable(CF, RF, S, mode)))
    assert n == 1
    assert_same(out.to_numpy(), oracle.convolve2_sep(s, cf, rf, C.F32, expand))


# ---------------------------------------------------------------------------
# 3-D
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("expand", [False, True], ids=["default", "expand"])
def test_conv3_256cube(af, oracle, expand):
    """The 256^3 volume with a 3x3x3 filter, every output bit for bit in the
    exact mode, and within 1e-6 * sum|s*f| in the fused mode."""
    g = C.rng(256)
    v = np.asfortranarray(g.random((256, 256, 256), dtype=np.float32))
    k3 = g.standard_normal((3, 3, 3))
    f = np.asfortranarray((k3 / k3.sum()).astype(np.float32))
    V, F = af.Array.from_numpy(v), af.Array.from_numpy(f)
    mode = af.AF_CONV_EXPAND if expand else af.AF_CONV_DEFAULT
    n, out = _exact(af, lambda: _ran(af, "conv3_tma_kernel",
                                     lambda: af.convolve3(V, F, mode, af.AF_CONV_SPATIAL)))
    assert n == 1
    ref = oracle.convolve(v, f, C.F32, 3, expand)
    assert_same(out.to_numpy(), ref)
    fused = af.convolve3(V, F, mode, af.AF_CONV_SPATIAL).to_numpy()
    assert _fused_ok(oracle, fused, v, f, 3, expand) <= 1e-6


# ---------------------------------------------------------------------------
# NN at the benchmarked shapes, sampled points against FP64
# ---------------------------------------------------------------------------
NN_BENCH = {
    # 128x128x64x32 * 3x3x64x128, stride 1, pad 1 (the headline workload)
    "3a": ((128, 128, 64, 32), (3, 3, 64, 128), (1, 1), (1, 1), (1, 1)),
    # 56x56x256x64 * 1x1x256x512
    "3b": ((56, 56, 256, 64), (1, 1, 256, 512), (1, 1), (0, 0), (1, 1)),
    # 64x64x128x16 * 3x3x128x256, stride 2, pad 1
    "4a": ((64, 64, 128, 16), (3, 3, 128, 256), (2, 2), (1, 1), (1, 1)),
    # 64x64x128x16 * 5x5x128x256, stride 2, pad 4, dilation 2
    "4b": ((64, 64, 128, 16), (5, 5, 128, 256), (2, 2), (4, 4), (2, 2)),
}

_nn_cache = {}


def _nn_data(key):
    if key not in _nn_cache:
        sd, fd, st, pd, dl = NN_BENCH[key]
        g = C.rng(4000 + sum(map(ord, key)))
        x = np.asfortranarray(g.standard_normal(sd, dtype=np.float32))
        w = np.asfortranarray((g.standard_normal(fd) * np.sqrt(2.0 / (fd[0] * fd[1] * fd[2])))
                              .astype(np.float32))
        od = C.nn_out_dims(list(sd), list(fd), st, pd, dl)
        gy = np.asfortranarray(g.standard_normal(od, dtype=np.float32))
        _nn_cache.clear()
        _nn_cache[key] = (x, w, gy)
    return _nn_cache[key]


def _sampled(got, ref, prec, what):
    got = np.asarray(got, np.float64)
    if prec == "fp32":
        err = np.abs(got - ref).max()
        assert err <= 1e-5 * np.abs(ref).max(), f"{what}: max abs {err:.3e}"
    else:
        rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
        assert rel <= (8e-2 if prec == "fp8" else 2e-2), f"{what}: rel {rel:.3e}"


FWD_KERNEL = {"fp32": "simt_fwd_kernel", "bf16": "tc_fwd_kernel", "fp8": "tc_fwd_fp8_kernel"}


@pytest.mark.parametrize("prec", ["fp32", "bf16", "fp8"])
@pytest.mark.parametrize("key", list(NN_BENCH))
def test_nn_forward_bench_shape(af, oracle, key, prec):
    x, w, _ = _nn_data(key)
    sd, fd, st, pd, dl = NN_BENCH[key]
    X, W = af.Array.from_numpy(x), af.Array.from_numpy(w)
    n, y = _ran(af, FWD_KERNEL[prec], lambda: af.convolve2_nn(X, W, st, pd, dl, precision=prec))
    assert n == 1
    y = y.to_numpy().ravel(order="F")
    idx = C.rng(11).integers(0, y.size, 384)
    ref = oracle.nn_forward_points_f64(x, w, st, pd, dl, idx)
    _sampled(y[idx], ref, prec, f"{key} {prec} fwd")


@pytest.mark.parametrize("prec", ["fp32", "bf16"])
@pytest.mark.parametrize("key", list(NN_BENCH))
def test_nn_gradients_bench_shape(af, oracle, key, prec):
    """Data and filter gradients through the combined call (the bench's
    step) and the per-gradient call, sampled against FP64."""
    x, w, gy = _nn_data(key)
    sd, fd, st, pd, dl = NN_BENCH[key]
    X, W, G = af.Array.from_numpy(x), af.Array.from_numpy(w), af.Array.from_numpy(gy)
    dx, dw, db = af.convolve2_gradients_nn(G, X, W, st, pd, dl, precision=prec, bias=True)
    dxn = dx.to_numpy().ravel(order="F")
    dwn = dw.to_numpy().ravel(order="F")
    g = C.rng(12)
    i1 = g.integers(0, dxn.size, 256)
    _sampled(dxn[i1], oracle.nn_data_grad_points_f64(gy, list(sd), w, st, pd, dl, i1), prec,
             f"{key} {prec} dgrad")
    i2 = g.integers(0, dwn.size, 96)
    _sampled(dwn[i2], oracle.nn_filter_grad_points_f64(gy, x, list(fd), st, pd, dl, i2), prec,
             f"{key} {prec} wgrad")
    dbr = gy.astype(np.float64).sum(axis=(0, 1, 3))
    assert np.abs(db.to_numpy().ravel() - dbr).max() <= 1e-5 * np.abs(gy).sum(axis=(0, 1, 3)).max()
    # the per-gradient entry point gives the same bits
    Y = af.convolve2_nn(X, W, st, pd, dl)
    dw1 = af.convolve2_gradient_nn(G, X, W, Y, st, pd, dl, af.AF_CONV_GRADIENT_FILTER,
                                   precision=prec).to_numpy().ravel(order="F")
    assert_same(dw1, dwn, "per-gradient call")
