"""GPU parity of af_convolve1/2/3 through the C ABI against the oracle.

* integer inputs: bit-exact against the oracle port and the reference's hash;
* f32/f64/c32/c64 with afgb_set_exact_fp(1): bit-exact (the reference's
  rounding order, no fused multiply-add);
* f32/f64/c32/c64 in the default fused mode: |gpu - ref| <= TOL * sum|s*f|
  per output element, TOL = 1e-6 (f32, c32) and 1e-14 (f64, c64).
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
DIRECT = json.loads((GOLD / "direct.json").read_text())
TOL = {C.F32: 1e-6, C.C32: 1e-6, C.F64: 1e-14, C.C64: 1e-14}
FLOATS = (C.F32, C.F64, C.C32, C.C64)


def digest(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


def run(af, s, f, dt, rank, expand, domain=None):
    S = af.Array.from_numpy(s, dt)
    F = af.Array.from_numpy(f)
    fn = {1: af.convolve1, 2: af.convolve2, 3: af.convolve3}[rank]
    mode = af.AF_CONV_EXPAND if expand else af.AF_CONV_DEFAULT
    out = fn(S, F, mode, af.AF_CONV_SPATIAL if domain is None else domain)
    return out.to_numpy()


def abs_bound(oracle, s, f, rank, expand):
    """sum over taps of |s*f| per output element, in FP64 (for complex
    operands (|re|+|im|)(|re|+|im|) bounds the four partial products)."""
    if np.iscomplexobj(s):
        sa = np.abs(s.real).astype(np.float64) + np.abs(s.imag)
        fa = np.abs(f.real).astype(np.float64) + np.abs(f.imag)
    else:
        sa = np.abs(s.astype(np.float64))
        fa = np.abs(f.astype(np.float64))
    return oracle.convolve(sa, fa, C.F64, rank, expand)


CASES = list(C.direct_cases())


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_direct_exact(af, oracle, case):
    cid, dt, rank, sd, fd, expand, seed = case
    s = C.make_signal(dt, sd, seed)
    f = C.make_filter(dt, fd, seed + 1, rank)
    af.set_exact_fp(True)
    try:
        out = run(af, s, f, dt, rank, expand)
    finally:
        af.set_exact_fp(False)
    ref = oracle.convolve(s, f, dt, rank, expand)
    assert out.shape == ref.shape
    assert out.tobytes() == ref.tobytes(), f"max diff {np.abs(out.astype(np.complex128) - ref).max()}"
    assert digest(out) == DIRECT[cid]["sha256"]


@pytest.mark.parametrize("case", [c for c in CASES if c[1] in FLOATS], ids=lambda c: c[0])
def test_direct_fused_within_tolerance(af, oracle, case):
    cid, dt, rank, sd, fd, expand, seed = case
    s = C.make_signal(dt, sd, seed)
    f = C.make_filter(dt, fd, seed + 1, rank)
    out = run(af, s, f, dt, rank, expand)
    ref = oracle.convolve(s, f, dt, rank, expand)
    bound = abs_bound(oracle, s, f, rank, expand)
    err = np.abs(out.astype(np.complex128) - ref.astype(np.complex128))
    assert np.all(err <= TOL[dt] * bound + 1e-30), float((err / (bound + 1e-30)).max())


@pytest.mark.parametrize("name,fn", [("config1a_gauss5_512", C.config1a),
                                     ("config1b_neighbour3_1024", C.config1b)])
def test_config1_full_size(af, oracle, name, fn):
    """The 512x512 Gaussian and 1024x1024 neighbour-count images at full
    size: bit-exact in the exact mode,
    within 1e-6 relative in the default mode."""
    s, f = fn()
    af.set_exact_fp(True)
    try:
        out = run(af, s, f, C.F32, 2, False)
    finally:
        af.set_exact_fp(False)
    assert digest(out) == DIRECT[name]["sha256"]
    fast = run(af, s, f, C.F32, 2, False)
    ref = oracle.convolve(s, f, C.F32, 2, False)
    # every term is non-negative here, so sum|s*f| is the result itself
    np.testing.assert_allclose(fast, ref, rtol=1e-6, atol=1e-7)


def test_large_batch_identity_filter(af):
    """test/convolve.cpp:750-783: identity filter over 65536 batch slices."""
    n, big = 10, 65536
    sig = np.ones((n, n, big), np.float32, order="F")
    filt = np.zeros((3, 3), np.float32)
    filt[1, 1] = 1
    out = run(af, sig, filt, C.F32, 2, False)
    assert out.sum(dtype=np.float64) == big * n * n
    out1 = run(af, np.ones((n, 1, big), np.float32, order="F"), np.array([0, 1, 0], np.float32),
               C.F32, 1, False)
    assert out1.sum(dtype=np.float64) == big * n


def test_auto_domain_takes_fft_route_for_batched_filters(af, oracle):
    """kbatch >= 10 makes the reference choose the frequency domain
    (src/api/c/convolve.cpp:112-115); AUTO then gives the FFT result, equal
    to the spatial one within rounding."""
    s = C.make_signal(C.F32, (40, 30, 12), 11)
    f = C.make_filter(C.F32, (5, 5, 12), 12, 2)
    out = run(af, s, f, C.F32, 2, False, domain=af.AF_CONV_AUTO)
    fft = af.fft_convolve2(af.Array.from_numpy(s), af.Array.from_numpy(f)).to_numpy()
    assert out.tobytes() == fft.tobytes()
    ref = oracle.convolve(s, f, C.F32, 2, False)
    bound = abs_bound(oracle, s, f, 2, False)
    assert np.all(np.abs(out - ref) <= 1e-5 * bound.max() + 1e-30)


def test_unsupported_filter_sizes(af):
    """Same limits and code as the reference CUDA backend
    (src/backend/cuda/kernel/convolve.hpp:149-157)."""
    S = af.Array.from_numpy(np.ones((40, 40), np.float32))
    for fshape in [(7, 3), (18, 18), (6, 5)]:
        F = af.Array.from_numpy(np.ones(fshape, np.float32))
        with pytest.raises(af.AfError) as e:
            af.convolve2(S, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)
        assert e.value.code == af.AF_ERR_NOT_SUPPORTED
    S3 = af.Array.from_numpy(np.ones((10, 10, 10), np.float32))
    F3 = af.Array.from_numpy(np.ones((6, 5, 5), np.float32))
    with pytest.raises(af.AfError) as e:
        af.convolve3(S3, F3, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)
    assert e.value.code == af.AF_ERR_NOT_SUPPORTED


def test_diff_batch_and_types_rejected(af):
    """test/convolve.cpp:309-367 style checks: DIFF batch -> AF_ERR_ARG,
    f16 signal -> AF_ERR_TYPE."""
    S = af.Array.from_numpy(np.ones((8, 8, 2), np.float32))
    F = af.Array.from_numpy(np.ones((3, 3, 3), np.float32))
    with pytest.raises(af.AfError) as e:
        af.convolve2(S, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)
    assert e.value.code == af.AF_ERR_ARG
    H = af.Array.from_numpy(np.ones((8, 8), np.float16))
    F2 = af.Array.from_numpy(np.ones((3, 3), np.float32))
    with pytest.raises(af.AfError) as e:
        af.convolve2(H, F2, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)
    assert e.value.code == af.AF_ERR_TYPE


def test_empty_signal_returns_signal(af):
    """src/api/c/convolve.cpp:143-145: an empty input returns the signal."""
    S = af.Array.empty([0, 4], af.f32)
    F = af.Array.from_numpy(np.ones((3, 3), np.float32))
    out = af.convolve2(S, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)
    assert out.dims == [0, 4, 1, 1]


def test_strided_view_input(af, oracle):
    """A non-contiguous view (every other column of a bigger buffer) gives the
    same result as its dense copy."""
    import torch

    base = torch.randn(64, 50, device="cuda")  # rows (dim1) x cols (dim0)
    view = af.Array.view_device(base.data_ptr(), [25, 64], af.f32, strides=[2, 50], keep=base)
    F = af.Array.from_numpy(C.make_filter(C.F32, (5, 5), 3, 2))
    af.set_exact_fp(True)
    try:
        out = af.convolve2(view, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL).to_numpy()
    finally:
        af.set_exact_fp(False)
    dense = base.cpu().numpy().T[::2, :]
    ref = oracle.convolve(np.asfortranarray(dense), C.make_filter(C.F32, (5, 5), 3, 2), C.F32, 2,
                          False)
    assert out.tobytes() == ref.tobytes()


def test_allocation_failure_reports_no_mem(af):
    S = af.Array.from_numpy(np.ones((16, 16), np.float32))
    F = af.Array.from_numpy(np.ones((3, 3), np.float32))
    af.lib().afgb_debug_fail_alloc_after(1)
    try:
        with pytest.raises(af.AfError) as e:
            af.convolve2(S, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)
        assert e.value.code == af.AF_ERR_NO_MEM
    finally:
        af.lib().afgb_debug_fail_alloc_after(0)
    # the library is still usable afterwards
    out = af.convolve2(S, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL).to_numpy()
    assert out[8, 8, 0, 0] == 9.0


def _ran(af, name, fn):
    """Runs fn with the library's kernel timing on; the number of launches
    recorded under `name`."""
    import ctypes

    L = af.lib()
    L.afgb_kernel_timing(1)
    try:
        fn()
        af.sync()
        c = ctypes.c_ulonglong()
        ms = ctypes.c_double()
        L.afgb_kernel_time(name.encode(), ctypes.byref(c), ctypes.byref(ms))
    finally:
        L.afgb_kernel_timing(0)
    return c.value


TMA_2D = [c for c in CASES if c[0].startswith("r_tma_") and c[1] in (C.F32, C.U8, C.S8)]


@pytest.mark.parametrize("case", TMA_2D, ids=lambda c: c[0])
def test_tma_2d_path_taken(af, oracle, case):
    """Dense images with 16-byte rows and 3/5/7 square filters run on the
    TMA-staged kernel, in every batch kind (a fallback would still be
    correct, so the path itself is checked)."""
    cid, dt, rank, sd, fd, expand, seed = case
    s = C.make_signal(dt, sd, seed)
    f = C.make_filter(dt, fd, seed + 1, rank)
    out = {}
    n = _ran(af, "conv2_tma_kernel", lambda: out.setdefault("o", run(af, s, f, dt, rank, expand)))
    assert n == 1
    if dt != C.F32:
        assert out["o"].tobytes() == oracle.convolve(s, f, dt, rank, expand).tobytes()


TMA_3D = [c for c in CASES if c[0].startswith("c_tma_") and c[1] == C.F32]


@pytest.mark.parametrize("case", TMA_3D, ids=lambda c: c[0])
def test_tma_3d_path_taken(af, oracle, case):
    """Dense f32 volumes with 16-byte rows and a 3x3x3 filter run on the
    TMA-staged 3-D kernel in every batch kind, bit-exact in the exact mode."""
    cid, dt, rank, sd, fd, expand, seed = case
    s = C.make_signal(dt, sd, seed)
    f = C.make_filter(dt, fd, seed + 1, rank)
    out = {}
    af.set_exact_fp(True)
    try:
        n = _ran(af, "conv3_tma_kernel", lambda: out.setdefault("o", run(af, s, f, dt, rank, expand)))
    finally:
        af.set_exact_fp(False)
    assert n == 1
    assert out["o"].tobytes() == oracle.convolve(s, f, dt, rank, expand).tobytes()


@pytest.mark.parametrize("kind", ["lhs", "same"])
def test_tma_3d_multi_tile_per_cta(af, oracle, kind):
    """More tiles than resident CTAs, so each CTA walks several tiles through
    both of its buffers (256x64x64 x 2 volumes = 512 tiles)."""
    g = np.random.Generator(np.random.Philox(71))
    s = np.asfortranarray(g.random((256, 64, 64, 2), dtype=np.float32))
    fshape = (3, 3, 3) if kind == "lhs" else (3, 3, 3, 2)
    f = np.asfortranarray(g.standard_normal(fshape).astype(np.float32))
    out = {}
    af.set_exact_fp(True)
    try:
        n = _ran(af, "conv3_tma_kernel", lambda: out.setdefault("o", run(af, s, f, C.F32, 3, False)))
    finally:
        af.set_exact_fp(False)
    assert n == 1
    assert out["o"].tobytes() == oracle.convolve(s, f, C.F32, 3, False).tobytes()
