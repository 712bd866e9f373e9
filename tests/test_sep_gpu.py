"""GPU parity of af_convolve2_sep through the C ABI against the oracle.

Semantics are the reference CPU backend's (src/backend/cpu/kernel/
convolve.hpp:213-289): for integer inputs the taps are converted to the input
type and the intermediate image is stored in the input type, so results are
compared bit for bit; f32 in the exact mode is bit-exact too, and in the
default fused mode within 1e-6 * sum|terms| (two passes, bound propagated).
"""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu
GOLD = Path(__file__).resolve().parent / "golden"
SEP = json.loads((GOLD / "sep.json").read_text())
CASES = list(C.sep_cases())


def digest(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


def run(af, s, cf, rf, dt, expand):
    S = af.Array.from_numpy(s, dt)
    Cf = af.Array.from_numpy(cf)
    Rf = af.Array.from_numpy(rf)
    return af.convolve2_separable(Cf, Rf, S, af.AF_CONV_EXPAND if expand else af.AF_CONV_DEFAULT
                                  ).to_numpy()


@pytest.mark.parametrize("case", CASES, ids=lambda c: c[0])
def test_sep_exact(af, oracle, case):
    cid, dt, sd, cl, rl, expand, seed = case
    s = C.sep_signal(dt, sd, seed)
    cf, rf = C.sep_taps(dt, cl, seed + 1), C.sep_taps(dt, rl, seed + 2)
    af.set_exact_fp(True)
    try:
        out = run(af, s, cf, rf, dt, expand)
    finally:
        af.set_exact_fp(False)
    ref = oracle.convolve2_sep(s, cf, rf, dt, expand)
    assert out.shape == ref.shape
    assert out.tobytes() == ref.tobytes()
    assert digest(out) == SEP[cid]["sha256"]


@pytest.mark.parametrize("case", [c for c in CASES if c[1] == C.F32], ids=lambda c: c[0])
def test_sep_fused_f32(af, oracle, case):
    cid, dt, sd, cl, rl, expand, seed = case
    s = C.sep_signal(dt, sd, seed)
    cf, rf = C.sep_taps(dt, cl, seed + 1), C.sep_taps(dt, rl, seed + 2)
    out = run(af, s, cf, rf, dt, expand)
    ref = oracle.convolve2_sep(s, cf, rf, dt, expand)
    bound = oracle.convolve2_sep(np.abs(s).astype(np.float64), np.abs(cf).astype(np.float64),
                                 np.abs(rf).astype(np.float64), C.F64, expand)
    assert np.all(np.abs(out.astype(np.float64) - ref) <= 2e-6 * bound + 1e-30)


def test_sep_u8_full_config_properties(af, oracle):
    """The u8 bench workload (64 images 2048x2048, 15-tap N(0,1)/sum taps) at
    full size: spot-check 3 slices against the oracle bit for bit."""
    g = C.rng(21)
    s = np.asfortranarray(g.integers(0, 256, (2048, 2048, 64)).astype(np.uint8))
    t = g.standard_normal(15)
    cf = (t / t.sum()).astype(np.float32)
    t = g.standard_normal(15)
    rf = (t / t.sum()).astype(np.float32)
    out = run(af, s, cf, rf, C.U8, False)
    for k in (0, 31, 63):
        ref = oracle.convolve2_sep(s[:, :, k], cf, rf, C.U8, False)
        assert out[:, :, k:k + 1, :].tobytes() == ref.tobytes()


def test_sep_scalar_filters(af, oracle):
    """Both filters scalar: element-wise shortcut (src/api/c/convolve.cpp:57-68)."""
    s = C.sep_signal(C.F32, (9, 7), 3)
    out = run(af, s, np.array([2.0], np.float32), np.array([0.5], np.float32), C.F32, True)
    np.testing.assert_array_equal(out[:, :, 0, 0], s[:, :, 0, 0] * np.float32(1.0))


def test_sep_rejections(af):
    """test/convolve.cpp:309-367: 1-D signal -> AF_ERR_ARG; non-vector filter
    -> AF_ERR_ARG; filters longer than 31 -> AF_ERR_NOT_SUPPORTED."""
    S1 = af.Array.from_numpy(np.ones(10, np.float32))
    f4 = af.Array.from_numpy(np.ones(4, np.int32))
    with pytest.raises(af.AfError) as e:
        af.convolve2_separable(f4, f4, S1, af.AF_CONV_EXPAND)
    assert e.value.code == af.AF_ERR_ARG
    S2 = af.Array.from_numpy(np.ones((10, 10), np.float32))
    m = af.Array.from_numpy(np.ones((3, 3), np.float32))
    with pytest.raises(af.AfError) as e:
        af.convolve2_separable(m, f4, S2, af.AF_CONV_DEFAULT)
    assert e.value.code == af.AF_ERR_ARG
    # a one-tap filter next to a longer one is not a vector and not a
    # scalar pair: AF_ERR_ARG (src/api/c/convolve.cpp:57-71)
    one = af.Array.from_numpy(np.ones(1, np.float32))
    with pytest.raises(af.AfError) as e:
        af.convolve2_separable(one, f4, S2, af.AF_CONV_DEFAULT)
    assert e.value.code == af.AF_ERR_ARG
    long = af.Array.from_numpy(np.ones(33, np.float32))
    with pytest.raises(af.AfError) as e:
        af.convolve2_separable(long, f4, S2, af.AF_CONV_DEFAULT)
    assert e.value.code == af.AF_ERR_NOT_SUPPORTED


TMA_SEP = [c for c in CASES if c[0].startswith("sep_") and "_tma_" in c[0]
           and c[1] in (C.F32, C.U8, C.S8)]


@pytest.mark.parametrize("case", TMA_SEP, ids=lambda c: c[0])
def test_sep_tma_path_taken(af, oracle, case):
    """Dense 16-byte-row images with equal 3/5/7/15-tap filters run on the
    fused TMA-staged kernel (no temporary image)."""
    import ctypes

    cid, dt, sd, cl, rl, expand, seed = case
    s = C.sep_signal(dt, sd, seed)
    cf, rf = C.sep_taps(dt, cl, seed + 1), C.sep_taps(dt, rl, seed + 2)
    L = af.lib()
    L.afgb_kernel_timing(1)
    try:
        out = run(af, s, cf, rf, dt, expand)
        c, ms = ctypes.c_ulonglong(), ctypes.c_double()
        L.afgb_kernel_time(b"sep_tma_kernel", ctypes.byref(c), ctypes.byref(ms))
    finally:
        L.afgb_kernel_timing(0)
    assert c.value == 1
    if dt != C.F32:
        assert out.tobytes() == oracle.convolve2_sep(s, cf, rf, dt, expand).tobytes()
