"""CPU tests of af_harris: the oracle port against the digests of the
reference's own CPU kernels (tests/golden/harris.json, written by
tests/golden/gen_golden.py with the port asserted identical to the
reference), the host-side window, and the argument checks of
src/api/c/harris.cpp:52-66 through the C ABI on a device view that is never
read (no device work)."""
import ctypes
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import cases as C

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "harris.json").read_text())
DIMS4 = ctypes.c_longlong * 4


def digest(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


@pytest.mark.parametrize("case", C.harris_cases(), ids=lambda c: c[0])
def test_harris_port_matches_reference_digests(oracle, case):
    cid, dt, shape, mc, mr, sg, bs, k, kind, seed = case
    x, y, s = oracle.harris(C.harris_image(dt, shape, kind, seed), dt, mc, mr, sg, bs, k)
    g = GOLD[cid]
    assert x.size == g["n"]
    assert (digest(x), digest(y), digest(s)) == (g["x"], g["y"], g["score"])


def test_sort_cases_keep_the_strongest_in_order(oracle):
    """Where max_corners cut the list, the kept scores are non-increasing and
    equal scores keep scan order (x-major, then y)."""
    seen_tie = False
    for cid, dt, shape, mc, mr, sg, bs, k, kind, seed in C.harris_cases():
        if mc == 0:
            continue
        img = C.harris_image(dt, shape, kind, seed)
        if oracle.harris(img, dt, mc + 1, mr, sg, bs, k)[0].size <= mc:
            continue  # no more than max_corners found: kept in scan order, unsorted
        x, y, s = oracle.harris(img, dt, mc, mr, sg, bs, k)
        assert np.all(np.diff(s) <= 0), cid
        for i in range(s.size - 1):
            if s[i] == s[i + 1]:
                seen_tie = True
                assert (x[i], y[i]) < (x[i + 1], y[i + 1]), cid
    assert seen_tie  # the tiled images produce exact ties


def test_window_lengths_and_taps(oracle):
    # floor(6 sigma) made odd, else block_size
    assert oracle.harris_filter_len(1.0, 0) == 5
    assert oracle.harris_filter_len(5.0, 0) == 29
    assert oracle.harris_filter_len(0.5, 0) == 3
    assert oracle.harris_filter_len(1.0, 7) == 7
    w = oracle.harris_window(5, 1.0, C.F64)
    x = np.arange(5) - 2
    e = np.exp(-x * x / 2.0)
    np.testing.assert_allclose(w, e / e.sum(), rtol=1e-15)
    assert oracle.harris_window(4, 0.3, C.F32).tolist() == [0.25] * 4


def _view(L, dims, dt=0):
    out = ctypes.c_void_p()
    d = DIMS4(*dims)
    strides = DIMS4(1, dims[0], dims[0] * dims[1], dims[0] * dims[1] * dims[2])
    assert L.afgb_device_array_view(ctypes.byref(out), ctypes.c_void_p(0x7F0000002000), 4, d,
                                    strides, dt) == 0
    return out


@pytest.mark.parametrize("args,code", [
    ((64, 64, 3, 1), 203),         # 3-D input: AF_ERR_SIZE
    ((64, 1, 1, 1), 203),          # 1-D input
])
def test_harris_rejects_non_2d_input(aflib_cpu, args, code):
    L = aflib_cpu
    v = _view(L, args)
    feat = ctypes.c_void_p()
    assert L.af_harris(ctypes.byref(feat), v, 500, ctypes.c_float(1e5), ctypes.c_float(1.0), 0,
                       ctypes.c_float(0.04)) == code
    L.af_release_array(v)


@pytest.mark.parametrize("mc,mr,sigma,bs,k,dt,code", [
    (0, 0.0, 1.0, 0, 0.04, 0, 202),      # neither max_corners nor min_response
    (10, 0.0, 1.0, 0, 0.005, 0, 202),    # k_thr below 0.01
    (10, 0.0, 0.4, 0, 0.04, 0, 202),     # sigma below 0.5 without a block
    (10, 0.0, 5.5, 0, 0.04, 0, 202),     # sigma above 5 without a block
    (10, 0.0, 0.2, 2, 0.04, 0, 202),     # block_size 2 needs sigma in [0.5, 5]
    (10, 0.0, 1.0, 33, 0.04, 0, 202),    # block_size above 32
    (10, 0.0, 1.0, 0, 0.04, 4, 204),     # u8 image: AF_ERR_TYPE
    (10, 0.0, 1.0, 0, 0.04, 5, 204),     # s32 image
])
def test_harris_argument_checks(aflib_cpu, mc, mr, sigma, bs, k, dt, code):
    L = aflib_cpu
    v = _view(L, (64, 64, 1, 1), dt)
    feat = ctypes.c_void_p()
    assert L.af_harris(ctypes.byref(feat), v, mc, ctypes.c_float(mr), ctypes.c_float(sigma), bs,
                       ctypes.c_float(k)) == code
    L.af_release_array(v)


def test_harris_window_larger_than_image(aflib_cpu):
    """Both dims below the window (2*edge+1): AF_ERR_ARG."""
    L = aflib_cpu
    v = _view(L, (6, 6, 1, 1))
    feat = ctypes.c_void_p()
    assert L.af_harris(ctypes.byref(feat), v, 10, ctypes.c_float(0), ctypes.c_float(1.0), 9,
                       ctypes.c_float(0.04)) == 202
    L.af_release_array(v)


def test_features_object_without_arrays(aflib_cpu):
    """af_create_features(0) holds no arrays; count, retain and release work
    without a device."""
    L = aflib_cpu
    f = ctypes.c_void_p()
    assert L.af_create_features(ctypes.byref(f), 0) == 0
    n = ctypes.c_longlong(-1)
    assert L.af_get_features_num(ctypes.byref(n), f) == 0 and n.value == 0
    a = ctypes.c_void_p(1)
    assert L.af_get_features_xpos(ctypes.byref(a), f) == 0 and not a.value
    g = ctypes.c_void_p()
    assert L.af_retain_features(ctypes.byref(g), f) == 0
    assert L.af_release_features(g) == 0
    assert L.af_release_features(f) == 0
    assert L.af_create_features(ctypes.byref(f), -1) == 202
    assert L.af_get_features_num(ctypes.byref(n), None) == 202
