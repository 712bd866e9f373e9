"""GPU tests for af_unwrap / af_wrap / af_wrap_v2 through the C ABI: bit-exact
against the reference's digests (tests/golden/patches.json) for every type,
the reference tests' known answers and argument checks (test/wrap.cpp,
test/unwrap.cpp), sub-array outputs, and the maximum-batch case."""
import ctypes
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "patches.json").read_text())


def digest(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


def _ran(af, name, fn):
    L = af.lib()
    L.afgb_kernel_timing(1)
    try:
        out = fn()
        af.sync()
        c = ctypes.c_ulonglong()
        ms = ctypes.c_double()
        L.afgb_kernel_time(name.encode(), ctypes.byref(c), ctypes.byref(ms))
    finally:
        L.afgb_kernel_timing(0)
    return c.value, out


@pytest.mark.parametrize("case", C.patch_cases(), ids=lambda c: c[0])
def test_patches_match_reference_hash(af, case):
    cid, dt, sd, wx, wy, sx, sy, px, py, col, seed = case
    g = GOLD[cid]
    img = af.Array.from_numpy(C.patch_values(dt, sd, seed), dt)
    U = af.unwrap(img, wx, wy, sx, sy, px, py, col)
    assert U.dims == g["unwrap_dims"]
    assert digest(U.to_numpy()) == g["unwrap"]
    pm = af.Array.from_numpy(C.patch_values(dt, C.patch_dims(case), seed + 1), dt)
    W = af.wrap(pm, sd[0], sd[1], wx, wy, sx, sy, px, py, col)
    assert W.dims == list(sd)
    assert digest(W.to_numpy()) == g["wrap"]
    base = af.Array.from_numpy(C.patch_values(dt, sd, seed + 2), dt)
    V = af.wrap_v2(base, pm, sd[0], sd[1], wx, wy, sx, sy, px, py, col)
    assert V is base
    assert digest(base.to_numpy()) == g["wrap_v2"]
    # v2 with a null output allocates, like af_wrap
    assert digest(af.wrap_v2(None, pm, sd[0], sd[1], wx, wy, sx, sy, px, py, col).to_numpy()) \
        == g["wrap"]


def test_kernels_launch(af):
    a = af.Array.from_numpy(np.ones((16, 16), np.float32))
    n, U = _ran(af, "unwrap_rows_kernel", lambda: af.unwrap(a, 3, 3, 1, 1, 1, 1))
    assert n == 1
    n, _ = _ran(af, "wrap_s1_kernel", lambda: af.wrap(U, 16, 16, 3, 3, 1, 1, 1, 1))
    assert n == 1
    U2 = af.unwrap(a, 3, 3, 2, 2, 1, 1)
    n, _ = _ran(af, "wrap_tiled_kernel", lambda: af.wrap(U2, 16, 16, 3, 3, 2, 2, 1, 1))
    assert n == 1
    R = af.unwrap(a, 3, 3, 1, 1, 1, 1, False)
    n, _ = _ran(af, "wrap_s1_kernel", lambda: af.wrap(R, 16, 16, 3, 3, 1, 1, 1, 1, False))
    assert n == 1
    R2 = af.unwrap(a, 3, 3, 2, 2, 1, 1, False)
    n, _ = _ran(af, "wrap_rows_kernel", lambda: af.wrap(R2, 16, 16, 3, 3, 2, 2, 1, 1, False))
    assert n == 1
    # windows too large to stage: the untiled kernels
    big = af.Array.from_numpy(np.ones((80, 70), np.complex128))
    n, B = _ran(af, "unwrap_kernel", lambda: af.unwrap(big, 64, 64, 1, 1))
    assert n == 1
    n, _ = _ran(af, "wrap_kernel", lambda: af.wrap(B, 80, 70, 64, 64, 1, 1))
    assert n == 1


def test_doc_snippets(af):
    """test/wrap.cpp:200-251."""
    A = np.arange(1, 10, dtype=np.float32).reshape(3, 3, order="F")
    U = af.unwrap(af.Array.from_numpy(A), 2, 2, 2, 2, 1, 1)
    gold_u = np.array([[0, 0, 0, 5], [0, 0, 4, 6], [0, 2, 0, 8], [1, 3, 7, 9]], np.float32)
    np.testing.assert_array_equal(U.to_numpy()[:, :, 0, 0], gold_u)
    np.testing.assert_array_equal(af.wrap(U, 3, 3, 2, 2, 2, 2, 1, 1).to_numpy()[:, :, 0, 0], A)
    B = af.unwrap(af.Array.from_numpy(np.ones((3, 3), np.float32)), 2, 2, 1, 1)
    gold = np.array([1, 2, 1, 2, 4, 2, 1, 2, 1], np.float32).reshape(3, 3, order="F")
    np.testing.assert_array_equal(af.wrap(B, 3, 3, 2, 2, 1, 1).to_numpy()[:, :, 0, 0], gold)


H_IN = np.array([10, 20, 20, 30, 30, 40, 40, 50, 30, 40, 40, 50, 50, 60, 60, 70],
                np.float32).reshape(4, 4, order="F")
H_GOLD = np.array([10, 20, 30, 40, 20, 30, 40, 50, 30, 40, 50, 60, 40, 50, 60, 70],
                  np.float32).reshape(4, 4, order="F")


@pytest.mark.parametrize("dt", C.PATCH_DTYPES, ids=lambda d: C.DT_NAME[d])
def test_wrap_v2_full_and_sub_array(af, dt):
    """test/wrap.cpp:264-400 (WrapV2Simple): null, full existing and sub-array
    outputs; the sub-array's surroundings stay untouched."""
    t = C.NP_OF[dt]
    pin = af.Array.from_numpy(H_IN.astype(t), dt)
    gold = H_GOLD.astype(t)
    np.testing.assert_array_equal(
        af.wrap_v2(None, pin, 4, 4, 2, 2, 2, 2, 0, 0).to_numpy()[:, :, 0, 0], gold)
    full = af.Array.from_numpy(np.zeros((4, 4), t), dt)
    af.wrap_v2(full, pin, 4, 4, 2, 2, 2, 2, 0, 0)
    np.testing.assert_array_equal(full.to_numpy()[:, :, 0, 0], gold)
    # a 4x4 window at offset (2, 3) of a 9x8 parent (column-major strides 1, 9)
    parent = af.Array.from_numpy(np.zeros((9, 8), t), dt)
    es = np.dtype(t).itemsize
    sub = af.Array.view_device(parent.device_ptr() + (2 + 3 * 9) * es, [4, 4], dt,
                               strides=[1, 9], keep=parent)
    af.wrap_v2(sub, pin, 4, 4, 2, 2, 2, 2, 0, 0)
    expect = np.zeros((9, 8), t, order="F")
    expect[2:6, 3:7] = gold
    np.testing.assert_array_equal(parent.to_numpy()[:, :, 0, 0], expect)


def test_wrap_null_args(af):
    """test/wrap.cpp:404-442."""
    L = af.lib()
    pin = af.Array.from_numpy(H_IN)
    out = af._lib.af_array()
    for fn in (L.af_wrap, L.af_wrap_v2):
        assert fn(None, pin.handle, 4, 4, 2, 2, 2, 2, 0, 0, True) == af.AF_ERR_ARG
        assert fn(ctypes.byref(out), None, 4, 4, 2, 2, 2, 2, 0, 0, True) == af.AF_ERR_ARG


@pytest.mark.parametrize("args,err", [
    # window, stride, padding, is_column -> error (test/wrap.cpp:526-540)
    ((2, 2, 2, 2, 0, 0, True), 0), ((2, 2, 2, 2, 0, 0, False), 0),
    ((-1, 2, 2, 2, 0, 0, True), 202), ((2, -1, 2, 2, 0, 0, True), 202),
    ((-1, -1, 2, 2, 0, 0, True), 202), ((2, 2, -1, 2, 0, 0, True), 202),
    ((2, 2, 2, -1, 0, 0, True), 202), ((2, 2, -1, -1, 0, 0, True), 202),
    ((2, 2, 2, 2, 1, 1, True), 203), ((2, 2, 2, 2, -1, 1, True), 203),
    ((2, 2, 2, 2, 1, -1, True), 203), ((2, 2, 2, 2, -1, -1, True), 203),
])
def test_wrap_argument_table(af, args, err):
    wx, wy, sx, sy, px, py, col = args
    pin = af.Array.from_numpy(H_IN)
    out = af._lib.af_array()
    rc = af.lib().af_wrap(ctypes.byref(out), pin.handle, 4, 4, wx, wy, sx, sy, px, py, col)
    assert rc == err
    if out.value:
        af.lib().af_release_array(out)


@pytest.mark.parametrize("args,err", [
    # wx, wy, sx, sy, px, py -> src/api/c/unwrap.cpp:46-51 argument order
    ((0, 3, 1, 1, 0, 0), 202), ((11, 3, 1, 1, 0, 0), 202), ((11, 3, 1, 1, 1, 0), 0),
    ((3, 0, 1, 1, 0, 0), 202), ((3, 9, 1, 1, 0, 0), 202), ((3, 3, 0, 1, 0, 0), 202),
    ((3, 3, 1, 0, 0, 0), 202), ((3, 3, 1, 1, -1, 0), 202), ((3, 3, 1, 1, 3, 0), 202),
    ((3, 3, 1, 1, 0, -1), 202), ((3, 3, 1, 1, 0, 3), 202), ((3, 3, 1, 1, 2, 2), 0),
])
def test_unwrap_argument_checks(af, args, err):
    img = af.Array.from_numpy(np.ones((10, 8), np.float32))
    out = af._lib.af_array()
    rc = af.lib().af_unwrap(ctypes.byref(out), img.handle, *args, True)
    assert rc == err
    if out.value:
        af.lib().af_release_array(out)


def test_f16_is_a_type_error(af):
    h = af.Array.from_numpy(np.ones((6, 6), np.float16), af.f16)
    out = af._lib.af_array()
    assert af.lib().af_unwrap(ctypes.byref(out), h.handle, 2, 2, 2, 2, 0, 0, True) \
        == af.AF_ERR_TYPE
    p = af.Array.from_numpy(np.ones((4, 9), np.float16), af.f16)
    assert af.lib().af_wrap(ctypes.byref(out), p.handle, 6, 6, 2, 2, 2, 2, 0, 0, True) \
        == af.AF_ERR_TYPE


def test_wrap_v2_existing_output_checks(af):
    pin = af.Array.from_numpy(H_IN)
    wrong_dims = af.Array.from_numpy(np.zeros((5, 4), np.float32))
    h = af._lib.af_array(wrong_dims.handle.value)
    assert af.lib().af_wrap_v2(ctypes.byref(h), pin.handle, 4, 4, 2, 2, 2, 2, 0, 0, True) \
        == af.AF_ERR_SIZE
    wrong_type = af.Array.from_numpy(np.zeros((4, 4), np.float64))
    h = af._lib.af_array(wrong_type.handle.value)
    assert af.lib().af_wrap_v2(ctypes.byref(h), pin.handle, 4, 4, 2, 2, 2, 2, 0, 0, True) != 0


def test_max_dim_round_trip(af):
    """test/wrap.cpp:183-198: 65536 batch slices of a 5x5 image, one patch each."""
    x = np.arange(5 * 5 * 65536, dtype=np.float32).reshape(5, 5, 1, 65536, order="F")
    a = af.Array.from_numpy(x)
    U = af.unwrap(a, 5, 5, 5, 5, 0, 0)
    assert U.dims == [25, 1, 1, 65536]
    np.testing.assert_array_equal(af.wrap(U, 5, 5, 5, 5, 5, 5, 0, 0).to_numpy(), x)


@pytest.mark.parametrize("geo", [(3, 3, 1, 1, 0, 0), (3, 3, 2, 2, 2, 2), (4, 4, 2, 2, 3, 3),
                                 (8, 8, 8, 8, 7, 7), (31, 31, 8, 8, 15, 15),
                                 (15, 10, 15, 10, 14, 9)])
@pytest.mark.parametrize("col", [True, False])
def test_wrap_of_unwrap_full_size(af, oracle, geo, col):
    """The reference's 300x100 property test (test/wrap.cpp:78-181) at its own
    size, checked bit for bit against the oracle."""
    wx, wy, sx, sy, px, py = geo
    x = (C.patch_values(C.S32, (300, 100), 11) % 1000).astype(np.int32)
    U = af.unwrap(af.Array.from_numpy(x), wx, wy, sx, sy, px, py, col)
    got = af.wrap(U, 300, 100, wx, wy, sx, sy, px, py, col).to_numpy()
    ref = oracle.wrap_patches(oracle.unwrap_patches(x, wx, wy, sx, sy, px, py, col), 300, 100,
                              wx, wy, sx, sy, px, py, col)
    np.testing.assert_array_equal(got.reshape(ref.shape, order="F"), ref)


def test_empty_and_strided_input(af):
    e = af.Array.from_numpy(np.zeros((6, 6, 0), np.float32))
    U = af.unwrap(e, 2, 2, 2, 2)
    assert U.dims[2] == 0
    # a strided input view (every other column of a 12x6 image) is densified
    import torch

    t = torch.arange(72, dtype=torch.float32, device="cuda").reshape(6, 12)
    v = af.Array.view_device(t.data_ptr(), [6, 6], af.f32, strides=[2, 12], keep=t)
    got = af.unwrap(v, 3, 3, 1, 1, 1, 1).to_numpy()
    host = np.asfortranarray(t.cpu().numpy().T[::2, :])
    import oracle as O

    np.testing.assert_array_equal(got.reshape(-1, order="F"),
                                  O.unwrap_patches(host, 3, 3, 1, 1, 1, 1).reshape(-1, order="F"))


@pytest.mark.parametrize("dt", [C.F32, C.U8, C.C64], ids=lambda d: C.DT_NAME[d])
@pytest.mark.parametrize("col", [True, False])
@pytest.mark.parametrize("shape,geo", [
    ((1100, 6, 2, 1), (3, 3, 1, 1, 1, 1)),      # 1100 windows per row: 512-window units
    ((264, 70, 1, 2), (64, 64, 1, 9, 0, 3)),    # 64x64 windows: 100-window units, short last unit
    ((90, 40, 3, 1), (5, 4, 3, 2, 2, 1)),
])
def test_patch_units_and_tiles_match_oracle(af, oracle, dt, col, shape, geo):
    """Geometries that split a window row into several units and tiles that
    fall back to the untiled wrap, bit for bit against the oracle."""
    wx, wy, sx, sy, px, py = geo
    x = C.patch_values(dt, shape, 4321)
    U = af.unwrap(af.Array.from_numpy(x, dt), wx, wy, sx, sy, px, py, col)
    ref_u = oracle.unwrap_patches(x, wx, wy, sx, sy, px, py, col)
    got_u = U.to_numpy()
    assert list(got_u.shape) == list(ref_u.shape)
    assert got_u.tobytes(order="F") == ref_u.tobytes(order="F")
    pm = C.patch_values(dt, list(ref_u.shape), 4322)
    W = af.wrap(af.Array.from_numpy(pm, dt), shape[0], shape[1], wx, wy, sx, sy, px, py, col)
    ref_w = oracle.wrap_patches(pm, shape[0], shape[1], wx, wy, sx, sy, px, py, col)
    assert W.to_numpy().tobytes(order="F") == ref_w.tobytes(order="F")


WRAP_S1 = [
    # (W, H, d2, d3), pad, dtype: several row tiles, ragged widths, every pad the kernel takes
    ((131, 77, 3, 2), 1, C.F32),
    ((128, 40, 2, 1), 0, C.F64),
    ((97, 35, 2, 2), 2, C.S16),
    ((64, 64, 1, 3), 1, C.C32),
]


@pytest.mark.parametrize("col", [True, False], ids=["col", "row"])
@pytest.mark.parametrize("case", WRAP_S1, ids=lambda c: f"{c[0][0]}x{c[0][1]}p{c[1]}_{C.DT_NAME[c[2]]}")
def test_wrap_s1_kernel_matches_oracle(af, oracle, case, col):
    """The stride-1 3x3 wrap (row tiles staged as contiguous runs of the patch
    matrix: one in the column layout, one per tap plane in the row layout)
    against the oracle, bit for bit, over several row tiles per slice; and
    wrap_v2 adding into an existing output."""
    (W, H, d2, d3), pad, dt = case
    nx, ny = W + 2 * pad - 2, H + 2 * pad - 2
    shape = (9, nx * ny, d2, d3) if col else (nx * ny, 9, d2, d3)
    pm = C.patch_values(dt, shape, 7700 + W)
    P = af.Array.from_numpy(pm)
    n, out = _ran(af, "wrap_s1_kernel", lambda: af.wrap(P, W, H, 3, 3, 1, 1, pad, pad, col))
    assert n == 1
    want = oracle.wrap_patches(pm, W, H, 3, 3, 1, 1, pad, pad, col)
    assert digest(out.to_numpy()) == digest(want)
    base_np = C.patch_values(dt, (W, H, d2, d3), 7800 + W)
    base = af.Array.from_numpy(base_np)
    af.wrap_v2(base, P, W, H, 3, 3, 1, 1, pad, pad, col)
    want2 = oracle.wrap_patches(pm, W, H, 3, 3, 1, 1, pad, pad, col, out=base_np)
    assert digest(base.to_numpy()) == digest(want2)
