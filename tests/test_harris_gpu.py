"""af_harris on the GPU against the oracle port (itself pinned to the
reference's CPU kernels by tests/golden/harris.json): the count, x, y and
score of every corner are bit-identical, in the same order, for f32 and f64
images -- on every golden case, at a 2048 x 2048 image, on a strided view,
and whatever the global exact-rounding setting."""
import ctypes

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu


def run(af, img, mc, mr, sg, bs, k):
    f = af.harris(af.Array.from_numpy(img), mc, mr, sg, bs, k)
    return f, (f.x(), f.y(), f.score())


def assert_same(got, want, what):
    assert got[0].size == want[0].size, f"{what}: {got[0].size} corners, oracle {want[0].size}"
    for name, a, b in zip(("x", "y", "score"), got, want):
        assert a.dtype == np.float32
        assert a.tobytes() == b.tobytes(), f"{what}: {name} differs"


@pytest.mark.parametrize("case", C.harris_cases(), ids=lambda c: c[0])
def test_harris_matches_oracle(af, oracle, case):
    cid, dt, shape, mc, mr, sg, bs, k, kind, seed = case
    img = C.harris_image(dt, shape, kind, seed)
    f, got = run(af, img, mc, mr, sg, bs, k)
    want = oracle.harris(img, dt, mc, mr, sg, bs, k)
    assert_same(got, want, cid)
    n = f.num()
    assert n == want[0].size
    if n:
        assert np.all(f.orientation() == 0) and np.all(f.size() == 1)
        assert f.orientation().size == n and f.size().size == n


@pytest.mark.parametrize("dt,mc,mr", [(C.F32, 500, 0.0), (C.F32, 0, 1e4), (C.F64, 300, 0.0)])
def test_harris_full_size_image(af, oracle, dt, mc, mr):
    """2048 x 2048 (f32) / 1024 x 1024 (f64) images of rectangles."""
    shape = (2048, 2048) if dt == C.F32 else (1024, 1024)
    img = C.harris_image(dt, shape, "blocks", 45001)
    _, got = run(af, img, mc, mr, 1.0, 0, 0.04)
    want = oracle.harris(img, dt, mc, mr, 1.0, 0, 0.04)
    assert want[0].size > 0
    assert_same(got, want, f"{shape} dt={dt}")


def test_harris_on_strided_view(af, oracle):
    """A column-strided device view reads like its dense copy."""
    import torch

    img = C.harris_image(C.F32, (130, 110), "blocks", 45002)
    big = np.zeros((130, 220), np.float32, order="F")
    big[:, ::2] = img
    t = torch.from_numpy(np.ascontiguousarray(big.T)).cuda()  # (220, 130) row-major = F (130, 220)
    V = af.Array.view_device(t.data_ptr(), [130, 110, 1, 1], C.F32, strides=[1, 260, 130 * 220,
                                                                             130 * 220], keep=t)
    f = af.harris(V, 30, 0.0, 1.0, 0, 0.04)
    want = oracle.harris(img, C.F32, 30, 0.0, 1.0, 0, 0.04)
    assert_same((f.x(), f.y(), f.score()), want, "strided view")


def test_harris_ignores_global_fast_math(af, oracle):
    """The window sums round like the reference even with exact rounding
    switched off globally (it is forced inside af_harris)."""
    img = C.harris_image(C.F32, (200, 170), "noise", 45003)
    af.set_exact_fp(False)
    _, got = run(af, img, 0, 1.0, 1.5, 0, 0.04)
    assert_same(got, oracle.harris(img, C.F32, 0, 1.0, 1.5, 0, 0.04), "fast-math off")


def test_features_create_retain_release(af):
    L = af.lib()
    f = ctypes.c_void_p()
    assert L.af_create_features(ctypes.byref(f), 7) == 0
    n = ctypes.c_longlong()
    assert L.af_get_features_num(ctypes.byref(n), f) == 0 and n.value == 7
    x = ctypes.c_void_p()
    assert L.af_get_features_score(ctypes.byref(x), f) == 0
    d = [ctypes.c_longlong() for _ in range(4)]
    assert L.af_get_dims(*[ctypes.byref(v) for v in d], x) == 0
    assert [v.value for v in d] == [7, 1, 1, 1]
    g = ctypes.c_void_p()
    assert L.af_retain_features(ctypes.byref(g), f) == 0
    assert L.af_release_features(f) == 0
    # the retained object holds its own handles on the same arrays, alive
    # after the original object is gone (af_retain_array makes new handles)
    y = ctypes.c_void_p()
    assert L.af_get_features_score(ctypes.byref(y), g) == 0 and y.value
    assert L.af_get_dims(*[ctypes.byref(v) for v in d], y) == 0
    assert [v.value for v in d] == [7, 1, 1, 1]
    assert L.af_release_features(g) == 0


def test_harris_empty_result_dims(af):
    """No corner: x/y/score of dims (0,0,0,0), orientation/size (0,1,1,1)."""
    img = C.harris_image(C.F32, (8, 40), "noise", 45004)
    f = af.harris(af.Array.from_numpy(img), 10, 0.0, 1.0, 0, 0.04)
    assert f.num() == 0
    L = af.lib()
    d = [ctypes.c_longlong() for _ in range(4)]
    for getter, dims in ((L.af_get_features_xpos, [0, 0, 0, 0]),
                         (L.af_get_features_size, [0, 1, 1, 1])):
        a = ctypes.c_void_p()
        assert getter(ctypes.byref(a), f.handle) == 0
        assert L.af_get_dims(*[ctypes.byref(v) for v in d], a) == 0
        assert [v.value for v in d] == dims
