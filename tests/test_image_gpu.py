"""GPU tests of af_gaussian_kernel, af_dog and af_sobel_operator through the
C ABI: Sobel bit for bit against the reference's digests (tests/golden/
image.json), the Gaussian within float rounding of the FP64 closed form, DoG
against the oracle's convolutions, and the reference's argument checks
(src/api/c/sobel.cpp:38-48, src/api/c/dog.cpp:56-63, test/dog.cpp)."""
import ctypes
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "image.json").read_text())


def digest(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


@pytest.mark.parametrize("case", C.sobel_cases(), ids=lambda c: c[0])
def test_sobel_matches_reference_hash(af, case):
    cid, dt, shape, seed = case
    x = C.sobel_input(dt, shape, seed)
    dx, dy = af.sobel_operator(af.Array.from_numpy(x, dt))
    assert dx.dims == C.af_shape(shape)
    assert digest(dx.to_numpy()) == GOLD[cid]["dx"]
    assert digest(dy.to_numpy()) == GOLD[cid]["dy"]


def test_sobel_large_image_and_view(af, oracle):
    x = np.asfortranarray(np.random.Generator(np.random.Philox(4)).random((1000, 700, 3))
                          .astype(np.float32))
    dx, dy = af.sobel_operator(af.Array.from_numpy(x))
    rx, ry = oracle.sobel(x, C.F32)
    assert dx.to_numpy()[:, :, :, 0].tobytes() == rx[:, :, :, 0].tobytes()
    assert dy.to_numpy()[:, :, :, 0].tobytes() == ry[:, :, :, 0].tobytes()
    import torch

    t = torch.arange(24 * 20, dtype=torch.float32, device="cuda").reshape(20, 24)
    v = af.Array.view_device(t.data_ptr(), [12, 20], af.f32, strides=[2, 24], keep=t)
    host = np.asfortranarray(t.cpu().numpy().T[::2, :])
    gx, gy = af.sobel_operator(v)
    hx, hy = oracle.sobel(host, C.F32)
    assert gx.to_numpy().tobytes() == hx.tobytes() and gy.to_numpy().tobytes() == hy.tobytes()


def test_sobel_checks(af):
    img = af.Array.from_numpy(np.ones((8, 8), np.float32))
    dx, dy = af._lib.af_array(), af._lib.af_array()
    L = af.lib()
    assert L.af_sobel_operator(ctypes.byref(dx), ctypes.byref(dy), img.handle, 5) == af.AF_ERR_ARG
    vec = af.Array.from_numpy(np.ones((8,), np.float32))
    assert L.af_sobel_operator(ctypes.byref(dx), ctypes.byref(dy), vec.handle, 3) == af.AF_ERR_SIZE
    c = af.Array.from_numpy(np.ones((8, 8), np.complex64))
    assert L.af_sobel_operator(ctypes.byref(dx), ctypes.byref(dy), c.handle, 3) == af.AF_ERR_TYPE


@pytest.mark.parametrize("rows,cols,sr,sc", [(5, 5, 1.0, 1.0), (7, 7, 0, 0), (15, 7, 0, 0),
                                             (1, 15, 0, 0), (15, 1, 2.5, 0), (31, 17, 3.0, 1.5),
                                             (64, 64, 0, 0)])
def test_gaussian_kernel(af, oracle, rows, cols, sr, sc):
    g = af.gaussian_kernel(rows, cols, sr, sc).to_numpy()[:, :, 0, 0]
    ref = oracle.gaussian_kernel(rows, cols, sr, sc)
    assert g.dtype == np.float32 and g.shape == ref.shape
    np.testing.assert_allclose(g, ref, rtol=2e-6, atol=1e-9)


@pytest.mark.parametrize("dt", [C.F32, C.F64, C.U8, C.S32, C.B8], ids=lambda d: C.DT_NAME[d])
@pytest.mark.parametrize("shape,r1,r2", [((64, 48), 3, 2), ((40, 30, 3), 2, 1), ((33, 29), 9, 4)])
def test_dog(af, oracle, dt, shape, r1, r2):
    x = C.make_signal(dt, shape, 77)
    out = af.dog(af.Array.from_numpy(x, dt), r1, r2).to_numpy()
    ref = oracle.dog(x, dt, r1, r2)
    assert out.dtype == (np.float64 if dt == C.F64 else np.float32)
    # the Gaussian taps are f32 for every type (the f64 path casts them), so a
    # tap's last-place difference from the oracle's bounds the error
    scale = float(np.abs(x.astype(np.float64)).max()) + 1e-30
    tol = 2e-6 * scale
    assert np.abs(out.astype(np.float64) - ref).max() <= tol


def test_dog_reference_checks(af):
    """test/dog.cpp:43-82: constant image, the difference of blurs; a vector is
    rejected (AF_ERR_ARG)."""
    img = af.Array.from_numpy(np.ones((512, 512, 3), np.float32))
    out = af.dog(img, 3, 2).to_numpy()
    k1 = af.gaussian_kernel(7, 7)
    k2 = af.gaussian_kernel(5, 5)
    a = af.convolve2(img, k1).to_numpy()
    b = af.convolve2(img, k2).to_numpy()
    assert float(np.sum(out - (a - b))) < 1e-2
    with pytest.raises(af.AfError) as e:
        af.dog(af.Array.from_numpy(np.ones((512,), np.float32)), 3, 2)
    assert e.value.code == af.AF_ERR_ARG
    with pytest.raises(af.AfError) as e:
        af.dog(af.Array.from_numpy(np.ones((8, 8), np.complex64)), 1, 2)
    assert e.value.code == af.AF_ERR_TYPE
