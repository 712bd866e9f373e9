"""af_canny on the GPU against the oracle port (itself pinned to the
reference's CPU kernels by tests/golden/canny.json): the edge map is
bit-identical for every accepted type, manual and Otsu thresholds, L1 and L2
magnitudes, batches of slices, wide slices (the reference's seed-scan
range), a 2048 x 2048 image and a strided view."""
import ctypes

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu


def run(af, img, otsu, t1, t2, isf):
    e = af.canny(af.Array.from_numpy(img), 1 if otsu else 0, t1, t2, 3, isf)
    assert e.dtype == 4  # b8
    return e.to_numpy().reshape(img.shape, order="F").astype(np.int8)


@pytest.mark.parametrize("case", C.canny_cases(), ids=lambda c: c[0])
def test_canny_matches_oracle(af, oracle, case):
    cid, dt, shape, otsu, t1, t2, isf, kind, seed = case
    img = C.canny_image(dt, shape, kind, seed)
    got = run(af, img, otsu, t1, t2, isf)
    want = oracle.canny(img, dt, otsu, t1, t2, isf).reshape(img.shape, order="F")
    assert int(got.sum()) == int(want.sum()), cid
    assert got.tobytes(order="F") == want.tobytes(order="F"), cid


@pytest.mark.parametrize("dt,otsu,isf", [(C.F32, False, False), (C.U8, True, False),
                                         (C.F32, True, True)])
def test_canny_full_size_image(af, oracle, dt, otsu, isf):
    img = C.canny_image(dt, (2048, 2048), "blocks", 55001)
    got = run(af, img, otsu, 0.1, 0.3, isf)
    want = oracle.canny(img, dt, otsu, 0.1, 0.3, isf).reshape(img.shape, order="F")
    assert want.sum() > 0
    assert got.tobytes(order="F") == want.tobytes(order="F")


def test_canny_on_strided_view(af, oracle):
    import torch

    img = C.canny_image(C.F32, (130, 110), "blocks", 55002)
    big = np.zeros((130, 220), np.float32, order="F")
    big[:, ::2] = img
    t = torch.from_numpy(np.ascontiguousarray(big.T)).cuda()
    V = af.Array.view_device(t.data_ptr(), [130, 110, 1, 1], C.F32,
                             strides=[1, 260, 130 * 220, 130 * 220], keep=t)
    e = af.canny(V, 0, 0.1, 0.3, 3, False).to_numpy().reshape(130, 110, order="F")
    want = oracle.canny(img, C.F32, False, 0.1, 0.3, False)[:, :, 0]
    assert e.astype(np.int8).tobytes(order="F") == want.tobytes(order="F")


def test_canny_otsu_needs_two_bins(af):
    """A gradient maximum below 2 (an image in [0, 0.01]) has no Otsu
    histogram; the call reports AF_ERR_NOT_SUPPORTED and the library stays
    usable."""
    img = (C.canny_image(C.F32, (64, 64), "blocks", 55003) * 1e-5).astype(np.float32)
    out = ctypes.c_void_p()
    L = af.lib()
    assert L.af_canny(ctypes.byref(out), af.Array.from_numpy(img).handle, 1, ctypes.c_float(0.3),
                      ctypes.c_float(0.0), 3, False) == af.AF_ERR_NOT_SUPPORTED
    assert run(af, img, False, 0.1, 0.3, False).shape == (64, 64)
