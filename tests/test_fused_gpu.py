"""GPU tests of the fused forward epilogue (afgb_convolve2_nn_fused): the
bias add and ReLU applied in the convolution's epilogue give the same bits as
the unfused convolution followed by the same float operations, on the
tensor-core paths (TMA-store, strided manual-store and folded RGB forms) and
the FP32 path."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu

SHAPES = [
    # (W, H, C, N), (fw, fh, K), stride, pad, dil
    ((64, 48, 64, 2), (3, 3, 96), (1, 1), (1, 1), (1, 1)),     # TMA-store epilogue
    ((57, 41, 32, 2), (3, 3, 64), (2, 2), (1, 1), (1, 1)),     # strided: manual stores
    ((96, 80, 3, 2), (3, 3, 32), (2, 2), (1, 1), (1, 1)),      # RGB: taps folded
    ((40, 36, 16, 1), (5, 5, 200), (1, 1), (4, 4), (2, 2)),    # two output-channel tiles
    ((128, 10, 64, 2), (3, 3, 96), (1, 1), (1, 1), (1, 1)),    # 128-pixel rows
]


def _run(af, x, w, b, geo, precision, relu):
    s, p, d = geo
    X = af.Array.view_torch(x)
    W = af.Array.view_torch(w)
    B = af.Array.view_torch(b) if b is not None else None
    fused = af.convolve2_nn(X, W, s, p, d, precision=precision, bias=B, relu=relu).to_torch()
    plain = af.convolve2_nn(X, W, s, p, d, precision=precision).to_torch().clone()
    if b is not None:
        plain = plain + b.view(1, -1, 1, 1)
    if relu:
        plain = torch.where(plain < 0, torch.zeros_like(plain), plain)
    return fused, plain


@pytest.mark.parametrize("precision", ["bf16", "fp32"])
@pytest.mark.parametrize("shape", SHAPES, ids=lambda v: f"{v[0]}x{v[1]}s{v[2][0]}")
@pytest.mark.parametrize("bias,relu", [(True, True), (True, False), (False, True)])
def test_fused_epilogue_matches_separate_ops(af, precision, shape, bias, relu):
    (W_, H_, C_, N_), (fw, fh, K), s, p, d = shape
    g = torch.Generator(device="cuda").manual_seed(W_ * 7 + K)
    x = torch.randn((N_, C_, H_, W_), device="cuda", generator=g)
    w = torch.randn((K, C_, fh, fw), device="cuda", generator=g) * (2.0 / (fw * fh * C_)) ** 0.5
    b = torch.randn((K,), device="cuda", generator=g) if bias else None
    fused, plain = _run(af, x, w, b, (s, p, d), precision, relu)
    af.sync()
    torch.cuda.synchronize()
    assert fused.shape == plain.shape
    assert torch.equal(fused, plain)
    if relu:
        assert bool((fused >= 0).all())


def test_fused_checks(af):
    x = af.Array.from_numpy(np.ones((8, 8, 4, 1), np.float32))
    w = af.Array.from_numpy(np.ones((3, 3, 4, 5), np.float32))
    bad_bias = af.Array.from_numpy(np.ones((4,), np.float32))
    with pytest.raises(af.AfError) as e:
        af.convolve2_nn(x, w, (1, 1), (1, 1), (1, 1), bias=bad_bias)
    assert e.value.code == af.AF_ERR_SIZE
    out = af._lib.af_array()
    st = (af._lib.dim_t * 2)(1, 1)
    rc = af.lib().afgb_convolve2_nn_fused(ctypes.byref(out), x.handle, w.handle, 2, st, 2, st, 2,
                                          st, 0, None, 2)
    assert rc == af.AF_ERR_ARG
    x64 = af.Array.from_numpy(np.ones((8, 8, 4, 1), np.float64))
    w64 = af.Array.from_numpy(np.ones((3, 3, 4, 5), np.float64))
    with pytest.raises(af.AfError) as e:
        af.convolve2_nn(x64, w64, (1, 1), (1, 1), (1, 1), relu=True)
    assert e.value.code == af.AF_ERR_TYPE
