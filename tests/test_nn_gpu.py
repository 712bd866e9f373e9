"""GPU parity of af_convolve2_nn / af_convolve2_gradient_nn (plain FP32 form)
through the C ABI against the FP64 oracle.

Tolerance (FP32 against FP64): |gpu - ref| <= 1e-5 * max|ref| + 1e-5 * sum|terms|
per element is the bound written below as `close`; in practice the GEMM
error is ~1e-7 relative.
"""
import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu


def nn_case(af, case, seed, dtype=np.float32):
    s, f = C.nn_inputs(case, seed, dtype)
    g = C.nn_grad(case, seed, dtype)
    return s, f, g


def close(out, ref, rel=1e-5):
    scale = max(1.0, float(np.abs(ref).max()))
    err = float(np.abs(out.astype(np.float64) - ref).max())
    assert err <= rel * scale, f"max abs err {err:.3e} vs scale {scale:.3e}"


@pytest.mark.parametrize("i,case", list(enumerate(C.NN_CASES)), ids=[c[0] for c in C.NN_CASES])
def test_nn_forward_fp32(af, oracle, i, case):
    name, sd, fd, st, pd, dl = case
    s, f, g = nn_case(af, case, 9000 + 10 * i)
    out = af.convolve2_nn(af.Array.from_numpy(s), af.Array.from_numpy(f), st, pd, dl).to_numpy()
    ref = oracle.nn_forward_f64(s, f, st, pd, dl)
    assert out.shape == ref.shape
    close(out, ref)


@pytest.mark.parametrize("i,case", list(enumerate(C.NN_CASES)), ids=[c[0] for c in C.NN_CASES])
def test_nn_gradients_fp32(af, oracle, i, case):
    name, sd, fd, st, pd, dl = case
    s, f, g = nn_case(af, case, 9000 + 10 * i)
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    O = af.convolve2_nn(S, F, st, pd, dl)
    dx = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_DATA).to_numpy()
    dw = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_FILTER).to_numpy()
    db = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_BIAS,
                                  real_bias=True).to_numpy()
    close(dx, oracle.nn_data_grad_f64(g, list(s.shape), f, st, pd, dl))
    close(dw, oracle.nn_filter_grad_f64(g, s, list(f.shape), st, pd, dl))
    close(db, oracle.nn_bias_grad_f64(g, list(s.shape), list(f.shape), st, pd, dl))
    # reference semantics: BIAS through the plain entry point returns the data
    # gradient (src/api/c/convolve.cpp:401-411)
    dxb = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_BIAS).to_numpy()
    assert dxb.tobytes() == dx.tobytes()


@pytest.mark.parametrize("dtype,rel", [(np.float64, 1e-12), (np.float16, 2e-2)])
def test_nn_other_dtypes(af, oracle, dtype, rel):
    case = C.NN_CASES[8]
    name, sd, fd, st, pd, dl = case
    s, f, g = nn_case(af, case, 123, dtype)
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    O = af.convolve2_nn(S, F, st, pd, dl)
    close(O.to_numpy(), oracle.nn_forward_f64(s, f, st, pd, dl), rel)
    dx = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_DATA).to_numpy()
    close(dx, oracle.nn_data_grad_f64(g, list(s.shape), f, st, pd, dl), rel)
    dw = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_FILTER).to_numpy()
    close(dw, oracle.nn_filter_grad_f64(g, s, list(f.shape), st, pd, dl), rel)


def test_zero_padding_issue2817(af):
    """test/convolve.cpp:1170-1185."""
    s = np.ones((5, 5), np.float32)
    f = np.full((3, 3), 1 / 9, np.float32)
    S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
    conv = af.convolve2_nn(S, F, (1, 1), (0, 0), (1, 1))
    c = conv.to_numpy()[:, :, 0, 0]
    assert np.abs(c - 1).sum() < 1e-5
    G = af.Array.from_numpy(np.full((3, 3), 1 / 9, np.float32))
    wg = af.convolve2_gradient_nn(G, S, F, conv, (1, 1), (0, 0), (1, 1),
                                  af.AF_CONV_GRADIENT_FILTER).to_numpy()[:, :, 0, 0]
    assert np.abs(wg - c).sum() < 1e-5


@pytest.mark.parametrize("n,fsz", [(10, 3), (11, 5), (12, 7), (19, 9), (33, 3), (255, 3),
                                   (256, 3), (257, 3)])
def test_conv2_consistency(af, n, fsz):
    """test/convolve.cpp:868-894: convolve2NN(pad=f/2) == convolve2 within 2e-5."""
    g = C.rng(n * 100 + fsz)
    s = g.standard_normal((n, n)).astype(np.float32)
    f = g.standard_normal((fsz, fsz)).astype(np.float32)
    S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
    native = af.convolve2(S, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL).to_numpy()
    nn = af.convolve2_nn(S, F, (1, 1), (fsz // 2, fsz // 2), (1, 1)).to_numpy()
    np.testing.assert_allclose(native, nn, atol=2e-5 * max(1.0, float(np.abs(nn).max())))


def test_nn_validation_codes(af):
    """src/api/c/convolve.cpp:365-370, 434-450 argument checks."""
    S = af.Array.from_numpy(np.ones((8, 8, 3, 1), np.float32))
    F = af.Array.from_numpy(np.ones((3, 3, 3, 2), np.float32))
    Fbad = af.Array.from_numpy(np.ones((3, 3, 4, 2), np.float32))
    with pytest.raises(af.AfError) as e:
        af.convolve2_nn(S, Fbad, (1, 1), (1, 1), (1, 1))
    assert e.value.code == af.AF_ERR_SIZE
    with pytest.raises(af.AfError) as e:
        af.convolve2_nn(S, F, (0, 1), (1, 1), (1, 1))  # stride ndims 0
    assert e.value.code == af.AF_ERR_ARG
    with pytest.raises(af.AfError) as e:
        af.convolve2_nn(S, F, (1, 1, 2), (1, 1), (1, 1))  # 3 stride dims
    assert e.value.code == af.AF_ERR_ARG
    with pytest.raises(af.AfError) as e:
        af.convolve2_nn(S, F, (1, 1), (1, 1), (0, 0))
    assert e.value.code == af.AF_ERR_ARG
    Si = af.Array.from_numpy(np.ones((8, 8, 3, 1), np.int32))
    with pytest.raises(af.AfError) as e:
        af.convolve2_nn(Si, F, (1, 1), (1, 1), (1, 1))
    assert e.value.code == af.AF_ERR_TYPE
    Fd = af.Array.from_numpy(np.ones((3, 3, 3, 2), np.float64))
    with pytest.raises(af.AfError) as e:
        af.convolve2_nn(S, Fd, (1, 1), (1, 1), (1, 1))
    assert e.value.code == af.AF_ERR_INTERNAL
    O = af.convolve2_nn(S, F, (1, 1), (1, 1), (1, 1))
    Gbad = af.Array.from_numpy(np.ones((8, 8, 3, 1), np.float32))
    with pytest.raises(af.AfError) as e:
        af.convolve2_gradient_nn(Gbad, S, F, O, (1, 1), (1, 1), (1, 1))
    assert e.value.code == af.AF_ERR_SIZE


def test_padding_dims_zero_means_ones(af, oracle):
    """dim4(0, ptr) is all ones (src/backend/common/dim4.cpp:35-37): padding
    with zero listed dims pads by one."""
    import ctypes

    s, f = C.nn_inputs(C.NN_CASES[7], 5)
    S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
    L = af.lib()
    out = ctypes.c_void_p()
    one = (ctypes.c_longlong * 2)(1, 1)
    rc = L.af_convolve2_nn(ctypes.byref(out), S.handle, F.handle, 2, one, 0, None, 2, one)
    assert rc == 0
    res = af.Array(out.value).to_numpy()
    close(res, oracle.nn_forward_f64(s, f, (1, 1), (1, 1), (1, 1)))
