"""GPU parity of the BF16 tensor-core (tcgen05) form of af_convolve2_nn and
its gradients, through the C ABI (afgb_convolve2_nn_ex /
afgb_convolve2_gradient_nn_ex), against the FP64 oracle.

Tolerance: norm-wise relative error ||gpu - ref|| / ||ref|| <= 2e-2 per
output (bf16 operands with FP32 accumulation give ~2-3e-3 on the larger
cases; a 25-term reduction with one channel reaches ~1.3e-2 because the
input rounding errors do not average out), and max-abs error
<= 8e-2 * max|ref|.
"""
import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu

REL = 2e-2

TC_CASES = C.NN_CASES + [
    ("tc_c64_k128", (24, 20, 64, 2), (3, 3, 64, 128), (1, 1), (1, 1), (1, 1)),
    ("tc_c128_k256_s2", (33, 31, 128, 2), (3, 3, 128, 256), (2, 2), (1, 1), (1, 1)),
    ("tc_5x5_d2_p4_s2", (30, 28, 32, 2), (5, 5, 32, 64), (2, 2), (4, 4), (2, 2)),
    ("tc_c200_k130", (17, 19, 200, 3), (3, 3, 200, 130), (1, 1), (1, 1), (1, 1)),
    ("tc_1x1_c256", (28, 28, 256, 2), (1, 1, 256, 192), (1, 1), (0, 0), (1, 1)),
    # C*fw*fh <= 64: taps folded into channels (1x1 problem on the output grid)
    ("tc_rgb_s2", (34, 30, 3, 2), (3, 3, 3, 32), (2, 2), (1, 1), (1, 1)),
    ("tc_fold_d2_s3", (29, 31, 6, 2), (3, 3, 6, 40), (3, 2), (2, 1), (2, 2)),
    ("tc_fold_5x5_c2", (23, 19, 2, 3), (5, 5, 2, 130), (1, 1), (2, 2), (1, 1)),
    # stride 4 with a 3x3 filter: data-gradient phases that no tap reaches are zero
    ("tc_s4_zero_phases", (21, 18, 16, 2), (3, 3, 16, 24), (4, 4), (1, 1), (1, 1)),
    ("tc_s2x3_c96", (35, 40, 96, 1), (3, 5, 96, 64), (2, 3), (1, 2), (1, 1)),
    # filter gradients on strips shared by the taps of a filter row
    ("tc_strip_5x5_d2", (30, 28, 32, 2), (5, 5, 32, 64), (1, 1), (4, 4), (2, 2)),
    ("tc_strip_7x7", (40, 36, 64, 1), (7, 7, 64, 128), (1, 1), (3, 3), (1, 1)),
    ("tc_strip_w16", (16, 40, 64, 2), (3, 3, 64, 128), (1, 1), (1, 1), (1, 1)),
    ("tc_strip_sy2", (33, 40, 64, 1), (3, 3, 64, 64), (1, 2), (1, 1), (1, 1)),
    # wide rows and edge rows at stride 1
    ("tc_w128_c64_k128", (128, 12, 64, 2), (3, 3, 64, 128), (1, 1), (1, 1), (1, 1)),
    ("tc_w120_c96_k96", (120, 9, 96, 1), (3, 3, 96, 96), (1, 1), (1, 1), (1, 1)),
    ("tc_1x5_w256", (256, 6, 64, 1), (5, 1, 64, 128), (1, 1), (2, 0), (1, 1)),
    ("tc_nopad_k32", (130, 10, 64, 1), (3, 3, 64, 32), (1, 1), (0, 0), (1, 1)),
    ("tc_fold_rgb_w128", (128, 10, 3, 2), (3, 3, 3, 64), (1, 1), (1, 1), (1, 1)),
    ("tc_d2_c16_k48", (124, 8, 16, 2), (3, 3, 16, 48), (1, 1), (2, 2), (2, 2)),
    # pixels-on-M strip kernel (stride 1, rows of 96+ pixels): two 128-pixel
    # segments with a ragged second, odd heights, N = 16 / 80 channels,
    # dilated and rectangular filters, four source chunks
    ("tc_strip_w200_k80", (200, 7, 48, 2), (3, 3, 48, 80), (1, 1), (1, 1), (1, 1)),
    ("tc_strip_w256_1x1", (256, 5, 128, 1), (1, 1, 128, 16), (1, 1), (0, 0), (1, 1)),
    ("tc_strip_5x3_dx2", (160, 9, 64, 1), (5, 3, 64, 32), (1, 1), (4, 1), (2, 1)),
    ("tc_strip_c256_k64", (128, 6, 256, 1), (3, 3, 256, 64), (1, 1), (1, 1), (1, 1)),
    ("tc_strip_w100_nopad", (100, 9, 64, 2), (3, 3, 64, 128), (1, 1), (0, 0), (1, 1)),
]


def check(out, ref, what):
    ref = np.asarray(ref, np.float64)
    out = np.asarray(out, np.float64)
    rel = np.linalg.norm(out - ref) / max(np.linalg.norm(ref), 1e-30)
    mx = np.abs(out - ref).max() / max(np.abs(ref).max(), 1e-30)
    assert rel <= REL and mx <= 4 * REL, f"{what}: rel {rel:.3e} max {mx:.3e}"
    return rel


@pytest.mark.parametrize("i,case", list(enumerate(TC_CASES)), ids=[c[0] for c in TC_CASES])
def test_bf16_forward(af, oracle, i, case):
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 7000 + 10 * i)
    out = af.convolve2_nn(af.Array.from_numpy(s), af.Array.from_numpy(f), st, pd, dl,
                          precision="bf16").to_numpy()
    ref = oracle.nn_forward_f64(s, f, st, pd, dl)
    assert out.shape == ref.shape
    check(out, ref, "fwd")


@pytest.mark.parametrize("i,case", list(enumerate(TC_CASES)), ids=[c[0] for c in TC_CASES])
def test_bf16_data_grad(af, oracle, i, case):
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 7000 + 10 * i)
    g = C.nn_grad(case, 7000 + 10 * i)
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    O = af.convolve2_nn(S, F, st, pd, dl)
    dx = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_DATA,
                                  precision="bf16").to_numpy()
    check(dx, oracle.nn_data_grad_f64(g, list(s.shape), f, st, pd, dl), "dgrad")


@pytest.mark.parametrize("i,case", list(enumerate(TC_CASES)), ids=[c[0] for c in TC_CASES])
def test_bf16_filter_grad(af, oracle, i, case):
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 7000 + 10 * i)
    g = C.nn_grad(case, 7000 + 10 * i)
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    O = af.convolve2_nn(S, F, st, pd, dl)
    dw = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_FILTER,
                                  precision="bf16").to_numpy()
    check(dw, oracle.nn_filter_grad_f64(g, s, list(f.shape), st, pd, dl), "wgrad")


def test_bf16_filter_grad_deterministic(af):
    """The split-K reduction order is fixed: two calls give identical bits."""
    case = TC_CASES[-4]
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 1)
    g = C.nn_grad(case, 1)
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    O = af.convolve2_nn(S, F, st, pd, dl)
    a = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_FILTER,
                                 precision="bf16").to_numpy()
    b = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_FILTER,
                                 precision="bf16").to_numpy()
    assert a.tobytes() == b.tobytes()


def test_bf16_bench_shape_sampled(af, oracle):
    """The benchmark forward shape (128x128x64x32 * 3x3x64x128) against FP64
    on 512 sampled outputs."""
    g = C.rng(33)
    s = np.asfortranarray(g.standard_normal((128, 128, 64, 32), dtype=np.float32))
    f = np.asfortranarray((g.standard_normal((3, 3, 64, 128)) * np.sqrt(2 / 576)).astype(np.float32))
    out = af.convolve2_nn(af.Array.from_numpy(s), af.Array.from_numpy(f), (1, 1), (1, 1), (1, 1),
                          precision="bf16").to_numpy().ravel(order="F")
    idx = g.integers(0, out.size, 512)
    ref = oracle.nn_forward_points_f64(s, f, (1, 1), (1, 1), (1, 1), idx)
    rel = np.linalg.norm(out[idx] - ref) / np.linalg.norm(ref)
    assert rel <= REL


# ---- FP8-E4M3 forward ------------------------------------------------------
# e4m3 keeps 3 mantissa bits: with amax scaling each operand carries up to
# 2^-4 relative rounding error (rms ~3.6%), so the norm-wise relative error of
# the forward is a few percent.  Bound: 8e-2 norm-wise, 0.3 * max|ref| max-abs.
FP8_REL = 8e-2
FP8_CASES = [c for c in TC_CASES if c[0] in ("nn_multi", "nn_s2_c16", "nn_1x1", "tc_c64_k128",
                                              "tc_c128_k256_s2", "tc_c200_k130", "tc_1x1_c256")]


@pytest.mark.parametrize("case", FP8_CASES, ids=[c[0] for c in FP8_CASES])
def test_fp8_forward(af, oracle, case):
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 8100)
    out = af.convolve2_nn(af.Array.from_numpy(s), af.Array.from_numpy(f), st, pd, dl,
                          precision="fp8").to_numpy()
    ref = oracle.nn_forward_f64(s, f, st, pd, dl)
    rel = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    mx = np.abs(out - ref).max() / np.abs(ref).max()
    assert rel <= FP8_REL and mx <= 0.3, f"rel {rel:.3e} max {mx:.3e}"


def test_fp8_forward_user_scales(af, oracle):
    """Per-output-channel scales supplied by the caller (afgb_convolve2_nn_ex
    out_channel_scales): same result quality as the device-derived scales."""
    case = FP8_CASES[3]
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 8200)
    scales = (np.abs(f).reshape(-1, fd[3], order="F").max(axis=0) / 448.0).astype(np.float32)
    out = af.convolve2_nn(af.Array.from_numpy(s), af.Array.from_numpy(f), st, pd, dl,
                          precision="fp8", scales=af.Array.from_numpy(scales)).to_numpy()
    ref = oracle.nn_forward_f64(s, f, st, pd, dl)
    rel = np.linalg.norm(out - ref) / np.linalg.norm(ref)
    assert rel <= FP8_REL


def test_fp8_gradients_not_supported(af):
    """FP8 is a forward-only form; gradients report AF_ERR_NOT_SUPPORTED."""
    case = C.NN_CASES[7]
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 1)
    g = C.nn_grad(case, 1)
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    O = af.convolve2_nn(S, F, st, pd, dl)
    with pytest.raises(af.AfError) as e:
        af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_DATA, precision="fp8")
    assert e.value.code == af.AF_ERR_NOT_SUPPORTED


def _launches(af, name, fn):
    import ctypes

    L = af.lib()
    L.afgb_kernel_timing(1)
    try:
        r = fn()
        af.sync()
        c, ms = ctypes.c_ulonglong(), ctypes.c_double()
        L.afgb_kernel_time(name.encode(), ctypes.byref(c), ctypes.byref(ms))
    finally:
        L.afgb_kernel_timing(0)
    return c.value, r


STRIDED = [("s2_c64", (33, 30, 64, 2), (3, 3, 64, 96), (2, 2), (1, 1), (1, 1)),
           ("s3x2_d2_c64", (40, 37, 64, 1), (3, 3, 64, 128), (3, 2), (2, 1), (2, 2)),
           ("s2_5x5_c128", (30, 28, 128, 2), (5, 5, 128, 64), (2, 2), (4, 4), (2, 2))]


@pytest.mark.parametrize("case", STRIDED, ids=lambda c: c[0])
def test_bf16_strided_tma_paths(af, oracle, case):
    """Strided forwards and filter gradients load the pixel operand by TMA
    with traversal strides (the map walks every s-th pixel); results against
    FP64 and the kernels that ran."""
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 6100)
    g = C.nn_grad(case, 6100)
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    n, Y = _launches(af, "tc_fwd_kernel", lambda: af.convolve2_nn(S, F, st, pd, dl, precision="bf16"))
    assert n == 1
    check(Y.to_numpy(), oracle.nn_forward_f64(s, f, st, pd, dl), name + " fwd")
    n, DW = _launches(af, "tc_wgrad_kernel", lambda: af.convolve2_gradient_nn(
        G, S, F, Y, st, pd, dl, af.AF_CONV_GRADIENT_FILTER, precision="bf16"))
    assert n == 1
    check(DW.to_numpy(), oracle.nn_filter_grad_f64(g, s, C.af_shape(fd), st, pd, dl), name + " wgrad")


COMBINED = [c for c in TC_CASES if c[0] in ("tc_c64_k128", "tc_c128_k256_s2", "tc_5x5_d2_p4_s2",
                                            "tc_c200_k130", "tc_rgb_s2", "nn_multi", "tc_strip_7x7")]


@pytest.mark.parametrize("precision", ["bf16", "fp32"])
@pytest.mark.parametrize("case", COMBINED, ids=lambda c: c[0])
def test_combined_gradients_match_separate(af, case, precision):
    """afgb_convolve2_gradients_nn returns the same bits as one
    afgb_convolve2_gradient_nn_ex call per gradient (BF16 shares the
    converted incoming gradient when its channel padding allows)."""
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 6300)
    g = C.nn_grad(case, 6300)
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    dx, dw, db = af.convolve2_gradients_nn(G, S, F, st, pd, dl, precision=precision, bias=True)
    sep = [af.convolve2_gradient_nn(G, S, F, G, st, pd, dl, t, precision=precision, real_bias=True)
           for t in (af.AF_CONV_GRADIENT_DATA, af.AF_CONV_GRADIENT_FILTER, af.AF_CONV_GRADIENT_BIAS)]
    for a, b in zip((dx, dw, db), sep):
        assert a.dims == b.dims
        assert a.to_numpy().tobytes() == b.to_numpy().tobytes()
    only_w = af.convolve2_gradients_nn(G, S, F, st, pd, dl, precision=precision, data=False)
    assert only_w[0] is None and only_w[2] is None
    assert only_w[1].to_numpy().tobytes() == sep[1].to_numpy().tobytes()


def test_combined_gradients_validation(af):
    case = TC_CASES[0]
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 1)
    S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
    bad = af.Array.from_numpy(np.zeros((3, 3, fd[3], sd[3]), np.float32, order="F"))
    with pytest.raises(af.AfError) as e:
        af.convolve2_gradients_nn(bad, S, F, st, pd, dl, precision="bf16")
    assert e.value.code == af.AF_ERR_SIZE
    with pytest.raises(af.AfError) as e:
        af.convolve2_gradients_nn(bad, S, F, st, pd, dl, data=False, filter=False, bias=False)
    assert e.value.code == af.AF_ERR_ARG


# ---- the signal's converted copy kept on its array --------------------------
def test_signal_copy_shared_and_invalidated(af, oracle):
    """A library-owned signal keeps its bf16 channels-last copy between the
    forward and the gradients of one step (same bits as a fresh array), and
    drops it when the buffer is written: through af_get_device_ptr (here a
    torch view writing new data) and by a library call writing in place
    (af_wrap_v2)."""
    import torch

    case = ("tc_c64_k128", (24, 20, 64, 2), (3, 3, 64, 128), (1, 1), (1, 1), (1, 1))
    name, sd, fd, st, pd, dl = case
    s1, f = C.nn_inputs(case, 91)
    s2, _ = C.nn_inputs(case, 92)
    g = C.nn_grad(case, 91)
    S, F, G = af.Array.from_numpy(s1), af.Array.from_numpy(f), af.Array.from_numpy(g)
    y1 = af.convolve2_nn(S, F, st, pd, dl, precision="bf16").to_numpy()
    dx, dw, _ = af.convolve2_gradients_nn(G, S, F, st, pd, dl, precision="bf16")
    S_fresh = af.Array.from_numpy(s1)
    dx0, dw0, _ = af.convolve2_gradients_nn(G, S_fresh, F, st, pd, dl, precision="bf16")
    assert dw.to_numpy().tobytes() == dw0.to_numpy().tobytes()
    assert dx.to_numpy().tobytes() == dx0.to_numpy().tobytes()
    # new contents through the device pointer
    t = torch.as_tensor(S, device="cuda")
    t.copy_(torch.from_numpy(np.ascontiguousarray(s2.transpose(3, 2, 1, 0))).cuda())
    torch.cuda.synchronize()
    y2 = af.convolve2_nn(S, F, st, pd, dl, precision="bf16").to_numpy()
    check(y2, oracle.nn_forward_f64(s2, f, st, pd, dl), "fwd after external write")
    assert np.abs(y2 - y1).max() > 0
    # new contents from a library call writing in place: wrap_v2 adds the
    # patches of s1 back into S (S becomes s2 + wrap(unwrap(s1)))
    U = af.unwrap(af.Array.from_numpy(s1), 1, 1, 1, 1, 0, 0)
    af.wrap_v2(S, U, sd[0], sd[1], 1, 1, 1, 1, 0, 0)
    y3 = af.convolve2_nn(S, F, st, pd, dl, precision="bf16").to_numpy()
    check(y3, oracle.nn_forward_f64(s1 + s2, f, st, pd, dl), "fwd after in-place library write")
