"""GPU tests of the frequency-domain convolution (af_fft_convolve1/2/3 and the
AUTO / FREQ routes of af_convolve1/2/3) against the oracle's FP64 restatement
of the reference's FFT semantics (oracle.fft_convolve): floating types within
a rounding bound, integer types bit for bit (rounded results of exact integer
sums), and the reference's argument checks."""
import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu

SHAPES = [
    (1, (50, 3), (7,)), (1, (64,), (9, 4)), (1, (33, 5), (6, 5)), (1, (40,), (129,)),
    (2, (20, 17, 2), (5, 5)), (2, (20, 17), (5, 5, 3)), (2, (16, 12, 3), (4, 6, 3)),
    (2, (19, 9, 2, 3), (3, 3, 2, 3)), (2, (45, 37), (21, 19)),
    (3, (9, 8, 7), (3, 3, 3)), (3, (9, 8, 7, 2), (3, 2, 3)), (3, (12, 10, 9), (7, 6, 8)),
]
FN = {1: "fft_convolve1", 2: "fft_convolve2", 3: "fft_convolve3"}


def bound(s, f, rank, expand, oracle):
    """max over outputs of sum |s||f| (FP64), the scale of the rounding error."""
    sa = np.abs(s).astype(np.float64)
    fa = np.abs(f).astype(np.float64)
    return float(np.abs(oracle.fft_convolve(sa, fa, C.F64, rank, expand)).max()) + 1e-30


def run_fft(af, s, f, dt, rank, expand, fdt=None):
    S = af.Array.from_numpy(s, dt)
    F = af.Array.from_numpy(f, fdt)
    mode = af.AF_CONV_EXPAND if expand else af.AF_CONV_DEFAULT
    return getattr(af, FN[rank])(S, F, mode).to_numpy()


def values(dt, shape, seed):
    if dt in (C.F32, C.F64, C.C32, C.C64):
        return C.make_signal(dt, shape, seed)
    g = np.random.Generator(np.random.Philox(seed))
    hi = {C.B8: 2, C.U8: 6, C.S8: 6}.get(dt, 50)
    return np.asfortranarray(g.integers(0, hi, C.af_shape(shape)).astype(C.NP_OF[dt]))


@pytest.mark.parametrize("dt", [C.F32, C.F64, C.C32, C.C64, C.S32, C.U8, C.S16, C.U64, C.B8],
                         ids=lambda d: C.DT_NAME[d])
@pytest.mark.parametrize("rank,sd,fd", SHAPES, ids=lambda v: str(v).replace(" ", ""))
@pytest.mark.parametrize("expand", [False, True])
def test_fft_matches_oracle(af, oracle, dt, rank, sd, fd, expand):
    s = values(dt, sd, 100 + rank)
    if dt in (C.C32, C.C64):
        f = C.make_signal(dt, fd, 200 + rank)
    elif dt in (C.F32, C.F64):
        f = C.make_filter(dt, fd, 200 + rank, rank)
    else:
        g = np.random.Generator(np.random.Philox(300 + rank))
        f = np.asfortranarray(g.integers(0, 3, C.af_shape(fd)).astype(np.float32) + 0.5)
    got = run_fft(af, s, f, dt, rank, expand)
    ref = oracle.fft_convolve(s, f, dt, rank, expand)
    assert got.shape == ref.shape and got.dtype == ref.dtype
    if dt in (C.F32, C.F64, C.C32, C.C64):
        eps = 1e-5 if dt in (C.F32, C.C32) else 1e-13
        tol = eps * bound(s, f, rank, expand, oracle)
        assert np.abs(got.astype(np.complex128) - ref).max() <= tol
    else:
        np.testing.assert_array_equal(got, ref)


@pytest.mark.parametrize("dt", [C.F32, C.S32], ids=lambda d: C.DT_NAME[d])
def test_fft_diff_batch(af, oracle, dt):
    """DIFF batches go through the reference's fallback (no tap truncation,
    truncating integer conversion): signal (.., 2, 1) x filter (.., 1, 3)."""
    s = values(dt, (30, 21, 2, 1), 5)
    f = np.asfortranarray(C.make_filter(C.F32, (5, 4, 1, 3), 6, 2))
    got = run_fft(af, s, f, dt, 2, True)
    ref = oracle.fft_convolve(s, f, dt, 2, True)
    assert got.shape == (34, 24, 2, 3)
    if dt == C.F32:
        assert np.abs(got - ref).max() <= 1e-5 * bound(s, f, 2, True, oracle)
    else:  # trunc of a float sum: +-1 where the sum sits on an integer
        assert np.abs(got.astype(np.int64) - ref.astype(np.int64)).max() <= 1


def test_auto_and_freq_route_to_fft(af, oracle):
    """src/api/c/convolve.cpp:99-130: kbatch >= 10, filters over 17 and
    non-square filters over 5 go to the frequency domain; FREQ always."""
    s = C.make_signal(C.F32, (40, 30, 12), 11)
    f = C.make_filter(C.F32, (5, 5, 12), 12, 2)
    S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
    auto = af.convolve2(S, F, af.AF_CONV_DEFAULT, af.AF_CONV_AUTO).to_numpy()
    fft = af.fft_convolve2(S, F, af.AF_CONV_DEFAULT).to_numpy()
    assert auto.tobytes() == fft.tobytes()
    ref = oracle.convolve(s, f, C.F32, 2, False)
    assert np.abs(auto - ref).max() <= 1e-5 * bound(s, f, 2, False, oracle)
    s2 = C.make_signal(C.F32, (64, 48), 13)
    f2 = C.make_filter(C.F32, (23, 23), 14, 2)
    S2, F2 = af.Array.from_numpy(s2), af.Array.from_numpy(f2)
    for dom in (af.AF_CONV_AUTO, af.AF_CONV_FREQ):
        got = af.convolve2(S2, F2, af.AF_CONV_EXPAND, dom).to_numpy()
        assert got.tobytes() == af.fft_convolve2(S2, F2, af.AF_CONV_EXPAND).to_numpy().tobytes()
    # a small filter with FREQ still takes the FFT route
    f3 = C.make_filter(C.F32, (3, 3), 15, 2)
    got = af.convolve2(S2, af.Array.from_numpy(f3), af.AF_CONV_DEFAULT, af.AF_CONV_FREQ)
    ref = oracle.convolve(s2, f3, C.F32, 2, False)
    assert np.abs(got.to_numpy() - ref).max() <= 1e-5 * bound(s2, f3, 2, False, oracle)
    # 1-D: a 200-tap filter (> 128) under AUTO
    s1 = C.make_signal(C.F32, (1000,), 16)
    f1 = C.make_filter(C.F32, (200,), 17, 1)
    got = af.convolve1(af.Array.from_numpy(s1), af.Array.from_numpy(f1), af.AF_CONV_DEFAULT,
                       af.AF_CONV_AUTO).to_numpy()
    ref = oracle.fft_convolve(s1, f1, C.F32, 1, False)
    assert np.abs(got - ref).max() <= 1e-5 * bound(s1, f1, 1, False, oracle)


def test_fft_rank_reduction(af):
    """af_fft_convolve2 on vectors is rank 1; af_fft_convolve3 on images is
    rank 2 (src/api/c/fftconvolve.cpp:244-266)."""
    s = C.make_signal(C.F32, (100,), 1)
    f = C.make_filter(C.F32, (9,), 2, 1)
    S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
    a = af.fft_convolve2(S, F, af.AF_CONV_EXPAND).to_numpy()
    b = af.fft_convolve1(S, F, af.AF_CONV_EXPAND).to_numpy()
    assert a.tobytes() == b.tobytes()
    s = C.make_signal(C.F32, (30, 20), 3)
    f = C.make_filter(C.F32, (5, 5), 4, 2)
    S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
    a = af.fft_convolve3(S, F, af.AF_CONV_DEFAULT).to_numpy()
    b = af.fft_convolve2(S, F, af.AF_CONV_DEFAULT).to_numpy()
    assert a.tobytes() == b.tobytes()


def test_fft_errors(af):
    S = af.Array.from_numpy(np.ones((8, 8, 2, 3), np.float32))
    F = af.Array.from_numpy(np.ones((3, 3, 3, 3), np.float32))
    with pytest.raises(af.AfError) as e:
        af.fft_convolve2(S, F)
    assert e.value.code == af.AF_ERR_ARG
    H = af.Array.from_numpy(np.ones((8, 8), np.float16))
    F2 = af.Array.from_numpy(np.ones((3, 3), np.float32))
    with pytest.raises(af.AfError) as e:
        af.fft_convolve2(H, F2)
    assert e.value.code == af.AF_ERR_TYPE


@pytest.mark.parametrize("rank,sdim,fdim,expand", [
    (1, 32768, 25, True), (1, 32768, 4095, False), (2, 1024, 25, True), (2, 1024, 129, False),
    (3, 64, 5, True), (3, 64, 31, False)])
def test_fft_large(af, oracle, rank, sdim, fdim, expand):
    """test/fftconvolve.cpp:107-225 sizes: uniform [0,1) signal and filter,
    checked against the FP64 oracle (the reference test allows 5e-2)."""
    g = np.random.Generator(np.random.Philox(rank * 1000 + fdim))
    s = np.asfortranarray(g.random((sdim,) * rank, dtype=np.float32))
    f = np.asfortranarray(g.random((fdim,) * rank, dtype=np.float32))
    got = run_fft(af, s, f, C.F32, rank, expand)
    ref = oracle.fft_convolve(s, f, C.F32, rank, expand)
    assert got.shape == ref.shape
    assert np.abs(got - ref).max() <= 2e-6 * float(np.abs(ref).max()) + 1e-6


def test_fft_strided_input_and_launches(af, oracle):
    import torch

    base = torch.randn(64, 50, device="cuda")
    v = af.Array.view_device(base.data_ptr(), [25, 64], af.f32, strides=[2, 50], keep=base)
    f = C.make_filter(C.F32, (7, 7, 3), 5, 2)
    n0 = af.launch_count()
    got = af.fft_convolve2(v, af.Array.from_numpy(f)).to_numpy()
    assert af.launch_count() > n0
    host = np.asfortranarray(base.cpu().numpy().T[::2, :])
    ref = oracle.fft_convolve(host, f, C.F32, 2, False)
    assert np.abs(got - ref).max() <= 1e-5 * bound(host, f, 2, False, oracle)


def test_fft_plan_cache_eviction(af, oracle):
    """More distinct transform shapes than the plan cache holds, twice over:
    every call keeps the plans it uses while older ones are evicted."""
    for rep in range(2):
        for n in range(20, 60, 2):
            s = C.make_signal(C.F32, (n, 3), n)
            f = C.make_filter(C.F32, (5,), n + 1, 1)
            got = af.fft_convolve1(af.Array.from_numpy(s), af.Array.from_numpy(f)).to_numpy()
            ref = oracle.fft_convolve(s, f, C.F32, 1, False)
            assert np.abs(got - ref).max() <= 1e-5 * bound(s, f, 1, False, oracle)


def _launches(af, names, fn):
    import ctypes

    L = af.lib()
    L.afgb_kernel_timing(1)
    try:
        r = fn()
        af.sync()
        counts = {}
        for name in names:
            c, ms = ctypes.c_ulonglong(), ctypes.c_double()
            L.afgb_kernel_time(name.encode(), ctypes.byref(c), ctypes.byref(ms))
            counts[name] = c.value
    finally:
        L.afgb_kernel_timing(0)
    return counts, r


OWN = ("fft_r2c_rows_kernel", "fft_c2r_rows_kernel", "fft_axis_kernel")


@pytest.mark.parametrize("dt,rank,sd,fd", [
    (C.F32, 1, (3000, 4), (77,)), (C.F64, 1, (513,), (40, 3)),
    (C.F32, 2, (300, 250, 2), (31, 17)), (C.F64, 2, (97, 130), (9, 9, 2)),
    (C.F32, 3, (40, 33, 20), (5, 4, 3)), (C.C32, 2, (120, 90), (11, 11)),
    (C.C64, 3, (20, 18, 10, 2), (3, 3, 3)), (C.S32, 2, (200, 150), (15, 15))],
    ids=lambda v: str(v).replace(" ", ""))
def test_own_transforms_serve_2a3b_sizes(af, oracle, dt, rank, sd, fd):
    """The padded lengths are 2^a 3^b, so this library's Stockham transforms
    run (no cuFFT): the real-row kernels for real data, the axis kernel for
    every other axis and for complex data; results within the rounding bound
    of the FP64 oracle (integers bit for bit)."""
    s = values(dt, sd, 70 + rank)
    if dt in (C.C32, C.C64):
        f = C.make_signal(dt, fd, 71 + rank)
    elif dt in (C.F32, C.F64):
        f = C.make_filter(dt, fd, 71 + rank, rank)
    else:
        f = np.asfortranarray(np.ones(fd, np.float32))
    counts, got = _launches(af, OWN, lambda: run_fft(af, s, f, dt, rank, True))
    real = dt not in (C.C32, C.C64)
    if real:
        assert counts["fft_r2c_rows_kernel"] > 0 and counts["fft_c2r_rows_kernel"] > 0
    if rank > 1 or not real:
        assert counts["fft_axis_kernel"] > 0
    ref = oracle.fft_convolve(s, f, dt, rank, True)
    if dt in (C.F32, C.F64, C.C32, C.C64):
        eps = 1e-5 if dt in (C.F32, C.C32) else 1e-13
        assert np.abs(got.astype(np.complex128) - ref).max() <= eps * bound(s, f, rank, True, oracle)
    else:
        np.testing.assert_array_equal(got, ref)


def test_cufft_serves_lengths_above_the_shared_memory_plan(af, oracle):
    """A 1-D length whose half does not fit one block's shared memory
    (36864 = 2^12 * 9 here) goes to cuFFT, with the same results."""
    g = np.random.Generator(np.random.Philox(9))
    s = np.asfortranarray(g.random(32768, dtype=np.float32))
    f = np.asfortranarray(g.random(4095, dtype=np.float32))
    counts, got = _launches(af, OWN, lambda: run_fft(af, s, f, C.F32, 1, False))
    assert counts["fft_r2c_rows_kernel"] == 0
    ref = oracle.fft_convolve(s, f, C.F32, 1, False)
    assert np.abs(got - ref).max() <= 2e-6 * float(np.abs(ref).max()) + 1e-6
