"""CPU tests of the frequency-domain oracle (oracle.fft_convolve).

The reference's FFT path cannot be compiled here (it needs FFTW), so the
oracle's FFT semantics are pinned through the spatial path, which is pinned to
the reference's own CPU kernels: both compute the same linear convolution, so
for floating types they agree to rounding, and for integer types with integer
taps (the FFT path first truncates the taps to the signal type) they agree
exactly."""
import numpy as np
import pytest

import cases as C

SHAPES = [
    (1, (50, 3), (7,)), (1, (64,), (9, 4)), (1, (33, 5), (6, 5)),
    (2, (20, 17, 2), (5, 5)), (2, (20, 17), (5, 5, 3)), (2, (16, 12, 3), (4, 6, 3)),
    (2, (19, 9, 2, 3), (3, 3, 2, 3)),
    (3, (9, 8, 7), (3, 3, 3)), (3, (9, 8, 7, 2), (3, 2, 3)),
]


@pytest.mark.parametrize("rank,sd,fd", SHAPES)
@pytest.mark.parametrize("expand", [False, True])
def test_fft_oracle_matches_spatial_float(oracle, rank, sd, fd, expand):
    s = C.make_signal(C.F64, sd, 5)
    f = C.make_filter(C.F64, fd, 6, rank)
    a = oracle.fft_convolve(s, f, C.F64, rank, expand)
    b = oracle.convolve(s, f, C.F64, rank, expand)
    assert a.shape == b.shape
    np.testing.assert_allclose(a, b, rtol=0, atol=1e-12 * max(1.0, np.abs(b).max()))


@pytest.mark.parametrize("dt", [C.S32, C.U8, C.S16, C.U32, C.S64, C.B8])
@pytest.mark.parametrize("rank,sd,fd", SHAPES[:7])
def test_fft_oracle_integer_rounds_truncated_taps(oracle, dt, rank, sd, fd):
    s = C.make_signal(dt, sd, 7)
    g = np.random.Generator(np.random.Philox(8))
    f = np.asfortranarray(g.integers(0, 3, C.af_shape(fd)).astype(np.float32) +
                          np.float32(0.75))  # the FFT path truncates these taps
    a = oracle.fft_convolve(s, f, dt, rank, False)
    taps = (f != 0).astype(np.float32) if dt == C.B8 else np.trunc(f)
    b = oracle.convolve(s, np.asfortranarray(taps), dt, rank, False)
    np.testing.assert_array_equal(a, b)


def test_fft_oracle_complex_and_diff(oracle):
    s = C.make_signal(C.C64, (12, 10, 2), 9)
    f = C.make_signal(C.C64, (3, 4, 2), 10)
    a = oracle.fft_convolve(s, f, C.C64, 2, True)
    b = oracle.convolve(s, f, C.C64, 2, True)
    np.testing.assert_allclose(a, b, atol=1e-12 * np.abs(b).max())
    # DIFF batch: signal (.., 2, 1), filter (.., 1, 3) -> output (.., 2, 3)
    s = C.make_signal(C.F64, (10, 9, 2, 1), 11)
    f = C.make_filter(C.F64, (3, 3, 1, 3), 12, 2)
    a = oracle.fft_convolve(s, f, C.F64, 2, False)
    assert a.shape == (10, 9, 2, 3)
    for i in range(2):
        for j in range(3):
            ref = oracle.convolve(np.asfortranarray(s[:, :, i, 0]), np.asfortranarray(f[:, :, 0, j]),
                                  C.F64, 2, False)
            np.testing.assert_allclose(a[:, :, i, j], ref[:, :, 0, 0], atol=1e-12)
