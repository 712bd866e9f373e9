"""Failure detection: a bounded device wait that runs out is reported, and
the library stays usable.

Every wait of the TMA and tensor-core kernels spins a bounded number of
times, then raises a device error word and lets the kernel return; af_sync
reads the word, returns AF_ERR_RUNTIME and clears it.  Here the limit is
lowered to a few thousand polls and block 0 of the TMA 2-D kernel is told
to issue no tile copies (afgb_debug_wait_limit), so its consumers' waits run
out with no copy in flight: nothing traps, faults or waits forever.
"""
import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu


def test_expired_wait_reports_runtime_error_and_recovers(af, oracle):
    L = af.lib()
    s = C.make_signal(C.F32, (128, 96, 3), 41)
    f = C.make_filter(C.F32, (5, 5), 42, 2)
    S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
    af.sync()
    assert L.afgb_debug_wait_limit(4096, 1) == 0
    try:
        out = af.convolve2(S, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)  # enqueued
        rc = L.af_sync(-1)
    finally:
        assert L.afgb_debug_wait_limit(0, 0) == 0
    assert rc == af.AF_ERR_RUNTIME
    del out
    assert L.af_sync(-1) == 0  # the error word was read and cleared
    af.set_exact_fp(True)
    try:
        again = af.convolve2(S, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL).to_numpy()
    finally:
        af.set_exact_fp(False)
    assert again.tobytes() == oracle.convolve(s, f, C.F32, 2, False).tobytes()


def test_wait_limit_without_skipped_copies_changes_nothing(af, oracle):
    """A lowered limit alone does not trip healthy waits on a small image
    (the copies land long before a few thousand polls)."""
    L = af.lib()
    s = C.make_signal(C.F32, (64, 64, 2), 43)
    f = C.make_filter(C.F32, (3, 3), 44, 2)
    af.sync()
    assert L.afgb_debug_wait_limit(1 << 16, 0) == 0
    try:
        af.set_exact_fp(True)
        out = af.convolve2(af.Array.from_numpy(s), af.Array.from_numpy(f), af.AF_CONV_DEFAULT,
                           af.AF_CONV_SPATIAL).to_numpy()
    finally:
        af.set_exact_fp(False)
        assert L.afgb_debug_wait_limit(0, 0) == 0
    assert out.tobytes() == oracle.convolve(s, f, C.F32, 2, False).tobytes()
