"""GPU tests of the runtime's host transfers: uploads (af_create_array) and
downloads (af_get_data_ptr) run on copy streams ordered by per-buffer events,
so they overlap compute; results must still be exactly the computed ones."""
import ctypes

import numpy as np
import pytest
import torch

pytestmark = pytest.mark.gpu


def test_upload_compute_download_chain(af):
    """Arrays used right after their upload, outputs read while later work is
    queued: every value is the one computed in order."""
    g = np.random.Generator(np.random.Philox(3))
    x = np.asfortranarray(g.standard_normal((96, 80, 8, 4), dtype=np.float32))
    w = np.asfortranarray(g.standard_normal((3, 3, 8, 16), dtype=np.float32))
    X, W = af.Array.from_numpy(x), af.Array.from_numpy(w)
    ys = [af.convolve2_nn(X, W, (1, 1), (1, 1), (1, 1)) for _ in range(3)]
    big = af.convolve2_nn(af.Array.from_numpy(x), W, (1, 1), (1, 1), (1, 1))  # queued after
    first = ys[0].to_numpy()
    for y in ys[1:] + [big]:
        assert y.to_numpy().tobytes() == first.tobytes()


def test_download_after_device_pointer_write(af):
    """A caller that writes through af_get_device_ptr on its own stream work
    sees its write in af_get_data_ptr (the download then waits on the whole
    stream, not on the library's last write)."""
    a = af.Array.from_numpy(np.zeros((256, 64), np.float32))
    b = af.convolve2(a, af.Array.from_numpy(np.ones((3, 3), np.float32)))
    ptr = b.device_ptr()
    t = torch.as_tensor(b, device="cuda")  # same memory
    assert t.data_ptr() == ptr
    t.fill_(7.0)
    out = b.to_numpy()
    assert (out == 7.0).all()


def test_many_small_round_trips(af):
    for n in (1, 3, 17, 1000, 65536):
        v = np.arange(n, dtype=np.float64)
        A = af.Array.from_numpy(v)
        assert np.array_equal(A.to_numpy().ravel(), v)
