"""The no-allocation filter-gradient entry point, through the C ABI.

afgb_convolve2_filter_grad_noalloc serves callers that cannot allocate GPU
memory (their device memory is wholly reserved by another allocator, or their
memory budget is fixed after start-up): it takes caller-owned device buffers
and keeps its split-K partial sums in a fixed device array inside the
library.  Its results must match the allocating entry point
(af_convolve2_gradient_nn with AF_CONV_GRADIENT_FILTER) within the FP32
tolerance the NN tests use, call after call, because every call reuses the
same scratch array; they are also checked against the FP64 oracle.

That it allocates nothing is checked directly: after a warm-up call (the
first call on a device places the scratch array, see the header), a call
runs with the library's allocation-failure injection armed and must still
succeed, and neither the device's free memory nor the library pool's
statistics change across it.

This file is collected last so that a failure here leaves every other test
already run.
"""
import ctypes

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu

CASES = [
    ("s2_c16", (17, 15, 16, 2), (3, 3, 16, 24), (2, 2), (1, 1), (1, 1)),
    ("s1_c64_k128", (24, 20, 64, 2), (3, 3, 64, 128), (1, 1), (1, 1), (1, 1)),
    ("d2_p4_s2", (20, 18, 8, 2), (5, 5, 8, 12), (2, 2), (4, 4), (2, 2)),
    # fw*fh*C*K = 2,096,640, just under the 2,097,152-float scratch: one split
    ("at_cap", (6, 5, 512, 1), (3, 3, 512, 455), (1, 1), (1, 1), (1, 1)),
]


def dims_arg(v):
    return (ctypes.c_longlong * len(v))(*[int(x) for x in v])


def noalloc_filter_grad(af, g_t, x_t, sdims, fdims, st, pd, dl, stream="torch", dw=None):
    """Call the entry point on torch-owned device buffers; returns (rc, dW).
    stream: "torch" passes torch's current stream, None passes 0 (the
    library's own stream)."""
    import torch

    if dw is None:
        dw = torch.empty(list(reversed(fdims)), dtype=torch.float32, device="cuda")
    if stream == "torch":
        sp = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream or 1)
    else:
        sp = None
    rc = af.lib().afgb_convolve2_filter_grad_noalloc(
        ctypes.c_void_p(dw.data_ptr()), ctypes.c_void_p(g_t.data_ptr()),
        ctypes.c_void_p(x_t.data_ptr()), dims_arg(sdims), dims_arg(fdims), dims_arg(st),
        dims_arg(pd), dims_arg(dl), sp)
    if stream == "torch":
        torch.cuda.synchronize()
    else:
        af.sync()
    return rc, dw


def _inputs(af, case):
    import torch

    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 4242)
    g = C.nn_grad(case, 4242)
    x_t = torch.from_numpy(np.ascontiguousarray(s.ravel(order="F"))).cuda()
    g_t = torch.from_numpy(np.ascontiguousarray(g.ravel(order="F"))).cuda()
    return s, f, g, x_t, g_t


def _as_filter(dw, f):
    return dw.cpu().numpy().reshape(-1).reshape(f.shape, order="F")


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_allocating_entry_point(af, oracle, case):
    name, sd, fd, st, pd, dl = case
    s, f, g, x_t, g_t = _inputs(af, case)
    # the allocating entry point on the same data
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    O = af.convolve2_nn(S, F, st, pd, dl)
    ref = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_FILTER).to_numpy()
    ref64 = oracle.nn_filter_grad_f64(g, s, list(f.shape), st, pd, dl)
    scale = max(1.0, float(np.abs(ref).max()))
    scale64 = max(1.0, float(np.abs(ref64).max()))
    for _ in range(2):  # two calls in a row share the scratch array
        rc, dw = noalloc_filter_grad(af, g_t, x_t, list(s.shape), list(f.shape), st, pd, dl)
        assert rc == 0
        got = _as_filter(dw, f)
        err = float(np.abs(got.astype(np.float64) - ref).max())
        assert err <= 1e-5 * scale, f"max abs err vs allocating path {err:.3e}"
        err64 = float(np.abs(got.astype(np.float64) - ref64).max())
        assert err64 <= 1e-5 * scale64, f"max abs err vs FP64 {err64:.3e}"


def test_noalloc_allocates_nothing(af):
    """A warmed-up call succeeds with every library allocation made to fail,
    and leaves the device's free memory and the pool statistics unchanged."""
    import torch

    case = CASES[1]
    name, sd, fd, st, pd, dl = case
    s, f, g, x_t, g_t = _inputs(af, case)
    dw = torch.empty(list(reversed(f.shape)), dtype=torch.float32, device="cuda")
    rc, ref = noalloc_filter_grad(af, g_t, x_t, list(s.shape), list(f.shape), st, pd, dl, dw=dw)
    assert rc == 0
    ref = _as_filter(ref, f)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    pool0 = af.device_mem_info()
    af.lib().afgb_debug_fail_alloc_after(1)
    try:
        rc, dw = noalloc_filter_grad(af, g_t, x_t, list(s.shape), list(f.shape), st, pd, dl, dw=dw)
    finally:
        af.lib().afgb_debug_fail_alloc_after(0)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert rc == 0
    assert free1 == free0
    assert af.device_mem_info() == pool0
    assert _as_filter(dw, f).tobytes() == ref.tobytes()


def test_noalloc_on_library_stream(af):
    """stream 0 runs on the library's current stream, with the same result."""
    import torch

    case = CASES[0]
    name, sd, fd, st, pd, dl = case
    s, f, g, x_t, g_t = _inputs(af, case)
    torch.cuda.synchronize()
    rc0, a = noalloc_filter_grad(af, g_t, x_t, list(s.shape), list(f.shape), st, pd, dl,
                                 stream=None)
    rc1, b = noalloc_filter_grad(af, g_t, x_t, list(s.shape), list(f.shape), st, pd, dl)
    assert rc0 == 0 and rc1 == 0
    assert _as_filter(a, f).tobytes() == _as_filter(b, f).tobytes()


def test_noalloc_rejects_oversized_filter(af):
    """fw*fh*C*K beyond the 2,097,152-float scratch gives AF_ERR_SIZE."""
    import torch

    dummy = torch.zeros(16, device="cuda")
    sdims, fdims = [8, 8, 512, 1], [3, 3, 512, 512]
    rc = af.lib().afgb_convolve2_filter_grad_noalloc(
        ctypes.c_void_p(dummy.data_ptr()), ctypes.c_void_p(dummy.data_ptr()),
        ctypes.c_void_p(dummy.data_ptr()), dims_arg(sdims), dims_arg(fdims), dims_arg([1, 1]),
        dims_arg([1, 1]), dims_arg([1, 1]), None)
    assert rc == af.AF_ERR_SIZE
