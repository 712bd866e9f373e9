"""The no-allocation filter-gradient entry point, through the C ABI.

afgb_convolve2_filter_grad_noalloc serves callers that cannot allocate GPU
memory (their device memory is wholly reserved by another allocator, or their
memory budget is fixed after start-up): it takes caller-owned device buffers
and keeps its split-K partial sums in a fixed device array inside the
library.  Its results must match the allocating entry point
(af_convolve2_gradient_nn with AF_CONV_GRADIENT_FILTER) within the FP32
tolerance the NN tests use, call after call, because every call reuses the
same scratch array.

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
]


def dims_arg(v):
    return (ctypes.c_longlong * len(v))(*[int(x) for x in v])


def noalloc_filter_grad(af, g_t, x_t, sdims, fdims, st, pd, dl):
    """Call the entry point on torch-owned device buffers; returns (rc, dW)."""
    import torch

    dw = torch.empty(list(reversed(fdims)), dtype=torch.float32, device="cuda")
    rc = af.lib().afgb_convolve2_filter_grad_noalloc(
        ctypes.c_void_p(dw.data_ptr()), ctypes.c_void_p(g_t.data_ptr()),
        ctypes.c_void_p(x_t.data_ptr()), dims_arg(sdims), dims_arg(fdims), dims_arg(st),
        dims_arg(pd), dims_arg(dl), ctypes.c_void_p(torch.cuda.current_stream().cuda_stream or 1))
    torch.cuda.synchronize()
    return rc, dw


@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_noalloc_matches_allocating_entry_point(af, case):
    import torch

    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 4242)
    g = C.nn_grad(case, 4242)
    # the allocating entry point on the same data
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    O = af.convolve2_nn(S, F, st, pd, dl)
    ref = af.convolve2_gradient_nn(G, S, F, O, st, pd, dl, af.AF_CONV_GRADIENT_FILTER).to_numpy()
    # caller-owned device buffers (ArrayFire layout: reversed torch shape)
    x_t = torch.from_numpy(np.ascontiguousarray(s.ravel(order="F"))).cuda()
    g_t = torch.from_numpy(np.ascontiguousarray(g.ravel(order="F"))).cuda()
    scale = max(1.0, float(np.abs(ref).max()))
    for _ in range(2):  # two calls in a row share the scratch array
        rc, dw = noalloc_filter_grad(af, g_t, x_t, list(s.shape), list(f.shape), st, pd, dl)
        assert rc == 0
        got = dw.cpu().numpy().reshape(-1).reshape(f.shape, order="F")
        err = float(np.abs(got.astype(np.float64) - ref).max())
        assert err <= 1e-5 * scale, f"max abs err {err:.3e}"


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
