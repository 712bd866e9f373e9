"""Pins the FP64 evaluation used by the finite-difference and CNN tests:
torch's float64 conv2d on the flipped filter, with stride / padding /
dilation pairs swapped into torch's (H, W) order, equals the oracle's FP64
NN forward (itself pinned to the reference's unwrap + GEMM), and torch's
float64 autograd gradients equal the oracle's data and filter gradients."""
import numpy as np
import pytest

import cases as C


def ref_conv64(x, w, s, p, d):
    import torch.nn.functional as F

    return F.conv2d(x, w.flip([2, 3]), stride=(s[1], s[0]), padding=(p[1], p[0]),
                    dilation=(d[1], d[0]))


@pytest.mark.parametrize("case", C.NN_CASES, ids=lambda c: c[0])
def test_torch_fp64_matches_oracle(oracle, case):
    torch = pytest.importorskip("torch")
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 17)
    g = C.nn_grad(case, 17)
    x = torch.from_numpy(np.ascontiguousarray(s.transpose(3, 2, 1, 0))).double().requires_grad_()
    w = torch.from_numpy(np.ascontiguousarray(f.transpose(3, 2, 1, 0))).double().requires_grad_()
    y = ref_conv64(x, w, st, pd, dl)
    y.backward(torch.from_numpy(np.ascontiguousarray(g.transpose(3, 2, 1, 0))).double())
    back = lambda t: np.asfortranarray(t.detach().numpy().transpose(3, 2, 1, 0))  # noqa: E731
    np.testing.assert_allclose(back(y), oracle.nn_forward_f64(s, f, st, pd, dl), rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(back(x.grad), oracle.nn_data_grad_f64(g, C.af_shape(sd), f, st, pd, dl),
                               rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(back(w.grad), oracle.nn_filter_grad_f64(g, s, C.af_shape(fd), st, pd, dl),
                               rtol=1e-12, atol=1e-12)
