"""The NN convolution pair inside torch.autograd (arrayfire_gb300.autograd),
checked three ways:

* against the FP64 oracle, whose NN formulas are pinned to the reference's own
  unwrap + GEMM and wrap_dilated (the reference's gradient call,
  src/backend/cpu/convolve.cpp:179-243);
* against FP64 central finite differences, h = 1e-3 on 256 random coordinates
  of the input, filter and bias, at the full backward shapes
  64x64x128x16 * 3x3x128x256 (stride 2, pad 1) and 5x5 with dilation 2, pad 4.
  The loss is L = sum(G * conv(x, w) + b), evaluated in FP64 with torch's
  float64 convolution (pinned to the oracle by
  tests/test_torch_reference_cpu.py); L is linear in each coordinate, so the
  central difference is exact up to FP64 rounding (~1e-10 relative);
* a four-layer conv2_nn + ReLU network with activation recomputation against
  the same network in FP64.

Tolerances: FP32 path 1e-5 relative (norm-wise) against FP64; BF16 path 2e-2
(bf16 operands, FP32 accumulation) per layer.  Through the four-layer
network the BF16 gradients stay within 5e-2 (each layer's activations are
re-rounded to bf16, so per-layer errors compound).
"""
import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu


def to_af(t):
    """torch (N,C,H,W) -> ArrayFire-layout numpy (W,H,C,N), Fortran order."""
    return np.asfortranarray(t.detach().cpu().numpy().transpose(3, 2, 1, 0))


def ref_conv64(x, w, s, p, d):
    import torch.nn.functional as F

    return F.conv2d(x.double(), w.double().flip([2, 3]), stride=(s[1], s[0]),
                    padding=(p[1], p[0]), dilation=(d[1], d[0]))


def rel(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


AG_CASES = [c for c in C.NN_CASES if c[0] in ("nn_s1p1", "nn_d2", "nn_35_s31_d21", "nn_multi",
                                               "nn_s2_c16", "nn_5x5_d2_s2", "nn_1x1", "nn_nopad")]


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("bf16", 2e-2)])
@pytest.mark.parametrize("case", AG_CASES, ids=lambda c: c[0])
def test_function_against_oracle(af, oracle, case, precision, tol):
    import torch

    from arrayfire_gb300.autograd import conv2_nn

    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 101)
    x = torch.from_numpy(np.ascontiguousarray(s.transpose(3, 2, 1, 0))).cuda().requires_grad_()
    w = torch.from_numpy(np.ascontiguousarray(f.transpose(3, 2, 1, 0))).cuda().requires_grad_()
    b = torch.randn(fd[3], device="cuda", requires_grad=True)
    y = conv2_nn(x, w, b, st, pd, dl, precision=precision)
    gnp = C.nn_grad(case, 101)
    g = torch.from_numpy(np.ascontiguousarray(gnp.transpose(3, 2, 1, 0))).cuda()
    y.backward(g)
    torch.cuda.synchronize()
    yref = oracle.nn_forward_f64(s, f, st, pd, dl) + b.detach().cpu().double().numpy()[None, None, :, None]
    assert rel(to_af(y), yref) <= tol
    assert rel(to_af(x.grad), oracle.nn_data_grad_f64(gnp, C.af_shape(sd), f, st, pd, dl)) <= tol
    assert rel(to_af(w.grad), oracle.nn_filter_grad_f64(gnp, s, C.af_shape(fd), st, pd, dl)) <= tol
    bref = oracle.nn_bias_grad_f64(gnp, C.af_shape(sd), C.af_shape(fd), st, pd, dl).ravel()
    assert rel(b.grad.cpu().numpy(), bref) <= max(tol, 1e-6)


def test_gradcheck_f64(af):
    """torch.autograd.gradcheck on the f64 path (the library computes f64
    convolutions in f64)."""
    import torch

    from arrayfire_gb300.autograd import Conv2NN

    g = torch.Generator(device="cpu").manual_seed(5)
    x = torch.randn(2, 3, 7, 6, generator=g, dtype=torch.float64).cuda().requires_grad_()
    w = torch.randn(4, 3, 3, 2, generator=g, dtype=torch.float64).cuda().requires_grad_()
    b = torch.randn(4, generator=g, dtype=torch.float64).cuda().requires_grad_()
    fn = lambda x_, w_, b_: Conv2NN.apply(x_, w_, b_, (2, 1), (1, 1), (1, 2), "fp32")  # noqa: E731
    assert torch.autograd.gradcheck(fn, (x, w, b), eps=1e-6, atol=1e-8, rtol=1e-6)


FD_SHAPES = [
    # (name, x (N,C,H,W), w (K,C,fh,fw), stride, padding, dilation) in ArrayFire order pairs
    ("bwd_3x3_s2", (16, 128, 64, 64), (256, 128, 3, 3), (2, 2), (1, 1), (1, 1)),
    ("bwd_5x5_d2_p4_s2", (16, 128, 64, 64), (256, 128, 5, 5), (2, 2), (4, 4), (2, 2)),
]


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-5), ("bf16", 2e-2)])
@pytest.mark.parametrize("shape", FD_SHAPES, ids=lambda s: s[0])
def test_finite_differences_full_size(af, shape, precision, tol):
    import torch

    from arrayfire_gb300.autograd import conv2_nn

    name, xs, ws, st, pd, dl = shape
    gen = torch.Generator(device="cuda").manual_seed(11)
    x = torch.randn(xs, device="cuda", generator=gen).requires_grad_()
    std = (2.0 / (ws[1] * ws[2] * ws[3])) ** 0.5
    w = (torch.randn(ws, device="cuda", generator=gen) * std).requires_grad_()
    b = torch.zeros(ws[0], device="cuda", requires_grad=True)
    y = conv2_nn(x, w, b, st, pd, dl, precision=precision)
    G = torch.randn(y.shape, device="cuda", generator=gen)
    y.backward(G)
    torch.cuda.synchronize()

    x64, w64, b64, G64 = x.detach().double(), w.detach().double(), b.detach().double(), G.double()

    def loss(xv, wv, bv, n=None):
        # images other than n do not change when a coordinate of image n moves
        if n is not None:
            return (G64[n:n + 1] * (ref_conv64(xv[n:n + 1], wv, st, pd, dl)
                                    + bv.view(1, -1, 1, 1))).sum().item()
        return (G64 * (ref_conv64(xv, wv, st, pd, dl) + bv.view(1, -1, 1, 1))).sum().item()

    rng = np.random.Generator(np.random.Philox(3))
    h = 1e-3
    fd_vals, an_vals = [], []
    # 160 input coordinates, 80 filter coordinates, 16 bias coordinates
    for _ in range(160):
        i = tuple(int(rng.integers(0, d)) for d in xs)
        xp, xm = x64.clone(), x64.clone()
        xp[i] += h
        xm[i] -= h
        fd_vals.append((loss(xp, w64, b64, i[0]) - loss(xm, w64, b64, i[0])) / (2 * h))
        an_vals.append(x.grad[i].item())
    for _ in range(80):
        i = tuple(int(rng.integers(0, d)) for d in ws)
        wp, wm = w64.clone(), w64.clone()
        wp[i] += h
        wm[i] -= h
        fd_vals.append((loss(x64, wp, b64) - loss(x64, wm, b64)) / (2 * h))
        an_vals.append(w.grad[i].item())
    for _ in range(16):
        k = int(rng.integers(0, ws[0]))
        bp, bm = b64.clone(), b64.clone()
        bp[k] += h
        bm[k] -= h
        fd_vals.append((loss(x64, w64, bp) - loss(x64, w64, bm)) / (2 * h))
        an_vals.append(b.grad[k].item())
    fd_vals, an_vals = np.array(fd_vals), np.array(an_vals)
    for sl, what in ((slice(0, 160), "input"), (slice(160, 240), "filter"), (slice(240, 256), "bias")):
        r = rel(an_vals[sl], fd_vals[sl])
        assert r <= (tol if what != "bias" else max(tol, 1e-6)), f"{name} {precision} {what}: {r:.3e}"


def _cnn_setup(n=2, hw=32, seed=0):
    import torch

    gen = torch.Generator(device="cuda").manual_seed(seed)
    x0 = torch.rand((n, 3, hw, hw), device="cuda", generator=gen) * 2 - 1
    chans = [(3, 32), (32, 64), (64, 128), (128, 128)]
    ws = [torch.randn((k, c, 3, 3), device="cuda", generator=gen) * (2.0 / (9 * c)) ** 0.5
          for c, k in chans]
    geoms = [((2, 2), (1, 1), (1, 1)), ((2, 2), (1, 1), (1, 1)), ((1, 1), (1, 1), (1, 1)),
             ((1, 1), (2, 2), (2, 2))]
    return x0, ws, geoms


def _cnn_ref64(x0, ws, geoms):
    import torch

    wl = [w.detach().double().requires_grad_() for w in ws]
    h = x0.double()
    for w, (s, p, d) in zip(wl, geoms):
        h = torch.relu(ref_conv64(h, w, s, p, d))
    loss = (h ** 2).sum()
    loss.backward()
    return loss.item(), [w.grad for w in wl]


@pytest.mark.parametrize("precision,tol", [("fp32", 1e-4), ("bf16", 5e-2)])
def test_cnn_step_against_fp64(af, precision, tol):
    from arrayfire_gb300.autograd import cnn_step

    x0, ws, geoms = _cnn_setup()
    loss, grads, rflops = cnn_step(x0, ws, geoms, precision=precision, recompute=True)
    ref_loss, ref_grads = _cnn_ref64(x0, ws, geoms)
    assert abs(loss.item() - ref_loss) <= tol * abs(ref_loss)
    for l, (g, r) in enumerate(zip(grads, ref_grads)):
        e = rel(g.cpu().numpy(), r.cpu().numpy())
        assert e <= tol, f"layer {l + 1}: {e:.3e}"
    assert rflops > 0


def test_cnn_recompute_matches_stored(af):
    """Recomputed layer inputs are the same bits as stored ones, so the
    gradients agree exactly."""
    from arrayfire_gb300.autograd import cnn_step

    x0, ws, geoms = _cnn_setup(seed=1)
    _, g1, r1 = cnn_step(x0, ws, geoms, precision="bf16", recompute=True)
    _, g2, r2 = cnn_step(x0, ws, geoms, precision="bf16", recompute=False)
    assert r1 > 0 and r2 == 0
    for a, b in zip(g1, g2):
        assert a.cpu().numpy().tobytes() == b.cpu().numpy().tobytes()
