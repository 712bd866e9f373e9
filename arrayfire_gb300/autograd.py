"""torch.autograd bindings of the NN convolution pair, and a multi-layer CNN
step built from it.

`Conv2NN` wraps af_convolve2_nn (src/api/c/convolve.cpp:344-392) as the
forward and af_convolve2_gradient_nn (src/api/c/convolve.cpp:394-477) as the
backward, exactly as a user of the reference would differentiate a layer:
the data gradient (AF_CONV_GRADIENT_DATA), the filter gradient
(AF_CONV_GRADIENT_FILTER) and, through the library's extension, the real bias
gradient -- all that are needed in one afgb_convolve2_gradients_nn call, whose
results equal the per-gradient calls bit for bit.  Tensors are passed
zero-copy: a torch tensor (N, C, H, W) is the ArrayFire array (W, H, C, N),
and the library runs on torch's current stream.

Semantics are ArrayFire's, not torch's: the filter is flipped (a true
convolution, src/backend/cpu/convolve.cpp:130-157), and stride, padding and
dilation pairs are given in ArrayFire order (dim 0 = W first).

`cnn_step` runs one forward and backward pass of a plain CNN (conv2_nn +
ReLU per layer, loss = sum of squares of the output) with activation
recomputation: the forward keeps only the network input and output, and the
backward recomputes each layer's input from the network input when it
needs it.  No im2col patch buffer is ever formed (the kernels gather their
operands implicitly), which is what the reference's unwrap + GEMM stores for
every layer (src/backend/cpu/convolve.cpp:213-243).
"""
from __future__ import annotations

from typing import Optional, Sequence

import torch

from . import Array, convolve2_gradients_nn, convolve2_nn, set_stream

__all__ = ["Conv2NN", "conv2_nn", "cnn_step", "nn_flops"]


def _view(t: torch.Tensor) -> Array:
    return Array.view_torch(t.contiguous())


def _grad_precision(precision: str) -> str:
    # the FP8 form has a forward only; its gradients run in BF16
    return "fp32" if precision == "fp32" else "bf16"


class Conv2NN(torch.autograd.Function):
    """y = af_convolve2_nn(x, w) (+ b per output channel)."""

    @staticmethod
    def forward(ctx, x, w, b, stride, padding, dilation, precision):
        set_stream(torch.cuda.current_stream())
        X, W = _view(x), _view(w)
        y = convolve2_nn(X, W, stride, padding, dilation, precision=precision).to_torch()
        if b is not None:
            y.add_(b.view(1, -1, 1, 1))
        ctx.save_for_backward(x, w)
        ctx.conf = (tuple(stride), tuple(padding), tuple(dilation), precision, b is not None)
        return y

    @staticmethod
    def backward(ctx, gy):
        x, w = ctx.saved_tensors
        stride, padding, dilation, precision, has_b = ctx.conf
        set_stream(torch.cuda.current_stream())
        gp = _grad_precision(precision)
        gy = gy.contiguous()
        # the gradient call takes the forward output only for its dims; the
        # incoming gradient has the same dims
        G, X, W = _view(gy), _view(x), _view(w)
        want = (ctx.needs_input_grad[0], ctx.needs_input_grad[1],
                has_b and ctx.needs_input_grad[2])
        gx = gw = gb = None
        if any(want):
            # one call for every gradient needed (each equals its
            # af_convolve2_gradient_nn result; BIAS is the real bias gradient)
            dX, dW, dB = convolve2_gradients_nn(G, X, W, stride, padding, dilation, precision=gp,
                                                data=want[0], filter=want[1], bias=want[2])
            gx = dX.to_torch() if dX is not None else None
            gw = dW.to_torch() if dW is not None else None
            gb = dB.to_torch().reshape(-1) if dB is not None else None
        return gx, gw, gb, None, None, None, None


def conv2_nn(x: torch.Tensor, w: torch.Tensor, b: Optional[torch.Tensor] = None,
             stride: Sequence[int] = (1, 1), padding: Sequence[int] = (0, 0),
             dilation: Sequence[int] = (1, 1), precision: str = "fp32") -> torch.Tensor:
    """Differentiable af_convolve2_nn on torch tensors x (N,C,H,W), w (K,C,fh,fw)."""
    return Conv2NN.apply(x, w, b, tuple(stride), tuple(padding), tuple(dilation), precision)


def nn_flops(x_shape, w_shape, stride, padding, dilation) -> float:
    """2*Wo*Ho*N*K*fw*fh*C: the multiply-adds of one forward (and of each gradient)."""
    n, c, h, wd = x_shape
    k, _, fh, fw = w_shape
    wo = 1 + (wd + 2 * padding[0] - ((fw - 1) * dilation[0] + 1)) // stride[0]
    ho = 1 + (h + 2 * padding[1] - ((fh - 1) * dilation[1] + 1)) // stride[1]
    return 2.0 * wo * ho * n * k * fw * fh * c


def _layer(h, w, geom, precision):
    """conv2_nn + ReLU, the ReLU fused into the convolution's epilogue."""
    s, p, d = geom
    return convolve2_nn(_view(h), _view(w), s, p, d, precision=precision, relu=True).to_torch()


def cnn_step(x0: torch.Tensor, weights: Sequence[torch.Tensor], geoms, precision: str = "bf16",
             recompute: bool = True):
    """One forward + backward pass of conv2_nn + ReLU layers with
    loss = sum(out**2).

    weights[l] is (K, C, fh, fw); geoms[l] = (stride, padding, dilation) in
    ArrayFire order.  With `recompute`, the forward keeps only x0 and the
    output, and the backward rebuilds each layer's input from x0.  Returns
    (loss, [dW_l], recompute_flops).
    """
    set_stream(torch.cuda.current_stream())
    L = len(weights)
    kept = [x0] + [None] * L
    h = x0
    for l in range(L):
        h = _layer(h, weights[l], geoms[l], precision)
        if not recompute or l == L - 1:
            kept[l + 1] = h
    out = h
    flat = out.reshape(-1)
    loss = torch.dot(flat, flat)       # sum of squares
    gp = _grad_precision(precision)
    grads = [None] * L
    g = out * 2.0                      # dL/d out
    above = out                        # ReLU output of the layer being differentiated
    rflops = 0.0
    for l in range(L - 1, -1, -1):
        x_l = kept[l]
        if x_l is None:                # recompute layer l's input from x0
            x_l = x0
            for j in range(l):
                rflops += nn_flops(x_l.shape, weights[j].shape, *geoms[j])
                x_l = _layer(x_l, weights[j], geoms[j], precision)
        s, p, d = geoms[l]
        # through the ReLU: dL/dz = dL/dh where h > 0 (one fused kernel)
        g = torch.ops.aten.threshold_backward(g, above, 0.0)
        G, X, W = _view(g), _view(x_l), _view(weights[l])
        dX, dW, _ = convolve2_gradients_nn(G, X, W, s, p, d, precision=gp, data=l > 0)
        grads[l] = dW.to_torch()
        if l > 0:
            g = dX.to_torch()
        above = x_l
        del G, X, W
    return loss, grads, rflops
