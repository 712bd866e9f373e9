"""The row kernel: stride-1 tensor-core forwards and data gradients with at
most 256 output channels (one CTA per group of 64), pixels on M and (filter
row, output channel) on N,
one TMEM buffer per source row and the partial output rows in the epilogue's
registers.  Against FP64 at the BF16 tolerance of the other tensor-core tests
(norm-wise relative error <= 2e-2, max-abs <= 8e-2 * max|ref|), on shapes
that reach its edge cases: several 128-pixel segments per row, output
channels that are not multiples of 64 (a partial last group), up to four
channel groups, filters one, two and three rows high, five tap columns
with horizontal dilation and the widest strip, padding of zero and of
fh - 1 rows, bands of output rows that cross from one image into the next,
and 1x1 filters.  Each case states which of its forward and data gradient
the row kernel serves (the others stay on the gather kernel); the gather
kernel (AFGB_NN_KERNEL=gather, in a child process) keeps its own parity check
on two of the shapes."""
import ctypes
import json
import os
import subprocess
import sys
from pathlib import Path

import numpy as np
import pytest

import cases as C

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]

# name, (W, H, C, N), (fw, fh, C, K), stride, pad, dilation; row kernel for (fwd, dgrad)
ROW_CASES = [
    (("w128_c64_k128", (128, 12, 64, 2), (3, 3, 64, 128), (1, 1), (1, 1), (1, 1)), (1, 1)),
    (("w128_c64_k64", (128, 12, 64, 2), (3, 3, 64, 64), (1, 1), (1, 1), (1, 1)), (1, 1)),
    (("w200_c48_k80", (200, 7, 48, 2), (3, 3, 48, 80), (1, 1), (1, 1), (1, 1)), (1, 1)),
    (("w200_c80_k48", (200, 7, 80, 2), (3, 3, 80, 48), (1, 1), (1, 1), (1, 1)), (1, 1)),
    (("w200_5x3_dx2", (200, 9, 64, 1), (5, 3, 64, 32), (1, 1), (4, 1), (2, 1)), (1, 1)),
    (("w100_nopad", (100, 9, 64, 2), (3, 3, 64, 64), (1, 1), (0, 0), (1, 1)), (1, 1)),
    (("w256_1x1_k16", (256, 5, 128, 1), (1, 1, 128, 16), (1, 1), (0, 0), (1, 1)), (1, 1)),
    (("w128_k200_four_groups", (128, 10, 64, 1), (3, 3, 64, 200), (1, 1), (1, 1), (1, 1)), (1, 0)),  # dgrad weights > smem
    (("w128_c256_k64", (128, 9, 256, 1), (3, 3, 256, 64), (1, 1), (1, 1), (1, 1)), (0, 1)),  # fwd weights > smem
    (("w128_bands_cross_images", (128, 6, 64, 3), (3, 3, 64, 64), (1, 1), (1, 1), (1, 1)), (1, 1)),
    (("w128_tall_py2", (128, 40, 64, 1), (3, 3, 64, 64), (1, 1), (1, 2), (1, 1)), (1, 1)),
    (("w128_3x1_k60", (128, 20, 64, 1), (3, 1, 64, 60), (1, 1), (1, 0), (1, 1)), (1, 1)),
    (("w128_3x2_c60", (128, 20, 60, 1), (3, 2, 60, 64), (1, 1), (1, 1), (1, 1)), (1, 1)),
]


def _err(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b)), float(np.abs(a - b).max() / np.abs(b).max())


def _check(got, ref, what):
    rel, mx = _err(got, ref)
    assert rel <= 2e-2 and mx <= 8e-2, f"{what}: rel {rel:.3e} max {mx:.3e}"


def _row_launches(af, fn):
    L = af.lib()
    L.afgb_kernel_timing(1)
    try:
        r = fn()
        af.sync()
        c, ms = ctypes.c_ulonglong(), ctypes.c_double()
        L.afgb_kernel_time(b"tc_row_kernel", ctypes.byref(c), ctypes.byref(ms))
    finally:
        L.afgb_kernel_timing(0)
    return c.value, r


@pytest.mark.parametrize("case,expect", ROW_CASES, ids=lambda c: c[0] if isinstance(c[0], str) else "")
def test_row_kernel_forward_and_data_gradient(af, oracle, case, expect):
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 7300)
    g = C.nn_grad(case, 7300)
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    n, Y = _row_launches(af, lambda: af.convolve2_nn(S, F, st, pd, dl, precision="bf16"))
    assert n == expect[0], f"forward: {n} row-kernel launches, expected {expect[0]}"
    _check(Y.to_numpy(), oracle.nn_forward_f64(s, f, st, pd, dl), name + " fwd")
    n, DX = _row_launches(af, lambda: af.convolve2_gradient_nn(
        G, S, F, Y, st, pd, dl, af.AF_CONV_GRADIENT_DATA, precision="bf16"))
    assert n == expect[1], f"data gradient: {n} row-kernel launches, expected {expect[1]}"
    ref = oracle.nn_data_grad_f64(g, list(s.shape), f, st, pd, dl)
    _check(DX.to_numpy(), ref, name + " dgrad")
    # the combined gradients call shares the incoming gradient's copy: same bits
    n, both = _row_launches(af, lambda: af.convolve2_gradients_nn(G, S, F, st, pd, dl, precision="bf16"))
    assert n == expect[1]
    assert both[0].to_numpy().tobytes() == DX.to_numpy().tobytes()


@pytest.mark.parametrize("relu", [True, False])
def test_row_kernel_bias_relu_epilogue(af, relu):
    case = ROW_CASES[3][0]
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 7400)
    rng = np.random.default_rng(7401)
    b = rng.standard_normal(fd[3]).astype(np.float32)
    S, F, B = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(b)
    n, Y = _row_launches(af, lambda: af.convolve2_nn(S, F, st, pd, dl, precision="bf16", bias=B, relu=relu))
    assert n == 1
    plain = af.convolve2_nn(S, F, st, pd, dl, precision="bf16").to_numpy()
    want = plain + b.reshape(1, 1, -1, 1)
    if relu:
        want = np.where(want < 0, np.float32(0), want)
    assert Y.to_numpy().tobytes() == want.astype(np.float32).tobytes()


def test_row_kernel_not_taken_outside_its_limits(af):
    """Strided, narrow, vertically dilated, five-row and over-256-channel shapes
    stay on the gather kernel."""
    for case in [("s2", (64, 30, 64, 1), (3, 3, 64, 64), (2, 2), (1, 1), (1, 1)),
                 ("narrow", (64, 30, 64, 1), (3, 3, 64, 64), (1, 1), (1, 1), (1, 1)),
                 ("dy2", (128, 20, 64, 1), (3, 3, 64, 64), (1, 1), (1, 2), (1, 2)),
                 ("w160_segment_waste", (160, 9, 64, 1), (3, 3, 64, 32), (1, 1), (1, 1), (1, 1)),
                 ("five_rows", (128, 20, 64, 1), (5, 5, 64, 64), (1, 1), (2, 2), (1, 1)),
                 ("k320", (128, 20, 64, 1), (3, 3, 64, 320), (1, 1), (1, 1), (1, 1))]:
        name, sd, fd, st, pd, dl = case
        s, f = C.nn_inputs(case, 7500)
        S, F = af.Array.from_numpy(s), af.Array.from_numpy(f)
        n, _ = _row_launches(af, lambda: af.convolve2_nn(S, F, st, pd, dl, precision="bf16"))
        assert n == 0, name


CHILD = r'''
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests/golden")
import torch
import arrayfire_gb300 as af
import oracle as O
import cases as C
af.lib(); torch.cuda.init(); af.set_stream(torch.cuda.current_stream())
CASES = json.loads(sys.argv[2])
res = {}
def err(a, b):
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    return [float(np.linalg.norm(a - b) / np.linalg.norm(b)), float(np.abs(a - b).max() / np.abs(b).max())]
for i, case in enumerate(CASES):
    case = tuple(tuple(c) if isinstance(c, list) else c for c in case)
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 7600 + i)
    g = C.nn_grad(case, 7600 + i)
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    y = af.convolve2_nn(S, F, st, pd, dl, precision="bf16").to_numpy()
    dx, dw, _ = af.convolve2_gradients_nn(G, S, F, st, pd, dl, precision="bf16")
    res[name] = {"fwd": err(y, O.nn_forward_f64(s, f, st, pd, dl)),
                 "dgrad": err(dx.to_numpy(), O.nn_data_grad_f64(g, list(s.shape), f, st, pd, dl))}
print(json.dumps(res))
'''


def test_gather_kernel_on_row_shapes_in_child_process():
    env = dict(os.environ, AFGB_NN_KERNEL="gather")
    cases = json.dumps([ROW_CASES[1][0], ROW_CASES[2][0]])
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT), cases], capture_output=True, text=True,
                       env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    assert len(res) == 2
    for name, e in res.items():
        for what in ("fwd", "dgrad"):
            rel, mx = e[what]
            assert rel <= 2e-2 and mx <= 8e-2, f"{name} {what}: rel {rel:.3e} max {mx:.3e}"
