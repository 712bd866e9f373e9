"""The pixels-on-M strip kernel (stride-1 tensor-core forward and data
gradient), selected with AFGB_NN_KERNEL=strip in a child process (the
library reads the switch once per process), against FP64 at the BF16
tolerance of the other tensor-core tests: norm-wise relative error <= 2e-2
and max-abs <= 8e-2 * max|ref|."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

pytestmark = pytest.mark.gpu
ROOT = Path(__file__).resolve().parents[1]

CHILD = r'''
import json, sys
import numpy as np
sys.path.insert(0, sys.argv[1]); sys.path.insert(0, sys.argv[1] + "/tests/golden")
import torch
import arrayfire_gb300 as af
import oracle as O
import cases as C
af.lib(); torch.cuda.init(); af.set_stream(torch.cuda.current_stream())
CASES = [
    ("w128_c64_k128", (128, 12, 64, 2), (3, 3, 64, 128), (1, 1), (1, 1), (1, 1)),
    ("w200_c48_k80", (200, 7, 48, 2), (3, 3, 48, 80), (1, 1), (1, 1), (1, 1)),
    ("w256_1x1_k16", (256, 5, 128, 1), (1, 1, 128, 16), (1, 1), (0, 0), (1, 1)),
    ("w160_5x3_dx2", (160, 9, 64, 1), (5, 3, 64, 32), (1, 1), (4, 1), (2, 1)),
    ("w100_nopad", (100, 9, 64, 2), (3, 3, 64, 128), (1, 1), (0, 0), (1, 1)),
]
res = {}
def err(a, b):
    a = np.asarray(a, np.float64); b = np.asarray(b, np.float64)
    return [float(np.linalg.norm(a - b) / np.linalg.norm(b)), float(np.abs(a - b).max() / np.abs(b).max())]
for i, case in enumerate(CASES):
    name, sd, fd, st, pd, dl = case
    s, f = C.nn_inputs(case, 900 + i)
    g = C.nn_grad(case, 900 + i)
    S, F, G = af.Array.from_numpy(s), af.Array.from_numpy(f), af.Array.from_numpy(g)
    y = af.convolve2_nn(S, F, st, pd, dl, precision="bf16").to_numpy()
    dx, dw, _ = af.convolve2_gradients_nn(G, S, F, st, pd, dl, precision="bf16")
    Y = af.convolve2_nn(S, F, st, pd, dl)
    dx1 = af.convolve2_gradient_nn(G, S, F, Y, st, pd, dl, af.AF_CONV_GRADIENT_DATA, precision="bf16").to_numpy()
    res[name] = {"fwd": err(y, O.nn_forward_f64(s, f, st, pd, dl)),
                 "dgrad": err(dx.to_numpy(), O.nn_data_grad_f64(g, list(s.shape), f, st, pd, dl)),
                 "dgrad_same": bool(dx1.tobytes() == dx.to_numpy().tobytes())}
print(json.dumps(res))
'''


def test_strip_kernel_parity_in_child_process():
    env = dict(os.environ, AFGB_NN_KERNEL="strip")
    r = subprocess.run([sys.executable, "-c", CHILD, str(ROOT)], capture_output=True, text=True,
                       env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    res = json.loads(r.stdout.strip().splitlines()[-1])
    for name, e in res.items():
        for what in ("fwd", "dgrad"):
            rel, mx = e[what]
            assert rel <= 2e-2 and mx <= 8e-2, f"{name} {what}: rel {rel:.3e} max {mx:.3e}"
        assert e["dgrad_same"], f"{name}: gradients call and per-gradient call differ"
