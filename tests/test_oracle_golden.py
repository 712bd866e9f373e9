"""CPU tests: the oracle port against the golden fixtures (made from the
reference's own CPU kernels) and against the reference's in-source known
answers.  No GPU."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import cases as C

GOLD = Path(__file__).resolve().parent / "golden"


def digest(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


DIRECT = json.loads((GOLD / "direct.json").read_text())
SEP = json.loads((GOLD / "sep.json").read_text())


@pytest.mark.parametrize("case", list(C.direct_cases()), ids=lambda c: c[0])
def test_port_direct_matches_reference_hash(oracle, case):
    cid, dt, rank, sd, fd, expand, seed = case
    s = C.make_signal(dt, sd, seed)
    f = C.make_filter(dt, fd, seed + 1, rank)
    out = oracle.convolve(s, f, dt, rank, expand, "port")
    assert list(out.shape) == DIRECT[cid]["dims"]
    assert digest(out) == DIRECT[cid]["sha256"]


@pytest.mark.parametrize("case", list(C.sep_cases()), ids=lambda c: c[0])
def test_port_sep_matches_reference_hash(oracle, case):
    cid, dt, sd, cl, rl, expand, seed = case
    s = C.sep_signal(dt, sd, seed)
    out = oracle.convolve2_sep(s, C.sep_taps(dt, cl, seed + 1), C.sep_taps(dt, rl, seed + 2), dt,
                               expand, "port")
    assert list(out.shape) == SEP[cid]["dims"]
    assert digest(out) == SEP[cid]["sha256"]


@pytest.mark.parametrize("name,fn", [("config1a_gauss5_512", C.config1a),
                                     ("config1b_neighbour3_1024", C.config1b)])
def test_port_config1_full_size(oracle, name, fn):
    s, f = fn()
    out = oracle.convolve(s, f, C.F32, 2, False, "port")
    assert digest(out) == DIRECT[name]["sha256"]


def test_nn_fp64_loops_match_fixture(oracle):
    gold = np.load(GOLD / "nn.npz")
    for i, case in enumerate(C.NN_CASES):
        name, sd, fd, st, pd, dl = case
        s, f = C.nn_inputs(case, 9000 + 10 * i, np.float64)
        g = C.nn_grad(case, 9000 + 10 * i, np.float64)
        np.testing.assert_allclose(oracle.nn_forward_f64(s, f, st, pd, dl), gold[f"{name}__fwd"],
                                   rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(oracle.nn_data_grad_f64(g, list(s.shape), f, st, pd, dl),
                                   gold[f"{name}__dgrad"], rtol=1e-12, atol=1e-12)
        np.testing.assert_allclose(oracle.nn_filter_grad_f64(g, s, list(f.shape), st, pd, dl),
                                   gold[f"{name}__wgrad"], rtol=1e-12, atol=1e-12)


# ---- in-source known answers of the reference (test/convolve.cpp)
def test_kat_doc_1d(oracle):
    # test/convolve.cpp:526-536 (values printed to 4 decimals)
    a = np.array([0.0000, 0.1315, 0.7556, 0.4587, 0.5328, 0.2190, 0.0470, 0.6789, 0.6793, 0.9347],
                 np.float32)
    b = np.array([0.3835, 0.5194, 0.8310, 0.0346], np.float32)
    c = np.array([0.3581, 0.6777, 1.0750, 0.7679, 0.5903, 0.4851, 0.6598, 1.2770, 1.0734, 0.8002])
    out = oracle.convolve(a, b, C.F32, 1, False)[:, 0, 0, 0]
    np.testing.assert_allclose(out, c, atol=2e-4)


def test_kat_doc_2d(oracle):
    # test/convolve.cpp:541-563
    out = oracle.convolve(np.full((5, 5), 0.5, np.float32), np.ones((2, 2), np.float32), C.F32, 2,
                          False)[:, :, 0, 0]
    gold = np.full((5, 5), 2.0)
    gold[4, :] = 1.0
    gold[:, 4] = 1.0
    gold[4, 4] = 0.5
    np.testing.assert_array_equal(out, gold)


def test_kat_doc_3d(oracle):
    # test/convolve.cpp:565-620
    out = oracle.convolve(np.ones((4, 4, 4), np.float32), np.full((2, 2, 2), 0.5, np.float32),
                          C.F32, 3, False)[:, :, :, 0]
    gold = np.full((4, 4, 4), 4.0)
    for ax in range(3):
        idx = [slice(None)] * 3
        idx[ax] = 3
        gold[tuple(idx)] /= 2
    np.testing.assert_array_equal(out, gold)


def test_kat_zero_padding_issue2817(oracle):
    # test/convolve.cpp:1170-1185
    s = np.ones((5, 5), np.float32)
    f = np.full((3, 3), 1 / 9, np.float32)
    conv = oracle.nn_forward_f64(s, f, (1, 1), (0, 0), (1, 1))[:, :, 0, 0]
    assert np.abs(conv - 1.0).sum() < 1e-5
    g = np.full((3, 3), 1 / 9, np.float32)
    wg = oracle.nn_filter_grad_f64(g, s, [3, 3, 1, 1], (1, 1), (0, 0), (1, 1))[:, :, 0, 0]
    assert np.abs(wg - conv).sum() < 1e-5


@pytest.mark.parametrize("n,fsz", [(10, 3), (11, 5), (12, 7), (19, 9), (33, 3), (255, 3),
                                   (256, 3), (257, 3)])
def test_kat_conv2_consistency(oracle, n, fsz):
    # test/convolve.cpp:868-894: convolve2NN(pad=f/2) == convolve2 within 2e-5
    g = C.rng(n * 100 + fsz)
    s = g.standard_normal((n, n)).astype(np.float32)
    f = g.standard_normal((fsz, fsz)).astype(np.float32)
    native = oracle.convolve(s, f, C.F32, 2, False)[:, :, 0, 0]
    nn = oracle.nn_forward_f64(s, f, (1, 1), (fsz // 2, fsz // 2), (1, 1))[:, :, 0, 0]
    np.testing.assert_allclose(native, nn, atol=2e-5 * max(1.0, np.abs(nn).max()))


def test_unwrap_port_shape_and_values(oracle):
    # test/unwrap.cpp:208-239 style check on a small ramp: every column of the
    # unwrapped matrix is the window of the padded image at its position
    s = np.arange(1, 26, dtype=np.float32).reshape(5, 5, order="F")
    cols = oracle.unwrap(s, 3, 3, 2, 2, 1, 1, 1, 1)[:, :, 0, 0]
    assert cols.shape == (9, 9)
    pad = np.zeros((7, 7), np.float32)
    pad[1:6, 1:6] = s
    for col in range(9):
        x0, y0 = (col % 3) * 2, (col // 3) * 2
        win = pad[x0:x0 + 3, y0:y0 + 3]
        np.testing.assert_array_equal(cols[:, col], win.ravel(order="F"))


@pytest.mark.skipif(not (Path(__file__).resolve().parents[1] / "oracle" / "_ref" / "libafref.so").exists(),
                    reason="reference kernels not compiled here")
def test_port_equals_reference_random(oracle):
    """Random extra shapes: the port and the reference's own kernels agree
    bit for bit (run where the reference tree is available)."""
    g = C.rng(77)
    for trial in range(60):
        rank = int(g.integers(1, 4))
        dt = [C.F32, C.F64, C.U8, C.S32, C.C32][trial % 5]
        sd = [int(g.integers(2, 20)) for _ in range(rank)]
        fd = [int(g.integers(2, 6)) for _ in range(rank)]
        if rank == 2 and fd[0] != fd[1] and max(fd) > 5:
            continue
        expand = bool(g.integers(0, 2))
        s = C.make_signal(dt, sd, 100 + trial)
        f = C.make_filter(dt, fd, 200 + trial, rank)
        a = oracle.convolve(s, f, dt, rank, expand, "port")
        b = oracle.convolve(s, f, dt, rank, expand, "ref")
        assert a.tobytes() == b.tobytes()
