"""CPU tests for af_unwrap / af_wrap / af_wrap_v2: the numpy port (oracle)
against the digests made from the reference's own CPU kernels
(tests/golden/patches.json) and against the reference tests' known answers
(test/wrap.cpp:200-251 DocSnippet, test/wrap.cpp:276-283 WrapV2 gold)."""
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import cases as C

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "patches.json").read_text())


def digest(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


@pytest.mark.parametrize("case", C.patch_cases(), ids=lambda c: c[0])
def test_port_patches_match_reference_hash(oracle, case):
    cid, dt, sd, wx, wy, sx, sy, px, py, col, seed = case
    g = GOLD[cid]
    geo = (wx, wy, sx, sy, px, py, col)
    img = C.patch_values(dt, sd, seed)
    u = oracle.unwrap_patches(img, *geo)
    assert list(u.shape) == g["unwrap_dims"] == C.patch_dims(case)
    assert digest(u) == g["unwrap"]
    pm = C.patch_values(dt, C.patch_dims(case), seed + 1)
    assert digest(oracle.wrap_patches(pm, sd[0], sd[1], *geo)) == g["wrap"]
    base = C.patch_values(dt, sd, seed + 2)
    assert digest(oracle.wrap_patches(pm, sd[0], sd[1], *geo, out=base)) == g["wrap_v2"]


def test_kat_doc_snippet_distinct(oracle):
    """test/wrap.cpp:200-226: 3x3 image, 2x2 windows at stride 2, padding 1."""
    A = np.arange(1, 10, dtype=np.float32).reshape(3, 3, order="F")
    U = oracle.unwrap_patches(A, 2, 2, 2, 2, 1, 1)
    gold_u = np.array([[0, 0, 0, 5], [0, 0, 4, 6], [0, 2, 0, 8], [1, 3, 7, 9]], np.float32)
    np.testing.assert_array_equal(U[:, :, 0, 0], gold_u)
    np.testing.assert_array_equal(oracle.wrap_patches(U, 3, 3, 2, 2, 2, 2, 1, 1)[:, :, 0, 0], A)


def test_kat_doc_snippet_sliding(oracle):
    """test/wrap.cpp:228-250: overlapping windows count each pixel's patches."""
    B = np.ones((3, 3), np.float32)
    U = oracle.unwrap_patches(B, 2, 2, 1, 1, 0, 0)
    assert U.shape[:2] == (4, 4) and (U == 1).all()
    W = oracle.wrap_patches(U, 3, 3, 2, 2, 1, 1, 0, 0)[:, :, 0, 0]
    gold = np.array([1, 2, 1, 2, 4, 2, 1, 2, 1], np.float32).reshape(3, 3, order="F")
    np.testing.assert_array_equal(W, gold)


def test_kat_wrap_v2_gold(oracle):
    """test/wrap.cpp:264-283: a 4x4 matrix of four 2x2 column patches wraps to
    the 4x4 image in tile order."""
    h_in = np.array([10, 20, 20, 30, 30, 40, 40, 50, 30, 40, 40, 50, 50, 60, 60, 70],
                    np.float32).reshape(4, 4, order="F")
    gold = np.array([10, 20, 30, 40, 20, 30, 40, 50, 30, 40, 50, 60, 40, 50, 60, 70],
                    np.float32).reshape(4, 4, order="F")
    np.testing.assert_array_equal(oracle.wrap_patches(h_in, 4, 4, 2, 2, 2, 2, 0, 0)[:, :, 0, 0],
                                  gold)
    # v2 into an existing image adds
    np.testing.assert_array_equal(
        oracle.wrap_patches(h_in, 4, 4, 2, 2, 2, 2, 0, 0, out=gold)[:, :, 0, 0], 2 * gold)


def factor_map(ix, iy, wx, wy, sx, sy, px, py):
    """How many patches cover each pixel (test/wrap.cpp:92-116)."""
    f = np.zeros((ix, iy), np.int64)
    nx = (ix + 2 * px - wx) // sx + 1
    ny = (iy + 2 * py - wy) // sy + 1
    for j in range(ny):
        for i in range(nx):
            x0, y0 = i * sx - px, j * sy - py
            f[max(x0, 0):min(x0 + wx, ix), max(y0, 0):min(y0 + wy, iy)] += 1
    return f


@pytest.mark.parametrize("geo", [(3, 3, 1, 1, 1, 1), (4, 4, 2, 2, 3, 3), (31, 31, 8, 8, 15, 15),
                                 (15, 10, 15, 10, 14, 9)])
@pytest.mark.parametrize("col", [True, False])
def test_port_wrap_of_unwrap_is_coverage_times_image(oracle, geo, col):
    """The reference's wrap test property (test/wrap.cpp:78-141): wrap(unwrap(x))
    equals x times the number of patches covering each pixel."""
    wx, wy, sx, sy, px, py = geo
    x = C.patch_values(C.S32, (60, 25), 7)[:, :, 0, 0] % 1000
    u = oracle.unwrap_patches(x, wx, wy, sx, sy, px, py, col)
    w = oracle.wrap_patches(u, 60, 25, wx, wy, sx, sy, px, py, col)[:, :, 0, 0]
    np.testing.assert_array_equal(w, x * factor_map(60, 25, wx, wy, sx, sy, px, py))


def test_port_patch_grid_truncates_like_c(oracle):
    """nx uses C's truncating division: a window wider than the padded image by
    less than the stride still yields one patch (src/api/c/wrap.cpp:51-52)."""
    assert oracle.patch_grid(4, 4, 5, 5, 2, 2, 0, 0) == (1, 1)
    assert oracle.patch_grid(4, 4, 6, 6, 2, 2, 0, 0) == (0, 0)
    assert oracle.patch_grid(4, 4, 7, 7, 2, 2, 0, 0) == (0, 0)
