"""CPU tests of af_canny: the oracle port against the digests of the
reference's own CPU kernels (tests/golden/canny.json, written by
tests/golden/gen_golden.py with the port asserted identical to the
reference), the seed-scan range of the reference's hysteresis, and the
argument checks of src/api/c/canny.cpp:236-244 through the C ABI on a device
view that is never read (no device work)."""
import ctypes
import hashlib
import json
from pathlib import Path

import numpy as np
import pytest

import cases as C

GOLD = json.loads((Path(__file__).resolve().parent / "golden" / "canny.json").read_text())
DIMS4 = ctypes.c_longlong * 4


def digest(a):
    return hashlib.sha256(np.asfortranarray(a).tobytes(order="F")).hexdigest()


@pytest.mark.parametrize("case", C.canny_cases(), ids=lambda c: c[0])
def test_canny_port_matches_reference_digests(oracle, case):
    cid, dt, shape, otsu, t1, t2, isf, kind, seed = case
    e = oracle.canny(C.canny_image(dt, shape, kind, seed), dt, otsu, t1, t2, isf)
    assert e.dtype == np.int8 and set(np.unique(e)) <= {0, 1}
    assert int(e.sum()) == GOLD[cid]["edges"]
    assert digest(e) == GOLD[cid]["digest"]


def test_hysteresis_seed_range(oracle):
    """The reference's seed scan covers linear indices [d0+1, d0+(d0-1)(d1-1)]:
    on a wide slice a strong pixel in the last interior columns is no seed
    (and, not being weak, no edge); one in range is."""
    d0, d1 = 10, 30
    strong = np.zeros((d0, d1), bool)
    weak = np.zeros((d0, d1), bool)
    strong[5, d1 - 2] = True   # index (d1-2)*d0 + 5 = 285 > d0 + 9*29 = 271
    strong[5, 10] = True       # in range
    weak[6, 11] = True         # traced from the in-range seed
    weak[4, d1 - 3] = True     # adjacent only to the out-of-range strong pixel
    e = oracle.canny_hysteresis(strong, weak)
    assert e[5, 10] == 1 and e[6, 11] == 1
    assert e[5, d1 - 2] == 0 and e[4, d1 - 3] == 0


def _view(L, dims, dt=0):
    out = ctypes.c_void_p()
    strides = DIMS4(1, dims[0], dims[0] * dims[1], dims[0] * dims[1] * dims[2])
    assert L.afgb_device_array_view(ctypes.byref(out), ctypes.c_void_p(0x7F0000003000), 4,
                                    DIMS4(*dims), strides, dt) == 0
    return out


@pytest.mark.parametrize("dims,dt,sw,code", [
    ((64, 1, 1, 1), 0, 3, 203),     # 1-D input: AF_ERR_SIZE
    ((4, 64, 1, 1), 0, 3, 203),     # below 5 rows
    ((64, 4, 1, 1), 0, 3, 203),     # below 5 columns
    ((64, 64, 1, 1), 0, 5, 202),    # sobel window other than 3: AF_ERR_ARG
    ((64, 64, 1, 1), 4, 3, 204),    # b8 image: AF_ERR_TYPE
    ((64, 64, 1, 1), 1, 3, 204),    # c32 image
])
def test_canny_argument_checks(aflib_cpu, dims, dt, sw, code):
    L = aflib_cpu
    v = _view(L, dims, dt)
    out = ctypes.c_void_p()
    assert L.af_canny(ctypes.byref(out), v, 0, ctypes.c_float(0.1), ctypes.c_float(0.2), sw,
                      False) == code
    L.af_release_array(v)
