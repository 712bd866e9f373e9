"""CPU tests of the C-ABI library: it loads without a GPU, exports every
symbol include/afgb300.h declares, and its host-only dispatch helpers make the
reference's decisions.  No compute call touches a device here."""
import re
from pathlib import Path

import numpy as np
import pytest

import cases as C

ROOT = Path(__file__).resolve().parents[1]


def declared_symbols():
    text = (ROOT / "include" / "afgb300.h").read_text()
    return sorted(set(re.findall(r"AFGB_API\s+[\w\s\*]*?\b((?:af|afgb)_\w+)\s*\(", text)))


def test_header_declares_the_six_entry_points():
    syms = declared_symbols()
    for s in ("af_convolve1", "af_convolve2", "af_convolve3", "af_convolve2_sep",
              "af_convolve2_nn", "af_convolve2_gradient_nn"):
        assert s in syms


def test_library_exports_every_declared_symbol(aflib_cpu):
    missing = [s for s in declared_symbols() if not hasattr(aflib_cpu, s)]
    assert not missing, missing


def test_ctypes_signatures_cover_header(aflib_cpu):
    from arrayfire_gb300 import _lib

    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(declared_symbols()) <= bound


def test_error_strings(aflib_cpu):
    import arrayfire_gb300 as A

    L = A.lib()
    assert L.af_err_to_string(0) == b"Success"
    assert L.af_err_to_string(202) == b"Invalid input argument"
    assert L.af_err_to_string(301) == b"Function not supported"


def test_null_handle_is_an_argument_error(aflib_cpu):
    import ctypes

    import arrayfire_gb300 as A

    L = A.lib()
    d = (ctypes.c_longlong * 4)()
    assert L.af_get_dims(d, d, d, d, None) == A.AF_ERR_ARG
    out = ctypes.c_void_p()
    assert L.af_convolve2(ctypes.byref(out), None, None, 0, 0) == A.AF_ERR_ARG
    # the thread-local message names the failure
    msg = ctypes.c_char_p()
    n = ctypes.c_longlong()
    L.af_get_last_error(ctypes.byref(msg), ctypes.byref(n))
    assert b"handle" in msg.value
    L.af_free_host(ctypes.cast(msg, ctypes.c_void_p))


def test_batch_kind_matches_reference_rule(aflib_cpu, oracle):
    import arrayfire_gb300 as A

    g = C.rng(3)
    for _ in range(2000):
        rank = int(g.integers(1, 4))
        sd = [int(v) for v in g.choice([1, 1, 2, 3, 5], 4)]
        fd = [int(v) for v in g.choice([1, 1, 2, 3, 5], 4)]
        assert A.identify_batch_kind(rank, sd, fd) == oracle.identify_batch_kind(rank, sd, fd)


def test_output_dims_match_reference_rule(aflib_cpu, oracle):
    import arrayfire_gb300 as A

    g = C.rng(4)
    for _ in range(500):
        rank = int(g.integers(1, 4))
        sd = [int(v) for v in g.integers(1, 9, 4)]
        fd = [int(v) for v in g.integers(1, 6, 4)]
        kind = int(g.integers(0, 4))
        for expand in (False, True):
            assert A.conv_output_dims(rank, kind, expand, sd, fd) == oracle.conv_output_dims(
                rank, kind, expand, sd, fd)


def test_nn_output_dims_match_reference_rule(aflib_cpu, oracle):
    import arrayfire_gb300 as A

    g = C.rng(5)
    for _ in range(500):
        sd = [int(v) for v in g.integers(1, 40, 4)]
        fd = [int(v) for v in g.integers(1, 7, 4)]
        st = [int(v) for v in g.integers(1, 4, 2)]
        pd = [int(v) for v in g.integers(0, 4, 2)]
        dl = [int(v) for v in g.integers(1, 4, 2)]
        assert A.nn_output_dims(sd, fd, st, pd, dl) == oracle.nn_output_dims(sd, fd, st, pd, dl)


def test_product_does_not_import_oracle():
    """The product package never loads the checker."""
    for p in (ROOT / "arrayfire_gb300").rglob("*.py"):
        text = p.read_text()
        assert "import oracle" not in text and "from oracle" not in text, p
    for p in list((ROOT / "arrayfire_gb300" / "csrc").glob("*")):
        assert "conv_oracle" not in p.read_text(errors="ignore"), p
