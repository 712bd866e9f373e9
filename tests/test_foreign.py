"""Handle interop with another ArrayFire backend library.

An af_array made by libafcuda (directly or through the unified libaf) is an
opaque object of that library (src/api/c/handle.hpp:50-83;
src/api/unified/symbol_manager.hpp:144-165 forwards handles unchanged).
afgb_import_foreign_array turns one into a view of this library by calling
that library's own af_get_device_ptr / af_get_dims / af_get_strides /
af_get_type (and af_sync); afgb_export_foreign_array copies a result into a
new array of that library (af_create_handle, af_get_device_ptr,
af_unlock_array).

ArrayFire itself is not installed here, so tests/c/foreign_backend_stub.c
stands in for it: a shared library exporting those entry points over its
own handle type.  The CPU tests check the handle translation without a
device; the GPU test runs a convolution on an imported array and exports the
result.
"""
import ctypes
import shutil
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
STUB = ROOT / "tests" / "c" / "foreign_backend_stub.c"
DIMS4 = ctypes.c_longlong * 4


@pytest.fixture(scope="module")
def stub(tmp_path_factory):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    so = tmp_path_factory.mktemp("stub") / "libforeign_stub.so"
    r = subprocess.run([cc, "-std=c99", "-O1", "-shared", "-fPIC", str(STUB), "-o", str(so)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    lib = ctypes.CDLL(str(so))  # RTLD_LOCAL: its af_* names stay private to it
    lib.stub_make_array.restype = ctypes.c_void_p
    lib.stub_make_array.argtypes = [ctypes.c_void_p, DIMS4, DIMS4, ctypes.c_int]
    lib.stub_data.restype = ctypes.c_void_p
    lib.stub_data.argtypes = [ctypes.c_void_p]
    lib.stub_is_locked.argtypes = [ctypes.c_void_p]
    lib.stub_set_pool.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    lib.af_release_array.argtypes = [ctypes.c_void_p]
    lib.af_get_dims.argtypes = [ctypes.POINTER(ctypes.c_longlong)] * 4 + [ctypes.c_void_p]
    lib.af_get_type.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_void_p]
    return lib


def _info(L, h):
    d = [ctypes.c_longlong() for _ in range(4)]
    s = [ctypes.c_longlong() for _ in range(4)]
    t = ctypes.c_int()
    p = ctypes.c_void_p()
    assert L.af_get_dims(*[ctypes.byref(x) for x in d], h) == 0
    assert L.af_get_strides(*[ctypes.byref(x) for x in s], h) == 0
    assert L.af_get_type(ctypes.byref(t), h) == 0
    assert L.af_get_device_ptr(ctypes.byref(p), h) == 0
    return [x.value for x in d], [x.value for x in s], t.value, p.value


def test_import_reads_the_foreign_handle(aflib_cpu, stub):
    """Pointer, dims, strides and type of a strided foreign array arrive
    unchanged in the view; the foreign buffer is locked (af_get_device_ptr)
    and the foreign queue synchronised."""
    L = aflib_cpu
    fake = 0x7F0000001000
    h = stub.stub_make_array(fake, DIMS4(30, 20, 3, 2), DIMS4(2, 64, 1280, 3840), 0)
    syncs = stub.stub_sync_count()
    out = ctypes.c_void_p()
    assert L.afgb_import_foreign_array(ctypes.byref(out), h, stub._handle) == 0
    d, s, t, p = _info(L, out)
    assert d == [30, 20, 3, 2] and s == [2, 64, 1280, 3840] and t == 0 and p == fake
    assert stub.stub_is_locked(h) == 1
    assert stub.stub_sync_count() == syncs + 1
    assert L.af_release_array(out) == 0
    assert stub.stub_data(h) == fake  # releasing the view left the foreign array alone
    stub.af_release_array(h)


def test_import_rejects_bad_arguments(aflib_cpu, stub, tmp_path):
    L = aflib_cpu
    out = ctypes.c_void_p()
    h = stub.stub_make_array(0x1000, DIMS4(4, 1, 1, 1), DIMS4(1, 4, 4, 4), 0)
    assert L.afgb_import_foreign_array(ctypes.byref(out), h, None) == 202  # AF_ERR_ARG
    assert L.afgb_import_foreign_array(None, h, stub._handle) == 202
    # a library without the entry points: AF_ERR_LOAD_SYM
    libm = ctypes.CDLL("libm.so.6")
    assert L.afgb_import_foreign_array(ctypes.byref(out), h, libm._handle) == 502
    # the foreign library's own error comes back unchanged
    bogus = ctypes.create_string_buffer(64)  # not a stub handle: its af_get_device_ptr says AF_ERR_ARG
    assert L.afgb_import_foreign_array(ctypes.byref(out), ctypes.addressof(bogus), stub._handle) == 202
    stub.af_release_array(h)


def test_header_declares_interop(aflib_cpu):
    text = (ROOT / "include" / "afgb300.h").read_text()
    for name in ("afgb_import_foreign_array", "afgb_export_foreign_array"):
        assert name in text
        assert hasattr(aflib_cpu, name)


@pytest.mark.gpu
def test_convolve_foreign_array_and_export(af, oracle, stub):
    """A foreign f32 image over device memory: af_convolve2 on its imported
    view equals the same call on a library array, and the exported result
    (a new foreign array) holds the same values."""
    import torch

    g = np.random.Generator(np.random.Philox(5))
    img = np.asfortranarray(g.random((64, 48, 3), dtype=np.float32))
    filt = np.asfortranarray(g.standard_normal((5, 5)).astype(np.float32))
    dev = torch.from_numpy(np.ascontiguousarray(img.transpose(2, 1, 0))).cuda()
    h = stub.stub_make_array(dev.data_ptr(), DIMS4(64, 48, 3, 1),
                             DIMS4(1, 64, 64 * 48, 64 * 48 * 3), 0)
    view = ctypes.c_void_p()
    L = af.lib()
    assert L.afgb_import_foreign_array(ctypes.byref(view), h, stub._handle) == 0
    V = af.Array(view.value)
    F = af.Array.from_numpy(filt)
    out = af.convolve2(V, F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)
    ref = af.convolve2(af.Array.from_numpy(img), F, af.AF_CONV_DEFAULT, af.AF_CONV_SPATIAL)
    np.testing.assert_array_equal(out.to_numpy(), ref.to_numpy())
    # export into the foreign library's memory
    pool = torch.zeros(1 << 20, dtype=torch.float32, device="cuda")
    stub.stub_set_pool(pool.data_ptr(), pool.numel() * 4)
    fh = ctypes.c_void_p()
    assert L.afgb_export_foreign_array(ctypes.byref(fh), out.handle, stub._handle) == 0
    assert stub.stub_is_locked(fh) == 0  # af_unlock_array after the copy
    d = [ctypes.c_longlong() for _ in range(4)]
    assert stub.af_get_dims(*[ctypes.byref(x) for x in d], fh) == 0
    assert [x.value for x in d] == [64, 48, 3, 1]
    got = pool[: 64 * 48 * 3].cpu().numpy().reshape(3, 48, 64).transpose(2, 1, 0)
    np.testing.assert_array_equal(got, ref.to_numpy()[..., 0])
    stub.af_release_array(fh)
    del V
    stub.af_release_array(h)
