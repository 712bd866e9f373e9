"""arrayfire_gb300 — GB300-native (sm_103a) backend for ArrayFire's spatial
convolution C API.

The compute lives in ``libafgb300.so`` (C ABI, ``include/afgb300.h``).  This
module is a thin Python mirror of the ArrayFire calls on that path, with the
same names, argument meaning and error codes:

    convolve1 / convolve2 / convolve3      af_convolve1/2/3   (include/af/signal.h:1391,1408,1460)
    convolve2_separable                    af_convolve2_sep   (include/af/signal.h:1478)
    convolve2_nn                           af_convolve2_nn    (include/af/signal.h:1440)
    convolve2_gradient_nn                  af_convolve2_gradient_nn (include/af/ml.h:84-92)
    fft_convolve1 / 2 / 3                  af_fft_convolve1/2/3 (include/af/signal.h:1492,1506,1520)
    unwrap / wrap / wrap_v2                af_unwrap / af_wrap / af_wrap_v2 (include/af/image.h:1483,1524,1570)
    gaussian_kernel / dog / sobel_operator af_gaussian_kernel, af_dog, af_sobel_operator

Arrays are ``Array`` handles over device memory with ArrayFire dims
(d0 fastest).  ``Array.from_numpy`` takes a numpy array laid out in
ArrayFire order (shape = dims, Fortran order); ``Array.view_torch`` wraps a
CUDA tensor without a copy (an NCHW tensor maps to dims (W,H,C,N)).
"""
from __future__ import annotations

import ctypes
from typing import Optional, Sequence

import numpy as np

from . import _lib
from ._lib import af_array, dims_arg, dim_t

# af_dtype (include/af/defines.h:211-233)
f32, c32, f64, c64, b8, s32, u32, u8, s64, u64, s16, u16, f16, s8 = range(14)
_NP = {f32: np.float32, c32: np.complex64, f64: np.float64, c64: np.complex128, b8: np.int8,
       s32: np.int32, u32: np.uint32, u8: np.uint8, s64: np.int64, u64: np.uint64,
       s16: np.int16, u16: np.uint16, f16: np.float16, s8: np.int8}
_FROM_NP = {np.dtype(np.float32): f32, np.dtype(np.complex64): c32, np.dtype(np.float64): f64,
            np.dtype(np.complex128): c64, np.dtype(np.int32): s32, np.dtype(np.uint32): u32,
            np.dtype(np.uint8): u8, np.dtype(np.int64): s64, np.dtype(np.uint64): u64,
            np.dtype(np.int16): s16, np.dtype(np.uint16): u16, np.dtype(np.float16): f16,
            np.dtype(np.int8): s8, np.dtype(np.bool_): b8}

AF_CONV_DEFAULT, AF_CONV_EXPAND = 0, 1
AF_CONV_AUTO, AF_CONV_SPATIAL, AF_CONV_FREQ = 0, 1, 2
AF_CONV_GRADIENT_DEFAULT, AF_CONV_GRADIENT_FILTER, AF_CONV_GRADIENT_DATA, AF_CONV_GRADIENT_BIAS = 0, 1, 2, 3
PRECISION = {"fp32": 0, "bf16": 1, "fp8": 2, "fp8_e4m3": 2}

AF_SUCCESS, AF_ERR_NO_MEM, AF_ERR_RUNTIME = 0, 101, 103
AF_ERR_ARG, AF_ERR_SIZE, AF_ERR_TYPE = 202, 203, 204
AF_ERR_NOT_SUPPORTED, AF_ERR_INTERNAL = 301, 998


class AfError(RuntimeError):
    """Raised for a non-zero af_err; ``code`` holds the value."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"af_err {code}: {msg}")
        self.code = code


def lib() -> ctypes.CDLL:
    return _lib.load()


def _check(code: int) -> None:
    if code != AF_SUCCESS:
        L = lib()
        msg = ctypes.c_char_p()
        ln = dim_t()
        L.af_get_last_error(ctypes.byref(msg), ctypes.byref(ln))
        text = msg.value.decode(errors="replace") if msg.value else ""
        if msg.value is not None:
            L.af_free_host(ctypes.cast(msg, ctypes.c_void_p))
        raise AfError(code, text or L.af_err_to_string(code).decode())


class Array:
    """Owning wrapper of an af_array handle (released on garbage collection)."""

    __slots__ = ("handle", "_keep")

    def __init__(self, handle: int, keep=None):
        self.handle = af_array(handle)
        self._keep = keep  # keeps a viewed tensor alive

    def __del__(self):
        h = getattr(self, "handle", None)
        if h is not None and h.value and _lib._lib is not None:
            try:
                _lib._lib.af_release_array(h)
            except Exception:
                pass
            self.handle = None

    # ---- construction
    @staticmethod
    def from_numpy(a: np.ndarray, dtype: Optional[int] = None) -> "Array":
        a = np.asarray(a)
        t = _FROM_NP[a.dtype] if dtype is None else dtype
        a = np.asfortranarray(a.astype(_NP[t], copy=False))
        dims = list(a.shape)[:4] if a.ndim else [1]
        out = af_array()
        _check(lib().af_create_array(ctypes.byref(out), a.ctypes.data_as(ctypes.c_void_p),
                                     len(dims), dims_arg(dims), t))
        return Array(out.value)

    @staticmethod
    def empty(dims: Sequence[int], dtype: int = f32) -> "Array":
        out = af_array()
        _check(lib().af_create_handle(ctypes.byref(out), len(dims), dims_arg(dims), dtype))
        return Array(out.value)

    @staticmethod
    def view_device(ptr: int, dims: Sequence[int], dtype: int, strides=None, keep=None) -> "Array":
        out = af_array()
        st = dims_arg(strides) if strides is not None else None
        _check(lib().afgb_device_array_view(ctypes.byref(out), ctypes.c_void_p(ptr), len(dims),
                                            dims_arg(dims), st, dtype))
        return Array(out.value, keep)

    @staticmethod
    def view_torch(t) -> "Array":
        """Zero-copy view of a contiguous CUDA tensor; dims are the tensor's
        shape reversed (NCHW -> (W,H,C,N))."""
        import torch

        if not t.is_cuda:
            raise ValueError("view_torch needs a CUDA tensor")
        t = t.contiguous()
        dt = {torch.float32: f32, torch.float64: f64, torch.float16: f16, torch.uint8: u8,
              torch.int8: s8, torch.int16: s16, torch.int32: s32, torch.int64: s64,
              torch.complex64: c32, torch.complex128: c64, torch.bool: b8}[t.dtype]
        dims = list(reversed(t.shape)) or [1]
        while len(dims) > 4:
            raise ValueError("at most 4 dims")
        return Array.view_device(t.data_ptr(), dims, dt, keep=t)

    # ---- inspection
    @property
    def dims(self) -> list[int]:
        d = [dim_t() for _ in range(4)]
        _check(lib().af_get_dims(*[ctypes.byref(x) for x in d], self.handle))
        return [x.value for x in d]

    @property
    def strides(self) -> list[int]:
        d = [dim_t() for _ in range(4)]
        _check(lib().af_get_strides(*[ctypes.byref(x) for x in d], self.handle))
        return [x.value for x in d]

    @property
    def dtype(self) -> int:
        t = ctypes.c_int()
        _check(lib().af_get_type(ctypes.byref(t), self.handle))
        return t.value

    @property
    def numdims(self) -> int:
        n = ctypes.c_uint()
        _check(lib().af_get_numdims(ctypes.byref(n), self.handle))
        return n.value

    def device_ptr(self) -> int:
        p = ctypes.c_void_p()
        _check(lib().af_get_device_ptr(ctypes.byref(p), self.handle))
        return p.value or 0

    def to_numpy(self) -> np.ndarray:
        dims = self.dims
        out = np.empty(dims, dtype=_NP[self.dtype], order="F")
        if out.size:
            _check(lib().af_get_data_ptr(out.ctypes.data_as(ctypes.c_void_p), self.handle))
        return out

    @property
    def __cuda_array_interface__(self):
        dims = self.dims
        strides = self.strides
        es = np.dtype(_NP[self.dtype]).itemsize
        return {
            "shape": tuple(reversed(dims)),
            "strides": tuple(s * es for s in reversed(strides)),
            "typestr": np.dtype(_NP[self.dtype]).str,
            "data": (self.device_ptr(), False),
            "version": 2,
        }

    def to_torch(self):
        """Zero-copy CUDA tensor of shape reversed(dims) over this array's
        memory (the tensor keeps the array alive).  Work on the library's
        stream is ordered with torch's when set_stream(torch stream) is used."""
        import torch

        return torch.as_tensor(self, device="cuda")


# ---------------------------------------------------------------------------
# module-level controls
# ---------------------------------------------------------------------------
def sync(device: int = -1) -> None:
    _check(lib().af_sync(device))


def set_stream(stream) -> None:
    """Run library work on `stream` (a torch.cuda.Stream, a raw cudaStream_t
    int where 0 means the legacy default stream, or None for the library's
    own stream)."""
    if stream is None:
        _check(lib().afgb_set_stream(None))
        return
    ptr = stream if isinstance(stream, int) else stream.cuda_stream
    # handle 0 is the legacy default stream (torch's default stream); pass it
    # as cudaStreamLegacy because a null handle selects the library's own
    # stream in afgb_set_stream
    _check(lib().afgb_set_stream(ctypes.c_void_p(ptr if ptr else 1)))


def set_exact_fp(exact: bool) -> None:
    _check(lib().afgb_set_exact_fp(1 if exact else 0))


def launch_count() -> int:
    return int(lib().afgb_kernel_launch_count())


def device_mem_info() -> dict:
    """af_device_mem_info: pool bytes reserved, bytes/buffers held by live arrays."""
    v = [ctypes.c_size_t() for _ in range(4)]
    _check(lib().af_device_mem_info(*[ctypes.byref(x) for x in v]))
    return {"alloc_bytes": v[0].value, "alloc_buffers": v[1].value,
            "lock_bytes": v[2].value, "lock_buffers": v[3].value}


def device_gc() -> None:
    _check(lib().af_device_gc())


def device_mem_peak(reset: bool = False) -> int:
    """Peak bytes held by this library's arrays and scratch since load or the last reset."""
    v = ctypes.c_size_t()
    _check(lib().afgb_device_mem_peak(ctypes.byref(v), 1 if reset else 0))
    return v.value


def device_mem_peak_breakdown() -> dict:
    """Bytes per allocation purpose at the peak of device_mem_peak."""
    buf = ctypes.create_string_buffer(4096)
    _check(lib().afgb_device_mem_peak_breakdown(buf, len(buf)))
    out = {}
    for ln in buf.value.decode().splitlines():
        k, _, v = ln.rpartition("=")
        out[k] = int(v)
    return out


def version() -> str:
    return lib().afgb_version().decode()


# ---------------------------------------------------------------------------
# the convolution path (af_* mirrors)
# ---------------------------------------------------------------------------
def _out_call(fn, *args) -> Array:
    out = af_array()
    _check(fn(ctypes.byref(out), *args))
    return Array(out.value)


def convolve1(signal: Array, filter: Array, mode=AF_CONV_DEFAULT, domain=AF_CONV_AUTO) -> Array:
    return _out_call(lib().af_convolve1, signal.handle, filter.handle, mode, domain)


def convolve2(signal: Array, filter: Array, mode=AF_CONV_DEFAULT, domain=AF_CONV_AUTO) -> Array:
    return _out_call(lib().af_convolve2, signal.handle, filter.handle, mode, domain)


def convolve3(signal: Array, filter: Array, mode=AF_CONV_DEFAULT, domain=AF_CONV_AUTO) -> Array:
    return _out_call(lib().af_convolve3, signal.handle, filter.handle, mode, domain)


def convolve2_separable(col_filter: Array, row_filter: Array, signal: Array,
                        mode=AF_CONV_DEFAULT) -> Array:
    return _out_call(lib().af_convolve2_sep, col_filter.handle, row_filter.handle, signal.handle,
                     mode)


def fft_convolve1(signal: Array, filter: Array, mode=AF_CONV_DEFAULT) -> Array:
    return _out_call(lib().af_fft_convolve1, signal.handle, filter.handle, mode)


def fft_convolve2(signal: Array, filter: Array, mode=AF_CONV_DEFAULT) -> Array:
    return _out_call(lib().af_fft_convolve2, signal.handle, filter.handle, mode)


def fft_convolve3(signal: Array, filter: Array, mode=AF_CONV_DEFAULT) -> Array:
    return _out_call(lib().af_fft_convolve3, signal.handle, filter.handle, mode)


def _dimargs(v: Sequence[int]):
    v = list(v)
    return len(v), dims_arg(v)


def convolve2_nn(signal: Array, filter: Array, stride=(1, 1), padding=(0, 0), dilation=(1, 1),
                 precision: str = "fp32", scales: Optional[Array] = None,
                 bias: Optional[Array] = None, relu: bool = False) -> Array:
    """af_convolve2_nn; `precision`/`scales` select afgb_convolve2_nn_ex, and
    `bias`/`relu` the fused epilogue of afgb_convolve2_nn_fused."""
    sn, sp = _dimargs(stride)
    pn, pp = _dimargs(padding)
    dn, dp = _dimargs(dilation)
    if bias is not None or relu:
        if scales is not None:
            raise ValueError("scales and a fused epilogue are separate entry points")
        return _out_call(lib().afgb_convolve2_nn_fused, signal.handle, filter.handle, sn, sp, pn,
                         pp, dn, dp, PRECISION[precision],
                         bias.handle if bias is not None else None, 1 if relu else 0)
    if precision == "fp32" and scales is None:
        return _out_call(lib().af_convolve2_nn, signal.handle, filter.handle, sn, sp, pn, pp, dn, dp)
    return _out_call(lib().afgb_convolve2_nn_ex, signal.handle, filter.handle, sn, sp, pn, pp, dn,
                     dp, PRECISION[precision], scales.handle if scales is not None else None)


def convolve2_gradient_nn(incoming_gradient: Array, original_signal: Array,
                          original_filter: Array, convolved_output: Array, stride=(1, 1),
                          padding=(0, 0), dilation=(1, 1), grad_type=AF_CONV_GRADIENT_FILTER,
                          precision: str = "fp32", real_bias: bool = False) -> Array:
    sn, sp = _dimargs(stride)
    pn, pp = _dimargs(padding)
    dn, dp = _dimargs(dilation)
    if precision == "fp32" and not real_bias:
        return _out_call(lib().af_convolve2_gradient_nn, incoming_gradient.handle,
                         original_signal.handle, original_filter.handle, convolved_output.handle,
                         sn, sp, pn, pp, dn, dp, grad_type)
    return _out_call(lib().afgb_convolve2_gradient_nn_ex, incoming_gradient.handle,
                     original_signal.handle, original_filter.handle, convolved_output.handle,
                     sn, sp, pn, pp, dn, dp, grad_type, PRECISION[precision])


def convolve2_gradients_nn(incoming_gradient: Array, original_signal: Array,
                           original_filter: Array, stride=(1, 1), padding=(0, 0),
                           dilation=(1, 1), precision: str = "fp32", data: bool = True,
                           filter: bool = True, bias: bool = False):
    """afgb_convolve2_gradients_nn: (data, filter, bias) gradients in one call,
    None for the ones not requested."""
    sn, sp = _dimargs(stride)
    pn, pp = _dimargs(padding)
    dn, dp = _dimargs(dilation)
    outs = [af_array() if want else None for want in (data, filter, bias)]
    _check(lib().afgb_convolve2_gradients_nn(
        *[ctypes.byref(o) if o is not None else None for o in outs], incoming_gradient.handle,
        original_signal.handle, original_filter.handle, sn, sp, pn, pp, dn, dp,
        PRECISION[precision]))
    return tuple(Array(o.value) if o is not None else None for o in outs)


def gaussian_kernel(rows: int, cols: int, sigma_r: float = 0.0, sigma_c: float = 0.0) -> Array:
    out = af_array()
    _check(lib().af_gaussian_kernel(ctypes.byref(out), rows, cols, sigma_r, sigma_c))
    return Array(out.value)


def dog(image: Array, radius1: int, radius2: int) -> Array:
    return _out_call(lib().af_dog, image.handle, radius1, radius2)


def sobel_operator(image: Array, ker_size: int = 3):
    dx, dy = af_array(), af_array()
    _check(lib().af_sobel_operator(ctypes.byref(dx), ctypes.byref(dy), image.handle, ker_size))
    return Array(dx.value), Array(dy.value)


class Features:
    """An af_features object (include/af/features.h): the count and five f32
    arrays, owned by the object; released with it."""

    def __init__(self, handle: int):
        self.handle = handle

    def __del__(self):
        h, self.handle = getattr(self, "handle", None), None
        if h:
            try:
                lib().af_release_features(h)
            except Exception:
                pass

    def num(self) -> int:
        n = ctypes.c_longlong()
        _check(lib().af_get_features_num(ctypes.byref(n), self.handle))
        return n.value

    def array(self, fn) -> Array:
        """One of the object's arrays, retained (an Array of its own)."""
        a, r = af_array(), af_array()
        _check(fn(ctypes.byref(a), self.handle))
        _check(lib().af_retain_array(ctypes.byref(r), a))
        return Array(r.value)

    def _get(self, fn) -> np.ndarray:
        return self.array(fn).to_numpy().ravel(order="F")

    def x(self) -> np.ndarray:
        return self._get(lib().af_get_features_xpos)

    def y(self) -> np.ndarray:
        return self._get(lib().af_get_features_ypos)

    def score(self) -> np.ndarray:
        return self._get(lib().af_get_features_score)

    def orientation(self) -> np.ndarray:
        return self._get(lib().af_get_features_orientation)

    def size(self) -> np.ndarray:
        return self._get(lib().af_get_features_size)


def harris(image: Array, max_corners: int = 500, min_response: float = 1e5, sigma: float = 1.0,
           block_size: int = 0, k_thr: float = 0.04) -> Features:
    """af_harris (include/af/vision.h:402; defaults of af::harris)."""
    out = ctypes.c_void_p()
    _check(lib().af_harris(ctypes.byref(out), image.handle, max_corners, min_response, sigma,
                           block_size, k_thr))
    return Features(out.value)


AF_CANNY_THRESHOLD_MANUAL, AF_CANNY_THRESHOLD_AUTO_OTSU = 0, 1


def canny(image: Array, threshold_type: int = AF_CANNY_THRESHOLD_MANUAL,
          low_threshold_ratio: float = 0.1, high_threshold_ratio: float = 0.2,
          sobel_window: int = 3, is_fast: bool = False) -> Array:
    """af_canny (include/af/image.h:1682; defaults of af::canny)."""
    return _out_call(lib().af_canny, image.handle, threshold_type, low_threshold_ratio,
                     high_threshold_ratio, sobel_window, is_fast)


def unwrap(signal: Array, wx: int, wy: int, sx: int, sy: int, px: int = 0, py: int = 0,
           is_column: bool = True) -> Array:
    """af_unwrap: wx x wy patches at strides (sx, sy), zero padding (px, py)."""
    return _out_call(lib().af_unwrap, signal.handle, wx, wy, sx, sy, px, py, bool(is_column))


def wrap(patches: Array, ox: int, oy: int, wx: int, wy: int, sx: int, sy: int, px: int = 0,
         py: int = 0, is_column: bool = True) -> Array:
    """af_wrap: accumulate patches into a new (ox, oy, d2, d3) image."""
    return _out_call(lib().af_wrap, patches.handle, ox, oy, wx, wy, sx, sy, px, py,
                     bool(is_column))


def wrap_v2(out: Optional[Array], patches: Array, ox: int, oy: int, wx: int, wy: int, sx: int,
            sy: int, px: int = 0, py: int = 0, is_column: bool = True) -> Array:
    """af_wrap_v2: as wrap, adding into `out` in place when it is given."""
    h = af_array(out.handle.value if out is not None else None)
    _check(lib().af_wrap_v2(ctypes.byref(h), patches.handle, ox, oy, wx, wy, sx, sy, px, py,
                            bool(is_column)))
    return out if out is not None else Array(h.value)


# host-only helpers (no GPU)
def identify_batch_kind(rank: int, sdims, fdims) -> int:
    return lib().afgb_identify_batch_kind(rank, dims_arg(list(sdims)), dims_arg(list(fdims)))


def conv_output_dims(rank, kind, expand, sdims, fdims) -> list[int]:
    out = (dim_t * 4)()
    lib().afgb_conv_output_dims(out, rank, kind, 1 if expand else 0, dims_arg(list(sdims)),
                                dims_arg(list(fdims)))
    return list(out)


def nn_output_dims(sdims, fdims, stride, padding, dilation) -> list[int]:
    out = (dim_t * 4)()
    lib().afgb_nn_output_dims(out, dims_arg(list(sdims)), dims_arg(list(fdims)),
                              dims_arg(list(stride)), dims_arg(list(padding)),
                              dims_arg(list(dilation)))
    return list(out)
