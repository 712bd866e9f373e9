"""ctypes binding of libafgb300.so — the C ABI declared in include/afgb300.h.

The shared library is the product; this module only loads it and declares
argument types.  It never substitutes another implementation: if the library
is missing, loading fails with an error naming the build step.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / "libafgb300.so"

dim_t = ctypes.c_longlong
af_array = ctypes.c_void_p
af_err = ctypes.c_int
_P = ctypes.c_void_p
_DP = ctypes.POINTER(dim_t)

_lib: ctypes.CDLL | None = None

# (name, restype, argtypes) for every exported symbol of include/afgb300.h
SIGNATURES = [
    ("af_create_array", af_err, [ctypes.POINTER(af_array), _P, ctypes.c_uint, _DP, ctypes.c_int]),
    ("af_create_handle", af_err, [ctypes.POINTER(af_array), ctypes.c_uint, _DP, ctypes.c_int]),
    ("af_device_array", af_err, [ctypes.POINTER(af_array), _P, ctypes.c_uint, _DP, ctypes.c_int]),
    ("af_get_data_ptr", af_err, [_P, af_array]),
    ("af_get_device_ptr", af_err, [ctypes.POINTER(_P), af_array]),
    ("af_release_array", af_err, [af_array]),
    ("af_retain_array", af_err, [ctypes.POINTER(af_array), af_array]),
    ("af_get_elements", af_err, [_DP, af_array]),
    ("af_get_type", af_err, [ctypes.POINTER(ctypes.c_int), af_array]),
    ("af_get_dims", af_err, [_DP, _DP, _DP, _DP, af_array]),
    ("af_get_numdims", af_err, [ctypes.POINTER(ctypes.c_uint), af_array]),
    ("af_get_strides", af_err, [_DP, _DP, _DP, _DP, af_array]),
    ("af_sync", af_err, [ctypes.c_int]),
    ("af_free_host", af_err, [_P]),
    ("af_get_last_error", None, [ctypes.POINTER(ctypes.c_char_p), _DP]),
    ("af_err_to_string", ctypes.c_char_p, [ctypes.c_int]),
    ("af_convolve1", af_err, [ctypes.POINTER(af_array), af_array, af_array, ctypes.c_int, ctypes.c_int]),
    ("af_convolve2", af_err, [ctypes.POINTER(af_array), af_array, af_array, ctypes.c_int, ctypes.c_int]),
    ("af_convolve3", af_err, [ctypes.POINTER(af_array), af_array, af_array, ctypes.c_int, ctypes.c_int]),
    ("af_convolve2_sep", af_err, [ctypes.POINTER(af_array), af_array, af_array, af_array, ctypes.c_int]),
    ("af_convolve2_nn", af_err, [ctypes.POINTER(af_array), af_array, af_array, ctypes.c_uint, _DP,
                                 ctypes.c_uint, _DP, ctypes.c_uint, _DP]),
    ("af_convolve2_gradient_nn", af_err, [ctypes.POINTER(af_array), af_array, af_array, af_array,
                                          af_array, ctypes.c_uint, _DP, ctypes.c_uint, _DP,
                                          ctypes.c_uint, _DP, ctypes.c_int]),
    ("af_fft_convolve1", af_err, [ctypes.POINTER(af_array), af_array, af_array, ctypes.c_int]),
    ("af_fft_convolve2", af_err, [ctypes.POINTER(af_array), af_array, af_array, ctypes.c_int]),
    ("af_fft_convolve3", af_err, [ctypes.POINTER(af_array), af_array, af_array, ctypes.c_int]),
    ("af_gaussian_kernel", af_err, [ctypes.POINTER(af_array), ctypes.c_int, ctypes.c_int,
                                    ctypes.c_double, ctypes.c_double]),
    ("af_dog", af_err, [ctypes.POINTER(af_array), af_array, ctypes.c_int, ctypes.c_int]),
    ("af_sobel_operator", af_err, [ctypes.POINTER(af_array), ctypes.POINTER(af_array), af_array,
                                   ctypes.c_uint]),
    ("af_harris", af_err, [ctypes.POINTER(_P), af_array, ctypes.c_uint, ctypes.c_float,
                           ctypes.c_float, ctypes.c_uint, ctypes.c_float]),
    ("af_create_features", af_err, [ctypes.POINTER(_P), dim_t]),
    ("af_retain_features", af_err, [ctypes.POINTER(_P), _P]),
    ("af_get_features_num", af_err, [ctypes.POINTER(dim_t), _P]),
    ("af_get_features_xpos", af_err, [ctypes.POINTER(af_array), _P]),
    ("af_get_features_ypos", af_err, [ctypes.POINTER(af_array), _P]),
    ("af_get_features_score", af_err, [ctypes.POINTER(af_array), _P]),
    ("af_get_features_orientation", af_err, [ctypes.POINTER(af_array), _P]),
    ("af_get_features_size", af_err, [ctypes.POINTER(af_array), _P]),
    ("af_release_features", af_err, [_P]),
    ("af_canny", af_err, [ctypes.POINTER(af_array), af_array, ctypes.c_int, ctypes.c_float,
                          ctypes.c_float, ctypes.c_uint, ctypes.c_bool]),
    ("af_unwrap", af_err, [ctypes.POINTER(af_array), af_array] + [dim_t] * 6 + [ctypes.c_bool]),
    ("af_wrap", af_err, [ctypes.POINTER(af_array), af_array] + [dim_t] * 8 + [ctypes.c_bool]),
    ("af_wrap_v2", af_err, [ctypes.POINTER(af_array), af_array] + [dim_t] * 8 + [ctypes.c_bool]),
    ("afgb_convolve2_nn_ex", af_err, [ctypes.POINTER(af_array), af_array, af_array, ctypes.c_uint, _DP,
                                      ctypes.c_uint, _DP, ctypes.c_uint, _DP, ctypes.c_int, af_array]),
    ("afgb_convolve2_nn_fused", af_err, [ctypes.POINTER(af_array), af_array, af_array, ctypes.c_uint,
                                         _DP, ctypes.c_uint, _DP, ctypes.c_uint, _DP, ctypes.c_int,
                                         af_array, ctypes.c_int]),
    ("afgb_convolve2_gradient_nn_ex", af_err, [ctypes.POINTER(af_array), af_array, af_array, af_array,
                                               af_array, ctypes.c_uint, _DP, ctypes.c_uint, _DP,
                                               ctypes.c_uint, _DP, ctypes.c_int, ctypes.c_int]),
    ("afgb_convolve2_gradients_nn", af_err, [ctypes.POINTER(af_array), ctypes.POINTER(af_array),
                                             ctypes.POINTER(af_array), af_array, af_array, af_array,
                                             ctypes.c_uint, _DP, ctypes.c_uint, _DP, ctypes.c_uint,
                                             _DP, ctypes.c_int]),
    ("afgb_device_array_view", af_err, [ctypes.POINTER(af_array), _P, ctypes.c_uint, _DP, _DP, ctypes.c_int]),
    ("afgb_set_stream", af_err, [_P]),
    ("afgb_debug_wait_limit", af_err, [ctypes.c_uint, ctypes.c_int]),
    ("afgb_device_mem_peak_breakdown", af_err, [ctypes.c_char_p, ctypes.c_size_t]),
    ("afgb_import_foreign_array", af_err, [ctypes.POINTER(af_array), _P, _P]),
    ("afgb_export_foreign_array", af_err, [ctypes.POINTER(af_array), _P, _P]),
    ("afgb_get_stream", af_err, [ctypes.POINTER(_P)]),
    ("afgb_set_exact_fp", af_err, [ctypes.c_int]),
    ("afgb_identify_batch_kind", ctypes.c_int, [ctypes.c_int, _DP, _DP]),
    ("afgb_conv_output_dims", ctypes.c_int, [_DP, ctypes.c_int, ctypes.c_int, ctypes.c_int, _DP, _DP]),
    ("afgb_nn_output_dims", ctypes.c_int, [_DP, _DP, _DP, _DP, _DP, _DP]),
    ("af_device_mem_info", ctypes.c_int, [ctypes.POINTER(ctypes.c_size_t)] * 4),
    ("af_device_gc", ctypes.c_int, []),
    ("afgb_device_mem_peak", ctypes.c_int, [ctypes.POINTER(ctypes.c_size_t), ctypes.c_int]),
    ("afgb_debug_fail_alloc_after", None, [ctypes.c_int]),
    ("afgb_kernel_launch_count", ctypes.c_ulonglong, []),
    ("afgb_convolve2_filter_grad_noalloc", af_err, [_P, _P, _P, _DP, _DP, _DP, _DP, _DP, _P]),
    ("afgb_kernel_timing", None, [ctypes.c_int]),
    ("afgb_kernel_time", af_err, [ctypes.c_char_p, ctypes.POINTER(ctypes.c_ulonglong),
                                  ctypes.POINTER(ctypes.c_double)]),
    ("afgb_version", ctypes.c_char_p, []),
]


def load() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    path = Path(os.environ.get("AFGB300_LIB", LIB_PATH))
    if not path.exists():
        raise ImportError(
            f"{path} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'` "
            "or `python arrayfire_gb300/build.py` (needs nvcc)")
    lib = ctypes.CDLL(str(path))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def dims_arg(vals) -> ctypes.Array:
    vals = [int(v) for v in vals]
    return (dim_t * max(1, len(vals)))(*vals) if vals else (dim_t * 1)(0)
