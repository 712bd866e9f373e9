/*
 * afgb300.h — C ABI of the GB300-native spatial-convolution backend.
 *
 * This library is a drop-in for ArrayFire v3.10's convolution entry points
 * on one GPU (sm_103a).  Every `af_*` symbol below has the same name,
 * signature, argument meaning and error codes as the ArrayFire declaration
 * cited beside it (paths are within the ArrayFire source tree).  The
 * `afgb_*` symbols are extensions with no ArrayFire counterpart; each says
 * what it adds.
 *
 * Data layout: arrays are column-major 4-D (d0 fastest), exactly as
 * ArrayFire's `af::dim4` + strides.  All compute runs on the library's
 * current CUDA stream (see afgb_set_stream); calls are asynchronous with
 * respect to the host, as in ArrayFire's CUDA backend, and af_get_data_ptr /
 * af_sync synchronise.
 */
#ifndef AFGB300_H
#define AFGB300_H

#include <stdbool.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(__GNUC__)
#define AFGB_API __attribute__((visibility("default")))
#else
#define AFGB_API
#endif

/* ---- types (include/af/defines.h) ------------------------------------ */

typedef long long dim_t;  /* include/af/defines.h:50 (64-bit dim_t) */
typedef void *af_array;   /* include/af/defines.h:243 */
typedef void *af_features; /* include/af/features.h:13 */

/* include/af/defines.h:75-202 — numeric values identical */
typedef enum {
    AF_SUCCESS = 0,
    AF_ERR_NO_MEM = 101,
    AF_ERR_DRIVER = 102,
    AF_ERR_RUNTIME = 103,
    AF_ERR_INVALID_ARRAY = 201,
    AF_ERR_ARG = 202,
    AF_ERR_SIZE = 203,
    AF_ERR_TYPE = 204,
    AF_ERR_DIFF_TYPE = 205,
    AF_ERR_BATCH = 207,
    AF_ERR_DEVICE = 208,
    AF_ERR_NOT_SUPPORTED = 301,
    AF_ERR_NOT_CONFIGURED = 302,
    AF_ERR_NONFREE = 303,
    AF_ERR_NO_DBL = 401,
    AF_ERR_NO_GFX = 402,
    AF_ERR_NO_HALF = 403,
    AF_ERR_LOAD_LIB = 501,
    AF_ERR_LOAD_SYM = 502,
    AF_ERR_ARR_BKND_MISMATCH = 503,
    AF_ERR_INTERNAL = 998,
    AF_ERR_UNKNOWN = 999
} af_err;

/* include/af/defines.h:211-233 — same order, same values */
typedef enum {
    f32 = 0, c32, f64, c64, b8, s32, u32, u8, s64, u64, s16, u16, f16, s8
} af_dtype;

/* include/af/defines.h:306-314 */
typedef enum { AF_CONV_DEFAULT = 0, AF_CONV_EXPAND = 1 } af_conv_mode;

/* include/af/defines.h:316-320 */
typedef enum { AF_CONV_AUTO = 0, AF_CONV_SPATIAL = 1, AF_CONV_FREQ = 2 } af_conv_domain;

/* include/af/defines.h:545-550 */
typedef enum {
    AF_CONV_GRADIENT_DEFAULT = 0,
    AF_CONV_GRADIENT_FILTER = 1,
    AF_CONV_GRADIENT_DATA = 2,
    AF_CONV_GRADIENT_BIAS = 3
} af_conv_gradient_type;

/* ---- array lifecycle (the subset the convolution path needs) -------- */

/* include/af/array.h:1657 — copies host data to a new device array */
AFGB_API af_err af_create_array(af_array *arr, const void *const data, const unsigned ndims,
                                const dim_t *const dims, const af_dtype type);
/* include/af/array.h:1672 — uninitialised device array */
AFGB_API af_err af_create_handle(af_array *arr, const unsigned ndims, const dim_t *const dims,
                                 const af_dtype type);
/* include/af/device.h:453 — adopts a cudaMalloc'd pointer; freed with the array */
AFGB_API af_err af_device_array(af_array *arr, void *data, const unsigned ndims,
                                const dim_t *const dims, const af_dtype type);
/* include/af/array.h:1689 — device-to-host copy; synchronises */
AFGB_API af_err af_get_data_ptr(void *data, const af_array arr);
/* include/af/device.h:576 */
AFGB_API af_err af_get_device_ptr(void **ptr, const af_array arr);
/* include/af/array.h:1696 */
AFGB_API af_err af_release_array(af_array arr);
/* include/af/array.h:1701 — new handle sharing the same buffer */
AFGB_API af_err af_retain_array(af_array *out, const af_array in);
/* include/af/array.h:1744 */
AFGB_API af_err af_get_elements(dim_t *elems, const af_array arr);
/* include/af/array.h:1754 */
AFGB_API af_err af_get_type(af_dtype *type, const af_array arr);
/* include/af/array.h:1767 */
AFGB_API af_err af_get_dims(dim_t *d0, dim_t *d1, dim_t *d2, dim_t *d3, const af_array arr);
/* include/af/array.h:1778 */
AFGB_API af_err af_get_numdims(unsigned *result, const af_array arr);
/* include/af/internal.h:134 */
AFGB_API af_err af_get_strides(dim_t *s0, dim_t *s1, dim_t *s2, dim_t *s3, const af_array arr);
/* include/af/device.h:354 — waits for all work queued by this library */
AFGB_API af_err af_sync(const int device);
/* include/af/device.h:446 — frees strings returned by af_get_last_error */
AFGB_API af_err af_free_host(void *ptr);
/* include/af/exception.h:65 — thread-local message of the last failure */
AFGB_API void af_get_last_error(char **msg, dim_t *len);
/* include/af/exception.h:70 */
AFGB_API const char *af_err_to_string(const af_err err);

/* ---- the convolution hot path --------------------------------------- */

/* include/af/signal.h:1391 (dispatcher src/api/c/convolve.cpp:217-226) */
AFGB_API af_err af_convolve1(af_array *out, const af_array signal, const af_array filter,
                             const af_conv_mode mode, af_conv_domain domain);
/* include/af/signal.h:1408 (src/api/c/convolve.cpp:228-241) */
AFGB_API af_err af_convolve2(af_array *out, const af_array signal, const af_array filter,
                             const af_conv_mode mode, af_conv_domain domain);
/* include/af/signal.h:1460 (src/api/c/convolve.cpp:243-256) */
AFGB_API af_err af_convolve3(af_array *out, const af_array signal, const af_array filter,
                             const af_conv_mode mode, af_conv_domain domain);
/* include/af/signal.h:1478 (src/api/c/convolve.cpp:258-334) */
AFGB_API af_err af_convolve2_sep(af_array *out, const af_array col_filter,
                                 const af_array row_filter, const af_array signal,
                                 const af_conv_mode mode);
/* include/af/signal.h:1440 (src/api/c/convolve.cpp:344-392) */
AFGB_API af_err af_convolve2_nn(af_array *out, const af_array signal, const af_array filter,
                                const unsigned stride_dims, const dim_t *strides,
                                const unsigned padding_dims, const dim_t *paddings,
                                const unsigned dilation_dims, const dim_t *dilations);
/* include/af/ml.h:84-92 (src/api/c/convolve.cpp:414-477).  As in the
 * reference, every grad_type other than AF_CONV_GRADIENT_FILTER returns the
 * data gradient; the real bias gradient is afgb_convolve2_gradient_nn_ex. */
AFGB_API af_err af_convolve2_gradient_nn(af_array *out, const af_array incoming_gradient,
                                         const af_array original_signal,
                                         const af_array original_filter,
                                         const af_array convolved_output,
                                         const unsigned stride_dims, const dim_t *strides,
                                         const unsigned padding_dims, const dim_t *paddings,
                                         const unsigned dilation_dims, const dim_t *dilations,
                                         af_conv_gradient_type grad_type);

/* ---- frequency-domain convolution ------------------------------------ */

/* include/af/signal.h:1492 (src/api/c/fftconvolve.cpp:239-242): FFT
 * convolution of rank 1; every batch kind including DIFF; integer types round
 * the result (DIFF truncates), as the reference's CPU backend. */
AFGB_API af_err af_fft_convolve1(af_array *out, const af_array signal, const af_array filter,
                                 const af_conv_mode mode);
/* include/af/signal.h:1506 (src/api/c/fftconvolve.cpp:244-254): rank 2, or 1
 * when both inputs have fewer than 2 dims.  af_convolve2 with AF_CONV_FREQ,
 * or AF_CONV_AUTO where the reference picks the frequency domain, calls this. */
AFGB_API af_err af_fft_convolve2(af_array *out, const af_array signal, const af_array filter,
                                 const af_conv_mode mode);
/* include/af/signal.h:1520 (src/api/c/fftconvolve.cpp:256-266): rank 3, or 2
 * when both inputs have fewer than 3 dims. */
AFGB_API af_err af_fft_convolve3(af_array *out, const af_array signal, const af_array filter,
                                 const af_conv_mode mode);

/* ---- image-processing callers of the convolution path ------------------ */

/* include/af/image.h:1404 (src/api/c/gaussian_kernel.cpp:29-99): rows x cols
 * f32 Gaussian, sigma <= 0 meaning a quarter of the size, normalised to unit
 * sum. */
AFGB_API af_err af_gaussian_kernel(af_array *out, const int rows, const int cols,
                                   const double sigma_r, const double sigma_c);
/* include/af/vision.h:635 (src/api/c/dog.cpp:30-85): difference of the input
 * convolved with the (2r1+1)^2 and (2r2+1)^2 Gaussians (DEFAULT mode); 2-D or
 * 3-D input (LHS batch), f32 result (f64 for f64). */
AFGB_API af_err af_dog(af_array *out, const af_array in, const int radius1, const int radius2);
/* include/af/image.h:1340 (src/api/c/sobel.cpp:38-87): 3x3 Sobel derivatives
 * with reflect-101 borders; ker_size must be 3. */
AFGB_API af_err af_sobel_operator(af_array *dx, af_array *dy, const af_array img,
                                  const unsigned ker_size);

/* ---- corner detection on the separable window (af_harris) and the
 * af_features object it returns ------------------------------------------ */

/* include/af/vision.h:402 (src/api/c/harris.cpp:42-95, CPU backend
 * src/backend/cpu/harris.cpp:28-144): Harris corners of a 2-D f32/f64 image.
 * Window length block_size, else floor(6 sigma) made odd: a box when
 * sigma < 0.5, else a Gaussian.  Responses det - k_thr tr^2, strict
 * 8-neighbour maxima of at least (unsigned)min_response (0 when
 * max_corners > 0) in column-major scan order, at most 20% of the pixels;
 * with max_corners > 0 the max_corners strongest (stable descending sort).
 * Feature x is the dim1 index, y the dim0 index; orientation 0, size 1.
 * Checks: 2-D input; d0 or d1 >= the window; max_corners > 0 or
 * min_response > 0; k_thr >= 0.01; block_size > 2 or sigma in [0.5, 5];
 * block_size <= 32. */
AFGB_API af_err af_harris(af_features *out, const af_array in, const unsigned max_corners,
                          const float min_response, const float sigma,
                          const unsigned block_size, const float k_thr);
/* include/af/features.h:92-154 (src/api/c/features.cpp:15-127): num > 0 gives
 * five uninitialised f32 arrays of num elements; the getters return the
 * object's own handles (not retained; released with the object). */
AFGB_API af_err af_create_features(af_features *feat, dim_t num);
AFGB_API af_err af_retain_features(af_features *out, const af_features feat);
AFGB_API af_err af_get_features_num(dim_t *num, const af_features feat);
AFGB_API af_err af_get_features_xpos(af_array *out, const af_features feat);
AFGB_API af_err af_get_features_ypos(af_array *out, const af_features feat);
AFGB_API af_err af_get_features_score(af_array *score, const af_features feat);
AFGB_API af_err af_get_features_orientation(af_array *orientation, const af_features feat);
AFGB_API af_err af_get_features_size(af_array *size, const af_features feat);
AFGB_API af_err af_release_features(af_features feat);

/* include/af/defines.h:486-489 */
typedef enum {
    AF_CANNY_THRESHOLD_MANUAL = 0,
    AF_CANNY_THRESHOLD_AUTO_OTSU = 1
} af_canny_threshold;

/* include/af/image.h:1682 (src/api/c/canny.cpp:232-285, CPU kernels
 * src/backend/cpu/kernel/canny.hpp): the b8 edge map (0/1) of each 2-D slice
 * (stacked along dim2): the image in float smoothed by the reference's 5-tap
 * separable filter, 3x3 Sobel derivatives, |gx| + |gy| (is_fast) or
 * sqrt(gx^2 + gy^2), non-maximum suppression, thresholds -- manual: ratios of
 * (s - min) / (max - min); AUTO_OTSU: the Otsu split T2 of a floor(max)-bin
 * histogram per slice and T1 = low_threshold_ratio * T2 -- and hysteresis.
 * Checks: at least 2-D, d0 and d1 >= 5, sobel_window == 3; f32, f64, s32,
 * u32, s16, u16, s8, u8.  AUTO_OTSU with a gradient maximum below 2 returns
 * AF_ERR_NOT_SUPPORTED (the reference's histogram then indexes outside its
 * arrays). */
AFGB_API af_err af_canny(af_array *out, const af_array in,
                         const af_canny_threshold threshold_type,
                         const float low_threshold_ratio, const float high_threshold_ratio,
                         const unsigned sobel_window, const bool is_fast);

/* ---- patch extraction and accumulation (the NN path's unwrap / wrap as
 * public calls; dilation 1) ----------------------------------------------- */

/* include/af/image.h:1483 (src/api/c/unwrap.cpp:37-103): patches of wx x wy
 * at strides (sx, sy) with zero padding (px, py); out dims (wx*wy, nx*ny, d2,
 * d3) with is_column, else (nx*ny, wx*wy, d2, d3); nx = (d0+2px-wx)/sx + 1. */
AFGB_API af_err af_unwrap(af_array *out, const af_array in, const dim_t wx, const dim_t wy,
                          const dim_t sx, const dim_t sy, const dim_t px, const dim_t py,
                          const bool is_column);
/* include/af/image.h:1524 (src/api/c/wrap.cpp:87-96): the inverse
 * accumulation into a new (ox, oy, d2, d3) array of zeros; overlapping patch
 * elements add in the element type. */
AFGB_API af_err af_wrap(af_array *out, const af_array in, const dim_t ox, const dim_t oy,
                        const dim_t wx, const dim_t wy, const dim_t sx, const dim_t sy,
                        const dim_t px, const dim_t py, const bool is_column);
/* include/af/image.h:1570 (src/api/c/wrap.cpp:98-109): as af_wrap, adding into
 * *out when it is not 0 (dense, same dims and type). */
AFGB_API af_err af_wrap_v2(af_array *out, const af_array in, const dim_t ox, const dim_t oy,
                           const dim_t wx, const dim_t wy, const dim_t sx, const dim_t sy,
                           const dim_t px, const dim_t py, const bool is_column);

/* ---- extensions (no ArrayFire counterpart) -------------------------- */

/* Arithmetic form of the NN convolution.  FP32 is the plain CUDA-core path
 * (the af_* entry points always use it).  BF16 and FP8_E4M3 run on the
 * tcgen05 tensor cores with FP32 accumulation; inputs and outputs stay f32
 * af_arrays, conversion happens on the device. */
typedef enum {
    AFGB_PRECISION_FP32 = 0,
    AFGB_PRECISION_BF16 = 1,
    AFGB_PRECISION_FP8_E4M3 = 2
} afgb_precision;

/* af_convolve2_nn with a precision knob.  For FP8_E4M3, `out_channel_scales`
 * (f32, K elements, may be 0) holds one dequantisation scale per output
 * channel: the filter of channel k is quantised as w/scale[k] and the
 * accumulator is multiplied back by scale[k].  When 0, the scales are derived
 * on the device as amax(|w[...,k]|)/448. */
AFGB_API af_err afgb_convolve2_nn_ex(af_array *out, const af_array signal, const af_array filter,
                                     const unsigned stride_dims, const dim_t *strides,
                                     const unsigned padding_dims, const dim_t *paddings,
                                     const unsigned dilation_dims, const dim_t *dilations,
                                     afgb_precision precision, const af_array out_channel_scales);

/* Extension: afgb_convolve2_nn_ex without scales, with a fused
 * epilogue: out = act(conv + bias[k]).  `bias` is 0 or an f32 array of K
 * elements; `activation` is 0 (none) or 1 (ReLU, max(v, 0) leaving NaN).  On
 * the tensor-core paths the bias and ReLU are applied in the kernel epilogue
 * before the output is stored; the FP32 path applies them in one extra pass.
 * f32 arrays only. */
AFGB_API af_err afgb_convolve2_nn_fused(af_array *out, const af_array signal,
                                       const af_array filter, const unsigned stride_dims,
                                       const dim_t *strides, const unsigned padding_dims,
                                       const dim_t *paddings, const unsigned dilation_dims,
                                       const dim_t *dilations, afgb_precision precision,
                                       const af_array bias, int activation);

/* af_convolve2_gradient_nn with a precision knob and a real bias gradient:
 * AF_CONV_GRADIENT_BIAS returns db[k] = sum_{x,y,n} g[x,y,k,n] as a
 * 1x1xKx1 array (FP32 compensated pairwise sum in a fixed order). */
AFGB_API af_err afgb_convolve2_gradient_nn_ex(
    af_array *out, const af_array incoming_gradient, const af_array original_signal,
    const af_array original_filter, const af_array convolved_output, const unsigned stride_dims,
    const dim_t *strides, const unsigned padding_dims, const dim_t *paddings,
    const unsigned dilation_dims, const dim_t *dilations, af_conv_gradient_type grad_type,
    afgb_precision precision);

/* The data, filter and bias gradients of one convolution in one call
 * (no counterpart in the reference, which computes one per
 * af_convolve2_gradient_nn call); any of the three outputs may be 0 to skip
 * it, and each result equals the afgb_convolve2_gradient_nn_ex call for its
 * type (BIAS as the real bias gradient).  The incoming gradient's dims must
 * be the forward output's (Wo, Ho, K, N).  In BF16 the data and filter
 * gradients share one bf16 copy of the incoming gradient. */
AFGB_API af_err afgb_convolve2_gradients_nn(af_array *data_grad, af_array *filter_grad,
                                           af_array *bias_grad, const af_array incoming_gradient,
                                           const af_array original_signal,
                                           const af_array original_filter,
                                           const unsigned stride_dims, const dim_t *strides,
                                           const unsigned padding_dims, const dim_t *paddings,
                                           const unsigned dilation_dims, const dim_t *dilations,
                                           afgb_precision precision);

/* Non-owning view of device memory with explicit strides (elements).  The
 * caller keeps ownership; releasing the view never frees `data`.  This is
 * how a framework tensor enters the library without a copy. */
AFGB_API af_err afgb_device_array_view(af_array *arr, void *data, const unsigned ndims,
                                       const dim_t *const dims, const dim_t *const strides,
                                       const af_dtype type);

/* Interop with another ArrayFire backend library in the same process
 * (libafcuda, or the unified libaf forwarding to it; its af_array handles are
 * opaque objects of that library, src/api/c/handle.hpp:50-83, passed through
 * unchanged by src/api/unified/symbol_manager.hpp:144-165).  `foreign_lib`
 * is that library's dlopen handle; its entry points are looked up with
 * dlsym (AF_ERR_LOAD_SYM when one is missing).
 *   afgb_import_foreign_array: a non-owning view of this library over the
 *     foreign array's device memory, without a copy.  Pointer, dims, strides
 *     and type come from the foreign af_get_device_ptr (src/api/c/
 *     memory.cpp:121: ArrayFire makes the array linear and locks its
 *     buffer), af_get_dims, af_get_strides and af_get_type; its af_sync, when
 *     exported, runs before the view is made.  Keep the foreign
 *     array alive while the view is used; release the view, then call the
 *     foreign af_unlock_array.
 *   afgb_export_foreign_array: a new af_array of the foreign library (its
 *     af_create_handle) holding a copy of `arr`, filled through its
 *     af_get_device_ptr and unlocked with its af_unlock_array when exported;
 *     the copy has completed when the call returns. */
AFGB_API af_err afgb_import_foreign_array(af_array *out, const af_array foreign,
                                          void *foreign_lib);
AFGB_API af_err afgb_export_foreign_array(af_array *foreign_out, const af_array arr,
                                          void *foreign_lib);

/* Route all subsequent work of the calling process to `stream`
 * (a cudaStream_t; 0 restores the library's own non-blocking stream). */
AFGB_API af_err afgb_set_stream(void *stream);
AFGB_API af_err afgb_get_stream(void **stream);

/* f32/f64/c32/c64 direct convolutions: 0 (default) lets the compiler fuse
 * multiply-add (results within a stated tolerance of the reference); 1
 * evaluates every product and sum separately in the reference's loop order,
 * which reproduces the reference CPU backend bit for bit.  Integer inputs
 * always use the exact order. */
AFGB_API af_err afgb_set_exact_fp(int exact);

/* Host-only helpers (no GPU needed): the reference's dispatch decisions,
 * exposed so they can be tested without a device.
 *   afgb_identify_batch_kind: src/api/c/convolve.cpp:77-97; returns
 *     0 NONE, 1 LHS, 2 RHS, 3 SAME, 4 DIFF, 5 UNSUPPORTED
 *     (src/backend/common/internal_enums.hpp:12-22 order).
 *   afgb_conv_output_dims: src/backend/cpu/convolve.cpp:38-58.
 *   afgb_nn_output_dims: src/backend/cpu/convolve.cpp:130-135. */
AFGB_API int afgb_identify_batch_kind(int rank, const dim_t *sdims, const dim_t *fdims);
AFGB_API int afgb_conv_output_dims(dim_t *odims, int rank, int kind, int expand,
                                   const dim_t *sdims, const dim_t *fdims);
AFGB_API int afgb_nn_output_dims(dim_t *odims, const dim_t *sdims, const dim_t *fdims,
                                 const dim_t *stride, const dim_t *padding,
                                 const dim_t *dilation);

/* Memory manager statistics of this library's device pool.
 *   af_device_mem_info: include/af/device.h:459 — alloc_bytes is the pool's
 *     reserved bytes, lock_bytes / lock_buffers the bytes and buffers held by
 *     live arrays and in-flight scratch (alloc_buffers = lock_buffers: a
 *     stream-ordered pool keeps no per-buffer free list).
 *   af_device_gc: include/af/device.h:492 — waits for the stream and returns
 *     unused pool memory to the device. */
AFGB_API af_err af_device_mem_info(size_t *alloc_bytes, size_t *alloc_buffers,
                                   size_t *lock_bytes, size_t *lock_buffers);
AFGB_API af_err af_device_gc(void);
/* Peak of lock_bytes since load or the last reset (reset != 0 restarts it at
 * the current value).  No counterpart in the reference. */
AFGB_API af_err afgb_device_mem_peak(size_t *peak_bytes, int reset);
/* What the bytes at that peak held, as "purpose=bytes" lines (arrays,
 * bf16 channels-last copies, weight operands, split-K partial sums, ...),
 * written to buf (len bytes, NUL-terminated, truncated if short). */
AFGB_API af_err afgb_device_mem_peak_breakdown(char *buf, size_t len);

/* Fault injection for tests: the n-th device allocation from now fails with
 * AF_ERR_NO_MEM (n <= 0 disables).  Host-side only. */
AFGB_API void afgb_debug_fail_alloc_after(int n);

/* Failure-path test hook: the bounded waits of the TMA and tensor-core
 * kernels give up after `polls` polls (0 restores the default, about
 * seconds), raising the device error word that af_sync / af_get_data_ptr
 * report as AF_ERR_RUNTIME and clear.  With skip_first_block_copies != 0,
 * block 0 of the TMA 2-D direct kernel issues no tile copies, so its waits
 * run out with nothing in flight and the kernel returns.  Call it while no
 * work of this library is in flight, on the current device. */
AFGB_API af_err afgb_debug_wait_limit(unsigned int polls, int skip_first_block_copies);

/* Number of kernels this library has launched since load (all devices). */
AFGB_API unsigned long long afgb_kernel_launch_count(void);

/* Filter gradient of the NN convolution (FP32) with no device allocation.
 * No counterpart in the reference.  It computes what af_convolve2_gradient_nn
 * returns for AF_CONV_GRADIENT_FILTER, for callers that cannot allocate GPU
 * memory — a host application whose device memory is wholly reserved by
 * another allocator, or a service with a fixed memory budget that forbids
 * allocation after start-up.  Inputs and the output are caller-owned device
 * buffers in ArrayFire layout: incoming_gradient (Wo,Ho,K,N), signal
 * (W,H,C,N) = signal_dims, filter_grad (fw,fh,C,K) = filter_dims; strides,
 * paddings and dilations hold two values each.  Work runs on `stream`
 * (0: the library's current stream, which the library creates on its first
 * use of the device — pass the caller's own stream to avoid that set-up).
 * Scratch: a fixed 8 MiB device array inside the library (2,097,152 floats;
 * fw*fh*C*K must not exceed that, else AF_ERR_SIZE).  CUDA loads a library's
 * kernel modules lazily by default (CUDA_MODULE_LOADING=LAZY since CUDA
 * 12.2), so the array, with the code of the module that holds it, is placed
 * in device memory by the FIRST call on each device, which also looks up the
 * array's device address; from then on it stays until the process exits.
 * Make that first call (a warm-up on small buffers will do) before the
 * caller's allocator reserves the device's memory and before any stream
 * capture, or run with CUDA_MODULE_LOADING=EAGER to place it when the
 * library is loaded.  Later calls allocate nothing.  All calls share the
 * array and leave their partial sums in it: calls that overlap on the GPU
 * (other streams, other host threads) race and give wrong results. */
AFGB_API af_err afgb_convolve2_filter_grad_noalloc(float *filter_grad, const float *incoming_gradient,
                                                   const float *signal, const dim_t *signal_dims,
                                                   const dim_t *filter_dims, const dim_t *strides,
                                                   const dim_t *paddings, const dim_t *dilations,
                                                   void *stream);

/* Device timing of the library's main kernels, for benchmarks: while
 * enabled, each main kernel launch is bracketed by CUDA events on its stream.
 * afgb_kernel_time sums the recorded launches whose kernel name equals
 * `name` (all launches when 0).  Disabling clears the record. */
AFGB_API void afgb_kernel_timing(int enable);
AFGB_API af_err afgb_kernel_time(const char *name, unsigned long long *count, double *total_ms);

/* Library version string. */
AFGB_API const char *afgb_version(void);

#ifdef __cplusplus
}
#endif
#endif /* AFGB300_H */
