// Launch interface of the direct (small-filter) convolution kernels.
#pragma once

#include "afgb_internal.hpp"

namespace afgb {

// One direct convolution of rank 1..3 over every batch slice, in one launch.
// `filt` has already been cast to the accumulator type of `sig`.
// Semantics: src/backend/cpu/kernel/convolve.hpp:19-211 (convolve_nd).
void launch_convolve_nd(const Array &sig, const Array &filt, Array &out, int kind, int rank,
                        bool expand);

// Separable 2-D convolution (column filter along dim0, then row filter along
// dim1) over every d2*d3 slice.  Filters are contiguous accumulator-typed
// vectors.  Semantics: src/backend/cpu/kernel/convolve.hpp:213-289.
void launch_convolve2_sep(const Array &sig, const Array &cfilt, const Array &rfilt, Array &out,
                          bool expand);

// Element-wise dtype conversion into a new dense array (castArray,
// src/api/c/handle.hpp:46; complex -> real takes the magnitude as in
// src/backend/cpu/cast.hpp:75-121).
Array cast_array(const Array &in, af_dtype to);

// Dense copy of a strided array (same dtype).
Array make_dense(const Array &in);

// af_unwrap / af_wrap kernels (unwrap_wrap.cu): `in` dense; wrap adds into
// `out` (any strides), or overwrites it with the sum alone when zero_init
void patches_unwrap(const Array &in, Array &out, long long wx, long long wy, long long sx,
                    long long sy, long long px, long long py, bool is_column);
void patches_wrap(const Array &in, Array &out, long long wx, long long wy, long long sx,
                  long long sy, long long px, long long py, bool is_column, bool zero_init);

// Frequency-domain convolution (fft_conv.cu) of rank 1..3 with the batch kind
// of the rank (not UNSUPPORTED); the reference's af_fft_convolve semantics.
Array fft_convolve(const Array &sig, const Array &filt, bool expand, int rank, int kind);

// Image-processing callers (image_ops.cu): the (rows x cols) f32 Gaussian of
// af_gaussian_kernel; af_dog's difference of Gaussian-blurred images; the 3x3
// Sobel derivatives of af_sobel_operator into dense dx, dy of the output type.
Array gaussian_kernel(int rows, int cols, double sigma_r, double sigma_c);
Array dog(const Array &in, int radius1, int radius2);
void sobel_3x3(const Array &img, Array &dx, Array &dy);

// af_harris (harris.cu): the corners of a 2-D f32/f64 image as dense f32
// vectors of n elements -- x along dim1, y along dim0, score, orientation 0,
// size 1 -- in the reference's order (src/backend/cpu/harris.cpp:28-144)
struct HarrisOut {
    long long n = 0;
    Array x, y, score, orientation, size;
};
void harris_corners(const Array &img, unsigned max_corners, float min_response, float sigma,
                    unsigned filter_len, float k_thr, HarrisOut &out);

// af_canny (canny.cu): the 0/1 (b8) edge map of each 2-D slice, threshold
// ratios manual or Otsu, L1 or L2 gradient magnitude (src/api/c/canny.cpp)
Array canny_edges(const Array &img, bool otsu, float t1, float t2, bool is_fast);

// out = T( s * (c * r) ) element-wise: the scalar-filter shortcut of
// af_convolve2_sep (src/api/c/convolve.cpp:57-68).
void launch_sep_scalar(const Array &sig, const Array &cfilt, const Array &rfilt, Array &out);

}  // namespace afgb
