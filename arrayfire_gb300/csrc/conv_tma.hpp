// TMA-staged direct convolutions (conv_tma.cu).  Each returns false when
// the inputs do not qualify (layout, alignment, dtype, filter size); the
// caller then runs the general kernels.
#pragma once

#include "afgb_internal.hpp"
#include "conv_params.cuh"

namespace afgb {
namespace dtma {

bool tma_convolve2(const DirectParams &p, af_dtype t, bool exact);
// 3x3x3 f32 volumes (dense, 16-byte rows)
bool tma_convolve3(const DirectParams &p, bool exact);
bool tma_convolve2_sep(const Array &sig, const float *cf, const float *rf, int cl, int rl,
                       Array &out, bool expand, bool exact);

}  // namespace dtma

// error word of the TMA-staged kernels (a tile wait that timed out)
unsigned int tma_take_error();

}  // namespace afgb
