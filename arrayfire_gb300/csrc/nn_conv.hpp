// Launch interface of the NN convolution (af_convolve2_nn and its
// gradients).  Layout is ArrayFire's: signal (W,H,C,N), filter (fw,fh,C,K),
// output (Wo,Ho,K,N), all column-major with dim 0 fastest.
#pragma once

#include "afgb_internal.hpp"

namespace afgb {

struct NNGeom {
    long long W, H, C, N;
    long long fw, fh, K;
    long long sx, sy, px, py, dx, dy;
    long long Wo, Ho;
};

// out[x,y,k,n] = sum_{c,u,v} in[x*sx-px+u*dx, y*sy-py+v*dy, c, n] *
//                w[fw-1-u, fh-1-v, c, k]   (src/backend/cpu/convolve.cpp:123-158)
// optional forward epilogue (afgb_convolve2_nn_fused): out = act(conv + bias[k])
struct NNEpilogue {
    const float *bias = nullptr;  // K floats on the device, or none
    int relu = 0;
};

void nn_forward(const NNGeom &g, const Array &sig, const Array &filt, Array &out,
                afgb_precision prec, const Array *scales, const NNEpilogue *ep = nullptr);
// dX = col2im(G * flip(W)^T)   (src/backend/cpu/convolve.cpp:179-211)
void nn_data_grad(const NNGeom &g, const Array &grad, const Array &filt, Array &dx,
                  afgb_precision prec);
// dW = flip(im2col(X)^T * G)   (src/backend/cpu/convolve.cpp:213-243)
void nn_filter_grad(const NNGeom &g, const Array &grad, const Array &sig, Array &dw,
                    afgb_precision prec);
// db[k] = sum_{x,y,n} g[x,y,k,n]  (no reference counterpart: the reference
// returns the data gradient for AF_CONV_GRADIENT_BIAS, src/api/c/convolve.cpp:401-411)
void nn_bias_grad(const NNGeom &g, const Array &grad, Array &db);
// any subset of the three gradients in one call (null outputs are skipped);
// the reduced precisions share one converted copy of the incoming gradient
void nn_gradients(const NNGeom &g, const Array &grad, const Array &sig, const Array &filt,
                  Array *dx, Array *dw, Array *db, afgb_precision prec);

// ---- plain CUDA-core implementations (nn_simt.cu)
void simt_forward(const NNGeom &g, const Array &sig, const Array &filt, Array &out);
void simt_data_grad(const NNGeom &g, const Array &grad, const Array &filt, Array &dx);
void simt_filter_grad(const NNGeom &g, const Array &grad, const Array &sig, Array &dw);

// ---- tensor-core implementations (nn_tc.cu); return false when the shape
// is outside what the tcgen05 kernels cover (the caller then reports
// AF_ERR_NOT_SUPPORTED; there is no silent fallback to another precision)
bool tc_forward(const NNGeom &g, const Array &sig, const Array &filt, Array &out,
                afgb_precision prec, const Array *scales, const NNEpilogue *ep = nullptr);
bool tc_data_grad(const NNGeom &g, const Array &grad, const Array &filt, Array &dx);
bool tc_filter_grad(const NNGeom &g, const Array &grad, const Array &sig, Array &dw);
bool tc_data_filter_grads(const NNGeom &g, const Array &grad, const Array &sig, const Array &filt,
                          Array &dx, Array &dw);

// fixed-order compensated sum of `splits` fp32 partials R[c + C*tap][k],
// written flipped into the (fw,fh,C,K) f32 filter gradient
void reduce_filter_partials(const NNGeom &g, const float *partials, int splits, float *dw);

// deterministic compensated reduction of `splits` fp32 partial matrices of
// `rows x cols` into `out` (pairwise tree over splits with TwoSum carries)
void reduce_partials(const float *partials, int splits, long long rows, long long cols,
                     float *out);

}  // namespace afgb
