// The six convolution entry points of the ArrayFire C API, with the
// reference's argument checks, batch-kind inference, domain choice and dtype
// dispatch (src/api/c/convolve.cpp), routed to this library's sm_103a
// kernels.  No CPU fallback: every path below launches device code.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstring>
#include <string>

#include "afgb_internal.hpp"
#include "conv_direct.hpp"
#include "nn_conv.hpp"

namespace afgb {

// src/api/c/convolve.cpp:77-97
static int identify_batch_kind(int rank, const dim_t *sd, const dim_t *fd) {
    dim_t sn = dim4_ndims(sd);
    dim_t fn = dim4_ndims(fd);
    if (sn == rank && fn == rank) return BATCH_NONE;
    if (sn == rank && (fn > rank && fn <= 4)) return BATCH_RHS;
    if ((sn > rank && sn <= 4) && fn == rank) return BATCH_LHS;
    if ((sn > rank && sn <= 4) && (fn > rank && fn <= 4)) {
        bool match = true, interleaved = true;
        for (int i = rank; i < 4; ++i) {
            match &= (sd[i] == fd[i]);
            interleaved &= (sd[i] == 1 || fd[i] == 1 || sd[i] == fd[i]);
        }
        if (match) return BATCH_SAME;
        return interleaved ? BATCH_DIFF : BATCH_UNSUPPORTED;
    }
    return BATCH_UNSUPPORTED;
}

// src/api/c/convolve.cpp:99-130 — true when the reference would take the
// frequency-domain route
static bool reference_picks_freq(int rank, const dim_t *sd, const dim_t *fd,
                                 af_conv_domain domain) {
    if (domain == AF_CONV_FREQ) return true;
    if (domain != AF_CONV_AUTO) return false;
    if (identify_batch_kind(rank, sd, fd) == BATCH_DIFF) return true;
    dim_t kbatch = 1;
    for (int i = 3; i >= rank; --i) kbatch *= fd[i];
    if (kbatch >= 10) return true;
    if (rank == 1 && fd[0] > 128) return true;
    if (rank == 2) {
        if (fd[0] > 17 || fd[1] > 17) return true;
        if (fd[0] != fd[1] && fd[0] > 5) return true;
    }
    if (rank == 3 && (fd[0] > 5 || fd[1] > 5 || fd[2] > 5)) return true;
    return false;
}

// filter sizes the spatial kernels accept: the same limits as the
// reference CUDA backend (src/backend/cuda/kernel/convolve.hpp:149-157,
// 242-266, 292-307), reported with the same error code
static bool spatial_supported(int rank, const dim_t *fd) {
    switch (rank) {
        case 1: return fd[0] <= 129;
        case 2: {
            if (fd[0] * fd[1] > 17 * 17) return false;
            bool small = fd[0] <= 5 && fd[1] <= 5;
            bool square = fd[0] == fd[1] && fd[0] > 5 && fd[0] < 18;
            return small || square;
        }
        case 3: return fd[0] * fd[1] * fd[2] <= 125;
    }
    return false;
}

static af_dtype acc_type(af_dtype t) {
    switch (t) {
        case f32: return f32;
        case f64: return f64;
        case c32: return c32;
        case c64: return c64;
        default: return f32;
    }
}

// src/backend/cpu/convolve.cpp:38-58 (same rule in src/backend/cuda/convolve.cpp:28-50)
static void conv_out_dims(dim_t *od, int rank, int kind, bool expand, const dim_t *sd,
                          const dim_t *fd) {
    if (expand) {
        for (int d = 0; d < 4; ++d) {
            if (kind == BATCH_NONE || kind == BATCH_RHS) od[d] = sd[d] + fd[d] - 1;
            else od[d] = (d < rank) ? sd[d] + fd[d] - 1 : sd[d];
        }
    } else {
        for (int d = 0; d < 4; ++d) od[d] = sd[d];
        if (kind == BATCH_RHS)
            for (int i = rank; i < 4; ++i) od[i] = fd[i];
    }
}

// convolve() of src/api/c/convolve.cpp:132-215
static af_err convolve_rank(af_array *out, const af_array signal, const af_array filter,
                            af_conv_mode mode, int rank) {
    Array *s = get_array(signal);
    Array *f = get_array(filter);
    if (dim4_ndims(f->dims) == 0 || dim4_ndims(s->dims) == 0) {
        return af_retain_array(out, signal);
    }
    int kind = identify_batch_kind(rank, s->dims, f->dims);
    AFGB_ARG_ASSERT(1, (kind != BATCH_UNSUPPORTED && kind != BATCH_DIFF));
    const bool expand = mode == AF_CONV_EXPAND;
    af_dtype st = s->type;
    if (st == f16 || !dtype_valid(st)) AFGB_TYPE_ERROR(1, st);
    if (!spatial_supported(rank, f->dims)) {
        AFGB_THROW(AF_ERR_NOT_SUPPORTED,
                   "CUDA N Dimensional Convolution doesn't support " + std::to_string(f->dims[0]) +
                       "x" + std::to_string(f->dims[1]) + "x" + std::to_string(f->dims[2]) +
                       " kernel");
    }
    Array filt = cast_array(*f, acc_type(st));
    dim_t od[4];
    conv_out_dims(od, rank, kind, expand, s->dims, f->dims);
    Array o = *create_array(st, od);
    launch_convolve_nd(*s, filt, o, kind, rank, expand);
    *out = make_handle(&o);
    return AF_SUCCESS;
}

// fft_convolve of src/api/c/fftconvolve.cpp:154-237: batch kind of the rank,
// then the signal's type (f16 is not accepted)
static af_err fft_convolve_impl(af_array *out, const af_array signal, const af_array filter,
                                bool expand, int rank) {
    Array *s = get_array(signal);
    Array *f = get_array(filter);
    const int kind = identify_batch_kind(rank, s->dims, f->dims);
    AFGB_ARG_ASSERT(1, (kind != BATCH_UNSUPPORTED));
    const af_dtype st = s->type;
    if (st == f16 || !dtype_valid(st)) AFGB_TYPE_ERROR(1, st);
    if (f->type == f16 || !dtype_valid(f->type)) AFGB_TYPE_ERROR(2, f->type);
    Array o = fft_convolve(*s, *f, expand, rank, kind);
    *out = make_handle(&o);
    return AF_SUCCESS;
}

static af_err convolve_domain(af_array *out, const af_array signal, const af_array filter,
                              af_conv_mode mode, af_conv_domain domain, int rank) {
    Array *s = get_array(signal);
    Array *f = get_array(filter);
    if (reference_picks_freq(rank, s->dims, f->dims, domain)) {
        switch (rank) {  // src/api/c/convolve.cpp:220-252
            case 1: return af_fft_convolve1(out, signal, filter, mode);
            case 2: return af_fft_convolve2(out, signal, filter, mode);
            default: return af_fft_convolve3(out, signal, filter, mode);
        }
    }
    return convolve_rank(out, signal, filter, mode, rank);
}

// src/api/c/convolve.cpp:50-75 and :258-334
static af_err convolve2_sep_impl(af_array *out, const af_array col_filter,
                                 const af_array row_filter, const af_array signal,
                                 af_conv_mode mode) {
    Array *s = get_array(signal);
    Array *cf = get_array(col_filter);
    Array *rf = get_array(row_filter);
    AFGB_ARG_ASSERT(1, (dim4_ndims(s->dims) >= 2));
    const bool expand = mode == AF_CONV_EXPAND;
    af_dtype st = s->type;
    if (st == f16 || !dtype_valid(st)) AFGB_TYPE_ERROR(1, st);
    af_dtype at = acc_type(st);
    Array c = cast_array(*cf, at);
    Array r = cast_array(*rf, at);
    auto is_vector = [](const Array &a) {
        int singular = 0, non_singular = 0;
        for (int i = 0; i < 4; ++i) {
            non_singular += (a.dims[i] != 0 && a.dims[i] != 1);
            singular += (a.dims[i] == 1);
        }
        return singular == 3 && non_singular == 1;
    };
    if (c.elements() == 1 && r.elements() == 1) {
        Array o = *create_array(st, s->dims);
        launch_sep_scalar(*s, c, r, o);
        *out = make_handle(&o);
        return AF_SUCCESS;
    }
    AFGB_ARG_ASSERT(2, is_vector(c));
    AFGB_ARG_ASSERT(3, is_vector(r));
    if (c.elements() > 31 || r.elements() > 31) {
        AFGB_THROW(AF_ERR_NOT_SUPPORTED, "CUDA convolution supports max kernel size of 31");
    }
    dim_t od[4] = {s->dims[0], s->dims[1], s->dims[2], s->dims[3]};
    if (expand) {
        od[0] += c.elements() - 1;
        od[1] += r.elements() - 1;
    }
    Array o = *create_array(st, od);
    launch_convolve2_sep(*s, c, r, o, expand);
    *out = make_handle(&o);
    return AF_SUCCESS;
}

// ---- NN: shared argument handling (src/api/c/convolve.cpp:344-392, 414-477)
struct NNArgs {
    dim_t stride[4], padding[4], dilation[4];
};

static NNArgs nn_args(unsigned stride_dims, const dim_t *strides, unsigned padding_dims,
                      const dim_t *paddings, unsigned dilation_dims, const dim_t *dilations) {
    NNArgs a;
    if (stride_dims && !strides) AFGB_THROW(AF_ERR_ARG, "null strides");
    if (padding_dims && !paddings) AFGB_THROW(AF_ERR_ARG, "null paddings");
    if (dilation_dims && !dilations) AFGB_THROW(AF_ERR_ARG, "null dilations");
    dim4_from(a.stride, stride_dims, strides);
    dim4_from(a.padding, padding_dims, paddings);
    dim4_from(a.dilation, dilation_dims, dilations);
    dim_t sn = dim4_ndims(a.stride), pn = dim4_ndims(a.padding), dn = dim4_ndims(a.dilation);
    AFGB_ARG_ASSERT(3, sn > 0 && sn <= 2);
    AFGB_ARG_ASSERT(5, pn >= 0 && pn <= 2);
    AFGB_ARG_ASSERT(7, dn > 0 && dn <= 2);
    return a;
}

// the reference's getArray<T> type check (src/api/c/handle.hpp:50-57)
static void require_type(const Array *a, af_dtype t) {
    if (a->type != t) AFGB_THROW(AF_ERR_INTERNAL, "Invalid type for input array.");
}

static void nn_geometry(NNGeom &g, const Array *s, const Array *f, const NNArgs &a) {
    std::memset(&g, 0, sizeof(g));
    g.W = s->dims[0];
    g.H = s->dims[1];
    g.C = s->dims[2];
    g.N = s->dims[3];
    g.fw = f->dims[0];
    g.fh = f->dims[1];
    g.K = f->dims[3];
    g.sx = a.stride[0];
    g.sy = a.stride[1];
    g.px = a.padding[0];
    g.py = a.padding[1];
    g.dx = a.dilation[0];
    g.dy = a.dilation[1];
    // src/backend/cpu/convolve.cpp:130-135 (C++ truncating division)
    g.Wo = 1 + (g.W + 2 * g.px - (((g.fw - 1) * g.dx) + 1)) / g.sx;
    g.Ho = 1 + (g.H + 2 * g.py - (((g.fh - 1) * g.dy) + 1)) / g.sy;
    if (g.Wo < 0) g.Wo = 0;
    if (g.Ho < 0) g.Ho = 0;
}

static af_err convolve2_nn_impl(af_array *out, const af_array signal, const af_array filter,
                                unsigned stride_dims, const dim_t *strides, unsigned padding_dims,
                                const dim_t *paddings, unsigned dilation_dims,
                                const dim_t *dilations, afgb_precision prec,
                                const af_array scales, const af_array bias = nullptr,
                                int activation = 0) {
    Array *s = get_array(signal);
    Array *f = get_array(filter);
    NNArgs a = nn_args(stride_dims, strides, padding_dims, paddings, dilation_dims, dilations);
    AFGB_DIM_ASSERT(1, s->dims[2] == f->dims[2]);
    af_dtype t = s->type;
    if (t != f32 && t != f64 && t != f16) AFGB_TYPE_ERROR(1, t);
    require_type(f, t);
    if (prec != AFGB_PRECISION_FP32 && t != f32) {
        AFGB_THROW(AF_ERR_TYPE, "tensor-core precisions take f32 arrays");
    }
    NNGeom g;
    nn_geometry(g, s, f, a);
    dim_t od[4] = {g.Wo, g.Ho, g.K, g.N};
    Array o = *create_array(t, od);
    Array sd = s->is_linear() ? *s : make_dense(*s);
    Array fd = f->is_linear() ? *f : make_dense(*f);
    const Array *sc = nullptr;
    Array scd;
    if (scales) {
        Array *sa = get_array(scales);
        require_type(sa, f32);
        AFGB_DIM_ASSERT(10, sa->elements() == g.K);
        scd = sa->is_linear() ? *sa : make_dense(*sa);
        sc = &scd;
    }
    NNEpilogue ep;
    Array bd;
    if (bias) {
        Array *ba = get_array(bias);
        require_type(ba, f32);
        AFGB_DIM_ASSERT(10, ba->elements() == g.K);
        if (t != f32) AFGB_TYPE_ERROR(1, t);
        bd = ba->is_linear() ? *ba : make_dense(*ba);
        ep.bias = bd.ptr<float>();
    }
    ep.relu = activation;
    if (activation && t != f32) AFGB_TYPE_ERROR(1, t);
    nn_forward(g, sd, fd, o, prec, sc, (bias || activation) ? &ep : nullptr);
    *out = make_handle(&o);
    return AF_SUCCESS;
}

static af_err convolve2_grad_impl(af_array *out, const af_array incoming_gradient,
                                  const af_array original_signal, const af_array original_filter,
                                  const af_array convolved_output, unsigned stride_dims,
                                  const dim_t *strides, unsigned padding_dims,
                                  const dim_t *paddings, unsigned dilation_dims,
                                  const dim_t *dilations, af_conv_gradient_type grad_type,
                                  afgb_precision prec, bool real_bias) {
    Array *gi = get_array(incoming_gradient);
    Array *s = get_array(original_signal);
    Array *f = get_array(original_filter);
    Array *o = get_array(convolved_output);
    bool same = true;
    for (int i = 0; i < 4; ++i) same &= gi->dims[i] == o->dims[i];
    AFGB_DIM_ASSERT(1, same);
    AFGB_DIM_ASSERT(3, o->dims[2] == f->dims[3]);
    AFGB_DIM_ASSERT(3, o->dims[3] == s->dims[3]);
    AFGB_DIM_ASSERT(2, s->dims[2] == f->dims[2]);
    NNArgs a = nn_args(stride_dims, strides, padding_dims, paddings, dilation_dims, dilations);
    af_dtype t = o->type;
    if (t != f32 && t != f64 && t != f16) AFGB_TYPE_ERROR(1, t);
    require_type(gi, t);
    require_type(s, t);
    require_type(f, t);
    if (prec != AFGB_PRECISION_FP32 && t != f32) {
        AFGB_THROW(AF_ERR_TYPE, "tensor-core precisions take f32 arrays");
    }
    NNGeom g;
    nn_geometry(g, s, f, a);
    // the reference does not compare the gradient's spatial size with the
    // forward geometry; a mismatch would index out of bounds here
    AFGB_DIM_ASSERT(1, gi->dims[0] == g.Wo && gi->dims[1] == g.Ho);
    Array gd = gi->is_linear() ? *gi : make_dense(*gi);
    Array sd = s->is_linear() ? *s : make_dense(*s);
    Array fd = f->is_linear() ? *f : make_dense(*f);
    if (grad_type == AF_CONV_GRADIENT_FILTER) {
        Array r = *create_array(t, f->dims);
        nn_filter_grad(g, gd, sd, r, prec);
        *out = make_handle(&r);
    } else if (grad_type == AF_CONV_GRADIENT_BIAS && real_bias) {
        dim_t bd[4] = {1, 1, g.K, 1};
        Array r = *create_array(t, bd);
        nn_bias_grad(g, gd, r);
        *out = make_handle(&r);
    } else {
        Array r = *create_array(t, s->dims);
        nn_data_grad(g, gd, fd, r, prec);
        *out = make_handle(&r);
    }
    return AF_SUCCESS;
}

static af_err convolve2_grads_impl(af_array *data_grad, af_array *filter_grad, af_array *bias_grad,
                                   const af_array incoming_gradient, const af_array original_signal,
                                   const af_array original_filter, unsigned stride_dims,
                                   const dim_t *strides, unsigned padding_dims,
                                   const dim_t *paddings, unsigned dilation_dims,
                                   const dim_t *dilations, afgb_precision prec) {
    Array *gi = get_array(incoming_gradient);
    Array *s = get_array(original_signal);
    Array *f = get_array(original_filter);
    AFGB_DIM_ASSERT(2, s->dims[2] == f->dims[2]);
    NNArgs a = nn_args(stride_dims, strides, padding_dims, paddings, dilation_dims, dilations);
    af_dtype t = s->type;
    if (t != f32 && t != f64 && t != f16) AFGB_TYPE_ERROR(1, t);
    require_type(gi, t);
    require_type(f, t);
    if (prec != AFGB_PRECISION_FP32 && t != f32) {
        AFGB_THROW(AF_ERR_TYPE, "tensor-core precisions take f32 arrays");
    }
    NNGeom g;
    nn_geometry(g, s, f, a);
    AFGB_DIM_ASSERT(1, gi->dims[0] == g.Wo && gi->dims[1] == g.Ho && gi->dims[2] == g.K &&
                           gi->dims[3] == g.N);
    Array gd = gi->is_linear() ? *gi : make_dense(*gi);
    Array sd = s->is_linear() ? *s : make_dense(*s);
    Array fd = f->is_linear() ? *f : make_dense(*f);
    Array dx, dw, db;
    if (data_grad) dx = *create_array(t, s->dims);
    if (filter_grad) dw = *create_array(t, f->dims);
    if (bias_grad) {
        dim_t bd[4] = {1, 1, g.K, 1};
        db = *create_array(t, bd);
    }
    nn_gradients(g, gd, sd, fd, data_grad ? &dx : nullptr, filter_grad ? &dw : nullptr,
                 bias_grad ? &db : nullptr, prec);
    if (data_grad) *data_grad = make_handle(&dx);
    if (filter_grad) *filter_grad = make_handle(&dw);
    if (bias_grad) *bias_grad = make_handle(&db);
    return AF_SUCCESS;
}

static bool patch_type(af_dtype t) { return t != f16 && dtype_valid(t); }

// af_wrap_common (src/api/c/wrap.cpp:33-85): argument checks in the
// reference's order, then out = (allocate ? zeros : *out) + wrap(in); a new
// output is written once by the kernel, without a zero fill first
static void wrap_impl(af_array *out, const af_array in, dim_t ox, dim_t oy, dim_t wx, dim_t wy,
                      dim_t sx, dim_t sy, dim_t px, dim_t py, bool is_column, bool allocate) {
    AFGB_ARG_ASSERT(0, out != nullptr);
    AFGB_ARG_ASSERT(1, in != nullptr);
    Array *a = get_array(in);
    const dim_t od[4] = {ox, oy, a->dims[2], a->dims[3]};
    AFGB_ARG_ASSERT(4, wx > 0);
    AFGB_ARG_ASSERT(5, wy > 0);
    AFGB_ARG_ASSERT(6, sx > 0);
    AFGB_ARG_ASSERT(7, sy > 0);
    const dim_t nx = (ox + 2 * px - wx) / sx + 1;
    const dim_t ny = (oy + 2 * py - wy) / sy + 1;
    const dim_t patch_size = is_column ? a->dims[0] : a->dims[1];
    const dim_t num_patches = is_column ? a->dims[1] : a->dims[0];
    AFGB_DIM_ASSERT(1, patch_size == wx * wy);
    AFGB_DIM_ASSERT(1, num_patches == nx * ny);
    // both counts negative (a window wider than the padded image by a stride or
    // more) multiply to a positive count; the reference then walks windows at
    // negative indices.  Rejected here as a size error.
    AFGB_DIM_ASSERT(1, nx >= 0 && ny >= 0);
    Array dst;
    if (allocate) {
        if (!patch_type(a->type)) AFGB_TYPE_ERROR(1, a->type);
        for (int i = 0; i < 4; ++i) AFGB_DIM_ASSERT(0, od[i] >= 0);
        dst = *create_array(a->type, od);  // every pixel is written by the kernel
    } else {
        dst = *get_array(*out);
        bool same = true;
        for (int i = 0; i < 4; ++i) same &= dst.dims[i] == od[i];
        AFGB_DIM_ASSERT(0, same);
        if (!patch_type(a->type)) AFGB_TYPE_ERROR(1, a->type);
        require_type(&dst, a->type);
    }
    Array src = a->is_linear() ? *a : make_dense(*a);
    patches_wrap(src, dst, wx, wy, sx, sy, px, py, is_column, allocate);
    if (allocate) *out = make_handle(&dst);
    else mark_written(dst);  // written in place
}

}  // namespace afgb

namespace afgb {
namespace {
struct FeaturesObj {
    dim_t n = 0;
    af_array x = nullptr, y = nullptr, score = nullptr, orientation = nullptr, size = nullptr;
    std::array<af_array *, 5> slots() { return {&x, &y, &score, &orientation, &size}; }
};

FeaturesObj *get_features(af_features f) {
    if (f == nullptr) AFGB_THROW(AF_ERR_ARG, "null af_features handle");
    return static_cast<FeaturesObj *>(f);
}

void release_features_arrays(FeaturesObj *f) {
    for (af_array *slot : f->slots()) {
        if (*slot) af_release_array(*slot);
        *slot = nullptr;
    }
}
}  // namespace
}  // namespace afgb

using namespace afgb;

extern "C" {

af_err af_convolve1(af_array *out, const af_array signal, const af_array filter,
                    const af_conv_mode mode, af_conv_domain domain) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    return convolve_domain(out, signal, filter, mode, domain, 1);
    AFGB_CATCHALL
}

af_err af_convolve2(af_array *out, const af_array signal, const af_array filter,
                    const af_conv_mode mode, af_conv_domain domain) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    Array *s = get_array(signal);
    Array *f = get_array(filter);
    if (dim4_ndims(s->dims) < 2 || dim4_ndims(f->dims) < 2) {
        return af_convolve1(out, signal, filter, mode, domain);
    }
    return convolve_domain(out, signal, filter, mode, domain, 2);
    AFGB_CATCHALL
}

af_err af_convolve3(af_array *out, const af_array signal, const af_array filter,
                    const af_conv_mode mode, af_conv_domain domain) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    Array *s = get_array(signal);
    Array *f = get_array(filter);
    if (dim4_ndims(s->dims) < 3 || dim4_ndims(f->dims) < 3) {
        return af_convolve2(out, signal, filter, mode, domain);
    }
    return convolve_domain(out, signal, filter, mode, domain, 3);
    AFGB_CATCHALL
}

af_err af_convolve2_sep(af_array *out, const af_array col_filter, const af_array row_filter,
                        const af_array signal, const af_conv_mode mode) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    return convolve2_sep_impl(out, col_filter, row_filter, signal, mode);
    AFGB_CATCHALL
}

af_err af_convolve2_nn(af_array *out, const af_array signal, const af_array filter,
                       const unsigned stride_dims, const dim_t *strides,
                       const unsigned padding_dims, const dim_t *paddings,
                       const unsigned dilation_dims, const dim_t *dilations) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    return convolve2_nn_impl(out, signal, filter, stride_dims, strides, padding_dims, paddings,
                             dilation_dims, dilations, AFGB_PRECISION_FP32, nullptr);
    AFGB_CATCHALL
}

af_err afgb_convolve2_nn_fused(af_array *out, const af_array signal, const af_array filter,
                               const unsigned stride_dims, const dim_t *strides,
                               const unsigned padding_dims, const dim_t *paddings,
                               const unsigned dilation_dims, const dim_t *dilations,
                               afgb_precision precision, const af_array bias, int activation) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    if ((int)precision < 0 || (int)precision > 2) AFGB_THROW(AF_ERR_ARG, "unknown precision");
    AFGB_ARG_ASSERT(11, activation == 0 || activation == 1);
    return convolve2_nn_impl(out, signal, filter, stride_dims, strides, padding_dims, paddings,
                             dilation_dims, dilations, precision, nullptr, bias, activation);
    AFGB_CATCHALL
}

af_err afgb_convolve2_nn_ex(af_array *out, const af_array signal, const af_array filter,
                            const unsigned stride_dims, const dim_t *strides,
                            const unsigned padding_dims, const dim_t *paddings,
                            const unsigned dilation_dims, const dim_t *dilations,
                            afgb_precision precision, const af_array out_channel_scales) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    if ((int)precision < 0 || (int)precision > 2) AFGB_THROW(AF_ERR_ARG, "unknown precision");
    return convolve2_nn_impl(out, signal, filter, stride_dims, strides, padding_dims, paddings,
                             dilation_dims, dilations, precision, out_channel_scales);
    AFGB_CATCHALL
}

af_err af_convolve2_gradient_nn(af_array *out, const af_array incoming_gradient,
                                const af_array original_signal, const af_array original_filter,
                                const af_array convolved_output, const unsigned stride_dims,
                                const dim_t *strides, const unsigned padding_dims,
                                const dim_t *paddings, const unsigned dilation_dims,
                                const dim_t *dilations, af_conv_gradient_type grad_type) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    return convolve2_grad_impl(out, incoming_gradient, original_signal, original_filter,
                               convolved_output, stride_dims, strides, padding_dims, paddings,
                               dilation_dims, dilations, grad_type, AFGB_PRECISION_FP32, false);
    AFGB_CATCHALL
}

af_err afgb_convolve2_gradient_nn_ex(af_array *out, const af_array incoming_gradient,
                                     const af_array original_signal,
                                     const af_array original_filter,
                                     const af_array convolved_output, const unsigned stride_dims,
                                     const dim_t *strides, const unsigned padding_dims,
                                     const dim_t *paddings, const unsigned dilation_dims,
                                     const dim_t *dilations, af_conv_gradient_type grad_type,
                                     afgb_precision precision) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    if ((int)precision < 0 || (int)precision > 2) AFGB_THROW(AF_ERR_ARG, "unknown precision");
    return convolve2_grad_impl(out, incoming_gradient, original_signal, original_filter,
                               convolved_output, stride_dims, strides, padding_dims, paddings,
                               dilation_dims, dilations, grad_type, precision, true);
    AFGB_CATCHALL
}

af_err afgb_convolve2_gradients_nn(af_array *data_grad, af_array *filter_grad,
                                   af_array *bias_grad, const af_array incoming_gradient,
                                   const af_array original_signal, const af_array original_filter,
                                   const unsigned stride_dims, const dim_t *strides,
                                   const unsigned padding_dims, const dim_t *paddings,
                                   const unsigned dilation_dims, const dim_t *dilations,
                                   afgb_precision precision) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, data_grad != nullptr || filter_grad != nullptr || bias_grad != nullptr);
    if ((int)precision < 0 || (int)precision > 2) AFGB_THROW(AF_ERR_ARG, "unknown precision");
    return convolve2_grads_impl(data_grad, filter_grad, bias_grad, incoming_gradient,
                                original_signal, original_filter, stride_dims, strides,
                                padding_dims, paddings, dilation_dims, dilations, precision);
    AFGB_CATCHALL
}

af_err af_fft_convolve1(af_array *out, const af_array signal, const af_array filter,
                        const af_conv_mode mode) {
    AFGB_TRY
    return fft_convolve_impl(out, signal, filter, mode == AF_CONV_EXPAND, 1);
    AFGB_CATCHALL
}

af_err af_fft_convolve2(af_array *out, const af_array signal, const af_array filter,
                        const af_conv_mode mode) {
    AFGB_TRY
    const bool low = dim4_ndims(get_array(signal)->dims) < 2 &&
                     dim4_ndims(get_array(filter)->dims) < 2;
    return fft_convolve_impl(out, signal, filter, mode == AF_CONV_EXPAND, low ? 1 : 2);
    AFGB_CATCHALL
}

af_err af_fft_convolve3(af_array *out, const af_array signal, const af_array filter,
                        const af_conv_mode mode) {
    AFGB_TRY
    const bool low = dim4_ndims(get_array(signal)->dims) < 3 &&
                     dim4_ndims(get_array(filter)->dims) < 3;
    return fft_convolve_impl(out, signal, filter, mode == AF_CONV_EXPAND, low ? 2 : 3);
    AFGB_CATCHALL
}

af_err af_gaussian_kernel(af_array *out, const int rows, const int cols, const double sigma_r,
                          const double sigma_c) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    AFGB_DIM_ASSERT(1, rows >= 0);
    AFGB_DIM_ASSERT(2, cols >= 0);
    Array g = gaussian_kernel(rows, cols, sigma_r, sigma_c);
    *out = make_handle(&g);
    AFGB_CATCHALL
}

// src/api/c/dog.cpp:56-85
af_err af_dog(af_array *out, const af_array in, const int radius1, const int radius2) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    Array *a = get_array(in);
    const dim_t nd = dim4_ndims(a->dims);
    AFGB_ARG_ASSERT(1, (nd >= 2));
    AFGB_ARG_ASSERT(1, (nd <= 3));
    switch (a->type) {
        case f32: case f64: case b8: case s32: case u32: case s16: case u16: case s8: case u8:
            break;
        default: AFGB_TYPE_ERROR(1, a->type);
    }
    AFGB_DIM_ASSERT(2, radius1 >= 0);
    AFGB_DIM_ASSERT(3, radius2 >= 0);
    Array o = dog(*a, radius1, radius2);
    *out = make_handle(&o);
    AFGB_CATCHALL
}

// src/api/c/sobel.cpp:38-87: dx, dy of the input's type for f32/f64/s32,
// s32 for the other integer types
af_err af_sobel_operator(af_array *dx, af_array *dy, const af_array img, const unsigned ker_size) {
    AFGB_TRY
    AFGB_ARG_ASSERT(4, (ker_size == 3));
    AFGB_ARG_ASSERT(0, dx != nullptr && dy != nullptr);
    Array *a = get_array(img);
    AFGB_DIM_ASSERT(3, (dim4_ndims(a->dims) >= 2));
    af_dtype ot;
    switch (a->type) {
        case f32: ot = f32; break;
        case f64: ot = f64; break;
        case s32: case u32: case s16: case u16: case b8: case s8: case u8: ot = s32; break;
        default: AFGB_TYPE_ERROR(1, a->type);
    }
    Array ox = *create_array(ot, a->dims);
    Array oy = *create_array(ot, a->dims);
    sobel_3x3(*a, ox, oy);
    *dx = make_handle(&ox);
    *dy = make_handle(&oy);
    AFGB_CATCHALL
}

af_err af_unwrap(af_array *out, const af_array in, const dim_t wx, const dim_t wy, const dim_t sx,
                 const dim_t sy, const dim_t px, const dim_t py, const bool is_column) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    Array *a = get_array(in);
    const dim_t *id = a->dims;
    AFGB_ARG_ASSERT(2, wx > 0 && wx <= id[0] + 2 * px);
    AFGB_ARG_ASSERT(3, wy > 0 && wy <= id[1] + 2 * py);
    AFGB_ARG_ASSERT(4, sx > 0);
    AFGB_ARG_ASSERT(5, sy > 0);
    AFGB_ARG_ASSERT(6, px >= 0 && px < wx);
    AFGB_ARG_ASSERT(7, py >= 0 && py < wy);
    if (!patch_type(a->type)) AFGB_TYPE_ERROR(1, a->type);
    const dim_t nx = (id[0] + 2 * px - wx) / sx + 1;
    const dim_t ny = (id[1] + 2 * py - wy) / sy + 1;
    dim_t od[4] = {wx * wy, nx * ny, id[2], id[3]};
    if (!is_column) std::swap(od[0], od[1]);
    Array src = a->is_linear() ? *a : make_dense(*a);
    Array r = *create_array(a->type, od);
    patches_unwrap(src, r, wx, wy, sx, sy, px, py, is_column);
    *out = make_handle(&r);
    AFGB_CATCHALL
}

af_err af_wrap(af_array *out, const af_array in, const dim_t ox, const dim_t oy, const dim_t wx,
               const dim_t wy, const dim_t sx, const dim_t sy, const dim_t px, const dim_t py,
               const bool is_column) {
    AFGB_TRY
    wrap_impl(out, in, ox, oy, wx, wy, sx, sy, px, py, is_column, true);
    AFGB_CATCHALL
}

af_err af_wrap_v2(af_array *out, const af_array in, const dim_t ox, const dim_t oy,
                  const dim_t wx, const dim_t wy, const dim_t sx, const dim_t sy, const dim_t px,
                  const dim_t py, const bool is_column) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    wrap_impl(out, in, ox, oy, wx, wy, sx, sy, px, py, is_column, *out == nullptr);
    AFGB_CATCHALL
}

// ---- af_features (src/api/c/features.cpp:15-127): five f32 arrays and a
// count; the getters hand out the object's own handles (not retained)
af_err af_create_features(af_features *feat, dim_t num) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, feat != nullptr);
    AFGB_ARG_ASSERT(1, num >= 0);
    auto *f = new FeaturesObj();
    f->n = num;
    if (num > 0) {
        const dim_t d[4] = {num, 1, 1, 1};
        try {
            for (af_array *slot : f->slots()) {
                Array a = *create_array(f32, d);
                *slot = make_handle(&a);
            }
        } catch (...) {
            release_features_arrays(f);
            delete f;
            throw;
        }
    }
    *feat = static_cast<af_features>(f);
    AFGB_CATCHALL
}

af_err af_release_features(af_features feat) {
    AFGB_TRY
    FeaturesObj *f = get_features(feat);
    release_features_arrays(f);
    delete f;
    AFGB_CATCHALL
}

af_err af_retain_features(af_features *out, const af_features feat) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    FeaturesObj *f = get_features(feat);
    auto *o = new FeaturesObj();
    o->n = f->n;
    auto src = f->slots(), dst = o->slots();
    for (size_t i = 0; i < src.size(); ++i) {
        if (*src[i] == nullptr) continue;
        const af_err e = af_retain_array(dst[i], *src[i]);
        if (e != AF_SUCCESS) {
            release_features_arrays(o);
            delete o;
            return e;
        }
    }
    *out = static_cast<af_features>(o);
    AFGB_CATCHALL
}

af_err af_get_features_num(dim_t *num, const af_features feat) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, num != nullptr);
    *num = get_features(feat)->n;
    AFGB_CATCHALL
}

#define AFGB_FEATURES_GETTER(NAME, FIELD)                      \
    af_err NAME(af_array *out, const af_features feat) {       \
        AFGB_TRY                                               \
        AFGB_ARG_ASSERT(0, out != nullptr);                    \
        *out = get_features(feat)->FIELD;                      \
        AFGB_CATCHALL                                          \
    }
AFGB_FEATURES_GETTER(af_get_features_xpos, x)
AFGB_FEATURES_GETTER(af_get_features_ypos, y)
AFGB_FEATURES_GETTER(af_get_features_score, score)
AFGB_FEATURES_GETTER(af_get_features_orientation, orientation)
AFGB_FEATURES_GETTER(af_get_features_size, size)
#undef AFGB_FEATURES_GETTER

// af_harris (src/api/c/harris.cpp:42-95): window length block_size, else
// floor(6 sigma) made odd; the reference's checks in its order; f32 and f64
af_err af_harris(af_features *out, const af_array in, const unsigned max_corners,
                 const float min_response, const float sigma, const unsigned block_size,
                 const float k_thr) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    Array *a = get_array(in);
    unsigned filter_len =
        (block_size == 0) ? static_cast<unsigned>(std::floor(6.f * sigma)) : block_size;
    if (block_size == 0 && filter_len % 2 == 0) filter_len--;
    const unsigned edge = (block_size > 0) ? block_size / 2 : filter_len / 2;
    AFGB_DIM_ASSERT(1, (a->ndims() == 2));
    AFGB_ARG_ASSERT(1, (a->dims[0] >= (dim_t)(2 * edge + 1) ||
                        a->dims[1] >= (dim_t)(2 * edge + 1)));
    AFGB_ARG_ASSERT(3, (max_corners > 0) || (min_response > 0.0f));
    AFGB_ARG_ASSERT(7, (k_thr >= 0.01f));
    AFGB_ARG_ASSERT(4, (block_size > 2) || (sigma >= 0.5f && sigma <= 5.f));
    AFGB_ARG_ASSERT(5, (block_size <= 32));
    if (a->type != f32 && a->type != f64) AFGB_TYPE_ERROR(1, a->type);
    HarrisOut r;
    harris_corners(*a, max_corners, min_response, sigma, filter_len, k_thr, r);
    if (r.n == 0) {
        // the reference's empty result: x, y, score of dims (0,0,0,0),
        // orientation and size of dims (0,1,1,1)
        const dim_t e0[4] = {0, 0, 0, 0}, e1[4] = {0, 1, 1, 1};
        r.x = *create_array(f32, e0);
        r.y = *create_array(f32, e0);
        r.score = *create_array(f32, e0);
        r.orientation = *create_array(f32, e1);
        r.size = *create_array(f32, e1);
    }
    auto *f = new FeaturesObj();
    f->n = r.n;
    f->x = make_handle(&r.x);
    f->y = make_handle(&r.y);
    f->score = make_handle(&r.score);
    f->orientation = make_handle(&r.orientation);
    f->size = make_handle(&r.size);
    *out = static_cast<af_features>(f);
    AFGB_CATCHALL
}

// af_canny (src/api/c/canny.cpp:232-285): the reference's checks in its
// order; any threshold type but AUTO_OTSU is manual; b8 result
af_err af_canny(af_array *out, const af_array in, const af_canny_threshold threshold_type,
                const float low_threshold_ratio, const float high_threshold_ratio,
                const unsigned sobel_window, const bool is_fast) {
    AFGB_TRY
    AFGB_ARG_ASSERT(0, out != nullptr);
    Array *a = get_array(in);
    AFGB_DIM_ASSERT(2, (a->ndims() >= 2));
    AFGB_DIM_ASSERT(2, (a->dims[0] >= 5 && a->dims[1] >= 5));
    AFGB_ARG_ASSERT(5, (sobel_window == 3));
    switch (a->type) {
        case f32: case f64: case s32: case u32: case s16: case u16: case s8: case u8: break;
        default: AFGB_TYPE_ERROR(1, a->type);
    }
    Array r = canny_edges(*a, threshold_type == AF_CANNY_THRESHOLD_AUTO_OTSU, low_threshold_ratio,
                          high_threshold_ratio, is_fast);
    *out = make_handle(&r);
    AFGB_CATCHALL
}

int afgb_identify_batch_kind(int rank, const dim_t *sdims, const dim_t *fdims) {
    return identify_batch_kind(rank, sdims, fdims);
}

int afgb_conv_output_dims(dim_t *odims, int rank, int kind, int expand, const dim_t *sdims,
                          const dim_t *fdims) {
    conv_out_dims(odims, rank, kind, expand != 0, sdims, fdims);
    return 0;
}

int afgb_nn_output_dims(dim_t *odims, const dim_t *sdims, const dim_t *fdims,
                        const dim_t *stride, const dim_t *padding, const dim_t *dilation) {
    dim_t Wo = 1 + (sdims[0] + 2 * padding[0] - (((fdims[0] - 1) * dilation[0]) + 1)) / stride[0];
    dim_t Ho = 1 + (sdims[1] + 2 * padding[1] - (((fdims[1] - 1) * dilation[1]) + 1)) / stride[1];
    odims[0] = Wo;
    odims[1] = Ho;
    odims[2] = fdims[3];
    odims[3] = sdims[3];
    return 0;
}

}  // extern "C"
