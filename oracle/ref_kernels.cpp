/*
 * ref_kernels.cpp — TEST INFRASTRUCTURE ONLY (oracle).  Exposes the
 * reference's own CPU kernel templates, compiled unchanged from an ArrayFire
 * v3.10.0 source tree, behind a C ABI so tests can pin the C restatement
 * (conv_oracle.c) and generate golden vectors.  Built by oracle/Makefile into
 * oracle/_ref/ only when the reference sources are present; it never ships
 * and the product never loads it.
 *
 * Entry points mirror the reference functions they call:
 *   ref_convolve_nd      -> arrayfire::cpu::kernel::convolve_nd
 *                           (src/backend/cpu/kernel/convolve.hpp:132-211)
 *   ref_convolve2_sep    -> arrayfire::cpu::kernel::convolve2<InT,AccT,Expand>
 *                           (src/backend/cpu/kernel/convolve.hpp:257-289), with
 *                           the temp sized as src/backend/cpu/convolve.cpp:68-99
 *   ref_unwrap_*         -> kernel::unwrap_dim  (src/backend/cpu/kernel/unwrap.hpp:19-80)
 *   ref_wrap_dilated_*   -> kernel::wrap_dim_dilated (src/backend/cpu/kernel/wrap.hpp:166-228)
 *   ref_unwrap_any       -> kernel::unwrap_dim with dilation 1 and d = is_column
 *                           (src/backend/cpu/unwrap.cpp:23-41), every af_unwrap type
 *   ref_wrap_any         -> kernel::wrap_dim<T, is_column> adding into `out`
 *                           (src/backend/cpu/wrap.cpp:24-37), every af_wrap type
 *   ref_sobel            -> kernel::derivative<Ti, To, isDX> for dx and dy
 *                           (src/backend/cpu/kernel/sobel.hpp:19-75), every
 *                           af_sobel_operator type
 *   ref_harris_f32/_f64  -> the corner pipeline of src/backend/cpu/harris.cpp:
 *                           gaussian1D / box window (cpu/utility.hpp:35-49),
 *                           kernel::gradient (cpu/kernel/gradient.hpp),
 *                           kernel::second_order_deriv, kernel::convolve2 (the
 *                           separable window), kernel::harris_responses,
 *                           kernel::non_maximal (cpu/kernel/harris.hpp), and the
 *                           stable descending sort + keep_corners of the
 *                           max_corners > 0 case (cpu/kernel/sort_by_key_impl.hpp)
 *   ref_canny            -> the edge pipeline of src/api/c/canny.cpp:205-230:
 *                           the 5-tap separable smoothing (kernel::convolve2),
 *                           kernel::derivative (Sobel), the gradient magnitude,
 *                           kernel::nonMaxSuppression, the manual or Otsu
 *                           thresholds (kernel::histogram; the array
 *                           arithmetic of canny.cpp:85-190 restated as loops in
 *                           its order), kernel::edgeTrackingHysteresis
 *                           (cpu/kernel/canny.hpp)
 */
#include <kernel/canny.hpp>
#include <kernel/convolve.hpp>
#include <kernel/gradient.hpp>
// kernel/histogram.hpp names dim4 unqualified, as its own includer
// (src/backend/cpu/histogram.cpp) arranges
#include <af/dim4.hpp>
using af::dim4;
#include <kernel/histogram.hpp>
#include <kernel/harris.hpp>
#include <kernel/sobel.hpp>
#include <kernel/sort_helper.hpp>
#include <utility.hpp>
#include <kernel/unwrap.hpp>
#include <kernel/wrap.hpp>

#include <algorithm>
#include <cmath>
#include <limits>
#include <complex>
#include <utility>
#include <cstring>
#include <vector>

#include <common/err_common.hpp>

// The kernels themselves never raise; dim4.cpp references these error
// classes, which live in the reference's error library.  Minimal bodies of
// our own let the shared object link without that library.
AfError::AfError(const char *const func, const char *const file, const int line,
                 const char *const message, af_err err, boost::stacktrace::stacktrace st)
    : std::logic_error(message), functionName(func), fileName(file), st_(st), lineNumber(line),
      error(err) {}
AfError::~AfError() noexcept {}
DimensionError::DimensionError(const char *const func, const char *const file, const int line,
                               const int index, const char *const expectString,
                               const boost::stacktrace::stacktrace &st)
    : AfError(func, file, line, "Invalid size", AF_ERR_SIZE, st),
      expected(expectString),
      argIndex(index) {}

using af::dim4;
namespace K = arrayfire::cpu::kernel;
using arrayfire::cpu::CParam;
using arrayfire::cpu::Param;

namespace {
dim4 d4(const long long *d) { return dim4(d[0], d[1], d[2], d[3]); }
dim4 dense(const long long *d) { return dim4(1, d[0], d[0] * d[1], d[0] * d[1] * d[2]); }

template <typename InT, typename AccT>
void nd(void *out, const long long *od, const long long *os, const void *sig, const long long *sd,
        const long long *ss, const void *filt, const long long *fd, const long long *fs, int kind,
        int rank, int expand) {
    Param<InT> o(static_cast<InT *>(out), d4(od), d4(os));
    CParam<InT> s(static_cast<const InT *>(sig), d4(sd), d4(ss));
    CParam<AccT> f(static_cast<const AccT *>(filt), d4(fd), d4(fs));
    K::convolve_nd<InT, AccT>(o, s, f, static_cast<AF_BATCH_KIND>(kind), rank, expand != 0);
}

template <typename InT, typename AccT>
void sep(void *out, const long long *od, const void *sig, const long long *sd, const void *cf,
         long long cflen, const void *rf, long long rflen, int expand) {
    long long td[4] = {sd[0] + (expand ? cflen - 1 : 0), sd[1], sd[2], sd[3]};
    std::vector<InT> temp((size_t)(td[0] * td[1] * td[2] * td[3]) + 1);
    long long cd[4] = {cflen, 1, 1, 1}, rd[4] = {rflen, 1, 1, 1};
    Param<InT> o(static_cast<InT *>(out), d4(od), dense(od));
    CParam<InT> s(static_cast<const InT *>(sig), d4(sd), dense(sd));
    CParam<AccT> c(static_cast<const AccT *>(cf), d4(cd), dense(cd));
    CParam<AccT> r(static_cast<const AccT *>(rf), d4(rd), dense(rd));
    Param<InT> t(temp.data(), d4(td), dense(td));
    if (expand) K::convolve2<InT, AccT, true>(o, s, c, r, t);
    else K::convolve2<InT, AccT, false>(o, s, c, r, t);
}
}  // namespace

namespace {
template <typename T>
void unwrap_any(void *out, const void *in, const long long *idims, long long wx, long long wy,
                long long sx, long long sy, long long px, long long py, int is_column) {
    long long nx = 1 + (idims[0] + 2 * px - wx) / sx;
    long long ny = 1 + (idims[1] + 2 * py - wy) / sy;
    long long od[4] = {wx * wy, nx * ny, idims[2], idims[3]};
    if (!is_column) std::swap(od[0], od[1]);
    Param<T> o(static_cast<T *>(out), d4(od), dense(od));
    CParam<T> i(static_cast<const T *>(in), d4(idims), dense(idims));
    K::unwrap_dim<T>(o, i, wx, wy, sx, sy, px, py, 1, 1, is_column ? 1 : 0);
}

template <typename T>
void wrap_any(void *out, const long long *odims, const void *in, const long long *idims,
              long long wx, long long wy, long long sx, long long sy, long long px, long long py,
              int is_column) {
    Param<T> o(static_cast<T *>(out), d4(odims), dense(odims));
    CParam<T> i(static_cast<const T *>(in), d4(idims), dense(idims));
    if (is_column) K::wrap_dim<T, 1>(o, i, wx, wy, sx, sy, px, py);
    else K::wrap_dim<T, 0>(o, i, wx, wy, sx, sy, px, py);
}
}  // namespace

namespace {
template <typename Ti, typename To>
void sobel_any(void *dx, void *dy, const void *in, const long long *dims) {
    Param<To> ox(static_cast<To *>(dx), d4(dims), dense(dims));
    Param<To> oy(static_cast<To *>(dy), d4(dims), dense(dims));
    CParam<Ti> i(static_cast<const Ti *>(in), d4(dims), dense(dims));
    K::derivative<Ti, To, true>(ox, i);
    K::derivative<Ti, To, false>(oy, i);
}
}  // namespace

extern "C" {

// dtype numbering: include/af/defines.h af_dtype
int ref_convolve_nd(int dtype, void *out, const long long *od, const long long *os,
                    const void *sig, const long long *sd, const long long *ss, const void *filt,
                    const long long *fd, const long long *fs, int kind, int rank, int expand) {
    switch (dtype) {
        case 0: nd<float, float>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 1: nd<std::complex<float>, std::complex<float>>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 2: nd<double, double>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 3: nd<std::complex<double>, std::complex<double>>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 4: nd<char, float>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 5: nd<int, float>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 6: nd<unsigned, float>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 7: nd<unsigned char, float>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 8: nd<long long, float>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 9: nd<unsigned long long, float>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 10: nd<short, float>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 11: nd<unsigned short, float>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        case 13: nd<signed char, float>(out, od, os, sig, sd, ss, filt, fd, fs, kind, rank, expand); break;
        default: return -1;
    }
    return 0;
}

int ref_convolve2_sep(int dtype, void *out, const long long *od, const void *sig,
                      const long long *sd, const void *cf, long long cflen, const void *rf,
                      long long rflen, int expand) {
    switch (dtype) {
        case 0: sep<float, float>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 1: sep<std::complex<float>, std::complex<float>>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 2: sep<double, double>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 3: sep<std::complex<double>, std::complex<double>>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 4: sep<char, float>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 5: sep<int, float>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 6: sep<unsigned, float>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 7: sep<unsigned char, float>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 8: sep<long long, float>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 9: sep<unsigned long long, float>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 10: sep<short, float>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 11: sep<unsigned short, float>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        case 13: sep<signed char, float>(out, od, sig, sd, cf, cflen, rf, rflen, expand); break;
        default: return -1;
    }
    return 0;
}

#define REF_UNWRAP(NAME, T)                                                                    \
    void NAME(T *out, const T *in, const long long *idims, long long wx, long long wy,         \
              long long sx, long long sy, long long px, long long py, long long dx,            \
              long long dy) {                                                                  \
        long long nx = 1 + (idims[0] + 2 * px - (((wx - 1) * dx) + 1)) / sx;                   \
        long long ny = 1 + (idims[1] + 2 * py - (((wy - 1) * dy) + 1)) / sy;                   \
        long long od[4] = {wx * wy, nx * ny, idims[2], idims[3]};                              \
        Param<T> o(out, d4(od), dense(od));                                                    \
        CParam<T> i(in, d4(idims), dense(idims));                                              \
        K::unwrap_dim<T>(o, i, wx, wy, sx, sy, px, py, dx, dy, 1);                             \
    }
REF_UNWRAP(ref_unwrap_f32, float)
REF_UNWRAP(ref_unwrap_f64, double)

#define REF_WRAP(NAME, T)                                                                      \
    void NAME(T *out, const long long *odims, const T *in, long long wx, long long wy,         \
              long long sx, long long sy, long long px, long long py, long long dx,            \
              long long dy) {                                                                  \
        long long nx = 1 + (odims[0] + 2 * px - (((wx - 1) * dx) + 1)) / sx;                   \
        long long ny = 1 + (odims[1] + 2 * py - (((wy - 1) * dy) + 1)) / sy;                   \
        long long id[4] = {wx * wy, nx * ny, odims[2], odims[3]};                              \
        Param<T> o(out, d4(odims), dense(odims));                                              \
        CParam<T> i(in, d4(id), dense(id));                                                    \
        K::wrap_dim_dilated<T>(o, i, wx, wy, sx, sy, px, py, dx, dy, 1);                       \
    }
REF_WRAP(ref_wrap_dilated_f32, float)
REF_WRAP(ref_wrap_dilated_f64, double)



// dtype numbering: include/af/defines.h af_dtype; outputs as af_sobel_operator
// (src/api/c/sobel.cpp:52-80)
int ref_sobel(int dtype, void *dx, void *dy, const void *in, const long long *dims) {
    switch (dtype) {
        case 0: sobel_any<float, float>(dx, dy, in, dims); break;
        case 2: sobel_any<double, double>(dx, dy, in, dims); break;
        case 5: sobel_any<int, int>(dx, dy, in, dims); break;
        case 6: sobel_any<unsigned, int>(dx, dy, in, dims); break;
        case 10: sobel_any<short, int>(dx, dy, in, dims); break;
        case 11: sobel_any<unsigned short, int>(dx, dy, in, dims); break;
        case 4: sobel_any<char, int>(dx, dy, in, dims); break;
        case 13: sobel_any<signed char, int>(dx, dy, in, dims); break;
        case 7: sobel_any<unsigned char, int>(dx, dy, in, dims); break;
        default: return -1;
    }
    return 0;
}

#define REF_PATCH_TYPES(FN, ...)                                   \
    switch (dtype) {                                               \
        case 0: FN<float>(__VA_ARGS__); break;                     \
        case 1: FN<std::complex<float>>(__VA_ARGS__); break;       \
        case 2: FN<double>(__VA_ARGS__); break;                    \
        case 3: FN<std::complex<double>>(__VA_ARGS__); break;      \
        case 4: FN<char>(__VA_ARGS__); break;                      \
        case 5: FN<int>(__VA_ARGS__); break;                       \
        case 6: FN<unsigned>(__VA_ARGS__); break;                  \
        case 7: FN<unsigned char>(__VA_ARGS__); break;             \
        case 8: FN<long long>(__VA_ARGS__); break;                 \
        case 9: FN<unsigned long long>(__VA_ARGS__); break;        \
        case 10: FN<short>(__VA_ARGS__); break;                    \
        case 11: FN<unsigned short>(__VA_ARGS__); break;           \
        case 13: FN<signed char>(__VA_ARGS__); break;              \
        default: return -1;                                        \
    }

int ref_unwrap_any(int dtype, void *out, const void *in, const long long *idims, long long wx,
                   long long wy, long long sx, long long sy, long long px, long long py,
                   int is_column) {
    REF_PATCH_TYPES(unwrap_any, out, in, idims, wx, wy, sx, sy, px, py, is_column)
    return 0;
}

int ref_wrap_any(int dtype, void *out, const long long *odims, const void *in,
                 const long long *idims, long long wx, long long wy, long long sx, long long sy,
                 long long px, long long py, int is_column) {
    REF_PATCH_TYPES(wrap_any, out, odims, in, idims, wx, wy, sx, sy, px, py, is_column)
    return 0;
}

}  // extern "C"

namespace {
// the steps of arrayfire::cpu::harris (src/backend/cpu/harris.cpp:28-144),
// each a reference kernel; returns the number of corners written
template <typename T>
int harris_any(const T *in, long long d0, long long d1, unsigned max_corners, float min_response,
               float sigma, unsigned filter_len, float k_thr, float *xo, float *yo, float *ro,
               long long cap) {
    const dim4 id(d0, d1, 1, 1), st(1, d0, d0 * d1, d0 * d1);
    const long long n = d0 * d1;
    std::vector<T> filt(filter_len);
    if (sigma < 0.5f) {
        for (unsigned i = 0; i < filter_len; i++) filt[i] = static_cast<T>(1) / (filter_len);
    } else {
        arrayfire::cpu::gaussian1D<T>(filt.data(), static_cast<int>(filter_len), sigma);
    }
    const unsigned border_len = filter_len / 2 + 1;
    std::vector<T> ix(n), iy(n), ixx(n), ixy(n), iyy(n), tmp(n);
    CParam<T> cin(in, id, st);
    K::gradient<T>(Param<T>(iy.data(), id, st), Param<T>(ix.data(), id, st), cin);
    K::second_order_deriv<T>(Param<T>(ixx.data(), id, st), Param<T>(ixy.data(), id, st),
                             Param<T>(iyy.data(), id, st), (unsigned)n,
                             CParam<T>(ix.data(), id, st), CParam<T>(iy.data(), id, st));
    const dim4 fd(filter_len, 1, 1, 1), fs(1, filter_len, filter_len, filter_len);
    CParam<T> cf(filt.data(), fd, fs);
    for (std::vector<T> *a : {&ixx, &ixy, &iyy}) {
        std::vector<T> t2(n), out(n);
        K::convolve2<T, T, false>(Param<T>(out.data(), id, st), CParam<T>(a->data(), id, st), cf,
                                  cf, Param<T>(t2.data(), id, st));
        *a = out;
    }
    std::vector<T> resp(n, T(0));
    K::harris_responses<T>(Param<T>(resp.data(), dim4(n, 1, 1, 1), dim4(1, n, n, n)),
                           (unsigned)d0, (unsigned)d1, CParam<T>(ixx.data(), id, st),
                           CParam<T>(ixy.data(), id, st), CParam<T>(iyy.data(), id, st), k_thr,
                           border_len);
    const unsigned corner_lim = (unsigned)(n * 0.2f);
    std::vector<float> xc(corner_lim + 1), yc(corner_lim + 1), rc(corner_lim + 1);
    const unsigned min_r = (max_corners > 0) ? 0U : static_cast<unsigned>(min_response);
    unsigned found = 0;
    const dim4 cd(corner_lim, 1, 1, 1), cs(1, corner_lim, corner_lim, corner_lim);
    K::non_maximal<T>(Param<float>(xc.data(), cd, cs), Param<float>(yc.data(), cd, cs),
                      Param<float>(rc.data(), cd, cs), &found, (unsigned)d0, (unsigned)d1,
                      CParam<T>(resp.data(), dim4(n, 1, 1, 1), dim4(1, n, n, n)), (float)min_r,
                      border_len, corner_lim);
    const unsigned out_n = std::min(found, (max_corners > 0) ? max_corners : corner_lim);
    if ((long long)out_n > cap) return -1;
    if (max_corners > 0 && found > out_n) {
        // sort_index(respCorners, descending): a stable sort of (value, index)
        const unsigned m = std::min(found, corner_lim);
        // with the reference's comparator (cpu/kernel/sort_by_key_impl.hpp:58-63)
        std::vector<K::IndexPair<float, unsigned>> kv(m);
        for (unsigned i = 0; i < m; ++i) kv[i] = std::make_tuple(rc[i], i);
        std::stable_sort(kv.begin(), kv.end(), K::IPCompare<float, unsigned, false>());
        for (unsigned f = 0; f < out_n; ++f) {
            xo[f] = xc[std::get<1>(kv[f])];
            yo[f] = yc[std::get<1>(kv[f])];
            ro[f] = std::get<0>(kv[f]);
        }
    } else {
        for (unsigned f = 0; f < out_n; ++f) {
            xo[f] = xc[f];
            yo[f] = yc[f];
            ro[f] = rc[f];
        }
    }
    return (int)out_n;
}
}  // namespace

extern "C" {
int ref_harris(int dtype, const void *in, long long d0, long long d1, unsigned max_corners,
               float min_response, float sigma, unsigned filter_len, float k_thr, float *xo,
               float *yo, float *ro, long long cap) {
    if (dtype == 0)
        return harris_any<float>(static_cast<const float *>(in), d0, d1, max_corners, min_response,
                                 sigma, filter_len, k_thr, xo, yo, ro, cap);
    if (dtype == 2)
        return harris_any<double>(static_cast<const double *>(in), d0, d1, max_corners,
                                  min_response, sigma, filter_len, k_thr, xo, yo, ro, cap);
    return -2;
}
}  // extern "C"

namespace {
// the array operations of src/api/c/canny.cpp around the reference's CPU
// kernels, on one or more 2-D slices stacked along dim2 (dims[3] == 1)
template <typename T>
int canny_any(const T *in, const long long *dims, int otsu, float t1, float t2, int isf,
              char *out) {
    const long long d0 = dims[0], d1 = dims[1], d2 = dims[2];
    if (dims[3] != 1) return -3;
    const long long n = d0 * d1 * d2;
    const dim4 id(d0, d1, d2, 1), st(1, d0, d0 * d1, d0 * d1 * d2);
    std::vector<float> x(n), t(n), smt(n), gx(n), gy(n), mag(n), sup(n, 0.f);
    for (long long i = 0; i < n; ++i) x[i] = static_cast<float>(in[i]);  // cast<float, T>
    static const float v[5] = {-0.11021f, -0.23691f, -0.30576f, -0.23691f, -0.11021f};
    CParam<float> cf(v, dim4(5, 1, 1, 1), dim4(1, 5, 5, 5));
    CParam<float> rf(v, dim4(1, 5, 1, 1), dim4(1, 1, 5, 5));
    K::convolve2<float, float, false>(Param<float>(smt.data(), id, st),
                                      CParam<float>(x.data(), id, st), cf, rf,
                                      Param<float>(t.data(), id, st));
    K::derivative<float, float, true>(Param<float>(gx.data(), id, st),
                                      CParam<float>(smt.data(), id, st));
    K::derivative<float, float, false>(Param<float>(gy.data(), id, st),
                                       CParam<float>(smt.data(), id, st));
    for (long long i = 0; i < n; ++i) {  // gradientMagnitude (canny.cpp:66-79)
        if (isf) {
            mag[i] = std::abs(gx[i]) + std::abs(gy[i]);
        } else {
            const float a = gx[i] * gx[i], b = gy[i] * gy[i];
            const float sg = a + b;
            mag[i] = std::sqrt(sg);
        }
    }
    K::nonMaxSuppression<float>(Param<float>(sup.data(), id, st),
                                CParam<float>(mag.data(), id, st),
                                CParam<float>(gx.data(), id, st), CParam<float>(gy.data(), id, st));
    // computeCandidates (canny.cpp:153-190)
    float maxVal = -std::numeric_limits<float>::infinity();
    for (long long i = 0; i < n; ++i) maxVal = std::max(sup[i], maxVal);
    std::vector<char> strong(n), weak(n);
    if (otsu) {
        const unsigned NB = static_cast<unsigned>(maxVal);
        if (NB < 2) return -4;  // the reference's Otsu loop needs two bins
        std::vector<unsigned> hist((size_t)NB * d2, 0u);
        K::histogram<float, true>(
            Param<unsigned>(hist.data(), dim4(NB, 1, d2, 1), dim4(1, NB, NB, NB * d2)),
            CParam<float>(sup.data(), id, st), NB, 0.0, maxVal);
        const float total = static_cast<float>(d0 * d1);
        for (long long z = 0; z < d2; ++z) {
            const unsigned *h = hist.data() + z * NB;
            std::vector<float> freqs(NB), cum(NB), prod(NB), cprod(NB), qlqh(NB);
            float c = 0.f, cp = 0.f, ws = 0.f;
            for (unsigned b = 0; b < NB; ++b) {
                freqs[b] = static_cast<float>(h[b]) / total;
                c = freqs[b] + c;  // scan: in + running
                cum[b] = c;
                qlqh[b] = cum[b] * (1.0f - cum[b]);
                prod[b] = static_cast<float>(b) * freqs[b];
                cp = prod[b] + cp;
                cprod[b] = cp;
                ws = prod[b] + ws;  // reduce: in + running
            }
            float best = 0.f;
            unsigned loc = 0;
            for (unsigned b = 0; b + 1 < NB; ++b) {
                const float qL = cum[b];
                const float qH = 1.0f - qL;
                const float muL = cprod[b] / qL;
                const float muH = (ws - cprod[b]) / qH;
                const float diff = muL - muH;
                const float sigma = (diff * diff) * qlqh[b];
                // ireduce<af_max_t> (cpu/kernel/ireduce.hpp:47-63)
                if (b == 0) {
                    best = std::isnan(sigma) ? -std::numeric_limits<float>::infinity() : sigma;
                    loc = 0;
                } else if (sigma > best) {
                    best = sigma;
                    loc = b;
                }
            }
            const float T2 = static_cast<float>(loc);
            const float T1 = T2 * t1;
            for (long long i = z * d0 * d1; i < (z + 1) * d0 * d1; ++i) {
                weak[i] = (sup[i] >= T1) && (sup[i] < T2);
                strong[i] = sup[i] >= T2;
            }
        }
    } else {
        float minVal = std::numeric_limits<float>::infinity();
        for (long long i = 0; i < n; ++i) minVal = std::min(sup[i], minVal);
        const float denom = maxVal - minVal;
        for (long long i = 0; i < n; ++i) {
            const float g = (sup[i] - minVal) / denom;
            weak[i] = (g >= t1) && (g < t2);
            strong[i] = g >= t2;
        }
    }
    std::fill(out, out + n, (char)0);
    K::edgeTrackingHysteresis<char>(Param<char>(out, id, st), CParam<char>(strong.data(), id, st),
                                    CParam<char>(weak.data(), id, st));
    return 0;
}
}  // namespace

extern "C" {
// af_canny: dtype numbering of include/af/defines.h; out holds 0/1 bytes
int ref_canny(int dtype, const void *in, const long long *dims, int otsu, float t1, float t2,
              int isf, char *out) {
    switch (dtype) {
        case 0: return canny_any<float>(static_cast<const float *>(in), dims, otsu, t1, t2, isf, out);
        case 2: return canny_any<double>(static_cast<const double *>(in), dims, otsu, t1, t2, isf, out);
        case 5: return canny_any<int>(static_cast<const int *>(in), dims, otsu, t1, t2, isf, out);
        case 6: return canny_any<unsigned>(static_cast<const unsigned *>(in), dims, otsu, t1, t2, isf, out);
        case 10: return canny_any<short>(static_cast<const short *>(in), dims, otsu, t1, t2, isf, out);
        case 11: return canny_any<unsigned short>(static_cast<const unsigned short *>(in), dims, otsu, t1, t2, isf, out);
        case 13: return canny_any<signed char>(static_cast<const signed char *>(in), dims, otsu, t1, t2, isf, out);
        case 7: return canny_any<unsigned char>(static_cast<const unsigned char *>(in), dims, otsu, t1, t2, isf, out);
        default: return -2;
    }
}
}  // extern "C"
