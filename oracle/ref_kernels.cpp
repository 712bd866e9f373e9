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
 */
#include <kernel/convolve.hpp>
#include <kernel/sobel.hpp>
#include <kernel/unwrap.hpp>
#include <kernel/wrap.hpp>

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
