/*
 * conv_oracle.c — TEST INFRASTRUCTURE ONLY.  This is the oracle that checks
 * the CUDA library; it is never part of the product path.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg load it.
 *
 * A plain-C restatement of ArrayFire's CPU convolution algorithms (v3.10.0),
 * written from the reference's loop structure so that rounding matches it:
 *
 *   oracle_convolve_nd   <- src/backend/cpu/kernel/convolve.hpp:19-211
 *                           (one2one_1d :19-37, one2one_2d :39-75,
 *                            one2one_3d :77-130, convolve_nd :132-211)
 *                           output dims: src/backend/cpu/convolve.cpp:38-58
 *   oracle_convolve2_sep <- src/backend/cpu/kernel/convolve.hpp:213-289
 *                           temp dims: src/backend/cpu/convolve.cpp:68-99
 *   oracle_unwrap        <- src/backend/cpu/kernel/unwrap.hpp:19-80
 *   oracle_wrap_dilated  <- src/backend/cpu/kernel/wrap.hpp:166-228
 *   oracle_nn_*_f64      <- FP64 direct loops of the formulas in
 *                           src/backend/cpu/convolve.cpp:123-243
 *                           (forward, data gradient, filter gradient) and the
 *                           bias gradient sum (no reference counterpart)
 *
 * Build with -ffp-contract=off: the reference's x86-64 build multiplies and
 * adds separately; a fused multiply-add would change the last bit.
 *
 * Out-of-range float->integer conversions are undefined in the reference
 * (`InT(accum)`); here they truncate toward zero and saturate, NaN -> 0,
 * which is the rule the CUDA library implements.  `b8` is treated as signed
 * char, as on the x86-64 build of the reference.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef long long dim_t;

enum { F32 = 0, C32, F64, C64, B8, S32, U32, U8, S64, U64, S16, U16, F16, S8 };
enum { BATCH_NONE = 0, BATCH_LHS, BATCH_RHS, BATCH_SAME };

typedef struct { float re, im; } cf32;
typedef struct { double re, im; } cf64;

/* ---- float -> integer (trunc toward zero, saturate, NaN -> 0) ---------- */
static double trunc_sat(double a, double lo, double hi) {
    if (a != a) return 0.0;
    double t = trunc(a);
    return t < lo ? lo : (t > hi ? hi : t);
}
static uint8_t to_u8(float a) { return (uint8_t)trunc_sat(a, 0.0, 255.0); }
static int8_t to_s8(float a) { return (int8_t)trunc_sat(a, -128.0, 127.0); }
static uint16_t to_u16(float a) { return (uint16_t)trunc_sat(a, 0.0, 65535.0); }
static int16_t to_s16(float a) { return (int16_t)trunc_sat(a, -32768.0, 32767.0); }
static int32_t to_s32(float a) { return (int32_t)trunc_sat(a, -2147483648.0, 2147483647.0); }
static uint32_t to_u32(float a) { return (uint32_t)trunc_sat(a, 0.0, 4294967295.0); }
static long long to_s64(float a) {
    if (a != a) return 0;
    if (a >= 9223372036854775807.0f) return 9223372036854775807LL;
    if (a <= -9223372036854775808.0f) return -9223372036854775807LL - 1;
    return (long long)a;
}
static unsigned long long to_u64(float a) {
    if (a != a || a <= 0.0f) return 0ull;
    if (a >= 18446744073709551615.0f) return 18446744073709551615ull;
    return (unsigned long long)a;
}

/* ---- complex helpers: (a+bi)(c+di) = (ac-bd) + (ad+bc)i ---------------- */
static cf32 cmul32(cf32 a, cf32 b) {
    float ac = a.re * b.re, bd = a.im * b.im, ad = a.re * b.im, bc = a.im * b.re;
    cf32 r = {ac - bd, ad + bc};
    return r;
}
static cf64 cmul64(cf64 a, cf64 b) {
    double ac = a.re * b.re, bd = a.im * b.im, ad = a.re * b.im, bc = a.im * b.re;
    cf64 r = {ac - bd, ad + bc};
    return r;
}

/* ====================================================================== */
/* convolve_nd                                                            */
/* ====================================================================== */

/*
 * One output element of one2one_{1,2,3}d: the loops run
 * wk (dim 2) outer, wj (dim 1), wi (dim 0) inner, each ascending, and
 * accumulate AccT(s_val * f) from zero.  Out-of-signal samples are zero but
 * still multiplied (the reference does not skip them).
 */
#define DEFINE_ND(NAME, InT, AccT, ZERO_ACC, LOAD_ACC, MAC, STORE)                          \
    static void NAME(InT *optr, const InT *iptr, const AccT *fptr, const dim_t *od,         \
                     const dim_t *sd, const dim_t *fd, const dim_t *os, const dim_t *ss,    \
                     const dim_t *fs, int rank, int expand) {                               \
        dim_t f0 = fd[0], f1 = rank >= 2 ? fd[1] : 1, f2 = rank >= 3 ? fd[2] : 1;           \
        dim_t iS = expand ? 0 : f0 / 2, iE = expand ? od[0] : iS + sd[0];                   \
        dim_t jS = rank >= 2 ? (expand ? 0 : f1 / 2) : 0;                                   \
        dim_t jE = rank >= 2 ? (expand ? od[1] : jS + sd[1]) : 1;                           \
        dim_t kS = rank >= 3 ? (expand ? 0 : f2 / 2) : 0;                                   \
        dim_t kE = rank >= 3 ? (expand ? od[2] : kS + sd[2]) : 1;                           \
        for (dim_t k = kS; k < kE; ++k)                                                     \
            for (dim_t j = jS; j < jE; ++j)                                                 \
                for (dim_t i = iS; i < iE; ++i) {                                           \
                    AccT acc = ZERO_ACC;                                                    \
                    for (dim_t wk = 0; wk < f2; ++wk) {                                     \
                        dim_t kI = k - wk;                                                  \
                        int kv = rank < 3 || (kI >= 0 && kI < sd[2]);                       \
                        for (dim_t wj = 0; wj < f1; ++wj) {                                 \
                            dim_t jI = j - wj;                                              \
                            int jv = rank < 2 || (jI >= 0 && jI < sd[1]);                   \
                            for (dim_t wi = 0; wi < f0; ++wi) {                             \
                                dim_t iI = i - wi;                                          \
                                InT s;                                                      \
                                memset(&s, 0, sizeof(s));                                   \
                                if (kv && jv && iI >= 0 && iI < sd[0]) {                    \
                                    dim_t off = iI * ss[0];                                 \
                                    if (rank >= 2) off += jI * ss[1];                       \
                                    if (rank >= 3) off += kI * ss[2];                       \
                                    s = iptr[off];                                          \
                                }                                                           \
                                dim_t foff = wi * fs[0];                                    \
                                if (rank >= 2) foff += wj * fs[1];                          \
                                if (rank >= 3) foff += wk * fs[2];                          \
                                AccT f = fptr[foff];                                        \
                                AccT sv = LOAD_ACC(s);                                      \
                                MAC(acc, sv, f);                                            \
                            }                                                               \
                        }                                                                   \
                    }                                                                       \
                    dim_t ooff = (i - iS);                                                  \
                    if (rank >= 2) ooff += (j - jS) * os[1];                                \
                    if (rank >= 3) ooff += (k - kS) * os[2];                                \
                    optr[ooff] = STORE(acc);                                                \
                }                                                                           \
    }

#define MAC_REAL(acc, s, f) \
    do {                    \
        acc += (s) * (f);   \
    } while (0)
#define MAC_C32(acc, s, f)              \
    do {                                \
        cf32 p_ = cmul32((s), (f));     \
        acc.re += p_.re;                \
        acc.im += p_.im;                \
    } while (0)
#define MAC_C64(acc, s, f)              \
    do {                                \
        cf64 p_ = cmul64((s), (f));     \
        acc.re += p_.re;                \
        acc.im += p_.im;                \
    } while (0)
#define ID(x) (x)
#define TOF(x) ((float)(x))
static const cf32 CZ32 = {0.f, 0.f};
static const cf64 CZ64 = {0.0, 0.0};

DEFINE_ND(nd_f32, float, float, 0.0f, ID, MAC_REAL, ID)
DEFINE_ND(nd_f64, double, double, 0.0, ID, MAC_REAL, ID)
DEFINE_ND(nd_c32, cf32, cf32, CZ32, ID, MAC_C32, ID)
DEFINE_ND(nd_c64, cf64, cf64, CZ64, ID, MAC_C64, ID)
DEFINE_ND(nd_u8, uint8_t, float, 0.0f, TOF, MAC_REAL, to_u8)
DEFINE_ND(nd_s8, int8_t, float, 0.0f, TOF, MAC_REAL, to_s8)
DEFINE_ND(nd_u16, uint16_t, float, 0.0f, TOF, MAC_REAL, to_u16)
DEFINE_ND(nd_s16, int16_t, float, 0.0f, TOF, MAC_REAL, to_s16)
DEFINE_ND(nd_s32, int32_t, float, 0.0f, TOF, MAC_REAL, to_s32)
DEFINE_ND(nd_u32, uint32_t, float, 0.0f, TOF, MAC_REAL, to_u32)
DEFINE_ND(nd_s64, long long, float, 0.0f, TOF, MAC_REAL, to_s64)
DEFINE_ND(nd_u64, unsigned long long, float, 0.0f, TOF, MAC_REAL, to_u64)

static size_t dtype_size(int t) {
    switch (t) {
        case F32: case S32: case U32: return 4;
        case C32: case F64: case S64: case U64: return 8;
        case C64: return 16;
        case B8: case U8: case S8: return 1;
        case S16: case U16: case F16: return 2;
    }
    return 0;
}
static size_t acc_size(int t) {
    switch (t) {
        case F64: return 8;
        case C32: return 8;
        case C64: return 16;
        default: return 4;
    }
}

/* convolve_nd (src/backend/cpu/kernel/convolve.hpp:132-211): batch steps per
 * kind, then one one2one call per (b1,b2,b3).  Strides are in elements. */
int oracle_convolve_nd(int dtype, void *out, const dim_t *od, const dim_t *os, const void *sig,
                       const dim_t *sd, const dim_t *ss, const void *filt, const dim_t *fd,
                       const dim_t *fs, int kind, int rank, int expand) {
    dim_t out_step[4] = {0, 0, 0, 0}, in_step[4] = {0, 0, 0, 0}, filt_step[4] = {0, 0, 0, 0};
    dim_t batch[4] = {0, 1, 1, 1};
    for (int i = 1; i < 4; ++i) {
        switch (kind) {
            case BATCH_LHS:
                out_step[i] = os[i];
                in_step[i] = ss[i];
                if (i >= rank) batch[i] = sd[i];
                break;
            case BATCH_SAME:
                out_step[i] = os[i];
                in_step[i] = ss[i];
                filt_step[i] = fs[i];
                if (i >= rank) batch[i] = sd[i];
                break;
            case BATCH_RHS:
                out_step[i] = os[i];
                filt_step[i] = fs[i];
                if (i >= rank) batch[i] = fd[i];
                break;
            default: break;
        }
    }
    size_t es = dtype_size(dtype), as = acc_size(dtype);
    for (dim_t b3 = 0; b3 < batch[3]; ++b3)
        for (dim_t b2 = 0; b2 < batch[2]; ++b2)
            for (dim_t b1 = 0; b1 < batch[1]; ++b1) {
                char *o = (char *)out + (b1 * out_step[1] + b2 * out_step[2] + b3 * out_step[3]) * es;
                const char *in =
                    (const char *)sig + (b1 * in_step[1] + b2 * in_step[2] + b3 * in_step[3]) * es;
                const char *f = (const char *)filt +
                                (b1 * filt_step[1] + b2 * filt_step[2] + b3 * filt_step[3]) * as;
#define CALL_ND(FN, InT, AccT) \
    FN((InT *)o, (const InT *)in, (const AccT *)f, od, sd, fd, os, ss, fs, rank, expand)
                switch (dtype) {
                    case F32: CALL_ND(nd_f32, float, float); break;
                    case F64: CALL_ND(nd_f64, double, double); break;
                    case C32: CALL_ND(nd_c32, cf32, cf32); break;
                    case C64: CALL_ND(nd_c64, cf64, cf64); break;
                    case U8: CALL_ND(nd_u8, uint8_t, float); break;
                    case B8:
                    case S8: CALL_ND(nd_s8, int8_t, float); break;
                    case U16: CALL_ND(nd_u16, uint16_t, float); break;
                    case S16: CALL_ND(nd_s16, int16_t, float); break;
                    case S32: CALL_ND(nd_s32, int32_t, float); break;
                    case U32: CALL_ND(nd_u32, uint32_t, float); break;
                    case S64: CALL_ND(nd_s64, long long, float); break;
                    case U64: CALL_ND(nd_u64, unsigned long long, float); break;
                    default: return -1;
                }
#undef CALL_ND
            }
    return 0;
}

/* ====================================================================== */
/* separable                                                              */
/* ====================================================================== */

/*
 * convolve2_separable<InT, AccT, Expand, ConvDim>
 * (src/backend/cpu/kernel/convolve.hpp:213-255).  The tap is converted to
 * the input type first (`InT f_val = fptr[f]`) and the product is taken in
 * the input type's arithmetic, then converted to AccT and added.
 * Narrow integer products promote to int; signed overflow wraps here.
 */
#define DEFINE_SEP(NAME, InT, AccT, ZERO_ACC, TAP, PROD, STORE)                                \
    static void NAME(InT *optr, const InT *iptr, const AccT *fptr, const dim_t *od,            \
                     const dim_t *sd, dim_t fdim, int expand, int conv_dim) {                  \
        for (dim_t j = 0; j < od[1]; ++j) {                                                    \
            dim_t cj = j + (conv_dim == 1) * (expand ? 0 : fdim >> 1);                         \
            for (dim_t i = 0; i < od[0]; ++i) {                                                \
                dim_t ci = i + (conv_dim == 0) * (expand ? 0 : fdim >> 1);                     \
                AccT acc = ZERO_ACC;                                                           \
                for (dim_t f = 0; f < fdim; ++f) {                                             \
                    InT fv = TAP(fptr[f]);                                                     \
                    InT s;                                                                     \
                    memset(&s, 0, sizeof(s));                                                  \
                    if (conv_dim == 0) {                                                       \
                        dim_t offi = ci - f;                                                   \
                        if (cj >= 0 && cj < sd[1] && offi >= 0 && offi < sd[0])                \
                            s = iptr[cj * sd[0] + offi];                                       \
                    } else {                                                                   \
                        dim_t offj = cj - f;                                                   \
                        if (ci >= 0 && ci < sd[0] && offj >= 0 && offj < sd[1])                \
                            s = iptr[offj * sd[0] + ci];                                       \
                    }                                                                          \
                    PROD(acc, s, fv);                                                          \
                }                                                                              \
                optr[j * od[0] + i] = STORE(acc);                                              \
            }                                                                                  \
        }                                                                                      \
    }

#define PROD_F(acc, s, f) acc += (s) * (f)
#define PROD_C32(acc, s, f) MAC_C32(acc, s, f)
#define PROD_C64(acc, s, f) MAC_C64(acc, s, f)
#define PROD_I(acc, s, f) acc += (float)((int)(s) * (int)(f))
#define PROD_U16(acc, s, f) acc += (float)(int)((unsigned)(s) * (unsigned)(f))
#define PROD_S32(acc, s, f) acc += (float)(int32_t)((uint32_t)(s) * (uint32_t)(f))
#define PROD_U32(acc, s, f) acc += (float)((uint32_t)(s) * (uint32_t)(f))
#define PROD_S64(acc, s, f) acc += (float)(long long)((unsigned long long)(s) * (unsigned long long)(f))
#define PROD_U64(acc, s, f) acc += (float)((unsigned long long)(s) * (unsigned long long)(f))

DEFINE_SEP(sep_f32, float, float, 0.0f, ID, PROD_F, ID)
DEFINE_SEP(sep_f64, double, double, 0.0, ID, PROD_F, ID)
DEFINE_SEP(sep_c32, cf32, cf32, CZ32, ID, PROD_C32, ID)
DEFINE_SEP(sep_c64, cf64, cf64, CZ64, ID, PROD_C64, ID)
DEFINE_SEP(sep_u8, uint8_t, float, 0.0f, to_u8, PROD_I, to_u8)
DEFINE_SEP(sep_s8, int8_t, float, 0.0f, to_s8, PROD_I, to_s8)
DEFINE_SEP(sep_u16, uint16_t, float, 0.0f, to_u16, PROD_U16, to_u16)
DEFINE_SEP(sep_s16, int16_t, float, 0.0f, to_s16, PROD_I, to_s16)
DEFINE_SEP(sep_s32, int32_t, float, 0.0f, to_s32, PROD_S32, to_s32)
DEFINE_SEP(sep_u32, uint32_t, float, 0.0f, to_u32, PROD_U32, to_u32)
DEFINE_SEP(sep_s64, long long, float, 0.0f, to_s64, PROD_S64, to_s64)
DEFINE_SEP(sep_u64, unsigned long long, float, 0.0f, to_u64, PROD_U64, to_u64)

/* convolve2 (src/backend/cpu/kernel/convolve.hpp:257-289): for every
 * (b2,b3) slice, column pass into an InT temp of dims
 * (sd0 + (expand ? cflen-1 : 0), sd1), then row pass.  Dense arrays. */
int oracle_convolve2_sep(int dtype, void *out, const dim_t *od, const void *sig, const dim_t *sd,
                         const void *cf, dim_t cflen, const void *rf, dim_t rflen, int expand) {
    size_t es = dtype_size(dtype);
    dim_t td[4] = {sd[0] + (expand ? cflen - 1 : 0), sd[1], sd[2], sd[3]};
    char *temp = (char *)malloc((size_t)(td[0] * td[1]) * es + 16);
    if (!temp) return -2;
    for (dim_t b3 = 0; b3 < od[3]; ++b3)
        for (dim_t b2 = 0; b2 < od[2]; ++b2) {
            const char *ip = (const char *)sig + ((b3 * sd[2] + b2) * sd[0] * sd[1]) * es;
            char *op = (char *)out + ((b3 * od[2] + b2) * od[0] * od[1]) * es;
#define CALL_SEP(FN, InT, AccT)                                                            \
    FN((InT *)temp, (const InT *)ip, (const AccT *)cf, td, sd, cflen, expand, 0);          \
    FN((InT *)op, (const InT *)temp, (const AccT *)rf, od, td, rflen, expand, 1)
            switch (dtype) {
                case F32: CALL_SEP(sep_f32, float, float); break;
                case F64: CALL_SEP(sep_f64, double, double); break;
                case C32: CALL_SEP(sep_c32, cf32, cf32); break;
                case C64: CALL_SEP(sep_c64, cf64, cf64); break;
                case U8: CALL_SEP(sep_u8, uint8_t, float); break;
                case B8:
                case S8: CALL_SEP(sep_s8, int8_t, float); break;
                case U16: CALL_SEP(sep_u16, uint16_t, float); break;
                case S16: CALL_SEP(sep_s16, int16_t, float); break;
                case S32: CALL_SEP(sep_s32, int32_t, float); break;
                case U32: CALL_SEP(sep_u32, uint32_t, float); break;
                case S64: CALL_SEP(sep_s64, long long, float); break;
                case U64: CALL_SEP(sep_u64, unsigned long long, float); break;
                default: free(temp); return -1;
            }
#undef CALL_SEP
        }
    free(temp);
    return 0;
}

/* ====================================================================== */
/* unwrap / wrap_dilated (f32 and f64)                                    */
/* ====================================================================== */

/* unwrap_dim with d = 1 (retCols = false): out (nx*ny, wx*wy, C, N) stored
 * as out[(y*wx + x) + wx*wy*col] per (C,N) slice.  Dense in/out. */
#define DEFINE_UNWRAP(NAME, T)                                                                    \
    void NAME(T *out, const T *in, const dim_t *idims, dim_t wx, dim_t wy, dim_t sx, dim_t sy,  \
              dim_t px, dim_t py, dim_t dx, dim_t dy) {                                          \
        dim_t nx = 1 + (idims[0] + 2 * px - (((wx - 1) * dx) + 1)) / sx;                         \
        dim_t ny = 1 + (idims[1] + 2 * py - (((wy - 1) * dy) + 1)) / sy;                         \
        dim_t ncols = nx * ny, wsz = wx * wy;                                                    \
        for (dim_t w = 0; w < idims[3]; ++w)                                                     \
            for (dim_t z = 0; z < idims[2]; ++z) {                                               \
                const T *ip = in + (w * idims[2] + z) * idims[0] * idims[1];                     \
                T *op = out + (w * idims[2] + z) * ncols * wsz;                                  \
                for (dim_t col = 0; col < ncols; ++col) {                                        \
                    dim_t spx = (col % nx) * sx - px, spy = (col / nx) * sy - py;                \
                    for (dim_t y = 0; y < wy; ++y)                                               \
                        for (dim_t x = 0; x < wx; ++x) {                                         \
                            dim_t xp = spx + x * dx, yp = spy + y * dy;                          \
                            T v = 0;                                                             \
                            if (xp >= 0 && xp < idims[0] && yp >= 0 && yp < idims[1])           \
                                v = ip[yp * idims[0] + xp];                                      \
                            op[col * wsz + y * wx + x] = v;                                      \
                        }                                                                        \
                }                                                                                \
            }                                                                                    \
    }
DEFINE_UNWRAP(oracle_unwrap_f32, float)
DEFINE_UNWRAP(oracle_unwrap_f64, double)

/* wrap_dim_dilated with d = 1: scatter-add in column order into out
 * (odims) which the caller zero-fills. */
#define DEFINE_WRAP(NAME, T)                                                                      \
    void NAME(T *out, const dim_t *odims, const T *in, dim_t wx, dim_t wy, dim_t sx, dim_t sy,  \
              dim_t px, dim_t py, dim_t dx, dim_t dy) {                                          \
        dim_t nx = 1 + (odims[0] + 2 * px - (((wx - 1) * dx) + 1)) / sx;                         \
        dim_t ny = 1 + (odims[1] + 2 * py - (((wy - 1) * dy) + 1)) / sy;                         \
        dim_t ncols = nx * ny, wsz = wx * wy;                                                    \
        for (dim_t w = 0; w < odims[3]; ++w)                                                     \
            for (dim_t z = 0; z < odims[2]; ++z) {                                               \
                const T *ip = in + (w * odims[2] + z) * ncols * wsz;                             \
                T *op = out + (w * odims[2] + z) * odims[0] * odims[1];                          \
                for (dim_t col = 0; col < ncols; ++col) {                                        \
                    dim_t spx = (col % nx) * sx - px, spy = (col / nx) * sy - py;                \
                    for (dim_t y = 0; y < wy; ++y)                                               \
                        for (dim_t x = 0; x < wx; ++x) {                                         \
                            dim_t xp = spx + x * dx, yp = spy + y * dy;                          \
                            if (xp >= 0 && xp < odims[0] && yp >= 0 && yp < odims[1])            \
                                op[yp * odims[0] + xp] += ip[col * wsz + y * wx + x];            \
                        }                                                                        \
                }                                                                                \
            }                                                                                    \
    }
DEFINE_WRAP(oracle_wrap_dilated_f32, float)
DEFINE_WRAP(oracle_wrap_dilated_f64, double)

/* ====================================================================== */
/* NN convolution in FP64                                                 */
/* ====================================================================== */
/* Geometry: signal (W,H,C,N), filter (fw,fh,C,K), out (Wo,Ho,K,N);
 * g[] = {W,H,C,N, fw,fh,K, sx,sy, px,py, dx,dy}.
 * Forward (src/backend/cpu/convolve.cpp:123-158):
 *   out[x,y,k,n] = sum_{c,v,u} in[x*sx-px+u*dx, y*sy-py+v*dy, c, n]
 *                              * w[fw-1-u, fh-1-v, c, k]                   */
static void nn_dims(const dim_t *g, dim_t *Wo, dim_t *Ho) {
    *Wo = 1 + (g[0] + 2 * g[9] - (((g[4] - 1) * g[11]) + 1)) / g[7];
    *Ho = 1 + (g[1] + 2 * g[10] - (((g[5] - 1) * g[12]) + 1)) / g[8];
}

static double nn_fwd_point(const double *in, const double *w, const dim_t *g, dim_t x, dim_t y,
                           dim_t k, dim_t n) {
    dim_t W = g[0], H = g[1], C = g[2], fw = g[4], fh = g[5];
    double acc = 0.0;
    for (dim_t c = 0; c < C; ++c)
        for (dim_t v = 0; v < fh; ++v) {
            dim_t ys = y * g[8] - g[10] + v * g[12];
            if (ys < 0 || ys >= H) continue;
            for (dim_t u = 0; u < fw; ++u) {
                dim_t xs = x * g[7] - g[9] + u * g[11];
                if (xs < 0 || xs >= W) continue;
                acc += in[xs + W * (ys + H * (c + C * n))] *
                       w[(fw - 1 - u) + fw * ((fh - 1 - v) + fh * (c + C * k))];
            }
        }
    return acc;
}

void oracle_nn_fwd_f64(double *out, const double *in, const double *w, const dim_t *g) {
    dim_t Wo, Ho;
    nn_dims(g, &Wo, &Ho);
    for (dim_t n = 0; n < g[3]; ++n)
        for (dim_t k = 0; k < g[6]; ++k)
            for (dim_t y = 0; y < Ho; ++y)
                for (dim_t x = 0; x < Wo; ++x)
                    out[x + Wo * (y + Ho * (k + g[6] * n))] = nn_fwd_point(in, w, g, x, y, k, n);
}

/* forward at selected output coordinates (linear indices into out) */
void oracle_nn_fwd_points_f64(double *vals, const dim_t *idx, dim_t npts, const double *in,
                              const double *w, const dim_t *g) {
    dim_t Wo, Ho;
    nn_dims(g, &Wo, &Ho);
    for (dim_t p = 0; p < npts; ++p) {
        dim_t t = idx[p];
        dim_t x = t % Wo, y = (t / Wo) % Ho, k = (t / (Wo * Ho)) % g[6], n = t / (Wo * Ho * g[6]);
        vals[p] = nn_fwd_point(in, w, g, x, y, k, n);
    }
}

/* data gradient: dx[x',y',c,n] = sum over (u,v,k) with
 * x' = x*sx - px + u*dx (x in [0,Wo)) of gr[x,y,k,n] * w[fw-1-u, fh-1-v, c, k] */
static double nn_dgrad_point(const double *gr, const double *w, const dim_t *g, dim_t xi,
                             dim_t yi, dim_t c, dim_t n) {
    dim_t C = g[2], fw = g[4], fh = g[5], K = g[6];
    dim_t Wo, Ho;
    nn_dims(g, &Wo, &Ho);
    double acc = 0.0;
    for (dim_t k = 0; k < K; ++k)
        for (dim_t v = 0; v < fh; ++v) {
            dim_t ty = yi + g[10] - v * g[12];
            if (ty < 0 || ty % g[8]) continue;
            dim_t y = ty / g[8];
            if (y >= Ho) continue;
            for (dim_t u = 0; u < fw; ++u) {
                dim_t tx = xi + g[9] - u * g[11];
                if (tx < 0 || tx % g[7]) continue;
                dim_t x = tx / g[7];
                if (x >= Wo) continue;
                acc += gr[x + Wo * (y + Ho * (k + K * n))] *
                       w[(fw - 1 - u) + fw * ((fh - 1 - v) + fh * (c + C * k))];
            }
        }
    return acc;
}

void oracle_nn_dgrad_f64(double *dx, const double *gr, const double *w, const dim_t *g) {
    for (dim_t n = 0; n < g[3]; ++n)
        for (dim_t c = 0; c < g[2]; ++c)
            for (dim_t y = 0; y < g[1]; ++y)
                for (dim_t x = 0; x < g[0]; ++x)
                    dx[x + g[0] * (y + g[1] * (c + g[2] * n))] = nn_dgrad_point(gr, w, g, x, y, c, n);
}

void oracle_nn_dgrad_points_f64(double *vals, const dim_t *idx, dim_t npts, const double *gr,
                                const double *w, const dim_t *g) {
    for (dim_t p = 0; p < npts; ++p) {
        dim_t t = idx[p];
        dim_t x = t % g[0], y = (t / g[0]) % g[1], c = (t / (g[0] * g[1])) % g[2],
              n = t / (g[0] * g[1] * g[2]);
        vals[p] = nn_dgrad_point(gr, w, g, x, y, c, n);
    }
}

/* filter gradient: dw[fw-1-u, fh-1-v, c, k] = sum_{x,y,n}
 *   in[x*sx-px+u*dx, y*sy-py+v*dy, c, n] * gr[x,y,k,n]
 * (src/backend/cpu/convolve.cpp:213-243: unwrap, GEMM, then flip) */
static double nn_wgrad_point(const double *in, const double *gr, const dim_t *g, dim_t ui,
                             dim_t vi, dim_t c, dim_t k) {
    dim_t W = g[0], H = g[1], C = g[2], N = g[3], fw = g[4], fh = g[5], K = g[6];
    dim_t Wo, Ho;
    nn_dims(g, &Wo, &Ho);
    dim_t u = fw - 1 - ui, v = fh - 1 - vi;
    double acc = 0.0;
    for (dim_t n = 0; n < N; ++n)
        for (dim_t y = 0; y < Ho; ++y) {
            dim_t ys = y * g[8] - g[10] + v * g[12];
            if (ys < 0 || ys >= H) continue;
            for (dim_t x = 0; x < Wo; ++x) {
                dim_t xs = x * g[7] - g[9] + u * g[11];
                if (xs < 0 || xs >= W) continue;
                acc += in[xs + W * (ys + H * (c + C * n))] * gr[x + Wo * (y + Ho * (k + K * n))];
            }
        }
    return acc;
}

void oracle_nn_wgrad_f64(double *dw, const double *in, const double *gr, const dim_t *g) {
    dim_t fw = g[4], fh = g[5], C = g[2];
    for (dim_t k = 0; k < g[6]; ++k)
        for (dim_t c = 0; c < C; ++c)
            for (dim_t v = 0; v < fh; ++v)
                for (dim_t u = 0; u < fw; ++u)
                    dw[u + fw * (v + fh * (c + C * k))] = nn_wgrad_point(in, gr, g, u, v, c, k);
}

void oracle_nn_wgrad_points_f64(double *vals, const dim_t *idx, dim_t npts, const double *in,
                                const double *gr, const dim_t *g) {
    dim_t fw = g[4], fh = g[5], C = g[2];
    for (dim_t p = 0; p < npts; ++p) {
        dim_t t = idx[p];
        dim_t u = t % fw, v = (t / fw) % fh, c = (t / (fw * fh)) % C, k = t / (fw * fh * C);
        vals[p] = nn_wgrad_point(in, gr, g, u, v, c, k);
    }
}

/* bias gradient: db[k] = sum_{x,y,n} gr[x,y,k,n] */
void oracle_nn_bgrad_f64(double *db, const double *gr, const dim_t *g) {
    dim_t Wo, Ho;
    nn_dims(g, &Wo, &Ho);
    for (dim_t k = 0; k < g[6]; ++k) {
        double acc = 0.0;
        for (dim_t n = 0; n < g[3]; ++n)
            for (dim_t p = 0; p < Wo * Ho; ++p) acc += gr[p + Wo * Ho * (k + g[6] * n)];
        db[k] = acc;
    }
}
