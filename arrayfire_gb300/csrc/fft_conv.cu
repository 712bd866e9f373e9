// Frequency-domain convolution: af_fft_convolve1/2/3 and the AUTO route of
// af_convolve1/2/3 (src/api/c/fftconvolve.cpp:38-260, CPU backend
// src/backend/cpu/fftconvolve.cpp:38-200, kernels
// src/backend/cpu/kernel/fftconvolve.hpp:19-250).
//
// What the reference computes, restated:
//   * real signals, batch kinds NONE / LHS / RHS / SAME: the filter is first
//     converted to the signal type (castArray<T>, so integer signals truncate
//     the taps), both are convolved exactly (linear convolution evaluated by
//     FFT in float, or double for f64), the result is divided by the
//     transform size and, for integer types, rounded (roundf) before the
//     conversion to the signal type;
//   * complex signals, and DIFF batches (fftconvolve_fallback): the filter
//     goes straight to the complex working type, and the real part (or the
//     complex value) is converted to the signal type without rounding;
//   * outputs: EXPAND keeps the full s+f-1 extent of the rank dims, DEFAULT
//     the window starting at f/2; batch dims are the elementwise maximum of the
//     signal's and the filter's (each batch dim of one side is 1 or equal).
//
// How it runs here: the reference halves the signal's dim 0 into a complex
// vector and uses complex transforms of power-of-two sizes.  This library
// uses real-to-complex transforms for real data, of the smallest 2^a 3^b sizes
// that hold s+f-1 (about half the work and memory of the power-of-two packing;
// measured faster than sizes with factors 5 and 7 as well), all on the
// library's stream:
//   pad      signal and filter -> zero-padded real (or complex) batches
//   forward  R2C / C2C transforms, batched over the slices
//   multiply one kernel, broadcasting the batch dims per batch kind
//   inverse  C2R / C2C transforms over the output slices
//   crop     one kernel: window, 1/size scale, rounding, type conversion
// The transforms are this library's (fft_own.cu) for every 2^a 3^b size that
// fits one block, the sizes picked by default; other sizes go to cuFFT,
// loaded at first use with dlopen, so the library still loads where cuFFT is
// absent (such calls then fail with AF_ERR_LOAD_LIB).  Padding, spectrum
// products and the output pass are this file's kernels.  Results equal the
// reference's up to floating-point rounding (the transform sizes and
// summation orders differ).
#include <cuda_runtime.h>
#include <cufft.h>
#include <dlfcn.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <type_traits>

#include "afgb_internal.hpp"
#include "conv_common.cuh"
#include "conv_direct.hpp"
#include "fft_own.hpp"

namespace afgb {

namespace {

// ---------------------------------------------------------------------------
// cuFFT, resolved at first use
// ---------------------------------------------------------------------------
struct CufftApi {
    bool ok = false;
    std::string why;
    cufftResult (*plan_many)(cufftHandle *, int, int *, int *, int, int, int *, int, int,
                             cufftType, int) = nullptr;
    cufftResult (*set_stream)(cufftHandle, cudaStream_t) = nullptr;
    cufftResult (*destroy)(cufftHandle) = nullptr;
    cufftResult (*r2c)(cufftHandle, cufftReal *, cufftComplex *) = nullptr;
    cufftResult (*c2r)(cufftHandle, cufftComplex *, cufftReal *) = nullptr;
    cufftResult (*d2z)(cufftHandle, cufftDoubleReal *, cufftDoubleComplex *) = nullptr;
    cufftResult (*z2d)(cufftHandle, cufftDoubleComplex *, cufftDoubleReal *) = nullptr;
    cufftResult (*c2c)(cufftHandle, cufftComplex *, cufftComplex *, int) = nullptr;
    cufftResult (*z2z)(cufftHandle, cufftDoubleComplex *, cufftDoubleComplex *, int) = nullptr;
};

CufftApi load_cufft() {
    CufftApi a;
    const char *names[] = {"libcufft.so.12", "libcufft.so.11", "libcufft.so",
                           "/usr/local/cuda/lib64/libcufft.so.12",
                           "/usr/local/cuda/targets/sbsa-linux/lib/libcufft.so.12",
                           "/usr/local/cuda/targets/x86_64-linux/lib/libcufft.so.12"};
    void *h = nullptr;
    for (const char *n : names) {
        h = dlopen(n, RTLD_NOW | RTLD_LOCAL);
        if (h) break;
    }
    if (!h) {
        a.why = "cuFFT (libcufft.so) could not be loaded";
        return a;
    }
    bool all = true;
    auto sym = [&](auto &fn, const char *name) {
        fn = reinterpret_cast<std::remove_reference_t<decltype(fn)>>(dlsym(h, name));
        all &= fn != nullptr;
    };
    sym(a.plan_many, "cufftPlanMany");
    sym(a.set_stream, "cufftSetStream");
    sym(a.destroy, "cufftDestroy");
    sym(a.r2c, "cufftExecR2C");
    sym(a.c2r, "cufftExecC2R");
    sym(a.d2z, "cufftExecD2Z");
    sym(a.z2d, "cufftExecZ2D");
    sym(a.c2c, "cufftExecC2C");
    sym(a.z2z, "cufftExecZ2Z");
    a.ok = all;
    if (!all) a.why = "cuFFT is missing an entry point";
    return a;
}

CufftApi &cufft() {
    static CufftApi api = load_cufft();
    if (!api.ok) AFGB_THROW(AF_ERR_LOAD_LIB, api.why);
    return api;
}

void cufft_check(cufftResult r, const char *what) {
    if (r != CUFFT_SUCCESS)
        AFGB_THROW(r == CUFFT_ALLOC_FAILED ? AF_ERR_NO_MEM : AF_ERR_RUNTIME,
                   std::string("cuFFT ") + what + " failed (" + std::to_string((int)r) + ")");
}

// plans by (device, rank, sizes, batch, type), kept for reuse (a cuFFT plan
// belongs to the device that was current when it was made).  Each convolution
// starts a new epoch; when the cache is full, plans not used in the current
// epoch are destroyed (never one the running convolution already holds).
struct PlanEntry {
    cufftHandle h;
    unsigned long long epoch;
};
std::mutex plan_mu;
std::map<std::tuple<int, int, int, int, int, int, int>, PlanEntry> plans;
unsigned long long plan_epoch = 0;
constexpr size_t kMaxPlans = 16;

// one frequency-domain convolution at a time per process: a plan's stream
// binding and its execution stay together, and no other call evicts the plans
// a running convolution holds (the work itself is asynchronous, so this only
// serialises host-side enqueueing)
std::mutex fft_call_mu;

unsigned long long begin_plan_epoch() {
    std::lock_guard<std::mutex> lk(plan_mu);
    return ++plan_epoch;
}

cufftHandle get_plan(int rank, const int *n_fast_first, int batch, cufftType type,
                     unsigned long long epoch) {
    std::lock_guard<std::mutex> lk(plan_mu);
    int dev = 0;
    AFGB_CUDA(cudaGetDevice(&dev));
    auto key = std::make_tuple(dev, rank, n_fast_first[0], n_fast_first[1], n_fast_first[2], batch,
                               (int)type);
    auto it = plans.find(key);
    if (it != plans.end()) {
        it->second.epoch = epoch;
        return it->second.h;
    }
    CufftApi &api = cufft();
    if (plans.size() >= kMaxPlans) {
        for (auto e = plans.begin(); e != plans.end();) {
            if (e->second.epoch != epoch) {
                api.destroy(e->second.h);
                e = plans.erase(e);
            } else {
                ++e;
            }
        }
    }
    int n[3];
    for (int k = 0; k < rank; ++k) n[k] = n_fast_first[rank - 1 - k];  // cuFFT: slowest first
    cufftHandle h;
    cufft_check(api.plan_many(&h, rank, n, nullptr, 1, 0, nullptr, 1, 0, type, batch), "plan");
    plans[key] = PlanEntry{h, epoch};
    return h;
}

// smallest n' >= n whose prime factors are all in the allowed set (even when
// `even`): 2 and 3 by default; AFGB_FFT_RADICES=2357, 235 or 2 changes the set
// (for comparing transform sizes)
long long good_size(long long n, bool even) {
    static const int radices = [] {
        const char *e = std::getenv("AFGB_FFT_RADICES");
        return e ? std::atoi(e) : 23;
    }();
    if (n <= 1) return 1;
    for (long long m = n;; ++m) {
        if (even && (m & 1)) continue;
        long long r = m;
        for (long long p : {2ll, 3ll, 5ll, 7ll}) {
            const bool ok = radices == 2 ? p == 2
                                         : (radices == 23 ? p <= 3 : (radices == 235 ? p <= 5 : true));
            if (ok)
                while (r % p == 0) r /= p;
        }
        if (r == 1) return m;
    }
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------
template <typename V> __device__ __forceinline__ V vzero() { return V{}; }

// one padded row (i1, i2, batch) per block iteration; the row's first d0
// elements come from the dense input, the rest are zero
template <typename V>
__global__ void fft_pad_kernel(const V *__restrict__ in, V *__restrict__ out, long long n0,
                               long long n1, long long n2, long long d0, long long d1,
                               long long d2, long long rows) {
    const long long slice = d0 * d1 * d2;
    for (long long row = blockIdx.x; row < rows; row += gridDim.x) {
        const long long i1 = row % n1, r = row / n1, i2 = r % n2, b = r / n2;
        V *o = out + row * n0;
        const bool inside = i1 < d1 && i2 < d2;
        const V *src = in + b * slice + d0 * (i1 + d1 * i2);
        for (long long i0 = threadIdx.x; i0 < n0; i0 += blockDim.x)
            o[i0] = (inside && i0 < d0) ? src[i0] : vzero<V>();
    }
}

// batch-dim broadcast of the spectrum product (up to three batch dims)
struct BatchMap {
    int nbd;
    long long od[3], sd[3], fd[3], ss[3], fs[3];
};

template <typename C> __device__ __forceinline__ C cmul(C a, C b) {
    return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}

template <typename C>
__global__ void fft_mul_kernel(const C *S, const C *F, C *P, long long nc, BatchMap bm,
                               long long obatch) {
    for (long long ob = blockIdx.y; ob < obatch; ob += gridDim.y) {
        long long r = ob, si = 0, fi = 0;
        for (int k = 0; k < bm.nbd; ++k) {
            const long long o = r % bm.od[k];
            r /= bm.od[k];
            si += (bm.sd[k] == 1 ? 0 : o) * bm.ss[k];
            fi += (bm.fd[k] == 1 ? 0 : o) * bm.fs[k];
        }
        const C *s = S + si * nc;
        const C *f = F + fi * nc;
        C *p = P + ob * nc;
        for (long long j = blockIdx.x * (long long)blockDim.x + threadIdx.x; j < nc;
             j += (long long)gridDim.x * blockDim.x)
            p[j] = cmul(s[j], f[j]);
    }
}

enum { CROP_PLAIN = 0, CROP_ROUND = 1, CROP_TRUNC = 2 };

template <typename To, int MODE> __device__ __forceinline__ To to_out(double v) {
    if constexpr (MODE == CROP_ROUND) return (To)roundf((float)v);
    else return (To)v;
}
template <typename To, int MODE> __device__ __forceinline__ To to_out(float v) {
    if constexpr (MODE == CROP_ROUND) return (To)roundf(v);
    else return (To)v;
}

template <typename V> struct ScalarOf { using type = V; };
template <> struct ScalarOf<cf32> { using type = float; };
template <> struct ScalarOf<cf64> { using type = double; };

// out[i0, i1, i2, b] = convert( buf[b][(i0+off0) + n0*((i1+off1) + n1*(i2+off2))] / scale ),
// one output row (i1, i2, b) per block iteration, threads along i0
template <typename V, typename To, int MODE>
__global__ void fft_crop_kernel(const V *__restrict__ buf, To *__restrict__ out, long long o0,
                                long long o1, long long o2, long long n0, long long n1,
                                long long n2, long long off0, long long off1, long long off2,
                                long long rows, typename ScalarOf<V>::type scale) {
    const long long nslice = n0 * n1 * n2;
    for (long long row = blockIdx.x; row < rows; row += gridDim.x) {
        const long long i1 = row % o1, r = row / o1, i2 = r % o2, b = r / o2;
        const V *src = buf + b * nslice + off0 + n0 * ((i1 + off1) + n1 * (i2 + off2));
        To *dst = out + row * o0;
        for (long long i0 = threadIdx.x; i0 < o0; i0 += blockDim.x) {
            const V v = src[i0];
            if constexpr (std::is_same<V, cf32>::value || std::is_same<V, cf64>::value) {
                if constexpr (std::is_same<To, cf32>::value || std::is_same<To, cf64>::value) {
                    using OS = decltype(To{}.x);
                    dst[i0] = To{(OS)(v.x / scale), (OS)(v.y / scale)};
                } else {
                    dst[i0] = to_out<To, MODE>(v.x / scale);  // the real part
                }
            } else {
                dst[i0] = to_out<To, MODE>(v / scale);
            }
        }
    }
}

unsigned blocks_for(long long n, int per_block) {
    return (unsigned)std::min<long long>(std::max<long long>((n + per_block - 1) / per_block, 1),
                                         (long long)num_sms() * 32);
}

// scratch buffer released when it goes out of scope (stream-ordered)
struct Scratch {
    void *p = nullptr;
    explicit Scratch(size_t bytes) : p(bytes ? tagged(bytes) : nullptr) {}
    static void *tagged(size_t bytes) {
        MemTag tag("frequency-domain buffers");
        return alloc_device(bytes);
    }
    ~Scratch() {
        if (p) free_device(p);
    }
    Scratch(const Scratch &) = delete;
    Scratch &operator=(const Scratch &) = delete;
    template <typename V> V *as() const { return static_cast<V *>(p); }
};

}  // namespace

// ---------------------------------------------------------------------------
// host driver
// ---------------------------------------------------------------------------
namespace {

struct FftGeom {
    unsigned long long epoch;  // plan-cache epoch of this convolution
    int rank;
    long long n[3];       // transform sizes, fastest first (1 beyond rank)
    long long nreal, ncplx;  // elements per slice: real input, spectrum
    long long sb, fb, ob;    // slices of signal, filter, output
    BatchMap bm;
};

template <typename V>
void pad_into(const Array &dense, V *dst, const FftGeom &g, long long nslices) {
    const long long d0 = dense.dims[0];
    const long long d1 = g.rank > 1 ? dense.dims[1] : 1;
    const long long d2 = g.rank > 2 ? dense.dims[2] : 1;
    const long long rows = g.n[1] * g.n[2] * nslices;
    if (rows == 0) return;
    const int threads = g.n[0] >= 256 ? 256 : (g.n[0] >= 64 ? 64 : 32);
    fft_pad_kernel<V><<<blocks_for(rows, 1), threads, 0, stream()>>>(
        dense.ptr<V>(), dst, g.n[0], g.n[1], g.n[2], d0, d1, d2, rows);
    count_launch();
    AFGB_POST_LAUNCH("fft_pad_kernel");
}

template <typename C>
void multiply(const C *S, const C *F, C *P, const FftGeom &g) {
    dim3 grid(blocks_for(g.ncplx, 256), (unsigned)std::min<long long>(g.ob, 65535));
    if (grid.x * (long long)grid.y > (long long)num_sms() * 64)
        grid.x = std::max<unsigned>(1, (unsigned)((long long)num_sms() * 64 / grid.y));
    fft_mul_kernel<C><<<grid, 256, 0, stream()>>>(S, F, P, g.ncplx, g.bm, g.ob);
    count_launch();
    AFGB_POST_LAUNCH("fft_mul_kernel");
}

template <typename V, typename To, int MODE>
void crop(const V *buf, Array &out, const FftGeom &g, bool expand, const dim_t *fd) {
    const long long o0 = out.dims[0];
    const long long o1 = g.rank > 1 ? out.dims[1] : 1;
    const long long o2 = g.rank > 2 ? out.dims[2] : 1;
    const long long total = out.elements();
    if (total == 0) return;
    long long off[3] = {0, 0, 0};
    if (!expand)
        for (int k = 0; k < g.rank; ++k) off[k] = fd[k] / 2;
    using S = typename ScalarOf<V>::type;
    const S scale = (S)((double)g.n[0] * (double)g.n[1] * (double)g.n[2]);
    const long long rows = total / o0;
    const int threads = o0 >= 256 ? 256 : (o0 >= 64 ? 64 : 32);
    fft_crop_kernel<V, To, MODE><<<blocks_for(rows, 1), threads, 0, stream()>>>(
        buf, out.ptr<To>(), o0, o1, o2, g.n[0], g.n[1], g.n[2], off[0], off[1], off[2], rows,
        scale);
    count_launch();
    AFGB_POST_LAUNCH("fft_crop_kernel");
}

template <typename V, int MODE>
void crop_to(const V *buf, Array &out, const FftGeom &g, bool expand, const dim_t *fd) {
    switch (out.type) {
        case f32: crop<V, float, MODE>(buf, out, g, expand, fd); break;
        case f64: crop<V, double, MODE>(buf, out, g, expand, fd); break;
        case c32:
            if constexpr (std::is_same<V, cf32>::value || std::is_same<V, cf64>::value)
                crop<V, cf32, MODE>(buf, out, g, expand, fd);
            break;
        case c64:
            if constexpr (std::is_same<V, cf32>::value || std::is_same<V, cf64>::value)
                crop<V, cf64, MODE>(buf, out, g, expand, fd);
            break;
        case s32: crop<V, int, MODE>(buf, out, g, expand, fd); break;
        case u32: crop<V, unsigned, MODE>(buf, out, g, expand, fd); break;
        case s64: crop<V, long long, MODE>(buf, out, g, expand, fd); break;
        case u64: crop<V, unsigned long long, MODE>(buf, out, g, expand, fd); break;
        case s16: crop<V, short, MODE>(buf, out, g, expand, fd); break;
        case u16: crop<V, unsigned short, MODE>(buf, out, g, expand, fd); break;
        case s8: crop<V, signed char, MODE>(buf, out, g, expand, fd); break;
        case u8: crop<V, unsigned char, MODE>(buf, out, g, expand, fd); break;
        case b8: crop<V, signed char, MODE>(buf, out, g, expand, fd); break;
        default: AFGB_TYPE_ERROR(1, out.type);
    }
}

// This library's transforms (fft_own.cu) serve every size whose lengths are
// 2^a 3^b and fit one block's shared memory, the sizes good_size picks by
// default; cuFFT serves the others (AFGB_FFT_RADICES with factors 5 or 7,
// or lengths above about 12800), or every size with AFGB_FFT_IMPL=cufft.
bool use_own_fft(const FftGeom &g, bool real, size_t csize) {
    static const bool force_cufft = [] {
        const char *e = std::getenv("AFGB_FFT_IMPL");
        return e && std::string(e) == "cufft";
    }();
    if (force_cufft) return false;
    for (int k = 0; k < g.rank; ++k)
        if (!fft_own_len_ok(g.n[k], real && k == 0, csize)) return false;
    return true;
}

// the rank-r transform of `b` slices over the axes above 0, in place on the
// (n0c, n1, n2, b) spectrum (n0c = n0/2+1 for real data, n0 for complex)
template <typename C>
void own_axes(C *spec, const FftGeom &g, long long n0c, long long b, bool inverse) {
    if (!inverse) {
        if (g.rank >= 2) fft_axis<C>(spec, g.n[1], n0c, g.n[2] * b, false);
        if (g.rank >= 3) fft_axis<C>(spec, g.n[2], n0c * g.n[1], b, false);
    } else {
        if (g.rank >= 3) fft_axis<C>(spec, g.n[2], n0c * g.n[1], b, true);
        if (g.rank >= 2) fft_axis<C>(spec, g.n[1], n0c, g.n[2] * b, true);
    }
}

template <typename R, typename C>
void own_forward_real(const R *in, C *spec, const FftGeom &g, long long b) {
    fft_real_forward<R, C>(in, spec, g.n[0], g.n[1] * g.n[2] * b);
    own_axes<C>(spec, g, g.n[0] / 2 + 1, b, false);
}

template <typename R, typename C>
void own_inverse_real(C *spec, R *out, const FftGeom &g, long long b) {
    own_axes<C>(spec, g, g.n[0] / 2 + 1, b, true);
    fft_real_inverse<R, C>(spec, out, g.n[0], g.n[1] * g.n[2] * b);
}

template <typename C>
void own_complex(C *spec, const FftGeom &g, long long b, bool inverse) {
    if (!inverse) fft_axis<C>(spec, g.n[0], 1, g.n[1] * g.n[2] * b, false);
    own_axes<C>(spec, g, g.n[0], b, inverse);
    if (inverse) fft_axis<C>(spec, g.n[0], 1, g.n[1] * g.n[2] * b, true);
}

// real data: R2C / C2R (float or double working type R, spectrum C)
template <typename R, typename C>
void run_real(const Array &s, const Array &f, Array &out, const FftGeom &g, bool expand, int mode,
              cufftType fwd, cufftType inv) {
    const bool own_fft = use_own_fft(g, true, sizeof(C));
    Scratch sreal(sizeof(R) * g.nreal * g.sb), freal(sizeof(R) * g.nreal * g.fb);
    Scratch sspec(sizeof(C) * g.ncplx * g.sb), fspec(sizeof(C) * g.ncplx * g.fb);
    pad_into<R>(s, sreal.as<R>(), g, g.sb);
    pad_into<R>(f, freal.as<R>(), g, g.fb);
    const int nf[3] = {(int)g.n[0], (int)g.n[1], (int)g.n[2]};
    if (own_fft) {
        own_forward_real<R, C>(sreal.as<R>(), sspec.as<C>(), g, g.sb);
        own_forward_real<R, C>(freal.as<R>(), fspec.as<C>(), g, g.fb);
    } else {
    CufftApi &api = cufft();
    cufftHandle ps = get_plan(g.rank, nf, (int)g.sb, fwd, g.epoch);
    cufftHandle pf = get_plan(g.rank, nf, (int)g.fb, fwd, g.epoch);
    cufft_check(api.set_stream(ps, stream()), "set stream");
    cufft_check(api.set_stream(pf, stream()), "set stream");
    if constexpr (std::is_same<R, float>::value) {
        cufft_check(api.r2c(ps, sreal.as<cufftReal>(), sspec.as<cufftComplex>()), "R2C");
        cufft_check(api.r2c(pf, freal.as<cufftReal>(), fspec.as<cufftComplex>()), "R2C");
    } else {
        cufft_check(api.d2z(ps, sreal.as<cufftDoubleReal>(), sspec.as<cufftDoubleComplex>()),
                    "D2Z");
        cufft_check(api.d2z(pf, freal.as<cufftDoubleReal>(), fspec.as<cufftDoubleComplex>()),
                    "D2Z");
    }
    }
    // product in place where one side's slices are the output's (NONE, LHS,
    // SAME: the signal's; RHS: the filter's), else (DIFF) in new buffers
    const bool s_is_out = g.ob == g.sb && std::equal(g.bm.sd, g.bm.sd + g.bm.nbd, g.bm.od);
    const bool f_is_out =
        !s_is_out && g.ob == g.fb && std::equal(g.bm.fd, g.bm.fd + g.bm.nbd, g.bm.od);
    const bool own = !s_is_out && !f_is_out;
    Scratch pspec(own ? sizeof(C) * g.ncplx * g.ob : 0);
    Scratch obuf(own ? sizeof(R) * g.nreal * g.ob : 0);
    C *P = s_is_out ? sspec.as<C>() : (f_is_out ? fspec.as<C>() : pspec.as<C>());
    R *oreal = s_is_out ? sreal.as<R>() : (f_is_out ? freal.as<R>() : obuf.as<R>());
    multiply<C>(sspec.as<C>(), fspec.as<C>(), P, g);
    if (own_fft) {
        own_inverse_real<R, C>(P, oreal, g, g.ob);
    } else {
    CufftApi &api = cufft();
    cufftHandle po = get_plan(g.rank, nf, (int)g.ob, inv, g.epoch);
    cufft_check(api.set_stream(po, stream()), "set stream");
    if constexpr (std::is_same<R, float>::value)
        cufft_check(api.c2r(po, reinterpret_cast<cufftComplex *>(P), reinterpret_cast<cufftReal *>(oreal)),
                    "C2R");
    else
        cufft_check(api.z2d(po, reinterpret_cast<cufftDoubleComplex *>(P),
                            reinterpret_cast<cufftDoubleReal *>(oreal)),
                    "Z2D");
    }
    if (mode == CROP_ROUND) crop_to<R, CROP_ROUND>(oreal, out, g, expand, f.dims);
    else if (mode == CROP_TRUNC) crop_to<R, CROP_TRUNC>(oreal, out, g, expand, f.dims);
    else crop_to<R, CROP_PLAIN>(oreal, out, g, expand, f.dims);
}

// complex data: C2C both ways
template <typename C>
void run_complex(const Array &s, const Array &f, Array &out, const FftGeom &g, bool expand,
                 int mode, cufftType type) {
    const bool own = use_own_fft(g, false, sizeof(C));
    Scratch sspec(sizeof(C) * g.ncplx * g.sb), fspec(sizeof(C) * g.ncplx * g.fb);
    pad_into<C>(s, sspec.as<C>(), g, g.sb);
    pad_into<C>(f, fspec.as<C>(), g, g.fb);
    const int nf[3] = {(int)g.n[0], (int)g.n[1], (int)g.n[2]};
    if (own) {
        own_complex<C>(sspec.as<C>(), g, g.sb, false);
        own_complex<C>(fspec.as<C>(), g, g.fb, false);
        const bool s_is_out = g.ob == g.sb && std::equal(g.bm.sd, g.bm.sd + g.bm.nbd, g.bm.od);
        const bool f_is_out =
            !s_is_out && g.ob == g.fb && std::equal(g.bm.fd, g.bm.fd + g.bm.nbd, g.bm.od);
        Scratch pspec(s_is_out || f_is_out ? 0 : sizeof(C) * g.ncplx * g.ob);
        C *P = s_is_out ? sspec.as<C>() : (f_is_out ? fspec.as<C>() : pspec.as<C>());
        multiply<C>(sspec.as<C>(), fspec.as<C>(), P, g);
        own_complex<C>(P, g, g.ob, true);
        if (mode == CROP_TRUNC) crop_to<C, CROP_TRUNC>(P, out, g, expand, f.dims);
        else crop_to<C, CROP_PLAIN>(P, out, g, expand, f.dims);
        return;
    }
    CufftApi &api = cufft();
    cufftHandle ps = get_plan(g.rank, nf, (int)g.sb, type, g.epoch);
    cufftHandle pf = get_plan(g.rank, nf, (int)g.fb, type, g.epoch);
    cufft_check(api.set_stream(ps, stream()), "set stream");
    cufft_check(api.set_stream(pf, stream()), "set stream");
    auto exec = [&](cufftHandle h, C *in, C *o, int dir) {
        if constexpr (std::is_same<C, cf32>::value)
            cufft_check(api.c2c(h, reinterpret_cast<cufftComplex *>(in),
                                reinterpret_cast<cufftComplex *>(o), dir),
                        "C2C");
        else
            cufft_check(api.z2z(h, reinterpret_cast<cufftDoubleComplex *>(in),
                                reinterpret_cast<cufftDoubleComplex *>(o), dir),
                        "Z2Z");
    };
    exec(ps, sspec.as<C>(), sspec.as<C>(), CUFFT_FORWARD);
    exec(pf, fspec.as<C>(), fspec.as<C>(), CUFFT_FORWARD);
    const bool s_is_out = g.ob == g.sb && std::equal(g.bm.sd, g.bm.sd + g.bm.nbd, g.bm.od);
    const bool f_is_out =
        !s_is_out && g.ob == g.fb && std::equal(g.bm.fd, g.bm.fd + g.bm.nbd, g.bm.od);
    Scratch pspec(s_is_out || f_is_out ? 0 : sizeof(C) * g.ncplx * g.ob);
    C *P = s_is_out ? sspec.as<C>() : (f_is_out ? fspec.as<C>() : pspec.as<C>());
    multiply<C>(sspec.as<C>(), fspec.as<C>(), P, g);
    cufftHandle po = get_plan(g.rank, nf, (int)g.ob, type, g.epoch);
    cufft_check(api.set_stream(po, stream()), "set stream");
    exec(po, P, P, CUFFT_INVERSE);
    if (mode == CROP_TRUNC) crop_to<C, CROP_TRUNC>(P, out, g, expand, f.dims);
    else crop_to<C, CROP_PLAIN>(P, out, g, expand, f.dims);
}

bool is_cplx(af_dtype t) { return t == c32 || t == c64; }

}  // namespace

Array fft_convolve(const Array &sig, const Array &filt, bool expand, int rank, int kind) {
    const af_dtype T = sig.type;
    const bool dbl = T == f64 || T == c64;
    const bool complex_path = is_cplx(T) || (kind == BATCH_DIFF && is_cplx(filt.type));
    const bool fallback = is_cplx(T) || kind == BATCH_DIFF;
    // working copies, dense, in the working type
    const af_dtype work = complex_path ? (dbl ? c64 : c32) : (dbl ? f64 : f32);
    Array s = cast_array(sig, work);
    Array f = fallback ? cast_array(filt, work) : cast_array(cast_array(filt, T), work);

    std::lock_guard<std::mutex> call_lock(fft_call_mu);
    FftGeom g{};
    g.epoch = begin_plan_epoch();
    g.rank = rank;
    for (int k = 0; k < 3; ++k) g.n[k] = 1;
    for (int k = 0; k < rank; ++k)
        g.n[k] = good_size(sig.dims[k] + filt.dims[k] - 1, k == 0 && !complex_path);
    g.nreal = g.n[0] * g.n[1] * g.n[2];
    g.ncplx = (complex_path ? g.n[0] : g.n[0] / 2 + 1) * g.n[1] * g.n[2];
    g.sb = g.fb = g.ob = 1;
    g.bm.nbd = 4 - rank;
    long long sstr = 1, fstr = 1;
    for (int k = rank; k < 4; ++k) {
        const int j = k - rank;
        g.bm.sd[j] = sig.dims[k];
        g.bm.fd[j] = filt.dims[k];
        g.bm.od[j] = std::max(sig.dims[k], filt.dims[k]);
        g.bm.ss[j] = sstr;
        g.bm.fs[j] = fstr;
        sstr *= sig.dims[k];
        fstr *= filt.dims[k];
        g.sb *= sig.dims[k];
        g.fb *= filt.dims[k];
        g.ob *= g.bm.od[j];
    }
    if (g.nreal * std::max(g.sb, std::max(g.fb, g.ob)) > (1ll << 40) ||
        std::max(g.sb, std::max(g.fb, g.ob)) > 0x7fffffffll || g.n[0] > 0x7fffffffll ||
        g.n[1] > 0x7fffffffll || g.n[2] > 0x7fffffffll)
        AFGB_THROW(AF_ERR_SIZE, "frequency-domain convolution too large");

    // output dims (src/backend/cpu/fftconvolve.cpp:164-181, fallback
    // src/api/c/fftconvolve.cpp:66-86)
    dim_t od[4];
    for (int d = 0; d < 4; ++d) {
        if (d < rank) od[d] = expand ? sig.dims[d] + filt.dims[d] - 1 : sig.dims[d];
        else od[d] = g.bm.od[d - rank];
    }
    Array out = *create_array(T, od);
    if (out.elements() == 0) return out;

    const bool integral = !(T == f32 || T == f64 || is_cplx(T));
    const int mode = integral ? (fallback ? CROP_TRUNC : CROP_ROUND) : CROP_PLAIN;
    KernelTimer kt("fft_pipeline");  // pads, transforms, product and crop
    if (complex_path) {
        if (dbl) run_complex<cf64>(s, f, out, g, expand, mode, CUFFT_Z2Z);
        else run_complex<cf32>(s, f, out, g, expand, mode, CUFFT_C2C);
    } else {
        if (dbl) run_real<double, cf64>(s, f, out, g, expand, mode, CUFFT_D2Z, CUFFT_Z2D);
        else run_real<float, cf32>(s, f, out, g, expand, mode, CUFFT_R2C, CUFFT_C2R);
    }
    return out;
}

}  // namespace afgb
