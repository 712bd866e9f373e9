// af_unwrap / af_wrap / af_wrap_v2: the patch extraction and patch
// accumulation that the reference's NN path is built on
// (src/api/c/unwrap.cpp:37, src/api/c/wrap.cpp:33-99; CPU kernels
// src/backend/cpu/kernel/unwrap.hpp:19-80, wrap.hpp:22-80).
//
// Patches: nx = (W + 2px - wx)/sx + 1 across, ny likewise; patch col =
// winx + nx*winy starts at (winx*sx - px, winy*sy - py).  With is_column the
// patch elements run along dim 0 (dims (wx*wy, nx*ny, d2, d3)), otherwise
// along dim 1 (dims (nx*ny, wx*wy, d2, d3)).
//
// unwrap is a copy (zero outside the image); `in` arrives dense.  wrap adds every patch element
// into its output pixel; one thread per output pixel visits the patches that
// cover it in increasing col order -- the order in which the reference's
// scatter loop reaches that pixel -- and adds in the element type, so float
// results are bit-identical and integer sums wrap exactly as T += T does.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "afgb_internal.hpp"
#include "conv_common.cuh"
#include "conv_direct.hpp"

namespace afgb {

struct PatchGeom {
    long long W, H;       // image dims 0, 1
    long long nx, ny;     // patches across, down
    long long wx, wy, sx, sy, px, py;
    long long slices;     // d2 * d3
    long long d2;         // dim 2 (splits a slice index into z, w)
    long long os[4];      // wrap: strides of the output image (may be a view)
    int is_column;
    int zero_init;        // wrap: start from 0 instead of reading `out` (af_wrap)
};

template <typename T> __device__ __forceinline__ T padd(T a, T b) { return (T)(a + b); }
template <> __device__ __forceinline__ cf32 padd<cf32>(cf32 a, cf32 b) { return cf32{a.x + b.x, a.y + b.y}; }
template <> __device__ __forceinline__ cf64 padd<cf64>(cf64 a, cf64 b) { return cf64{a.x + b.x, a.y + b.y}; }
template <typename T> __device__ __forceinline__ T pzero() { return T{}; }

// the index decompositions by multiply-high when every index is below 2^31
// (FAST), else by 64-bit division
struct PatchDivs {
    FastDiv wsz, np, nx, wx, W, H, d2;
};

// one thread per output element; in: image slices of W*H, out: patches
template <typename T, bool FAST>
__global__ void unwrap_kernel(const T *__restrict__ in, T *__restrict__ out, PatchGeom g,
                              PatchDivs f) {
    const long long wsz = g.wx * g.wy, np = g.nx * g.ny;
    const long long total = wsz * np * g.slices;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        long long k, col, s, winx, winy, kx, ky;
        if constexpr (FAST) {
            const uint32_t u = (uint32_t)t;
            uint32_t k32, c32, s32;
            if (g.is_column) {  // out[k + wsz*(col + np*s)]
                const uint32_t r = fdiv(u, f.wsz);
                k32 = u - r * f.wsz.d;
                s32 = fdiv(r, f.np);
                c32 = r - s32 * f.np.d;
            } else {            // out[col + np*(k + wsz*s)]
                const uint32_t r = fdiv(u, f.np);
                c32 = u - r * f.np.d;
                s32 = fdiv(r, f.wsz);
                k32 = r - s32 * f.wsz.d;
            }
            const uint32_t wy32 = fdiv(c32, f.nx), ky32 = fdiv(k32, f.wx);
            winy = wy32;
            winx = c32 - wy32 * f.nx.d;
            ky = ky32;
            kx = k32 - ky32 * f.wx.d;
            s = s32;
        } else {
            if (g.is_column) {
                k = t % wsz;
                const long long r = t / wsz;
                col = r % np;
                s = r / np;
            } else {
                col = t % np;
                const long long r = t / np;
                k = r % wsz;
                s = r / wsz;
            }
            winx = col % g.nx;
            winy = col / g.nx;
            kx = k % g.wx;
            ky = k / g.wx;
        }
        const long long x = winx * g.sx - g.px + kx;
        const long long y = winy * g.sy - g.py + ky;
        T v = pzero<T>();
        if (x >= 0 && x < g.W && y >= 0 && y < g.H) v = in[x + g.W * (y + g.H * s)];
        out[t] = v;
    }
}

// one thread per output pixel: out = out + (sum over covering patches in col
// order); `out` is addressed through its strides, so af_wrap_v2 can add into a
// sub-array view in place
template <typename T, bool FAST>
__global__ void wrap_kernel(const T *__restrict__ in, T *__restrict__ out, PatchGeom g,
                            PatchDivs f) {
    const long long wsz = g.wx * g.wy, np = g.nx * g.ny;
    const long long total = g.W * g.H * g.slices;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        long long x, y, z, w;
        if constexpr (FAST) {
            const uint32_t u = (uint32_t)t;
            const uint32_t r = fdiv(u, f.W);
            const uint32_t s = fdiv(r, f.H);
            const uint32_t w32 = fdiv(s, f.d2);
            x = u - r * f.W.d;
            y = r - s * f.H.d;
            z = s - w32 * f.d2.d;
            w = w32;
        } else {
            x = t % g.W;
            const long long r = t / g.W;
            y = r % g.H;
            const long long s = r / g.H;
            z = s % g.d2;
            w = s / g.d2;
        }
        const long long s = z + g.d2 * w;
        const long long o = x * g.os[0] + y * g.os[1] + z * g.os[2] + w * g.os[3];
        // patches with winx*sx - px <= x <= winx*sx - px + wx - 1, likewise in y
        const long long ax = x + g.px, ay = y + g.py;
        const long long x_lo = ax - g.wx + 1 > 0 ? (ax - g.wx + 1 + g.sx - 1) / g.sx : 0;
        const long long y_lo = ay - g.wy + 1 > 0 ? (ay - g.wy + 1 + g.sy - 1) / g.sy : 0;
        long long x_hi = ax >= 0 ? ax / g.sx : -1;  // af_wrap allows negative padding
        long long y_hi = ay >= 0 ? ay / g.sy : -1;
        if (x_hi > g.nx - 1) x_hi = g.nx - 1;
        if (y_hi > g.ny - 1) y_hi = g.ny - 1;
        T acc = g.zero_init ? pzero<T>() : out[o];
        for (long long wy_ = y_lo; wy_ <= y_hi; ++wy_) {
            const long long ky = ay - wy_ * g.sy;
            for (long long wx_ = x_lo; wx_ <= x_hi; ++wx_) {
                const long long kx = ax - wx_ * g.sx;
                const long long k = kx + g.wx * ky, col = wx_ + g.nx * wy_;
                const long long idx = g.is_column ? k + wsz * (col + np * s) : col + np * (k + wsz * s);
                acc = padd<T>(acc, in[idx]);
            }
        }
        out[o] = acc;
    }
}

static PatchDivs patch_divs(const PatchGeom &g) {
    auto d = [](long long v) { return make_fastdiv((uint32_t)std::max<long long>(v, 1)); };
    return PatchDivs{d(g.wx * g.wy), d(g.nx * g.ny), d(g.nx), d(g.wx), d(g.W), d(g.H), d(g.d2)};
}

static constexpr long long kFastLimit = 1ll << 31;

template <typename T>
static void launch_unwrap(const Array &in, Array &out, const PatchGeom &g) {
    const long long total = g.wx * g.wy * g.nx * g.ny * g.slices;
    if (total == 0) return;
    const unsigned blocks = (unsigned)std::min<long long>((total + 255) / 256, (long long)num_sms() * 16);
    const PatchDivs f = patch_divs(g);
    {
        KernelTimer kt("unwrap_kernel");
        if (total < kFastLimit)
            unwrap_kernel<T, true><<<blocks, 256, 0, stream()>>>(in.ptr<T>(), out.ptr<T>(), g, f);
        else
            unwrap_kernel<T, false><<<blocks, 256, 0, stream()>>>(in.ptr<T>(), out.ptr<T>(), g, f);
    }
    count_launch();
    AFGB_POST_LAUNCH("unwrap_kernel");
}

template <typename T>
static void launch_wrap(const Array &in, Array &out, const PatchGeom &g) {
    const long long total = g.W * g.H * g.slices;
    if (total == 0) return;
    const unsigned blocks = (unsigned)std::min<long long>((total + 255) / 256, (long long)num_sms() * 16);
    const PatchDivs f = patch_divs(g);
    {
        KernelTimer kt("wrap_kernel");
        if (total < kFastLimit)
            wrap_kernel<T, true><<<blocks, 256, 0, stream()>>>(in.ptr<T>(), out.ptr<T>(), g, f);
        else
            wrap_kernel<T, false><<<blocks, 256, 0, stream()>>>(in.ptr<T>(), out.ptr<T>(), g, f);
    }
    count_launch();
    AFGB_POST_LAUNCH("wrap_kernel");
}

#define AFGB_PATCH_DISPATCH(t, FN, ...)               \
    switch (t) {                                      \
        case f32: FN<float>(__VA_ARGS__); break;      \
        case f64: FN<double>(__VA_ARGS__); break;     \
        case c32: FN<cf32>(__VA_ARGS__); break;       \
        case c64: FN<cf64>(__VA_ARGS__); break;       \
        case s32: FN<int>(__VA_ARGS__); break;        \
        case u32: FN<unsigned>(__VA_ARGS__); break;   \
        case s64: FN<long long>(__VA_ARGS__); break;  \
        case u64: FN<unsigned long long>(__VA_ARGS__); break; \
        case s16: FN<short>(__VA_ARGS__); break;      \
        case u16: FN<unsigned short>(__VA_ARGS__); break; \
        case s8: FN<int8_t>(__VA_ARGS__); break;      \
        case u8: FN<uint8_t>(__VA_ARGS__); break;     \
        case b8: FN<int8_t>(__VA_ARGS__); break;      \
        default: AFGB_TYPE_ERROR(1, t);               \
    }

void patches_unwrap(const Array &in, Array &out, long long wx, long long wy, long long sx,
                    long long sy, long long px, long long py, bool is_column) {
    PatchGeom g;
    g.W = in.dims[0];
    g.H = in.dims[1];
    g.wx = wx; g.wy = wy; g.sx = sx; g.sy = sy; g.px = px; g.py = py;
    g.nx = (g.W + 2 * px - wx) / sx + 1;
    g.ny = (g.H + 2 * py - wy) / sy + 1;
    g.slices = in.dims[2] * in.dims[3];
    g.d2 = in.dims[2] > 0 ? in.dims[2] : 1;
    g.is_column = is_column ? 1 : 0;
    g.zero_init = 0;
    AFGB_PATCH_DISPATCH(in.type, launch_unwrap, in, out, g);
}

void patches_wrap(const Array &in, Array &out, long long wx, long long wy, long long sx,
                  long long sy, long long px, long long py, bool is_column, bool zero_init) {
    PatchGeom g;
    g.W = out.dims[0];
    g.H = out.dims[1];
    g.wx = wx; g.wy = wy; g.sx = sx; g.sy = sy; g.px = px; g.py = py;
    g.nx = (g.W + 2 * px - wx) / sx + 1;
    g.ny = (g.H + 2 * py - wy) / sy + 1;
    g.slices = out.dims[2] * out.dims[3];
    g.d2 = out.dims[2] > 0 ? out.dims[2] : 1;
    for (int i = 0; i < 4; ++i) g.os[i] = out.strides[i];
    g.is_column = is_column ? 1 : 0;
    g.zero_init = zero_init ? 1 : 0;
    AFGB_PATCH_DISPATCH(in.type, launch_wrap, in, out, g);
}

}  // namespace afgb
