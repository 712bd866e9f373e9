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

// elements per 16-byte vector of T (1 for 16-byte complex double)
template <typename T> constexpr int vec_of() { return sizeof(T) >= 16 ? 1 : 16 / (int)sizeof(T); }

template <typename T> struct alignas(16) VecT { T v[vec_of<T>()]; };

// VEC consecutive output elements per thread: the first element's (k, col,
// slice) comes from one decomposition, the rest by stepping the counters, and
// the VEC values leave in one 16-byte store (scalar stores for the tail or an
// unaligned output)
template <typename T, bool FAST>
__global__ void __launch_bounds__(256) unwrap_kernel(const T *__restrict__ in, T *__restrict__ out,
                                                     PatchGeom g, PatchDivs f, int vec_store) {
    constexpr int VEC = vec_of<T>();
    const long long wsz = g.wx * g.wy, np = g.nx * g.ny;
    const long long total = wsz * np * g.slices;
    const long long nvec = (total + VEC - 1) / VEC;
    for (long long v = blockIdx.x * (long long)blockDim.x + threadIdx.x; v < nvec;
         v += (long long)gridDim.x * blockDim.x) {
        const long long t0 = v * VEC;
        long long k, col, s;
        if constexpr (FAST) {
            const uint32_t u = (uint32_t)t0;
            if (g.is_column) {  // out[k + wsz*(col + np*s)]
                const uint32_t r = fdiv(u, f.wsz);
                k = u - r * f.wsz.d;
                const uint32_t s32 = fdiv(r, f.np);
                col = r - s32 * f.np.d;
                s = s32;
            } else {            // out[col + np*(k + wsz*s)]
                const uint32_t r = fdiv(u, f.np);
                col = u - r * f.np.d;
                const uint32_t s32 = fdiv(r, f.wsz);
                k = r - s32 * f.wsz.d;
                s = s32;
            }
        } else {
            if (g.is_column) {
                k = t0 % wsz;
                const long long r = t0 / wsz;
                col = r % np;
                s = r / np;
            } else {
                col = t0 % np;
                const long long r = t0 / np;
                k = r % wsz;
                s = r / wsz;
            }
        }
        long long winy = col / g.nx, winx = col - winy * g.nx;
        long long ky = k / g.wx, kx = k - ky * g.wx;
        VecT<T> o;
#pragma unroll
        for (int j = 0; j < VEC; ++j) {
            const long long x = winx * g.sx - g.px + kx;
            const long long y = winy * g.sy - g.py + ky;
            T val = pzero<T>();
            if (x >= 0 && x < g.W && y >= 0 && y < g.H && s < g.slices)
                val = in[x + g.W * (y + g.H * s)];
            o.v[j] = val;
            // step to the next output element
            if (g.is_column) {
                if (++kx == g.wx) {
                    kx = 0;
                    if (++ky == g.wy) {
                        ky = 0;
                        if (++winx == g.nx) {
                            winx = 0;
                            if (++winy == g.ny) { winy = 0; ++s; }
                        }
                    }
                }
            } else {
                if (++winx == g.nx) {
                    winx = 0;
                    if (++winy == g.ny) {
                        winy = 0;
                        if (++kx == g.wx) {
                            kx = 0;
                            if (++ky == g.wy) { ky = 0; ++s; }
                        }
                    }
                }
            }
        }
        if (vec_store && t0 + VEC <= total) {
            *reinterpret_cast<VecT<T> *>(out + t0) = o;
        } else {
#pragma unroll
            for (int j = 0; j < VEC; ++j)
                if (t0 + j < total) out[t0 + j] = o.v[j];
        }
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

// af_wrap with is_column on a TX x TY pixel tile of one slice: the patches
// covering the tile are, row by row of windows, contiguous runs of
// wsz * nwx elements; the block stages them in shared memory with 16-byte
// copies (each row keeps its global 16-byte phase, so the copies stay
// aligned), then each thread sums its pixels' patch elements in col order
// from shared memory
constexpr int WT_X = 32, WT_Y = 32, WT_THREADS = 256;

struct WrapTile {
    int tiles_x, tiles_y;
    int nwx_max, nwy_max;
    int run_pad;          // staged row pitch (elements, a multiple of VEC)
};

__host__ __device__ inline long long cdiv_pos(long long a, long long b) { return (a + b - 1) / b; }

template <typename T>
__global__ void __launch_bounds__(WT_THREADS) wrap_tiled_kernel(const T *__restrict__ in,
                                                                T *__restrict__ out, PatchGeom g,
                                                                WrapTile wt) {
    constexpr int VEC = vec_of<T>();
    extern __shared__ __align__(16) unsigned char wrap_smem[];
    T *sm = reinterpret_cast<T *>(wrap_smem);
    const long long wsz = g.wx * g.wy, np = g.nx * g.ny;
    long long tile = blockIdx.x;
    const int tx = (int)(tile % wt.tiles_x);
    tile /= wt.tiles_x;
    const int ty = (int)(tile % wt.tiles_y);
    const long long s = tile / wt.tiles_y;
    const long long x0 = (long long)tx * WT_X, y0 = (long long)ty * WT_Y;
    const long long x1 = min(x0 + WT_X, g.W) - 1, y1 = min(y0 + WT_Y, g.H) - 1;
    // windows covering any pixel of the tile
    const long long ax0 = x0 + g.px, ay0 = y0 + g.py, ax1 = x1 + g.px, ay1 = y1 + g.py;
    const long long wx_lo = ax0 - g.wx + 1 > 0 ? cdiv_pos(ax0 - g.wx + 1, g.sx) : 0;
    const long long wy_lo = ay0 - g.wy + 1 > 0 ? cdiv_pos(ay0 - g.wy + 1, g.sy) : 0;
    const long long wx_hi = min(ax1 >= 0 ? ax1 / g.sx : -1, g.nx - 1);
    const long long wy_hi = min(ay1 >= 0 ? ay1 / g.sy : -1, g.ny - 1);
    const int nwx = (int)max(0ll, wx_hi - wx_lo + 1), nwy = (int)max(0ll, wy_hi - wy_lo + 1);
    const int run = (int)wsz * nwx;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // stage: window row rr of the tile -> sm[rr*run_pad + phase(rr) + e], e < run
    for (int rr = warp; rr < nwy; rr += WT_THREADS / 32) {
        const long long gstart = wsz * (wx_lo + g.nx * (wy_lo + rr) + np * s);
        const int phase = (int)(gstart & (VEC - 1));
        const T *src = in + (gstart - phase);
        T *dst = sm + rr * wt.run_pad;
        const int nchunks = (phase + run + VEC - 1) / VEC;
        for (int c = lane; c < nchunks; c += 32) {
            const int e0 = c * VEC - phase;
            if (e0 >= 0 && e0 + VEC <= run) {
                *reinterpret_cast<VecT<T> *>(dst + c * VEC) =
                    *reinterpret_cast<const VecT<T> *>(src + c * VEC);
            } else {
#pragma unroll
                for (int j = 0; j < VEC; ++j)
                    if (e0 + j >= 0 && e0 + j < run) dst[c * VEC + j] = src[c * VEC + j];
            }
        }
    }
    __syncthreads();
    const int lx = threadIdx.x & (WT_X - 1);
    for (int ly = threadIdx.x / WT_X; ly < WT_Y; ly += WT_THREADS / WT_X) {
        const long long x = x0 + lx, y = y0 + ly;
        if (x > x1 || y > y1) continue;
        const long long ax = x + g.px, ay = y + g.py;
        const long long px_lo = ax - g.wx + 1 > 0 ? cdiv_pos(ax - g.wx + 1, g.sx) : 0;
        const long long py_lo = ay - g.wy + 1 > 0 ? cdiv_pos(ay - g.wy + 1, g.sy) : 0;
        const long long px_hi = min(ax >= 0 ? ax / g.sx : -1, g.nx - 1);
        const long long py_hi = min(ay >= 0 ? ay / g.sy : -1, g.ny - 1);
        const long long z = s % g.d2, w = s / g.d2;
        const long long o = x * g.os[0] + y * g.os[1] + z * g.os[2] + w * g.os[3];
        T acc = g.zero_init ? pzero<T>() : out[o];
        for (long long wy_ = py_lo; wy_ <= py_hi; ++wy_) {
            const int rr = (int)(wy_ - wy_lo);
            const long long gstart = wsz * (wx_lo + g.nx * wy_ + np * s);
            const T *row = sm + rr * wt.run_pad + (int)(gstart & (VEC - 1));
            const int ky = (int)(ay - wy_ * g.sy);
            for (long long wx_ = px_lo; wx_ <= px_hi; ++wx_) {
                const int kx = (int)(ax - wx_ * g.sx);
                acc = padd<T>(acc, row[kx + (int)g.wx * ky + (int)wsz * (int)(wx_ - wx_lo)]);
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
    constexpr int VEC = vec_of<T>();
    const long long total = g.wx * g.wy * g.nx * g.ny * g.slices;
    if (total == 0) return;
    const long long nvec = (total + VEC - 1) / VEC;
    const unsigned blocks = (unsigned)std::min<long long>((nvec + 255) / 256, (long long)num_sms() * 16);
    const PatchDivs f = patch_divs(g);
    const int vec_store = ((uintptr_t)out.data() % 16) == 0;
    {
        KernelTimer kt("unwrap_kernel");
        if (total < kFastLimit)
            unwrap_kernel<T, true><<<blocks, 256, 0, stream()>>>(in.ptr<T>(), out.ptr<T>(), g, f,
                                                                 vec_store);
        else
            unwrap_kernel<T, false><<<blocks, 256, 0, stream()>>>(in.ptr<T>(), out.ptr<T>(), g, f,
                                                                  vec_store);
    }
    count_launch();
    AFGB_POST_LAUNCH("unwrap_kernel");
}

// the tiled kernel when the window rows of a tile fit in 64 KB of shared
// memory, the patch matrix starts on a 16-byte boundary and the tile count
// fits a grid
static bool wrap_tiled_plan(const PatchGeom &g, size_t esize, const void *in, WrapTile &wt,
                            size_t &smem) {
    if (!g.is_column || ((uintptr_t)in % 16) != 0) return false;
    const long long vec = esize >= 16 ? 1 : 16 / (long long)esize;
    wt.tiles_x = (int)((g.W + WT_X - 1) / WT_X);
    wt.tiles_y = (int)((g.H + WT_Y - 1) / WT_Y);
    const long long nwx = std::min<long long>((WT_X + g.wx - 2) / g.sx + 1, g.nx);
    const long long nwy = std::min<long long>((WT_Y + g.wy - 2) / g.sy + 1, g.ny);
    if (nwx <= 0 || nwy <= 0) return false;
    const long long run_pad = (g.wx * g.wy * nwx + 2 * vec - 1) / vec * vec;
    smem = (size_t)(run_pad * nwy) * esize;
    const long long blocks = (long long)wt.tiles_x * wt.tiles_y * g.slices;
    if (smem > 64 * 1024 || blocks > 0x7fffffffll || run_pad * nwy > 0x7fffffffll) return false;
    wt.nwx_max = (int)nwx;
    wt.nwy_max = (int)nwy;
    wt.run_pad = (int)run_pad;
    return true;
}

template <typename T>
static void launch_wrap(const Array &in, Array &out, const PatchGeom &g) {
    const long long total = g.W * g.H * g.slices;
    if (total == 0) return;
    WrapTile wt;
    size_t smem = 0;
    if (wrap_tiled_plan(g, sizeof(T), in.data(), wt, smem)) {
        const unsigned blocks = (unsigned)((long long)wt.tiles_x * wt.tiles_y * g.slices);
        AFGB_CUDA(cudaFuncSetAttribute(wrap_tiled_kernel<T>,
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        {
            KernelTimer kt("wrap_tiled_kernel");
            wrap_tiled_kernel<T><<<blocks, WT_THREADS, smem, stream()>>>(in.ptr<T>(), out.ptr<T>(),
                                                                         g, wt);
        }
        count_launch();
        AFGB_POST_LAUNCH("wrap_tiled_kernel");
        return;
    }
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
