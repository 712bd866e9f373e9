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
#include <cstdlib>

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
    FastDiv wsz, np, nx, wx, W, H, d2, sx, sy;
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

// asynchronous global -> shared copy of one element (cp.async for 4-, 8- and
// 16-byte types, zero-filled when !valid; a plain load for 1- and 2-byte types),
// so a staging loop issues all its loads before waiting on any
template <typename T>
__device__ __forceinline__ void stage_elem(T *dst, const T *src, bool valid) {
    if constexpr (sizeof(T) >= 4) {
        const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
        const int n = valid ? (int)sizeof(T) : 0;
        if constexpr (sizeof(T) == 16)
            asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(n)
                         : "memory");
        else
            asm volatile("cp.async.ca.shared.global [%0], [%1], %2, %3;" ::"r"(d), "l"(src),
                         "n"((int)sizeof(T)), "r"(n)
                         : "memory");
    } else {
        *dst = valid ? *src : pzero<T>();
    }
}
// 16 bytes at once (both addresses 16-byte aligned)
__device__ __forceinline__ void stage16(void *dst, const void *src) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void stage_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// af_unwrap by window rows: a unit is one slice, nr <= R consecutive window
// rows and a chunk of nc <= ncols windows of each.  The block stages the
// (nr-1)*sy + wy input rows the unit reads (zero outside the image) in shared
// memory with asynchronous copies, then writes the unit's outputs -- per window
// row one contiguous run in the column layout, per tap runs of nc in the row
// layout -- one warp per run, each element read from shared memory through a
// per-tap offset table.  All per-element arithmetic is 32-bit and incremental.
struct UnwrapPlan {
    int ncols, nchunks, rows, nrowgroups, span_pad;
    long long units;
};

template <typename T, bool COL>
__global__ void __launch_bounds__(256) unwrap_rows_kernel(const T *__restrict__ in,
                                                          T *__restrict__ out, PatchGeom g,
                                                          UnwrapPlan up) {
    extern __shared__ __align__(16) unsigned char uw_smem[];
    const int wx = (int)g.wx, wy = (int)g.wy, sx = (int)g.sx, sy = (int)g.sy, wsz = wx * wy;
    int *ktab = reinterpret_cast<int *>(uw_smem);
    T *sm = reinterpret_cast<T *>(uw_smem + ((wsz * 4 + 15) & ~15));
    for (int k = threadIdx.x; k < wsz; k += blockDim.x) ktab[k] = (k / wx) * up.span_pad + k % wx;
    const long long np = g.nx * g.ny;
    const int nthr = blockDim.x;
    const int rstride = sy * up.span_pad;  // shared-memory step between window rows
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, nwarps = blockDim.x >> 5;
    // (window, tap) of element `lane` of a column-layout run and its 32-element step
    const int b0 = lane / wsz, k0 = lane - b0 * wsz, db = 32 / wsz, dk = 32 - db * wsz;
    for (long long u = blockIdx.x; u < up.units; u += gridDim.x) {
        const int chunk = (int)(u % up.nchunks);
        const long long r1 = u / up.nchunks;
        const long long rg = r1 % up.nrowgroups, s = r1 / up.nrowgroups;
        const long long winy0 = rg * up.rows;
        const int nr = (int)min((long long)up.rows, g.ny - winy0);
        const int cx0 = chunk * up.ncols;
        const int nc = (int)min((long long)up.ncols, g.nx - cx0);
        const long long xs = (long long)cx0 * g.sx - g.px, ys = winy0 * g.sy - g.py;
        const int span = (nc - 1) * sx + wx;
        const int rows_in = (nr - 1) * sy + wy;
        __syncthreads();  // the previous unit's readers are done (and ktab is written)
        for (int ry = 0; ry < rows_in; ++ry) {
            const long long y = ys + ry;
            const bool yok = y >= 0 && y < g.H;
            const T *row = in + g.W * ((yok ? y : 0) + g.H * s);
            for (int xx = threadIdx.x; xx < span; xx += nthr) {
                const long long x = xs + xx;
                const bool ok = yok && x >= 0 && x < g.W;
                stage_elem<T>(sm + ry * up.span_pad + xx, ok ? row + x : in, ok);
            }
        }
        stage_wait();
        __syncthreads();
        // one warp per output run: in the column layout a run is one window
        // row's wsz*nc elements (e = b*wsz + k, the lane's (b, k) stepping by
        // 32 elements); in the row layout one tap's nc windows of one row
        if constexpr (COL) {
            const int L = wsz * nc;
            for (int a = warp; a < nr; a += nwarps) {
                T *o = out + wsz * (cx0 + g.nx * (winy0 + a) + np * s);
                const T *srow = sm + a * rstride;
                int b = b0, k = k0;
#pragma unroll 4
                for (int e = lane; e < L; e += 32) {
                    o[e] = srow[ktab[k] + b * sx];
                    k += dk;
                    b += db;
                    if (k >= wsz) { k -= wsz; ++b; }
                }
            }
        } else {
            const int nrun = wsz * nr;
            for (int rn = warp; rn < nrun; rn += nwarps) {
                const int k = rn / nr, a = rn - k * nr;
                T *o = out + (cx0 + g.nx * (winy0 + a)) + np * (k + (long long)wsz * s);
                const T *src = sm + a * rstride + ktab[k];
#pragma unroll 4
                for (int c = lane; c < nc; c += 32) o[c] = src[c * sx];
            }
        }
    }
}

// Windows covering pixel coordinate a (already offset by the padding) along
// one axis: lo..hi, empty when hi < lo.  32-bit, divisions by multiply-high;
// valid while |a| + w + s < 2^31.
__device__ __forceinline__ void covering(int a, int w, int n, const FastDiv &fs, int &lo, int &hi) {
    lo = a - w + 1 > 0 ? (int)fdiv((uint32_t)(a - w + fs.d), fs) : 0;
    hi = a >= 0 ? min((int)fdiv((uint32_t)a, fs), n - 1) : -1;
}

// acc + the patch elements of one pixel in col order: window rows r = 0..nr-1
// (first element at p + r*row_step) of cnt windows each (next window at
// + win_step).  Elements are loaded WB at a time before they are added, so
// WB loads are in flight per thread; the additions keep their order.
constexpr int WB = 8;
template <typename T, typename Off>
__device__ __forceinline__ T sum_patch_elems(T acc, const T *p, int nr, int cnt, Off row_step,
                                             Off win_step) {
    const int total = nr * cnt;
    int j = 0;
    const T *rowp = p;
    for (int t0 = 0; t0 < total; t0 += WB) {
        T v[WB];
#pragma unroll
        for (int i = 0; i < WB; ++i) {
            if (t0 + i < total) {
                v[i] = rowp[(Off)j * win_step];
                if (++j == cnt) {
                    j = 0;
                    rowp += row_step;
                }
            }
        }
#pragma unroll
        for (int i = 0; i < WB; ++i)
            if (t0 + i < total) acc = padd<T>(acc, v[i]);
    }
    return acc;
}

// the same for at most 4 x 4 covering windows (every stride >= window/4, so
// 3x3 at stride 1 included): a fully unrolled, predicated 4 x 4 loop, all
// loads issued before the adds, offsets from precomputed row and window steps
template <typename T, typename Off>
__device__ __forceinline__ T sum_patch_small(T acc, const T *p, int nr, int cnt, Off row_step,
                                             Off win_step) {
    T v[16];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (r < nr && j < cnt) v[4 * r + j] = p[(Off)r * row_step + (Off)j * win_step];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int j = 0; j < 4; ++j)
            if (r < nr && j < cnt) acc = padd<T>(acc, v[4 * r + j]);
    return acc;
}

template <typename T, typename Off>
__device__ __forceinline__ T sum_patch(T acc, const T *p, int nr, int cnt, Off row_step,
                                       Off win_step) {
    if (nr <= 4 && cnt <= 4) return sum_patch_small<T, Off>(acc, p, nr, cnt, row_step, win_step);
    return sum_patch_elems<T, Off>(acc, p, nr, cnt, row_step, win_step);
}

// af_wrap, column layout, on a TX x TY pixel tile of one slice.  The patches
// covering the tile are, row by row of windows, contiguous runs of
// wsz * nwx elements: the block stages them in shared memory with 16-byte
// asynchronous copies (each row keeps its global 16-byte phase, so the copies
// stay aligned), then each thread sums its pixels' patch elements in col
// order from shared memory, with 32-bit incremental indexing.
constexpr int WT_X = 32, WT_Y = 32, WT_THREADS = 256;

struct WrapTile {
    int tiles_x, tiles_y;
    int run_pad;          // staged window-row pitch (elements, a multiple of VEC)
};

template <typename T>
__global__ void __launch_bounds__(WT_THREADS) wrap_tiled_kernel(const T *__restrict__ in,
                                                                T *__restrict__ out, PatchGeom g,
                                                                PatchDivs f, WrapTile wt) {
    constexpr int VEC = vec_of<T>();
    extern __shared__ __align__(16) unsigned char wrap_smem[];
    T *sm = reinterpret_cast<T *>(wrap_smem);
    const int wx = (int)g.wx, wy = (int)g.wy, sx = (int)g.sx, sy = (int)g.sy, wsz = wx * wy;
    const int nx = (int)g.nx, ny = (int)g.ny;
    const long long np = g.nx * g.ny;
    long long tile = blockIdx.x;
    const int tx = (int)(tile % wt.tiles_x);
    tile /= wt.tiles_x;
    const int ty = (int)(tile % wt.tiles_y);
    const long long s = tile / wt.tiles_y;
    const int x0 = tx * WT_X, y0 = ty * WT_Y;
    const int x1 = min(x0 + WT_X, (int)g.W) - 1, y1 = min(y0 + WT_Y, (int)g.H) - 1;
    const int px = (int)g.px, py = (int)g.py;
    // windows covering any pixel of the tile
    int wx_lo, wx_hi, wy_lo, wy_hi, tmp;
    covering(x0 + px, wx, nx, f.sx, wx_lo, tmp);
    covering(x1 + px, wx, nx, f.sx, tmp, wx_hi);
    covering(y0 + py, wy, ny, f.sy, wy_lo, tmp);
    covering(y1 + py, wy, ny, f.sy, tmp, wy_hi);
    const int nwx = max(0, wx_hi - wx_lo + 1), nwy = max(0, wy_hi - wy_lo + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // window row rr -> sm[rr*run_pad + phase(rr) + e], e < wsz*nwx
    const int run = wsz * nwx;
    for (int rr = warp; rr < nwy; rr += WT_THREADS / 32) {
        const long long gstart = wsz * (wx_lo + (long long)nx * (wy_lo + rr) + np * s);
        const int phase = (int)(gstart & (VEC - 1));
        const T *src = in + (gstart - phase);
        T *dst = sm + rr * wt.run_pad;
        const int nchunks = (phase + run + VEC - 1) / VEC;
        for (int c = lane; c < nchunks; c += 32) {
            const int e0 = c * VEC - phase;
            if (e0 >= 0 && e0 + VEC <= run) {
                stage16(dst + c * VEC, src + c * VEC);
            } else {
#pragma unroll
                for (int j = 0; j < VEC; ++j)
                    if (e0 + j >= 0 && e0 + j < run) dst[c * VEC + j] = src[c * VEC + j];
            }
        }
    }
    stage_wait();
    __syncthreads();
    // row rr of windows starts at sm + rr*run_pad + phase(rr); phase(rr) =
    // (slice offset + wsz*(wx_lo + nx*(wy_lo + rr))) mod VEC
    const int phase0 =
        (int)((np * wsz * s + (long long)wsz * (wx_lo + (long long)nx * wy_lo)) & (VEC - 1));
    const int phase_step = (int)(((long long)wsz * nx) & (VEC - 1));
    const int step = wsz - sx;  // next window along x: tap x - sx, window + 1
    const int lx = threadIdx.x & (WT_X - 1);
    const long long z = s % g.d2, w = s / g.d2;
    T *oslice = out + z * g.os[2] + w * g.os[3];
    const int x = x0 + lx;
    if (x > x1) return;
    int cx_lo, cx_hi;
    covering(x + px, wx, nx, f.sx, cx_lo, cx_hi);
    const int cnt = cx_hi - cx_lo + 1;
    const int kx0 = x + px - cx_lo * sx, p0 = cx_lo - wx_lo;
    for (int ly = threadIdx.x / WT_X; ly < WT_Y; ly += WT_THREADS / WT_X) {
        const int y = y0 + ly;
        if (y > y1) break;
        int cy_lo, cy_hi;
        covering(y + py, wy, ny, f.sy, cy_lo, cy_hi);
        T *op = oslice + x * g.os[0] + y * g.os[1];
        T acc = g.zero_init ? pzero<T>() : *op;
        if (cnt > 0 && cy_hi >= cy_lo) {
            // staged rows are run_pad apart plus a per-row phase, so the rows
            // are summed one at a time unless every row has the same phase
            if (phase_step == 0) {
                const int rr = cy_lo - wy_lo;
                const int base = rr * wt.run_pad + phase0;
                const int ky = y + py - cy_lo * sy;
                acc = sum_patch<T, int>(acc, sm + base + kx0 + wx * ky + p0 * wsz,
                                        cy_hi - cy_lo + 1, cnt, wt.run_pad - wx * sy, step);
            } else {
                for (int wy_ = cy_lo; wy_ <= cy_hi; ++wy_) {
                    const int rr = wy_ - wy_lo;
                    const int ky = y + py - wy_ * sy;
                    const int base = rr * wt.run_pad + ((phase0 + rr * phase_step) & (VEC - 1));
                    acc = sum_patch<T, int>(acc, sm + base + kx0 + wx * ky + p0 * wsz, 1, cnt,
                                                  0, step);
                }
            }
        }
        *op = acc;
    }
}

// af_wrap, stride 1 and WX x WY windows (3 x 3: the NN im2col geometry): a
// tile is TY output rows across the whole image width.  The patches of the
// window rows covering it are contiguous in the patch matrix: one run of
// nwy rows x nx windows x WX*WY elements in the column layout, one run of
// nwy x nx windows per tap plane in the row layout.  The block stages the
// run(s) with 16-byte asynchronous copies (each run keeps its global 16-byte
// phase); then each thread sums its pixels' elements from shared memory,
// window rows ascending and windows along x ascending (the reference's
// order, as the tiled kernel sums them), with fixed offsets for interior
// pixels: about 180 instructions per pixel instead of the tiled kernel's 470.
// 8 warps (column layout) or 9 (row layout: one warp per tap plane's run)
constexpr int WS1_THREADS = 288;

template <typename T, int WX, int WY, bool COL>
__global__ void __launch_bounds__(WS1_THREADS) wrap_s1_kernel(const T *__restrict__ in,
                                                              T *__restrict__ out, PatchGeom g,
                                                              PatchDivs f, int TY, int tiles_y,
                                                              int pitch) {
    constexpr int WSZ = WX * WY;
    constexpr int VEC = vec_of<T>();
    extern __shared__ __align__(16) unsigned char wrap_smem[];
    T *sm = reinterpret_cast<T *>(wrap_smem);
    const int nx = (int)g.nx, ny = (int)g.ny, W = (int)g.W, H = (int)g.H;
    const int px = (int)g.px, py = (int)g.py;
    const long long np = g.nx * g.ny;
    const int ty = (int)(blockIdx.x % (unsigned)tiles_y);
    const long long s = blockIdx.x / (unsigned)tiles_y;
    const int y0 = ty * TY, y1 = min(y0 + TY, H) - 1;
    const int wy_lo = max(0, y0 + py - WY + 1), wy_hi = min(ny - 1, y1 + py);
    const int nwy = max(0, wy_hi - wy_lo + 1);
    // run q (COL: the one run; ROW: tap plane q) starts at global element
    // gs(q) and is staged at sm + q * pitch, its phase first
    auto gs = [&](int q) {
        return COL ? (long long)WSZ * ((long long)nx * wy_lo + np * s)
                   : np * ((long long)q + WSZ * s) + (long long)nx * wy_lo;
    };
    constexpr int NRUN = COL ? 1 : WSZ;
    const int run = (COL ? WSZ : 1) * nx * nwy;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (nwy > 0) {
        for (int q = COL ? 0 : warp; q < NRUN; q += (COL ? NRUN : (int)(blockDim.x >> 5))) {
            const long long g0 = gs(q);
            const int phase = (int)(g0 & (VEC - 1));
            const T *src = in + (g0 - phase);
            T *dst = sm + q * pitch;
            const int nchunks = (phase + run + VEC - 1) / VEC;
            const int t0 = COL ? threadIdx.x : lane, tstep = COL ? (int)blockDim.x : 32;
            for (int c = t0; c < nchunks; c += tstep) {
                const int e0 = c * VEC - phase;
                if (e0 >= 0 && e0 + VEC <= run) {
                    stage16(dst + c * VEC, src + c * VEC);
                } else {
#pragma unroll
                    for (int j = 0; j < VEC; ++j)
                        if (e0 + j >= 0 && e0 + j < run) dst[c * VEC + j] = src[c * VEC + j];
                }
            }
        }
    }
    stage_wait();
    __syncthreads();
    const long long z = s % g.d2, w = s / g.d2;
    T *oslice = out + z * g.os[2] + w * g.os[3];
    const int npix = (y1 - y0 + 1) * W;
    int pb[COL ? 1 : WSZ];  // row layout: tap plane k's staged window 0
#pragma unroll
    for (int k = 0; k < (COL ? 1 : WSZ); ++k) pb[k] = k * pitch + (int)(gs(k) & (VEC - 1));
    for (int qp = threadIdx.x; qp < npix; qp += blockDim.x) {
        const int ly = (int)fdiv((uint32_t)qp, f.W), x = qp - ly * W, y = y0 + ly;
        const int ax = x + px, ay = y + py;
        const int cx_lo = max(0, ax - WX + 1), cx_hi = min(nx - 1, ax);
        const int cy_lo = max(0, ay - WY + 1), cy_hi = min(ny - 1, ay);
        T *op = oslice + x * g.os[0] + y * g.os[1];
        T acc = g.zero_init ? pzero<T>() : *op;
        const int nr = cy_hi - cy_lo + 1, nc = cx_hi - cx_lo + 1;
        const bool full = nr == WY && nc == WX;
        if (COL) {
            // element of window (cx_lo, cy_lo) at tap (ax - cx_lo, ay - cy_lo);
            // next window along x: + WSZ - 1, next window row: + nx*WSZ - WX
            const T *p0 = sm + (int)(gs(0) & (VEC - 1)) + ((cy_lo - wy_lo) * nx + cx_lo) * WSZ +
                          (ax - cx_lo) + WX * (ay - cy_lo);
            const int rstep = nx * WSZ - WX;
            if (full) {
                T v[WSZ];
#pragma unroll
                for (int r = 0; r < WY; ++r)
#pragma unroll
                    for (int j = 0; j < WX; ++j) v[r * WX + j] = p0[r * rstep + j * (WSZ - 1)];
#pragma unroll
                for (int e = 0; e < WSZ; ++e) acc = padd<T>(acc, v[e]);
            } else {
#pragma unroll
                for (int r = 0; r < WY; ++r)
#pragma unroll
                    for (int j = 0; j < WX; ++j)
                        if (r < nr && j < nc) acc = padd<T>(acc, p0[r * rstep + j * (WSZ - 1)]);
            }
        } else {
            // window (cx_lo + j, cy_lo + r) holds the pixel at tap
            // (ax - cx_lo - j, ay - cy_lo - r), in that tap's plane
            const int wbase = (cy_lo - wy_lo) * nx + cx_lo;
            if (full) {  // interior: tap (WX-1-j, WY-1-r) of window (cx_lo + j, cy_lo + r)
                T v[WSZ];
#pragma unroll
                for (int r = 0; r < WY; ++r)
#pragma unroll
                    for (int j = 0; j < WX; ++j)
                        v[r * WX + j] = sm[pb[(WX - 1 - j) + WX * (WY - 1 - r)] + wbase + r * nx + j];
#pragma unroll
                for (int e = 0; e < WSZ; ++e) acc = padd<T>(acc, v[e]);
            } else {
                const int k0 = (ax - cx_lo) + WX * (ay - cy_lo);
                for (int r = 0; r < nr; ++r)
                    for (int j = 0; j < nc; ++j) {
                        const int k = k0 - j - WX * r;
                        acc = padd<T>(acc, sm[k * pitch + (int)(gs(k) & (VEC - 1)) + wbase + r * nx + j]);
                    }
            }
        }
        *op = acc;
    }
}

// af_wrap, row layout: one thread per pixel of a 32 x 8 tile, reading the
// patch elements straight from global memory -- for a given tap consecutive
// windows are consecutive elements, so a warp's reads coalesce when sx = 1 --
// with 32-bit window arithmetic and 64-bit incremental element offsets.
template <typename T>
__global__ void __launch_bounds__(256) wrap_rows_kernel(const T *__restrict__ in,
                                                        T *__restrict__ out, PatchGeom g,
                                                        PatchDivs f, WrapTile wt) {
    const int wx = (int)g.wx, wy = (int)g.wy, sx = (int)g.sx, sy = (int)g.sy, wsz = wx * wy;
    const int nx = (int)g.nx, ny = (int)g.ny;
    const long long np = g.nx * g.ny;
    long long tile = blockIdx.x;
    const int tx = (int)(tile % wt.tiles_x);
    tile /= wt.tiles_x;
    const int ty = (int)(tile % wt.tiles_y);
    const long long s = tile / wt.tiles_y;
    const int x = tx * 32 + (threadIdx.x & 31), y = ty * 8 + (threadIdx.x >> 5);
    if (x >= (int)g.W || y >= (int)g.H) return;
    const int ax = x + (int)g.px, ay = y + (int)g.py;
    int cx_lo, cx_hi, cy_lo, cy_hi;
    covering(ax, wx, nx, f.sx, cx_lo, cx_hi);
    covering(ay, wy, ny, f.sy, cy_lo, cy_hi);
    const long long z = s % g.d2, w = s / g.d2;
    T *op = out + x * g.os[0] + y * g.os[1] + z * g.os[2] + w * g.os[3];
    T acc = g.zero_init ? pzero<T>() : *op;
    const int cnt = cx_hi - cx_lo + 1;
    if (cnt > 0 && cy_hi >= cy_lo) {
        const T *slice = in + np * wsz * s;
        const int ky = ay - cy_lo * sy, kx = ax - cx_lo * sx;
        const T *pp = slice + (cx_lo + (long long)nx * cy_lo) + np * (kx + wx * ky);
        // next window along x: col + 1, tap - sx; next window row: col + nx, tap - wx*sy
        acc = sum_patch<T, long long>(acc, pp, cy_hi - cy_lo + 1, cnt,
                                      (long long)nx - np * wx * sy, 1 - (long long)sx * np);
    }
    *op = acc;
}

static PatchDivs patch_divs(const PatchGeom &g) {
    auto d = [](long long v) { return make_fastdiv((uint32_t)std::max<long long>(v, 1)); };
    return PatchDivs{d(g.wx * g.wy), d(g.nx * g.ny), d(g.nx), d(g.wx), d(g.W), d(g.H), d(g.d2),
                     d(g.sx), d(g.sy)};
}

static constexpr long long kFastLimit = 1ll << 31;

// the window-row kernel when a unit's input rows and tap table fit in 48 KB of
// shared memory: windows per unit halved until one window row fits, then up to
// 16 window rows per unit while they still fit
static bool unwrap_rows_plan(const PatchGeom &g, size_t esize, UnwrapPlan &up, size_t &smem) {
    const long long wsz = g.wx * g.wy;
    if (wsz > 16384 || g.wx > (1 << 20) || g.sx > (1 << 20) || g.sy > (1 << 20)) return false;
    const long long budget = 48 * 1024 - ((wsz * 4 + 15) & ~15ll);
    long long ncols = std::min<long long>(g.nx, 512);
    while (ncols >= 1) {
        const long long span = (ncols - 1) * g.sx + g.wx;
        const long long span_pad = (span + 3) / 4 * 4;
        if (g.wy * span_pad * (long long)esize <= budget) {
            long long rows = 1;
            while (rows < 16 && rows < g.ny &&
                   (rows * g.sy + g.wy) * span_pad * (long long)esize <= budget)
                ++rows;
            up.ncols = (int)ncols;
            up.nchunks = (int)((g.nx + ncols - 1) / ncols);
            up.rows = (int)rows;
            up.nrowgroups = (int)((g.ny + rows - 1) / rows);
            up.span_pad = (int)span_pad;
            up.units = (long long)up.nchunks * up.nrowgroups * g.slices;
            smem = (size_t)(((wsz * 4 + 15) & ~15ll) + ((rows - 1) * g.sy + g.wy) * span_pad *
                                                           (long long)esize);
            // per-element counters and offsets stay within 32 bits
            return wsz * ncols * rows < (1ll << 30) && (rows * g.sy + g.wy) * span_pad < (1ll << 30);
        }
        ncols /= 2;
    }
    return false;
}

template <typename T>
static void launch_unwrap(const Array &in, Array &out, const PatchGeom &g) {
    constexpr int VEC = vec_of<T>();
    const long long total = g.wx * g.wy * g.nx * g.ny * g.slices;
    if (total == 0) return;
    UnwrapPlan up;
    size_t smem = 0;
    if (unwrap_rows_plan(g, sizeof(T), up, smem)) {
        const unsigned blocks = (unsigned)std::min<long long>(up.units, (long long)num_sms() * 8);
        {
            KernelTimer kt("unwrap_rows_kernel");
            if (g.is_column)
                unwrap_rows_kernel<T, true><<<blocks, 256, smem, stream()>>>(in.ptr<T>(),
                                                                             out.ptr<T>(), g, up);
            else
                unwrap_rows_kernel<T, false><<<blocks, 256, smem, stream()>>>(in.ptr<T>(),
                                                                              out.ptr<T>(), g, up);
        }
        count_launch();
        AFGB_POST_LAUNCH("unwrap_rows_kernel");
        return;
    }
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

// the staged / row kernels when every coordinate, window count and offset
// they form in 32 bits stays below 2^30, and (column layout) the tile's staged
// windows fit in 64 KB of shared memory with the patch matrix on a 16-byte
// boundary
static bool wrap_tiled_plan(const PatchGeom &g, size_t esize, const void *in, WrapTile &wt,
                            size_t &smem) {
    const long long lim = 1ll << 30;
    if (g.W + std::llabs(g.px) + g.wx + g.sx >= lim || g.H + std::llabs(g.py) + g.wy + g.sy >= lim ||
        g.nx >= lim || g.ny >= lim || g.wx * g.wy >= lim)
        return false;
    const long long tx = g.is_column ? WT_X : 32, ty = g.is_column ? WT_Y : 8;
    wt.tiles_x = (int)((g.W + tx - 1) / tx);
    wt.tiles_y = (int)((g.H + ty - 1) / ty);
    wt.run_pad = 0;
    smem = 0;
    const long long blocks = (long long)wt.tiles_x * wt.tiles_y * g.slices;
    if (blocks > 0x7fffffffll) return false;
    if (!g.is_column) return true;
    if (((uintptr_t)in % 16) != 0) return false;
    const long long vec = esize >= 16 ? 1 : 16 / (long long)esize;
    const long long nwx = std::min<long long>((WT_X + g.wx - 2) / g.sx + 1, g.nx);
    const long long nwy = std::min<long long>((WT_Y + g.wy - 2) / g.sy + 1, g.ny);
    if (nwx <= 0 || nwy <= 0) return false;
    const long long run_pad = (g.wx * g.wy * nwx + 2 * vec - 1) / vec * vec;
    smem = (size_t)(run_pad * nwy) * esize;
    if (smem > 64 * 1024) return false;
    wt.run_pad = (int)run_pad;
    return true;
}

// the stride-1 3 x 3 kernel: row tiles up to 16 deep whose staged runs fit
// 48 KB (four blocks per SM), 32-bit offsets; `pitch` is the staged run pitch
// (elements, room for the phase) of the row layout's tap planes
static bool wrap_s1_plan(const PatchGeom &g, size_t esize, const void *in, int &TY, int &tiles_y,
                         int &pitch, size_t &smem) {
    if (g.sx != 1 || g.sy != 1 || g.wx != 3 || g.wy != 3) return false;
    if (((uintptr_t)in % 16) != 0 || g.W <= 0 || g.H <= 0 || g.nx <= 0 || g.ny <= 0) return false;
    if (g.W >= (1 << 24) || g.H >= (1 << 24) || std::llabs(g.px) > 2 || std::llabs(g.py) > 2) return false;
    const long long vec = esize >= 16 ? 1 : 16 / (long long)esize;
    const long long row_bytes = 9 * g.nx * (long long)esize;
    const long long budget = 48 * 1024 - 16 - 9 * 2 * vec * (long long)esize;
    TY = (int)std::min<long long>(16, budget / row_bytes - 2);
    if (TY < 1) return false;
    TY = (int)std::min<long long>(TY, g.H);
    tiles_y = (int)((g.H + TY - 1) / TY);
    if ((long long)tiles_y * g.slices > 0x7fffffffll) return false;
    if ((long long)(TY + 2) * g.W >= (1 << 30)) return false;
    const long long plane = (TY + 2) * g.nx;  // a tap plane's staged windows
    pitch = (int)((plane + 2 * vec - 1) / vec * vec);
    smem = g.is_column ? (size_t)((TY + 2) * row_bytes + 16) : (size_t)(9 * pitch) * esize;
    return true;
}

template <typename T>
static void launch_wrap(const Array &in, Array &out, const PatchGeom &g) {
    const long long total = g.W * g.H * g.slices;
    if (total == 0) return;
    WrapTile wt;
    size_t smem = 0;
    const PatchDivs f = patch_divs(g);
    int TY = 0, tiles_y = 0, pitch = 0;
    if (wrap_s1_plan(g, sizeof(T), in.data(), TY, tiles_y, pitch, smem)) {
        const unsigned blocks = (unsigned)((long long)tiles_y * g.slices);
        auto k = g.is_column ? wrap_s1_kernel<T, 3, 3, true> : wrap_s1_kernel<T, 3, 3, false>;
        AFGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        {
            KernelTimer kt("wrap_s1_kernel");
            k<<<blocks, g.is_column ? 256 : WS1_THREADS, smem, stream()>>>(in.ptr<T>(), out.ptr<T>(),
                                                                             g, f, TY, tiles_y, pitch);
        }
        count_launch();
        AFGB_POST_LAUNCH("wrap_s1_kernel");
        return;
    }
    if (wrap_tiled_plan(g, sizeof(T), in.data(), wt, smem)) {
        const unsigned blocks = (unsigned)((long long)wt.tiles_x * wt.tiles_y * g.slices);
        if (g.is_column) {
            AFGB_CUDA(cudaFuncSetAttribute(wrap_tiled_kernel<T>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            {
                KernelTimer kt("wrap_tiled_kernel");
                wrap_tiled_kernel<T><<<blocks, WT_THREADS, smem, stream()>>>(in.ptr<T>(),
                                                                             out.ptr<T>(), g, f, wt);
            }
            count_launch();
            AFGB_POST_LAUNCH("wrap_tiled_kernel");
        } else {
            {
                KernelTimer kt("wrap_rows_kernel");
                wrap_rows_kernel<T><<<blocks, 256, 0, stream()>>>(in.ptr<T>(), out.ptr<T>(), g, f,
                                                                  wt);
            }
            count_launch();
            AFGB_POST_LAUNCH("wrap_rows_kernel");
        }
        return;
    }
    const unsigned blocks = (unsigned)std::min<long long>((total + 255) / 256, (long long)num_sms() * 16);
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
