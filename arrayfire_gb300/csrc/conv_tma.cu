// TMA-staged direct convolutions (2-D filters and the fused separable pair)
// for dense, 16-byte-aligned f32 and 8-bit images.
//
// Each CTA is persistent: it walks output tiles (64 rows of 64 outputs, or
// of 128 for 7x7 filters) in an order shared by the grid (the separable
// kernel strides by the grid; the 2-D kernel takes runs of consecutive tiles
// per round), and one thread keeps the next tile's haloed input window in
// flight with a 3-D TMA box load (x, y, image) while the CTA computes the
// current one.  The TMA fills coordinates outside the image with zeros, which is the
// convolution's zero padding, so no thread computes an address or a bounds
// check for the input.  The box's x origin is rounded down to the 16-byte
// TMA alignment; the compute loops absorb that shift with compile-time
// indices.
//
// Arithmetic is the reference's (src/backend/cpu/kernel/convolve.hpp):
// products accumulate from zero with the outer-dimension taps outside and
// dim-0 taps inside.  Both kernels run one scalar FMA (exact mode: a rounded
// product and sum) per tap and output.  Packed f32x2 FMAs occupy the FMA pipe
// for two cycles, so they raise no FMA throughput on this part; their
// register-pair moves for odd-aligned windows cost issue slots, and both
// kernels measured slower with them.
#include <cuda.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "conv_common.cuh"
#include "conv_params.cuh"
#include "conv_tma.hpp"
#include "tc_ptx.cuh"

namespace afgb {
namespace dtma {

using tc::fence_barrier_init;
using tc::mbar_arrive_expect_tx;
using tc::mbar_init;
using tc::mbar_try_wait;
using tc::smem_u32;

constexpr int TILE = 64;
constexpr int THREADS = 256;
// tile buffers per CTA (one computed, the rest in flight): two for the 2-D
// kernel (its scalar-FMA form needs few registers, so shared memory sets the
// CTAs per SM: five at two 21 KB buffers, each CTA's next tile loading during
// a whole tile of compute); two for the separable kernel, whose shared temp
// image would otherwise cost a CTA per SM
constexpr int NST_2D = 2;
constexpr int NST_SEP = 2;
// separable temp-image pitch (floats): 17 16-byte words, odd for the same reason
constexpr int SEP_TP = TILE + 4;


// tile -> (x tile, y tile, batch) decoding shared by both kernels; every
// thread decodes its tile with a few multiply-high steps
struct TileGrid {
    FastDiv tx, ty;       // tiles along x, along y
    FastDiv b1, b2;       // batch extents of dims 2 and 3 (2-D kernel)
    int ntiles;
    int zstep[4];         // slice index step per batch coordinate (2-D kernel)
    FastDiv run;          // consecutive tiles per CTA and round (2-D kernel)
};
// tile of a CTA's k-th step in the 2-D kernel: rounds of `run` consecutive
// tiles per CTA (CTA c takes tiles c*run .. c*run + run-1 of each round of
// gridDim.x * run).  Consecutive tiles of a CTA then mostly share one image
// and its filter, and the CTAs running together still cover neighbouring
// tiles, whose shared halo rows meet in L2.  Increasing in k, so a CTA is
// done at its first tile past the end.
__device__ __forceinline__ int run_tile(int k, const FastDiv &run) {
    const int r = (int)fdiv((uint32_t)k, run);
    const int n = (int)run.d;
    return (r * (int)gridDim.x + (int)blockIdx.x) * n + (k - r * n);
}
struct TileRec {
    int tx, ty, z;
    long long out, filt;  // element offsets of the tile's output slice and filter
};
__device__ __forceinline__ TileRec decode_tile(int t, const TileGrid &tg, const long long *out_step,
                                               const long long *filt_step) {
    const uint32_t r = fdiv((uint32_t)t, tg.tx);
    const uint32_t b = fdiv(r, tg.ty);
    const uint32_t r2 = fdiv(b, tg.b1);
    const uint32_t b3 = fdiv(r2, tg.b2);
    const uint32_t b1 = b - r2 * tg.b1.d, b2 = r2 - b3 * tg.b2.d;
    TileRec tr;
    tr.tx = (int)((uint32_t)t - r * tg.tx.d);
    tr.ty = (int)(r - b * tg.ty.d);
    tr.z = (int)b1 * tg.zstep[1] + (int)b2 * tg.zstep[2] + (int)b3 * tg.zstep[3];
    tr.out = (long long)b1 * out_step[1] + (long long)b2 * out_step[2] + (long long)b3 * out_step[3];
    tr.filt = (long long)b1 * filt_step[1] + (long long)b2 * filt_step[2] +
              (long long)b3 * filt_step[3];
    return tr;
}

__device__ __forceinline__ void tma_load_3d(uint32_t dst, const CUtensorMap *map, uint64_t *bar,
                                            int c0, int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%3, %4, %5}], [%2];" ::"r"(dst),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(smem_u32(bar)), "r"(c0), "r"(c1), "r"(c2)
        : "memory");
}

// test hook (afgb_debug_wait_limit): when set, block 0 of the 2-D kernel
// issues no tile copies, so its consumers' bounded waits run out with no copy
// in flight
__device__ int g_debug_skip_block0 = 0;

// bounded wait on a TMA barrier; false (and the error word raised) on timeout
__device__ __forceinline__ bool wait_tile(uint64_t *bar, uint32_t parity) {
    unsigned n = 0;
    const unsigned limit = tc::g_spin_limit;
    while (!mbar_try_wait(bar, parity)) {
        if (++n > limit) {
            atomicOr(&tc::g_tc_error, 256u);
            return false;
        }
    }
    return true;
}

template <typename T> __device__ __forceinline__ float to_f(T v) { return (float)v; }



// geometry of a haloed tile for an F0 x F1 filter, TW outputs wide (shared by
// both kernels)
template <typename T, int F0, int F1, bool EXPAND, int TW = TILE>
struct Halo {
    static constexpr int ES = sizeof(T);
    static constexpr int A = 16 / ES;                 // TMA x alignment (elements)
    static constexpr int C0 = EXPAND ? 0 : F0 / 2;
    static constexpr int C1 = EXPAND ? 0 : F1 / 2;
    static constexpr int LX = F0 - 1 - C0;            // halo left of the tile
    static constexpr int LY = F1 - 1 - C1;            // halo above the tile
    static constexpr int LT = (LX + A - 1) / A * A;   // TMA lead (aligned)
    static constexpr int LF = (LX + 3) / 4 * 4;       // float tile lead
    static constexpr int OFF = LF - LX;               // window shift, 0..3
    static constexpr int BH = TILE + F1 - 1;
    // float tile pitch: covers the right halo; an odd number of 16-byte
    // words, so eight rows at the same column fall in eight different bank
    // groups (a conflict-free 128-bit access by eight lanes on eight rows)
    static constexpr int PF0 = (LF + TW + C0 + 3) / 4 * 4;
    static constexpr int PF = (PF0 / 4) % 2 ? PF0 : PF0 + 4;
    // TMA box width (elements); f32 loads straight into the float layout
    static constexpr int BW = ES == 4 ? PF : (LT + TW + C0 + A - 1) / A * A;
    static constexpr int TBYTES = BH * BW * ES;
    static constexpr int TB_ALIGNED = (TBYTES + 127) / 128 * 128;
    static constexpr int FT_BYTES = ES == 4 ? 0 : (BH * PF * 4 + 127) / 128 * 128;
};

// 8-bit tile -> float tile (shifted so that the float tile starts at x0 - LF),
// four bytes per shared load; LT, LF, BW and PF are multiples of four
template <typename T, typename H>
__device__ __forceinline__ void widen_tile(const T *tb, float *ft) {
    constexpr int SHIFT = H::LT - H::LF;
    constexpr int Q = H::PF / 4, BQ = H::BW / 4;
    static_assert(SHIFT % 4 == 0 && H::PF % 4 == 0 && H::BW % 4 == 0, "widening needs 4-byte words");
    const uint32_t *tw = reinterpret_cast<const uint32_t *>(tb);
    constexpr int RPP = THREADS / Q;  // rows per pass
    if (threadIdx.x >= RPP * Q) return;
    for (int r = threadIdx.x / Q; r < H::BH; r += RPP) {
        const int c4 = threadIdx.x % Q;
        const int src = c4 + SHIFT / 4;
        float4 o = make_float4(0.f, 0.f, 0.f, 0.f);
        if (src < BQ) {
            const uint32_t w = tw[r * BQ + src];
            if constexpr (std::is_same<T, uint8_t>::value) {
                o = make_float4((float)(w & 0xFFu), (float)((w >> 8) & 0xFFu),
                                (float)((w >> 16) & 0xFFu), (float)(w >> 24));
            } else {
                o = make_float4((float)(int8_t)(w & 0xFFu), (float)(int8_t)((w >> 8) & 0xFFu),
                                (float)(int8_t)((w >> 16) & 0xFFu), (float)(int8_t)(w >> 24));
            }
        }
        reinterpret_cast<float4 *>(ft)[r * Q + c4] = o;
    }
}

// ===========================================================================
// 2-D direct convolution, F0 x F1 filter, 64 x (64 CG) tile, 4 x 4 CG outputs
// per thread
// ===========================================================================
// Filters above 5x5 keep all their taps in registers at two CTAs per SM; under
// a three-CTA cap (85 registers) the 7x7 taps do not fit and are fetched again
// inside the tap loop.  They also take two 64-column groups per tile (CG = 2:
// a 128 x 64 tile, each thread 4 rows of columns 4 tx.. and 64 + 4 tx..): the
// per-tile work outside the FMAs (tile decode, waits, barrier, stores' address
// arithmetic) then spreads over twice the outputs, which matters where the
// FMAs alone already fill most issue slots (49 per output at 7x7).
template <typename T, int F0, int F1, bool EXACT> struct Conv2Shape {
    // the exact mode's separate products and sums leave room for one group
    static constexpr int CG = (!EXACT && F0 * F1 > 25) ? 2 : 1;
};
template <typename T, int F0, int F1, bool EXACT, bool EXPAND>
using Conv2Halo = Halo<T, F0, F1, EXPAND, TILE * Conv2Shape<T, F0, F1, EXACT>::CG>;

template <typename T, int F0, int F1, bool EXACT, bool EXPAND>
__global__ void __launch_bounds__(THREADS, (F0 * F1 > 25) ? 2 : 3)
    conv2_tma_kernel(const __grid_constant__ CUtensorMap smap,
                                                            const DirectParams p,
                                                            const TileGrid tg) {
    using H = Conv2Halo<T, F0, F1, EXACT, EXPAND>;
    constexpr int CG = Conv2Shape<T, F0, F1, EXACT>::CG;
    constexpr int TWX = TILE * CG;
    constexpr int NST = NST_2D;
    constexpr int NW4 = (H::OFF + 4 + F0 - 1 + 3) / 4;
    static_assert(TILE * (CG - 1) + 60 + 4 * NW4 <= H::PF, "window exceeds the tile pitch");
    extern __shared__ __align__(128) unsigned char sm[];
    auto tb = [&](int i) { return reinterpret_cast<T *>(sm + i * H::TB_ALIGNED); };
    float *ft = reinterpret_cast<float *>(sm + NST * H::TB_ALIGNED);
    uint64_t *full = reinterpret_cast<uint64_t *>(sm + NST * H::TB_ALIGNED + H::FT_BYTES);
    const int tid = threadIdx.x;

    if (tid == 0) {
        for (int i = 0; i < NST; ++i) mbar_init(&full[i], 1);
        fence_barrier_init();
    }
    __syncthreads();

    const bool skip_copies = g_debug_skip_block0 && blockIdx.x == 0;
    auto issue = [&](int t, int buf) {
        if (skip_copies) return;
        const TileRec tr = decode_tile(t, tg, p.out_step, p.filt_step);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive_expect_tx(&full[buf], H::TBYTES);
        tma_load_3d(smem_u32(tb(buf)), &smap, &full[buf], tr.tx * TWX - H::LT,
                    tr.ty * TILE - H::LY, tr.z);
    };

    if (tid == 0)
        for (int i = 0; i < NST - 1; ++i) {
            const int t = run_tile(i, tg.run);
            if (t < tg.ntiles) issue(t, i);
        }
    const int tx = tid & 15, ty = tid >> 4;
    // the taps stay in registers from tile to tile and are reloaded only when
    // a tile's filter differs from the previous one (consecutive tiles of a
    // CTA mostly belong to one image)
    long long cur_filt = -1;
    float wr[F0 * F1];
    for (int k = 0;; ++k) {
        const int tile = run_tile(k, tg.run);
        if (tile >= tg.ntiles) break;
        const int buf = k % NST;
        const int ahead = run_tile(k + NST - 1, tg.run);
        if (tid == 0 && ahead < tg.ntiles) issue(ahead, (k + NST - 1) % NST);
        const TileRec tr = decode_tile(tile, tg, p.out_step, p.filt_step);
        const int ttx = tr.tx, tty = tr.ty;
        const long long out_off = tr.out;
        // taps go to registers before the wait, overlapping the tile load
        if (tr.filt != cur_filt) {
            const float *w = static_cast<const float *>(p.filt) + tr.filt;
#pragma unroll
            for (int fj = 0; fj < F1; ++fj)
#pragma unroll
                for (int fi = 0; fi < F0; ++fi)
                    wr[fj * F0 + fi] = __ldg(w + fi * p.fs[0] + fj * p.fs[1]);
            cur_filt = tr.filt;
        }
        if (!wait_tile(&full[buf], (k / NST) & 1)) break;
        const float *tile_f;
        if (sizeof(T) == 4) {
            tile_f = reinterpret_cast<const float *>(tb(buf));
        } else {
            widen_tile<T, H>(tb(buf), ft);
            __syncthreads();
            tile_f = ft;
        }

        float acc[CG][4][4];
        // one scalar FMA (or, in the exact mode, a rounded product and sum) per
        // tap and output; fused mode only changes the rounding
#pragma unroll
        for (int g = 0; g < CG; ++g)
#pragma unroll
            for (int a = 0; a < 4; ++a)
#pragma unroll
                for (int c = 0; c < 4; ++c) acc[g][a][c] = 0.0f;
#pragma unroll
        for (int q = 3 + F1 - 1; q >= 0; --q) {
#pragma unroll
            for (int g = 0; g < CG; ++g) {
                float v[NW4 * 4];
                const float *row = tile_f + (4 * ty + q) * H::PF + TILE * g + 4 * tx;
#pragma unroll
                for (int u = 0; u < NW4; ++u) {
                    const float4 t4 = *reinterpret_cast<const float4 *>(row + 4 * u);
                    v[4 * u] = t4.x;
                    v[4 * u + 1] = t4.y;
                    v[4 * u + 2] = t4.z;
                    v[4 * u + 3] = t4.w;
                }
#pragma unroll
                for (int rr = 0; rr < 4; ++rr) {
                    const int fj = rr + F1 - 1 - q;
                    if (fj >= 0 && fj < F1) {
#pragma unroll
                        for (int fi = 0; fi < F0; ++fi) {
                            const float wv = wr[fj * F0 + fi];
#pragma unroll
                            for (int cc = 0; cc < 4; ++cc)
                                acc[g][rr][cc] =
                                    mac<EXACT>(acc[g][rr][cc], v[cc + H::OFF + F0 - 1 - fi], wv);
                        }
                    }
                }
            }
        }
        T *out = static_cast<T *>(p.out) + out_off;
        const bool row_vec = ((p.os[1] & 3) == 0) &&
                             ((reinterpret_cast<uintptr_t>(out) % (4 * sizeof(T))) == 0);
#pragma unroll
        for (int g = 0; g < CG; ++g) {
            const long long x = (long long)ttx * TWX + TILE * g + 4 * tx;
            const bool vec = row_vec && (x + 3 < p.od[0]);
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
                const long long y = (long long)tty * TILE + 4 * ty + rr;
                if (y >= p.od[1] || x >= p.od[0]) continue;
                T *dst = out + y * p.os[1] + x;
                if (vec) {
                    if constexpr (sizeof(T) == 4) {
                        *reinterpret_cast<float4 *>(dst) =
                            make_float4(acc[g][rr][0], acc[g][rr][1], acc[g][rr][2], acc[g][rr][3]);
                    } else {
                        const uint32_t w4 = (uint32_t)(uint8_t)from_acc<T>(acc[g][rr][0]) |
                                            ((uint32_t)(uint8_t)from_acc<T>(acc[g][rr][1]) << 8) |
                                            ((uint32_t)(uint8_t)from_acc<T>(acc[g][rr][2]) << 16) |
                                            ((uint32_t)(uint8_t)from_acc<T>(acc[g][rr][3]) << 24);
                        *reinterpret_cast<uint32_t *>(dst) = w4;
                    }
                } else {
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc)
                        if (x + cc < p.od[0]) dst[cc] = from_acc_any(acc[g][rr][cc], T{});
                }
            }
        }
        __syncthreads();  // this buffer is reloaded at the next iteration's issue
    }
}

// ===========================================================================
// fused separable convolution: column pass (dim 0) into a shared temp image,
// row pass (dim 1) to the output; CFL/RFL compile-time filter lengths
// ===========================================================================
template <typename T>
__device__ __forceinline__ float sep_tap(float f) {
    if constexpr (IsInt<T>::value) return (float)from_acc<T>(f);
    return f;
}
// InT(accum) of the separable passes.  8-bit inputs: taps and samples are
// integers, so every sum is an exact integer and the conversion reduces to
// saturation (NaN cannot arise).
template <typename T>
__device__ __forceinline__ float sep_round(float a) {
    if constexpr (std::is_same<T, uint8_t>::value) return fminf(fmaxf(a, 0.0f), 255.0f);
    if constexpr (std::is_same<T, int8_t>::value) return fminf(fmaxf(a, -128.0f), 127.0f);
    return a;
}

template <typename T, int CFL, int RFL, bool EXACT, bool EXPAND>
__global__ void __launch_bounds__(THREADS) sep_tma_kernel(const __grid_constant__ CUtensorMap smap,
                                                          const SepTmaParams p,
                                                          const TileGrid tg) {
    using H = Halo<T, CFL, RFL, EXPAND>;
    constexpr int NST = NST_SEP;
    constexpr int NWP = (H::OFF + 8 + CFL - 1 + 3) / 4;  // pass-1 window (float4 chunks)
    static_assert(56 + 4 * NWP <= H::PF, "window exceeds the tile pitch");
    extern __shared__ __align__(128) unsigned char sm[];
    auto tb = [&](int i) { return reinterpret_cast<T *>(sm + i * H::TB_ALIGNED); };
    float *ft = reinterpret_cast<float *>(sm + NST * H::TB_ALIGNED);
    float *temp = reinterpret_cast<float *>(sm + NST * H::TB_ALIGNED + H::FT_BYTES);  // BH x TP
    uint64_t *full = reinterpret_cast<uint64_t *>(temp + H::BH * SEP_TP);
    __shared__ float ctap[CFL], rtap[RFL];
    const int tid = threadIdx.x;

    if (tid == 0) {
        for (int i = 0; i < NST; ++i) mbar_init(&full[i], 1);
        fence_barrier_init();
    }
    if (tid < CFL) ctap[tid] = sep_tap<T>(p.cf[tid]);
    if (tid < RFL) rtap[tid] = sep_tap<T>(p.rf[tid]);
    __syncthreads();
    float cr[CFL], rr_[RFL];
#pragma unroll
    for (int f = 0; f < CFL; ++f) cr[f] = ctap[f];
#pragma unroll
    for (int f = 0; f < RFL; ++f) rr_[f] = rtap[f];

    auto issue = [&](int t, int buf) {
        const uint32_t r = fdiv((uint32_t)t, tg.tx);
        const uint32_t b = fdiv(r, tg.ty);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive_expect_tx(&full[buf], H::TBYTES);
        tma_load_3d(smem_u32(tb(buf)), &smap, &full[buf], (int)((uint32_t)t - r * tg.tx.d) * TILE - H::LT,
                    (int)(r - b * tg.ty.d) * TILE - H::LY, (int)b);
    };

    int tile = blockIdx.x;
    if (tid == 0)
        for (int i = 0; i < NST - 1; ++i)
            if (tile + i * (int)gridDim.x < tg.ntiles) issue(tile + i * (int)gridDim.x, i);
    for (int k = 0; tile < tg.ntiles; tile += gridDim.x, ++k) {
        const int buf = k % NST;
        const int ahead = tile + (NST - 1) * (int)gridDim.x;
        if (tid == 0 && ahead < tg.ntiles) issue(ahead, (k + NST - 1) % NST);
        const uint32_t tr_ = fdiv((uint32_t)tile, tg.tx);
        const uint32_t tb_ = fdiv(tr_, tg.ty);
        const int ttx = (int)((uint32_t)tile - tr_ * tg.tx.d), tty = (int)(tr_ - tb_ * tg.ty.d);
        const long long out_off = (long long)tb_ * p.out_slice;
        if (!wait_tile(&full[buf], (k / NST) & 1)) break;
        const float *tile_f;
        if (sizeof(T) == 4) {
            tile_f = reinterpret_cast<const float *>(tb(buf));
        } else {
            widen_tile<T, H>(tb(buf), ft);
            __syncthreads();
            tile_f = ft;
        }
        // pass 1: temp[row][x] = IN( sum_f tile[row][x + OFF + CFL-1-f] * c[f] ),
        // 8 consecutive x per item; rows outside the image stay zero (the
        // reference reads zero for them in its second pass)
        // Items go eight rows to a group of eight lanes (same 8-column group
        // g), so each 128-bit access of eight lanes hits eight bank groups.
        const long long y_top = (long long)tty * TILE - H::LY;
        constexpr int ITEMS = (H::BH + 7) / 8 * 64;
        for (int it = tid; it < ITEMS; it += THREADS) {
            const int row = (it >> 6) * 8 + (it & 7), g = (it >> 3) & 7;
            if (row >= H::BH) continue;
            const long long gy = y_top + row;
            float a[8];
#pragma unroll
            for (int e = 0; e < 8; ++e) a[e] = 0.0f;
            if (gy >= 0 && gy < p.sd1) {
                float v[NWP * 4];
                const float *src = tile_f + row * H::PF + 8 * g;
#pragma unroll
                for (int u = 0; u < NWP; ++u) {
                    const float4 t4 = *reinterpret_cast<const float4 *>(src + 4 * u);
                    v[4 * u] = t4.x;
                    v[4 * u + 1] = t4.y;
                    v[4 * u + 2] = t4.z;
                    v[4 * u + 3] = t4.w;
                }
#pragma unroll
                for (int f = 0; f < CFL; ++f) {
                    const int j0 = H::OFF + CFL - 1 - f;  // window index of output 0
#pragma unroll
                    for (int e = 0; e < 8; ++e) a[e] = mac<EXACT>(a[e], v[j0 + e], cr[f]);
                }
            }
#pragma unroll
            for (int e = 0; e < 8; ++e) a[e] = sep_round<T>(a[e]);
            float *trow = temp + row * SEP_TP + 8 * g;
            *reinterpret_cast<float4 *>(trow) = make_float4(a[0], a[1], a[2], a[3]);
            *reinterpret_cast<float4 *>(trow + 4) = make_float4(a[4], a[5], a[6], a[7]);
        }
        __syncthreads();
        // pass 2: out[x][y] = IN( sum_g temp[y + RFL-1-g][x] * r[g] ), 4x4 per thread
        const int tx = tid & 15, ty = tid >> 4;
        float acc[4][4];
#pragma unroll
        for (int rr = 0; rr < 4; ++rr)
#pragma unroll
            for (int cc = 0; cc < 4; ++cc) acc[rr][cc] = 0.0f;
#pragma unroll
        for (int q = 3 + RFL - 1; q >= 0; --q) {
            const float4 t4 = *reinterpret_cast<const float4 *>(temp + (4 * ty + q) * SEP_TP + 4 * tx);
            const float tv[4] = {t4.x, t4.y, t4.z, t4.w};
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
                const int g = rr + RFL - 1 - q;
                if (g >= 0 && g < RFL) {
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc) acc[rr][cc] = mac<EXACT>(acc[rr][cc], tv[cc], rr_[g]);
                }
            }
        }
        T *out = static_cast<T *>(p.out) + out_off;
        const long long x = (long long)ttx * TILE + 4 * tx;
        const bool vec = (x + 3 < p.od0) && ((p.od0 & 3) == 0) &&
                         ((reinterpret_cast<uintptr_t>(out) % (4 * sizeof(T))) == 0);
#pragma unroll
        for (int rr = 0; rr < 4; ++rr) {
            const long long y = (long long)tty * TILE + 4 * ty + rr;
            if (y >= p.od1 || x >= p.od0) continue;
            const float *o = acc[rr];
            T *dst = out + y * p.od0 + x;
            if (vec) {
                if constexpr (sizeof(T) == 4) {
                    *reinterpret_cast<float4 *>(dst) = make_float4(o[0], o[1], o[2], o[3]);
                } else {
                    const uint32_t w4 = (uint32_t)(uint8_t)(int)sep_round<T>(o[0]) |
                                        ((uint32_t)(uint8_t)(int)sep_round<T>(o[1]) << 8) |
                                        ((uint32_t)(uint8_t)(int)sep_round<T>(o[2]) << 16) |
                                        ((uint32_t)(uint8_t)(int)sep_round<T>(o[3]) << 24);
                    *reinterpret_cast<uint32_t *>(dst) = w4;
                }
            } else {
#pragma unroll
                for (int cc = 0; cc < 4; ++cc)
                    if (x + cc < p.od0) dst[cc] = from_acc_any(o[cc], T{});
            }
        }
        __syncthreads();
    }
}

// ===========================================================================
// fused separable convolution on 8-bit images with integer dot products
// ===========================================================================
// The reference's 8-bit semantics (src/backend/cpu/kernel/convolve.hpp:233,
// src/backend/cpu/convolve.cpp:88-97) keep the taps and the intermediate
// image in the input type, so every product and sum is a small exact
// integer: each pass is dp4a over four bytes of the window and four reversed
// taps, and InT(sum) is a clamp to the type's range.  The column pass
// writes its result transposed (tempT[x][row], bytes) so that the row pass
// reads its windows as consecutive bytes too.  Unaligned windows come from
// two aligned words with one byte_perm.
template <typename T>
__device__ __forceinline__ int dp4(uint32_t a, uint32_t b, int c) {
    if constexpr (std::is_same<T, uint8_t>::value) return (int)__dp4a(a, b, (unsigned)c);
    return __dp4a((int)a, (int)b, c);
}
template <typename T>
__device__ __forceinline__ uint32_t clamp_byte(int v) {
    if constexpr (std::is_same<T, uint8_t>::value) return (uint32_t)min(v, 255);
    return (uint32_t)(uint8_t)(int8_t)max(min(v, 127), -128);
}
// bytes k..k+3 of the 8-byte little-endian pair (lo, hi), k in 0..3
__device__ __forceinline__ uint32_t window_word(uint32_t lo, uint32_t hi, int k) {
    return k == 0 ? lo : __byte_perm(lo, hi, 0x3210u + 0x1111u * (uint32_t)k);
}
// reversed taps packed four to a word: word i holds taps L-1-4i .. L-4-4i
template <typename T, int L>
__device__ __forceinline__ void pack_taps(const float *f, uint32_t (&w)[(L + 3) / 4]) {
#pragma unroll
    for (int i = 0; i < (L + 3) / 4; ++i) {
        uint32_t v = 0;
#pragma unroll
        for (int e = 0; e < 4; ++e) {
            const int j = 4 * i + e;  // window position; tap index L-1-j
            const uint32_t b = j < L ? (uint32_t)(uint8_t)from_acc<T>(f[L - 1 - j]) : 0u;
            v |= b << (8 * e);
        }
        w[i] = v;
    }
}

// transposed intermediate pitch: every pass-2 word read stays in its row,
// and an odd word count spreads 32 lanes' rows over the banks
__host__ __device__ constexpr int sep8_pitch(int nrb, int nrw) {
    return (((nrb * 4 > 64 + 4 * nrw ? nrb * 4 : 64 + 4 * nrw) + 3) / 4 | 1) * 4;
}

template <typename T, int CFL, int RFL, bool EXPAND>
__global__ void __launch_bounds__(THREADS) sep_dp4a_kernel(const __grid_constant__ CUtensorMap smap,
                                                           const SepTmaParams p,
                                                           const TileGrid tg) {
    using H = Halo<T, CFL, RFL, EXPAND>;
    constexpr int NST = NST_SEP;
    constexpr int OFF8 = H::LT - H::LX;           // tile byte of output 0's window
    constexpr int NCW = (CFL + 3) / 4, NRW = (RFL + 3) / 4;
    constexpr int NA = (OFF8 % 4 + 3) / 4 + NCW + 1;  // aligned words per pass-1 row
    constexpr int NRB = (H::BH + 3) / 4;          // 4-row blocks of the tile
    constexpr int TPT = sep8_pitch(NRB, NRW);     // tempT pitch (bytes)
    // the bytes that meet nonzero taps lie inside the row; the aligned word
    // loads may run up to 8 bytes past it (into the next row, or the buffer
    // that follows the last one), where the packed taps are zero
    static_assert(TILE - 1 + OFF8 + CFL - 1 < H::BW, "window exceeds the tile row");
    static_assert(4 * (15 + OFF8 / 4 + NA) <= H::BW + 8, "pass-1 words exceed the row by too much");
    static_assert(4 * (TILE / 4 + NRW) <= TPT, "pass-2 words exceed the transposed pitch");
    extern __shared__ __align__(128) unsigned char sm[];
    auto tb = [&](int i) { return sm + i * H::TB_ALIGNED; };
    unsigned char *tempT = sm + NST * H::TB_ALIGNED;  // TILE rows (x) of TPT bytes (tile rows)
    uint64_t *full = reinterpret_cast<uint64_t *>(tempT + ((TILE * TPT + 127) / 128) * 128);
    const int tid = threadIdx.x;

    uint32_t cw[NCW], rw[NRW];
    pack_taps<T, CFL>(p.cf, cw);
    pack_taps<T, RFL>(p.rf, rw);
    if (tid == 0) {
        for (int i = 0; i < NST; ++i) mbar_init(&full[i], 1);
        fence_barrier_init();
    }
    __syncthreads();

    auto issue = [&](int t, int buf) {
        const uint32_t r = fdiv((uint32_t)t, tg.tx);
        const uint32_t b = fdiv(r, tg.ty);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive_expect_tx(&full[buf], H::TBYTES);
        tma_load_3d(smem_u32(tb(buf)), &smap, &full[buf], (int)((uint32_t)t - r * tg.tx.d) * TILE - H::LT,
                    (int)(r - b * tg.ty.d) * TILE - H::LY, (int)b);
    };

    int tile = blockIdx.x;
    if (tid == 0)
        for (int i = 0; i < NST - 1; ++i)
            if (tile + i * (int)gridDim.x < tg.ntiles) issue(tile + i * (int)gridDim.x, i);
    for (int k = 0; tile < tg.ntiles; tile += gridDim.x, ++k) {
        const int buf = k % NST;
        const int ahead = tile + (NST - 1) * (int)gridDim.x;
        if (tid == 0 && ahead < tg.ntiles) issue(ahead, (k + NST - 1) % NST);
        const uint32_t tr_ = fdiv((uint32_t)tile, tg.tx);
        const uint32_t tb_ = fdiv(tr_, tg.ty);
        const int ttx = (int)((uint32_t)tile - tr_ * tg.tx.d), tty = (int)(tr_ - tb_ * tg.ty.d);
        const long long out_off = (long long)tb_ * p.out_slice;
        if (!wait_tile(&full[buf], (k / NST) & 1)) break;
        const unsigned char *tile_b = tb(buf);

        // pass 1: a 4-row x 4-column block per item; column blocks fastest
        for (int it = tid; it < NRB * (TILE / 4); it += THREADS) {
            const int cb = it % (TILE / 4), rb = it / (TILE / 4);
            uint32_t res[4] = {0u, 0u, 0u, 0u};  // res[s]: rows 4rb..4rb+3 of column 4cb+s
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int row = 4 * rb + i;
                if (row >= H::BH) break;
                const uint32_t *src =
                    reinterpret_cast<const uint32_t *>(tile_b + row * H::BW) + cb + OFF8 / 4;
                uint32_t a[NA];
#pragma unroll
                for (int w = 0; w < NA; ++w) a[w] = src[w];
#pragma unroll
                for (int sidx = 0; sidx < 4; ++sidx) {
                    constexpr int R0 = OFF8 % 4;
                    const int q = (R0 + sidx) / 4, sh = (R0 + sidx) % 4;
                    int acc = 0;
#pragma unroll
                    for (int w = 0; w < NCW; ++w) acc = dp4<T>(window_word(a[q + w], a[q + w + 1], sh), cw[w], acc);
                    res[sidx] |= clamp_byte<T>(acc) << (8 * i);
                }
            }
#pragma unroll
            for (int sidx = 0; sidx < 4; ++sidx)
                *reinterpret_cast<uint32_t *>(tempT + (4 * cb + sidx) * TPT + 4 * rb) = res[sidx];
        }
        __syncthreads();
        // pass 2: 4 x by 4 y outputs per thread
        const int tx = tid & 15, ty = tid >> 4;
        uint32_t outw[4] = {0u, 0u, 0u, 0u};  // outw[s]: row 4ty+s, columns 4tx..4tx+3
#pragma unroll
        for (int c = 0; c < 4; ++c) {
            const uint32_t *src = reinterpret_cast<const uint32_t *>(tempT + (4 * tx + c) * TPT) + ty;
            uint32_t a[NRW + 1];
#pragma unroll
            for (int w = 0; w <= NRW; ++w) a[w] = src[w];
#pragma unroll
            for (int sidx = 0; sidx < 4; ++sidx) {
                int acc = 0;
#pragma unroll
                for (int w = 0; w < NRW; ++w) acc = dp4<T>(window_word(a[w], a[w + 1], sidx), rw[w], acc);
                outw[sidx] |= clamp_byte<T>(acc) << (8 * c);
            }
        }
        T *out = static_cast<T *>(p.out) + out_off;
        const long long x = (long long)ttx * TILE + 4 * tx;
        const bool vec = (x + 3 < p.od0) && ((p.od0 & 3) == 0) &&
                         ((reinterpret_cast<uintptr_t>(out) & 3) == 0);
#pragma unroll
        for (int sidx = 0; sidx < 4; ++sidx) {
            const long long y = (long long)tty * TILE + 4 * ty + sidx;
            if (y >= p.od1 || x >= p.od0) continue;
            T *dst = out + y * p.od0 + x;
            if (vec) {
                *reinterpret_cast<uint32_t *>(dst) = outw[sidx];
            } else {
#pragma unroll
                for (int c = 0; c < 4; ++c)
                    if (x + c < p.od0) dst[c] = (T)(uint8_t)(outw[sidx] >> (8 * c));
            }
        }
        __syncthreads();
    }
}

// ===========================================================================
// 3-D direct convolution, 3x3x3 f32 filter, persistent over 64x8x8 tiles
// ===========================================================================
// One 4-D TMA box (x, y, z, volume) brings a tile's haloed input block, the
// next tile's box in flight while the CTA computes the current one; the box's
// x origin is the tile origin minus 4 (16-byte aligned), so the window shift
// OFF = 4 - (2 - c0) is absorbed by compile-time indices, and coordinates
// outside the volume read as zero.  Each thread computes 4 x by 4 z outputs
// of one row: input planes high to low, dim-1 taps ascending, dim-0 taps
// inside (the reference order, src/backend/cpu/kernel/convolve.hpp:45-73).
constexpr int C3_BX = 64, C3_BY = 8, C3_BZ = 8;
constexpr int C3_PF = 76;              // box width: an odd number of 16-byte words
constexpr int C3_TH = C3_BY + 2, C3_TD = C3_BZ + 2;
constexpr int C3_BYTES = C3_PF * C3_TH * C3_TD * 4;
constexpr int C3_BUF = (C3_BYTES + 1023) / 1024 * 1024;  // TMA destinations stay 1024-aligned
// input boxes per CTA: the one computed and the next in flight, three CTAs
// per SM (three boxes at two CTAs per SM measured slower: 0.050 against
// 0.047 ms on 256^3)
constexpr int C3_NB = 2;

struct Conv3Tma {
    FastDiv ntx, nty, nz;    // tiles along x, y, z
    int ntiles;
    long long vstep;         // volume index step per batch
};

template <bool EXACT, bool EXPAND>
__global__ void __launch_bounds__(256) conv3_tma_kernel(const __grid_constant__ CUtensorMap smap,
                                                        const DirectParams p, const Conv3Tma t3) {
    constexpr int C0 = EXPAND ? 0 : 1;
    constexpr int OFF = 4 - (2 - C0);  // window index of tap offset 0
    constexpr int NW4 = (OFF + 3 + 2 + 4) / 4;
    static_assert(60 + 4 * NW4 <= C3_PF, "window exceeds the box width");
    extern __shared__ __align__(1024) unsigned char sm3_raw[];
    unsigned char *sm3 = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(sm3_raw) + 1023) & ~uintptr_t(1023));
    uint64_t *bar = reinterpret_cast<uint64_t *>(sm3 + C3_NB * C3_BUF);

    // tile t -> (x tile, y tile, z tile, batch)
    auto decode = [&](int t, long long &i0, long long &j0, long long &k0, long long &b) {
        const uint32_t r = fdiv((uint32_t)t, t3.ntx);
        const uint32_t r2 = fdiv(r, t3.nty);
        const uint32_t bb = fdiv(r2, t3.nz);
        i0 = (long long)((uint32_t)t - r * t3.ntx.d) * C3_BX;
        j0 = (long long)(r - r2 * t3.nty.d) * C3_BY;
        k0 = (long long)(r2 - bb * t3.nz.d) * C3_BZ;
        b = bb;
    };
    auto issue = [&](int t, int buf) {
        long long i0, j0, k0, b;
        decode(t, i0, j0, k0, b);
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        tc::mbar_arrive_expect_tx(&bar[buf], C3_BYTES);
        tc::tma_load_4d(smem_u32(sm3 + buf * C3_BUF), &smap, &bar[buf], (int)(i0 - 4),
                        (int)(j0 + C0 - 2), (int)(k0 + C0 - 2), (int)(b * t3.vstep));
    };
    if (threadIdx.x == 0) {
        for (int i = 0; i < C3_NB; ++i) tc::mbar_init(&bar[i], 1);
        tc::fence_barrier_init();
        for (int i = 0; i < C3_NB - 1; ++i) {
            const long long t = blockIdx.x + (long long)i * gridDim.x;
            if (t < t3.ntiles) issue((int)t, i);
        }
    }
    __syncthreads();  // barriers initialised before anyone waits on them

    int k = 0;
    // filter taps of the tile's volume (SAME batches: one filter per volume)
    // in shared memory, rewritten only when the volume's filter changes; the
    // reads are broadcasts.  (Taps held in registers through __ldg were
    // re-fetched from global memory at every use by the compiled code.)
    __shared__ float wsm[27];
    long long cur_filt = -1;
    for (int t = blockIdx.x; t < t3.ntiles; t += gridDim.x, ++k) {
        const int buf = k % C3_NB;
        // the buffer of the previous tile, released by its closing barrier
        const long long ahead = t + (long long)(C3_NB - 1) * gridDim.x;
        if (threadIdx.x == 0 && ahead < t3.ntiles) issue((int)ahead, (k + C3_NB - 1) % C3_NB);
        long long i0, j0, k0, b;
        decode(t, i0, j0, k0, b);
        const long long foff = b * p.filt_step[3];
        if (foff != cur_filt) {  // the same for the whole CTA: the barrier is uniform
            if (threadIdx.x < 27) {
                const int fi = threadIdx.x % 3, fj = (threadIdx.x / 3) % 3, fk = threadIdx.x / 9;
                wsm[threadIdx.x] = __ldg(static_cast<const float *>(p.filt) + foff + fi * p.fs[0] +
                                         fj * p.fs[1] + fk * p.fs[2]);
            }
            __syncthreads();  // the previous tile's reads ended at its closing barrier
            cur_filt = foff;
        }
        if (!wait_tile(&bar[buf], (k / C3_NB) & 1)) {
            // a box that never landed: give the later boxes this CTA issued
            // a bounded chance to land before the CTA exits
            if (threadIdx.x == 0)
                for (int j = k + 1; j < k + C3_NB; ++j) {
                    if (blockIdx.x + (long long)j * gridDim.x >= t3.ntiles) break;
                    unsigned n = 0;
                    while (!mbar_try_wait(&bar[j % C3_NB], (j / C3_NB) & 1) && ++n < (1u << 16)) {
                    }
                }
            break;
        }
        const float *tile = reinterpret_cast<const float *>(sm3 + buf * C3_BUF);
        const int tx = threadIdx.x & 15;
        const int ty = (threadIdx.x >> 4) & 7;
        const int tz = threadIdx.x >> 7;  // 0..1, four z each
        float acc[4][4];
#pragma unroll
        for (int a = 0; a < 4; ++a)
#pragma unroll
            for (int c = 0; c < 4; ++c) acc[a][c] = 0.0f;
#pragma unroll
        for (int q = 5; q >= 0; --q) {      // input plane (relative), high to low
#pragma unroll
            for (int fj = 0; fj < 3; ++fj) {  // dim-1 tap, ascending
                float v[NW4 * 4];
                const float *row = tile + ((4 * tz + q) * C3_TH + (ty + 2 - fj)) * C3_PF + 4 * tx;
#pragma unroll
                for (int u = 0; u < NW4; ++u) {
                    const float4 t4 = *reinterpret_cast<const float4 *>(row + 4 * u);
                    v[4 * u] = t4.x;
                    v[4 * u + 1] = t4.y;
                    v[4 * u + 2] = t4.z;
                    v[4 * u + 3] = t4.w;
                }
#pragma unroll
                for (int rz = 0; rz < 4; ++rz) {
                    const int fk = rz + 2 - q;
                    if (fk >= 0 && fk < 3) {
#pragma unroll
                        for (int fi = 0; fi < 3; ++fi) {
                            const float wv = wsm[(fk * 3 + fj) * 3 + fi];
#pragma unroll
                            for (int cc = 0; cc < 4; ++cc)
                                acc[rz][cc] = mac<EXACT>(acc[rz][cc], v[OFF + cc + 2 - fi], wv);
                        }
                    }
                }
            }
        }
        float *out = static_cast<float *>(p.out) + b * p.out_step[3];
        const long long x = i0 + 4 * tx, y = j0 + ty;
        if (y < p.od[1]) {
            const bool vec_ok = (x + 3 < p.od[0]) && ((p.os[1] & 3) == 0) &&
                                ((p.os[2] & 3) == 0) &&
                                ((reinterpret_cast<uintptr_t>(out) & 15) == 0);
            // even row pitches (EXPAND's 258-wide rows): two 8-byte stores
            const bool vec2_ok = (x + 3 < p.od[0]) && ((p.os[1] & 1) == 0) &&
                                 ((p.os[2] & 1) == 0) &&
                                 ((reinterpret_cast<uintptr_t>(out) & 7) == 0);
#pragma unroll
            for (int rz = 0; rz < 4; ++rz) {
                const long long z = k0 + 4 * tz + rz;
                if (z >= p.od[2]) break;
                float *dst = out + x + y * p.os[1] + z * p.os[2];
                if (vec_ok) {
                    *reinterpret_cast<float4 *>(dst) =
                        make_float4(acc[rz][0], acc[rz][1], acc[rz][2], acc[rz][3]);
                } else if (vec2_ok) {
                    reinterpret_cast<float2 *>(dst)[0] = make_float2(acc[rz][0], acc[rz][1]);
                    reinterpret_cast<float2 *>(dst)[1] = make_float2(acc[rz][2], acc[rz][3]);
                } else {
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc)
                        if (x + cc < p.od[0]) dst[cc] = acc[rz][cc];
                }
            }
        }
        __syncthreads();  // every thread is done with this buffer before it is reloaded
    }
}

// ===========================================================================
// host side
// ===========================================================================
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *,
                                  const cuuint64_t *, const cuuint64_t *, const cuuint32_t *,
                                  const cuuint32_t *, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

static EncodeTiledFn encode_fn() {
    static EncodeTiledFn fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void *ptr = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &ptr, 12000,
                                             cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(ptr);
    });
    return fn;
}

// 3-D map over dense images (W, H, slices) with a BW x BH x 1 box
static bool make_map(CUtensorMap &m, const void *base, int esize, long long W, long long Hh,
                     long long slices, int bw, int bh) {
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    cuuint64_t dims[3] = {(cuuint64_t)W, (cuuint64_t)Hh, (cuuint64_t)slices};
    cuuint64_t strides[2] = {(cuuint64_t)(W * esize), (cuuint64_t)(W * Hh * esize)};
    cuuint32_t box[3] = {(cuuint32_t)bw, (cuuint32_t)bh, 1};
    cuuint32_t es[3] = {1, 1, 1};
    CUresult r = fn(&m, esize == 4 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_UINT8,
                    3, const_cast<void *>(base), dims, strides, box, es,
                    CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                    CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    return r == CUDA_SUCCESS;
}

static bool dense_aligned(const void *base, int esize, long long W) {
    return (reinterpret_cast<uintptr_t>(base) & 15) == 0 && ((W * esize) & 15) == 0;
}

template <typename K>
static int persistent_grid(K kernel, size_t smem, long long ntiles) {
    int per_sm = 1;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, THREADS, smem) != cudaSuccess ||
        per_sm < 1)
        per_sm = 1;
    return (int)std::max(1LL, std::min<long long>(ntiles, (long long)num_sms() * per_sm));
}

// tile grid of a launch; false when a count exceeds the decoder's range
// (tile indices, and the 2-D kernel's run order past the last tile, stay
// below 2^31)
static bool make_grid(TileGrid &tg, long long tiles_x, long long tiles_y, long long nbatch,
                      long long b1 = 1, long long b2 = 1) {
    const long long lim = 1LL << 30;
    if (tiles_x < 1 || tiles_y < 1 || b1 < 1 || b2 < 1) return false;
    if (tiles_x * tiles_y * nbatch >= lim || b1 >= lim || b2 >= lim) return false;
    std::memset(&tg, 0, sizeof(tg));
    tg.tx = make_fastdiv((uint32_t)tiles_x);
    tg.ty = make_fastdiv((uint32_t)tiles_y);
    tg.b1 = make_fastdiv((uint32_t)b1);
    tg.b2 = make_fastdiv((uint32_t)b2);
    tg.ntiles = (int)(tiles_x * tiles_y * nbatch);
    tg.run = make_fastdiv(1);
    return true;
}

// run length of the 2-D kernel's tile order: the longest of 8, 4, 2 whose
// last, partial round costs at most 3 % more steps on the busiest CTA than
// single tiles do (AFGB_TILE_RUN overrides, for tests)
static int tile_run(long long ntiles, int grid) {
    static const int forced = [] {
        const char *e = std::getenv("AFGB_TILE_RUN");
        const int v = e ? std::atoi(e) : 0;
        return v >= 1 && v <= 64 ? v : 0;
    }();
    if (forced) return forced;
    const long long g = std::max(1, grid);
    const long long base = (ntiles + g - 1) / g;
    for (int r = 8; r > 1; r /= 2) {
        const long long steps = (ntiles + g * r - 1) / (g * r) * r;
        if (steps * 100 <= base * 103) return r;
    }
    return 1;
}

template <typename T, int F0, int F1, bool EXACT, bool EXPAND>
static bool run_conv2(const DirectParams &p) {
    using H = Conv2Halo<T, F0, F1, EXACT, EXPAND>;
    constexpr int TWX = TILE * Conv2Shape<T, F0, F1, EXACT>::CG;
    const long long slice = p.sd[0] * p.sd[1];
    const long long slices = p.sd[2] * p.sd[3];
    const long long tx = (p.od[0] + TWX - 1) / TWX, ty = (p.od[1] + TILE - 1) / TILE;
    TileGrid tg;
    if (!make_grid(tg, tx, ty, p.nbatch, p.batch[1], p.batch[2])) return false;
    // slice index of a batch coordinate: the signal is dense, so each batch
    // step is a whole number of W x H slices
    for (int i = 1; i < 4; ++i) {
        if (p.batch[i] <= 1) continue;  // coordinate always 0
        if (p.in_step[i] % slice != 0 || p.in_step[i] / slice >= (1LL << 31)) return false;
        tg.zstep[i] = (int)(p.in_step[i] / slice);
    }
    if (slices >= (1LL << 31)) return false;
    CUtensorMap m;
    if (!make_map(m, p.sig, (int)sizeof(T), p.sd[0], p.sd[1], slices, H::BW, H::BH)) return false;
    const size_t smem = NST_2D * H::TB_ALIGNED + H::FT_BYTES + 8 * NST_2D;
    auto kfn = conv2_tma_kernel<T, F0, F1, EXACT, EXPAND>;
    AFGB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int grid = persistent_grid(kfn, smem, tg.ntiles);
    tg.run = make_fastdiv((uint32_t)tile_run(tg.ntiles, grid));
    {
        KernelTimer kt("conv2_tma_kernel");
        kfn<<<grid, THREADS, smem, stream()>>>(m, p, tg);
    }
    count_launch();
    AFGB_POST_LAUNCH("conv2_tma_kernel");
    return true;
}

template <typename T, int F, bool EXACT>
static bool conv2_square(const DirectParams &p) {
    return p.expand ? run_conv2<T, F, F, EXACT, true>(p) : run_conv2<T, F, F, EXACT, false>(p);
}

bool tma_convolve2(const DirectParams &p, af_dtype t, bool exact) {
    // dense signal and output (the tile's slice index and output offsets
    // assume column-major packing), TMA-aligned rows
    const int es = (t == f32) ? 4 : 1;
    if (!(t == f32 || t == u8 || t == s8 || t == b8)) return false;
    if (p.ss[0] != 1 || p.ss[1] != p.sd[0] || p.ss[2] != p.sd[0] * p.sd[1] ||
        p.ss[3] != p.sd[0] * p.sd[1] * p.sd[2])
        return false;
    if (p.os[0] != 1 || p.os[1] != p.od[0]) return false;
    if (!dense_aligned(p.sig, es, p.sd[0])) return false;
    if (p.sd[0] > (1LL << 30) || p.sd[1] > (1LL << 30)) return false;
    const long long f0 = p.fd[0], f1 = p.fd[1];
    if (f0 != f1 || !(f0 == 3 || f0 == 5 || f0 == 7)) return false;
    const bool ex = exact || es == 1;
#define AFGB_SQ(T, E)                                                    \
    switch (f0) {                                                        \
        case 3: return conv2_square<T, 3, E>(p);                         \
        case 5: return conv2_square<T, 5, E>(p);                         \
        default: return conv2_square<T, 7, E>(p);                        \
    }
    if (t == f32) {
        if (ex) { AFGB_SQ(float, true) }
        else { AFGB_SQ(float, false) }
    } else if (t == u8) {
        AFGB_SQ(uint8_t, true)
    } else {
        AFGB_SQ(int8_t, true)
    }
#undef AFGB_SQ
}

template <typename T, int CL, int RL, bool EXACT, bool EXPAND>
static bool run_sep(SepTmaParams p, const void *sig, long long W, long long Hh, long long slices) {
    using H = Halo<T, CL, RL, EXPAND>;
    TileGrid tg;
    if (!make_grid(tg, p.tiles_x, p.tiles_y, slices)) return false;
    CUtensorMap m;
    if (!make_map(m, sig, (int)sizeof(T), W, Hh, slices, H::BW, H::BH)) return false;
    const size_t smem = NST_SEP * H::TB_ALIGNED + H::FT_BYTES + (size_t)H::BH * SEP_TP * 4 +
                        8 * NST_SEP;
    auto kfn = sep_tma_kernel<T, CL, RL, EXACT, EXPAND>;
    AFGB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int grid = persistent_grid(kfn, smem, tg.ntiles);
    {
        KernelTimer kt("sep_tma_kernel");
        kfn<<<grid, THREADS, smem, stream()>>>(m, p, tg);
    }
    count_launch();
    AFGB_POST_LAUNCH("sep_tma_kernel");
    return true;
}

template <typename T, int CL, int RL, bool EXPAND>
static bool run_sep_dp4a(SepTmaParams p, const void *sig, long long W, long long Hh,
                         long long slices) {
    using H = Halo<T, CL, RL, EXPAND>;
    TileGrid tg;
    if (!make_grid(tg, p.tiles_x, p.tiles_y, slices)) return false;
    CUtensorMap m;
    if (!make_map(m, sig, 1, W, Hh, slices, H::BW, H::BH)) return false;
    constexpr int NRB = (H::BH + 3) / 4;
    constexpr int TPT = sep8_pitch(NRB, (RL + 3) / 4);
    const size_t smem = NST_SEP * H::TB_ALIGNED + ((TILE * TPT + 127) / 128) * 128 + 8 * NST_SEP;
    auto kfn = sep_dp4a_kernel<T, CL, RL, EXPAND>;
    AFGB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const int grid = persistent_grid(kfn, smem, tg.ntiles);
    {
        KernelTimer kt("sep_tma_kernel");
        kfn<<<grid, THREADS, smem, stream()>>>(m, p, tg);
    }
    count_launch();
    AFGB_POST_LAUNCH("sep_dp4a_kernel");
    return true;
}

template <typename T, int L, bool EXACT>
static bool sep_len(const SepTmaParams &p, bool expand, const void *sig, long long W, long long Hh,
                    long long slices) {
    if constexpr (sizeof(T) == 1) {  // exact integer arithmetic: dp4a
        return expand ? run_sep_dp4a<T, L, L, true>(p, sig, W, Hh, slices)
                      : run_sep_dp4a<T, L, L, false>(p, sig, W, Hh, slices);
    }
    return expand ? run_sep<T, L, L, EXACT, true>(p, sig, W, Hh, slices)
                  : run_sep<T, L, L, EXACT, false>(p, sig, W, Hh, slices);
}

bool tma_convolve2_sep(const Array &sig, const float *cf, const float *rf, int cl, int rl,
                       Array &out, bool expand, bool exact) {
    const af_dtype t = sig.type;
    const int es = (t == f32) ? 4 : 1;
    if (!(t == f32 || t == u8 || t == s8 || t == b8)) return false;
    if (cl != rl || !(cl == 3 || cl == 5 || cl == 7 || cl == 15)) return false;
    if (!sig.is_linear() || !dense_aligned(sig.data(), es, sig.dims[0])) return false;
    if (sig.dims[0] > (1LL << 30) || sig.dims[1] > (1LL << 30)) return false;
    SepTmaParams p;
    std::memset(&p, 0, sizeof(p));
    p.cf = cf;
    p.rf = rf;
    p.out = out.data();
    p.od0 = out.dims[0];
    p.od1 = out.dims[1];
    p.out_slice = out.dims[0] * out.dims[1];
    p.sd1 = sig.dims[1];
    p.tiles_x = (p.od0 + TILE - 1) / TILE;
    p.tiles_y = (p.od1 + TILE - 1) / TILE;
    const long long slices = sig.dims[2] * sig.dims[3];
    p.ntiles = p.tiles_x * p.tiles_y * slices;
    if (p.ntiles == 0) return true;
    const bool ex = exact && es == 4;  // 8-bit sums are exact integers either way
#define AFGB_SEPL(T, E)                                                                   \
    switch (cl) {                                                                         \
        case 3: return sep_len<T, 3, E>(p, expand, sig.data(), sig.dims[0], sig.dims[1], slices);   \
        case 5: return sep_len<T, 5, E>(p, expand, sig.data(), sig.dims[0], sig.dims[1], slices);   \
        case 7: return sep_len<T, 7, E>(p, expand, sig.data(), sig.dims[0], sig.dims[1], slices);   \
        default: return sep_len<T, 15, E>(p, expand, sig.data(), sig.dims[0], sig.dims[1], slices); \
    }
    if (t == f32) {
        if (ex) { AFGB_SEPL(float, true) }
        else { AFGB_SEPL(float, false) }
    } else if (t == u8) {
        AFGB_SEPL(uint8_t, false)
    } else {
        AFGB_SEPL(int8_t, false)
    }
#undef AFGB_SEPL
}

// 3x3x3 f32 volumes: dense, 16-byte rows; false when not applicable
bool tma_convolve3(const DirectParams &p, bool exact) {
    if (p.rank != 3 || p.fd[0] != 3 || p.fd[1] != 3 || p.fd[2] != 3) return false;
    if (p.ss[0] != 1 || p.ss[1] != p.sd[0] || p.ss[2] != p.sd[0] * p.sd[1] ||
        p.ss[3] != p.sd[0] * p.sd[1] * p.sd[2])
        return false;
    if (p.os[0] != 1 || !dense_aligned(p.sig, 4, p.sd[0])) return false;
    if (p.sd[0] >= (1LL << 30) || p.sd[1] >= (1LL << 30) || p.sd[2] >= (1LL << 30) ||
        p.sd[3] >= (1LL << 30))
        return false;
    const long long vol = p.sd[0] * p.sd[1] * p.sd[2];
    if (p.in_step[3] % vol != 0) return false;
    const long long ntx = (p.od[0] + C3_BX - 1) / C3_BX, nty = (p.od[1] + C3_BY - 1) / C3_BY,
                    nz = (p.od[2] + C3_BZ - 1) / C3_BZ;
    if (p.nbatch < 1 || ntx * nty * nz * p.nbatch >= (1LL << 31)) return false;
    Conv3Tma t3;
    t3.ntx = make_fastdiv((uint32_t)ntx);
    t3.nty = make_fastdiv((uint32_t)nty);
    t3.nz = make_fastdiv((uint32_t)nz);
    t3.ntiles = (int)(ntx * nty * nz * p.nbatch);
    t3.vstep = p.in_step[3] / vol;
    EncodeTiledFn fn = encode_fn();
    if (!fn) return false;
    CUtensorMap m;
    cuuint64_t dims[4] = {(cuuint64_t)p.sd[0], (cuuint64_t)p.sd[1], (cuuint64_t)p.sd[2],
                          (cuuint64_t)p.sd[3]};
    cuuint64_t strides[3] = {(cuuint64_t)(p.sd[0] * 4), (cuuint64_t)(p.sd[0] * p.sd[1] * 4),
                             (cuuint64_t)(vol * 4)};
    cuuint32_t box[4] = {(cuuint32_t)C3_PF, (cuuint32_t)C3_TH, (cuuint32_t)C3_TD, 1};
    cuuint32_t es[4] = {1, 1, 1, 1};
    if (fn(&m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, const_cast<void *>(p.sig), dims, strides, box, es,
           CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
           CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
        return false;
    const size_t smem = 1024 + C3_NB * C3_BUF + 8 * C3_NB;
#define AFGB_C3(E, X)                                                                           \
    do {                                                                                        \
        AFGB_CUDA(cudaFuncSetAttribute(conv3_tma_kernel<E, X>,                                  \
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
        const int grid = persistent_grid(conv3_tma_kernel<E, X>, smem, t3.ntiles);             \
        conv3_tma_kernel<E, X><<<grid, 256, smem, stream()>>>(m, p, t3);                       \
    } while (0)
    {
        KernelTimer kt("conv3_tma_kernel");
        if (exact) {
            if (p.expand) AFGB_C3(true, true);
            else AFGB_C3(true, false);
        } else {
            if (p.expand) AFGB_C3(false, true);
            else AFGB_C3(false, false);
        }
    }
#undef AFGB_C3
    count_launch();
    AFGB_POST_LAUNCH("conv3_tma_kernel");
    return true;
}

}  // namespace dtma

void tma_set_wait_limit(unsigned int polls, int skip_block0) {
    const unsigned int v = polls ? polls : tc::kSpinLimit;
    AFGB_CUDA(cudaMemcpyToSymbol(tc::g_spin_limit, &v, sizeof(v)));
    AFGB_CUDA(cudaMemcpyToSymbol(dtma::g_debug_skip_block0, &skip_block0, sizeof(skip_block0)));
}

unsigned int tma_take_error() {
    unsigned int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, tc::g_tc_error, sizeof(v)) != cudaSuccess) return 0;
    if (v) (void)cudaMemcpyToSymbol(tc::g_tc_error, &zero, sizeof(zero));
    return v;
}

}  // namespace afgb
