// Tensor-core (tcgen05 / TMEM) NN convolution for sm_103a: the BF16 form of
// af_convolve2_nn and both of its input gradients, plus the filter gradient.
//
// The reference runs these as unwrap + GEMM (src/backend/cpu/convolve.cpp:
// 123-243, src/backend/cuda/convolveNN.cpp:175-407) or hands them to cuDNN.
// Here each is one implicit GEMM whose operands are fetched straight from the
// image, so no unwrapped patch matrix exists:
//
//   gather kernel  D[och][pixel] = sum_{cchunk, tap} Wt[och][tap, c] * Img[pixel@tap][c]
//       forward:   Img = signal (NHWC bf16), och = filter K, taps all (u,v)
//       data grad: Img = incoming gradient, och = C; with stride > 1 one
//                  launch covers every stride phase (x' mod sx, y' mod sy)
//                  with that phase's taps, so no zero-stuffed products run
//     MMA M=128 output channels (weights: TMA, K-major, 128B swizzle),
//     N=256 output pixels, K=64 channels per stage, 4 stages.
//     Pixel operand: for stride 1 a 4-D TMA box {64 ch, BX, BY, 1} over the
//     NHWC tensor — a BX x BY pixel rectangle shifted by the tap, zero-filled
//     outside the image (the convolution's padding); for other strides a
//     cp.async row gather by four producer warps.
//     Persistent CTAs, warp-specialised (producers, 4 epilogue warps, one MMA
//     warp, one TMA warp); the 256-column accumulator is double-buffered in
//     TMEM (512 columns) so one tile's epilogue overlaps the next main loop.
//
//   wgrad kernel   D[k][(tap,c)] = sum_{pixels} G[pixel][k] * X[pixel@tap][c]
//     reduction over pixels: both operands are pixel rows, i.e. MN-major
//     shared-memory tiles (TMA boxes for stride 1, cp.async rows otherwise);
//     split-K over pixel blocks, FP32 partials combined by a fixed-order
//     compensated reduction (deterministic).
//
// Inputs and outputs stay f32 ArrayFire arrays; conversion to bf16
// channels-last happens on the device in bandwidth-bound pre-passes.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_fp8.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "nn_conv.hpp"
#include "tc_ptx.cuh"

namespace afgb {
namespace tc {

constexpr int BM = 128;               // output channels per tile (MMA M)
constexpr int BN = 256;               // output pixels per tile (MMA N)
constexpr int BK = 64;                // input channels per stage (128 bytes of bf16)
constexpr int STAGES = 4;
constexpr int A_BYTES = BM * BK * 2;  // 16 KB weight tile
constexpr int B_BYTES = BN * BK * 2;  // 32 KB pixel tile
constexpr int LAG = 2;                // cp.async groups in flight per producer
constexpr int MAX_PH = 64;
constexpr int MAX_T = 256;
constexpr int NUM_THREADS = 320;      // warps 0-3 gather, 4-7 epilogue, 8 MMA, 9 TMA
constexpr int EP_PITCH = 20;          // epilogue staging row pitch (floats): 16 pixels + 4
constexpr int EP_WARPS = 8;           // epilogue warps of the TMA path (two per TMEM quadrant)
// Column groups (stride 1, filters at most three taps high): the taps of one
// filter column read the same pixel columns one row apart, so they share one
// TMA box BY + 2 rows high; tap v's operand is the view (oy_v - oy_min) * BX
// pixel rows into it (an MMA operand may start at any 128-byte row).  Three
// taps per stage, one box load instead of three: the L2-to-shared traffic of
// the pixel operand drops from 9 to 3.75 boxes per tile and chunk.
constexpr int CG_STAGES = 2;
constexpr int CG_GT = 3;                                 // taps per group at most
constexpr int CG_BX = 32, CG_BY = 8;                      // 256-pixel rectangles
constexpr int CG_BOX_BYTES = CG_BX * (CG_BY + 2) * 128;  // 40 KB
constexpr int CG_STAGE_A = CG_GT * A_BYTES;              // 48 KB
constexpr int MAX_G = 16;
constexpr int EP_SLOT = 768;          // floats of staging per warp: 3 KB, 1024-byte aligned slots

struct GatherParams {
    const unsigned char *src;  // [N][SH][SW][SCpad] elements (bf16, or e4m3 bytes)
    float *dst;                // ArrayFire layout (DW, DH, DC, N)
    const float *out_scale;    // FP8: per-output-channel dequantisation factor
    const float *bias;         // forward: per-output-channel bias added in the epilogue
    int relu;                  // forward: max(v, 0) in the epilogue
    int SW, SH, SCpad, N;
    int DW, DH, DC;
    int mode;  // 0 forward, 1 data gradient
    int tma_store;  // epilogue writes by TMA through the output map (unit-stride outputs)
    int a_rows;     // weight rows loaded per stage: 128, or 64 when the output has at most 64
                    // channels (the upper half of each weight tile is zero, set once)
    int sx, sy, px, py, dx, dy, fw;
    int nchunk;       // SCpad / 64
    int n_och_tiles;  // ceil(DC / 128)
    int nphase, nphx;
    int total_tiles;
    int BX, BY;            // pixel rectangles (TMA path)
    int ph_ntx[MAX_PH], ph_nty[MAX_PH];  // rectangles per stride phase (TMA path)
    int phase_tile_begin[MAX_PH + 1];
    int phase_tap_begin[MAX_PH + 1];
    short tap_u[MAX_T], tap_v[MAX_T];
    short tap_ox[MAX_T], tap_oy[MAX_T];  // operand offset of each tap (TMA path)
    // column groups (cg != 0): group g holds taps cg_begin[g] .. cg_begin[g+1]-1
    // of the one phase, its box at (cg_ox[g], cg_oymin[g]); the j-th tap's
    // view starts cg_view[g * CG_GT + j] pixel rows into the box
    int cg, cg_ngroups, cg_box_bytes;
    short cg_begin[MAX_G + 1], cg_ox[MAX_G], cg_oymin[MAX_G];
    short cg_view[MAX_G * CG_GT];
};

struct Smem {
    uint64_t full[STAGES];
    uint64_t empty[STAGES];
    uint64_t tmem_full[2];
    uint64_t tmem_empty[2];
    uint64_t final_bar;
    uint32_t tmem_base;
    int abort;
};

struct TileInfo {
    int rx, ry, tap_begin, ntaps;
    int och0;
    // gather path: linear pixel range of one stride phase
    long long p0, npix;
    int MX, MY;
    // TMA path: pixel rectangle
    int x0, y0, n;
};

template <bool TMA_B>
__device__ __forceinline__ TileInfo decode_tile(const GatherParams &p, int tile) {
    TileInfo t;
    if (TMA_B) {
        // rectangles of one stride phase (a single phase for the forward):
        // the phase's outputs are (rx + sx*i, ry + sy*j), i < MX, j < MY
        int ph = 0;
        while (ph + 1 < p.nphase && tile >= p.phase_tile_begin[ph + 1]) ++ph;
        t.rx = ph % p.nphx;
        t.ry = ph / p.nphx;
        t.tap_begin = p.phase_tap_begin[ph];
        t.ntaps = p.phase_tap_begin[ph + 1] - p.phase_tap_begin[ph];
        const int local = tile - p.phase_tile_begin[ph];
        t.och0 = (local % p.n_och_tiles) * BM;
        int r = local / p.n_och_tiles;
        const int ntx = p.ph_ntx[ph], nty = p.ph_nty[ph];
        const int tx = r % ntx;
        r /= ntx;
        const int ty = r % nty;
        t.n = r / nty;
        t.x0 = tx * p.BX;
        t.y0 = ty * p.BY;
        t.p0 = 0;
        t.npix = 0;
        if (p.mode == 0) {
            t.MX = p.DW;
            t.MY = p.DH;
        } else {
            t.MX = (p.DW - t.rx + p.sx - 1) / p.sx;
            t.MY = (p.DH - t.ry + p.sy - 1) / p.sy;
        }
        return t;
    }
    int ph = 0;
    while (ph + 1 < p.nphase && tile >= p.phase_tile_begin[ph + 1]) ++ph;
    t.rx = ph % p.nphx;
    t.ry = ph / p.nphx;
    t.tap_begin = p.phase_tap_begin[ph];
    t.ntaps = p.phase_tap_begin[ph + 1] - p.phase_tap_begin[ph];
    const int local = tile - p.phase_tile_begin[ph];
    t.och0 = (local % p.n_och_tiles) * BM;
    const int ptile = local / p.n_och_tiles;
    if (p.mode == 0) {
        t.MX = p.DW;
        t.MY = p.DH;
    } else {
        t.MX = (p.DW - t.rx + p.sx - 1) / p.sx;
        t.MY = (p.DH - t.ry + p.sy - 1) / p.sy;
    }
    t.npix = (long long)t.MX * t.MY * p.N;
    t.p0 = (long long)ptile * BN;
    t.x0 = t.y0 = t.n = 0;
    return t;
}

__device__ __forceinline__ void tap_offsets(const GatherParams &p, const TileInfo &ti, int u, int v,
                                            int &offx, int &offy) {
    if (p.mode == 0) {
        offx = u * p.dx - p.px;
        offy = v * p.dy - p.py;
    } else {
        offx = (ti.rx + p.px - u * p.dx) / p.sx;
        offy = (ti.ry + p.py - v * p.dy) / p.sy;
    }
}

// FP8: e4m3 operands, 128 channels per 128-byte row, kind::f8f6f4 MMA;
// CG: column groups (stride-1 TMA path, bf16)
template <bool TMA_B, bool FP8, bool CG = false>
__global__ void __launch_bounds__(NUM_THREADS, 1)
    gather_conv_kernel(const __grid_constant__ GatherParams p,
                       const __grid_constant__ CUtensorMap wmap,
                       const __grid_constant__ CUtensorMap xmap,
                       const __grid_constant__ CUtensorMap omap) {
    static_assert(!CG || (TMA_B && !FP8), "column groups: TMA path, bf16");
    static_assert(CG_STAGES * (CG_STAGE_A + CG_BOX_BYTES) <= STAGES * (A_BYTES + B_BYTES),
                  "column-group stages fit the stage area");
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    // STAGES x 16 KB weight tiles then STAGES x 32 KB pixel tiles; column
    // groups: CG_STAGES x 3 x 16 KB weight tiles then CG_STAGES x 40 KB boxes
    unsigned char *a_stage = base;
    unsigned char *b_stage = base + (CG ? CG_STAGES * CG_STAGE_A : STAGES * A_BYTES);
    float *ep_stage = reinterpret_cast<float *>(base + STAGES * (A_BYTES + B_BYTES));  // 8 x 32 x 20
    Smem *sm = reinterpret_cast<Smem *>(ep_stage + EP_WARPS * EP_SLOT);
    volatile int *abort = &sm->abort;

    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;

    if (threadIdx.x == 0) {
        for (int s = 0; s < STAGES; ++s) {
            mbar_init(&sm->full[s], TMA_B ? 1 : 128 + 1);
            mbar_init(&sm->empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&sm->tmem_full[b], 1);
            mbar_init(&sm->tmem_empty[b], TMA_B ? 32 * EP_WARPS : 128);
        }
        mbar_init(&sm->final_bar, 1);
        sm->abort = 0;
        fence_barrier_init();
    }
    if (warp == 8) tmem_alloc(&sm->tmem_base, 512);
    if (warp == 9 && lane == 0) {
        prefetch_tmap(&wmap);
        if (TMA_B) prefetch_tmap(&xmap);
    }
    if (p.a_rows < BM) {
        // rows a_rows..127 of every weight tile are zero padding: written once
        // here, never loaded (the tensor core reads them through the async proxy)
        const int half_bytes = (BM - p.a_rows) * 128;
        const int nslots = CG ? CG_STAGES * CG_GT : STAGES;  // weight tiles, A_BYTES apart
        for (int i = threadIdx.x; i < nslots * half_bytes / 16; i += blockDim.x) {
            const int st = i / (half_bytes / 16), off = i - st * (half_bytes / 16);
            *reinterpret_cast<uint4 *>(a_stage + st * A_BYTES + p.a_rows * 128 + off * 16) =
                make_uint4(0u, 0u, 0u, 0u);
        }
        fence_proxy_async_smem();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = sm->tmem_base;

    if (warp < 4 && !TMA_B) {
        {
            // ---------------- pixel-row gather (128 threads)
            const int t = threadIdx.x;
            const int j = t & 7;    // 16-byte chunk within the 128-byte row
            const int r0 = t >> 3;  // rows r0 + 16 i
            const int alpha_x = p.mode == 0 ? p.sx : 1;
            const int alpha_y = p.mode == 0 ? p.sy : 1;
            constexpr int ES = FP8 ? 1 : 2;  // bytes per element
            const long long img_stride = (long long)p.SH * p.SW * p.SCpad * ES;
            const long long pix_stride = (long long)p.SCpad * ES;
            uint32_t it = 0;
            for (int tile = blockIdx.x; tile < p.total_tiles && !*abort; tile += gridDim.x) {
                TileInfo ti = decode_tile<false>(p, tile);
                if (ti.ntaps == 0) continue;
                int xb[16], yb[16], nb[16];
                uint32_t vmask = 0;
#pragma unroll
                for (int i = 0; i < 16; ++i) {
                    const long long pix = ti.p0 + r0 + 16 * i;
                    if (pix < ti.npix) {
                        const int X = (int)(pix % ti.MX);
                        const long long rest = pix / ti.MX;
                        const int Y = (int)(rest % ti.MY);
                        nb[i] = (int)(rest / ti.MY);
                        xb[i] = X * alpha_x;
                        yb[i] = Y * alpha_y;
                        vmask |= 1u << i;
                    } else {
                        xb[i] = yb[i] = nb[i] = 0;
                    }
                }
                const int iters = p.nchunk * ti.ntaps;
                for (int kb = 0; kb < iters; ++kb, ++it) {
                    const int s = it % STAGES;
                    if (!mbar_wait(&sm->empty[s], ((it / STAGES) & 1) ^ 1, abort, 1u)) break;
                    const int cchunk = kb / ti.ntaps;
                    const int tq = ti.tap_begin + (kb - cchunk * ti.ntaps);
                    int offx, offy;
                    tap_offsets(p, ti, p.tap_u[tq], p.tap_v[tq], offx, offy);
                    const uint32_t sb = smem_u32(b_stage + s * B_BYTES);
                    const unsigned char *cbase = p.src + cchunk * 128 + 16 * j;
#pragma unroll
                    for (int i = 0; i < 16; ++i) {
                        const int r = r0 + 16 * i;
                        const int xs = xb[i] + offx, ys = yb[i] + offy;
                        const bool ok = ((vmask >> i) & 1u) && xs >= 0 && xs < p.SW && ys >= 0 &&
                                        ys < p.SH;
                        const unsigned char *src =
                            ok ? cbase + nb[i] * img_stride + ((long long)ys * p.SW + xs) * pix_stride
                               : p.src;
                        cp_async_16(sb + r * 128 + ((j ^ (r & 7)) << 4), src, ok ? 16u : 0u);
                    }
                    cp_async_commit();
                    if (it >= LAG) {
                        cp_async_wait<LAG>();
                        fence_proxy_async_smem();
                        mbar_arrive(&sm->full[(it - LAG) % STAGES]);
                    }
                }
            }
            cp_async_wait_all();
            fence_proxy_async_smem();
            for (uint32_t k = (it >= LAG ? it - LAG : 0); k < it; ++k)
                mbar_arrive(&sm->full[k % STAGES]);
        }
    } else if (warp < 8) {
        // ---------------- epilogue: TMEM lanes 32*(warp%4) ..; on the TMA
        // path warps 0-3 join warps 4-7 (the gather warps are idle there),
        // the two warps of a TMEM quadrant taking alternate 16-pixel chunks
        const int q = warp & 3;
        const int half = TMA_B ? (warp >> 2) : 0;
        uint32_t acc_it = 0;
        const long long plane = (long long)p.DW * p.DH;
        const bool vec_rows = (p.DW & 3) == 0;
        for (int tile = blockIdx.x; tile < p.total_tiles && !*abort; tile += gridDim.x) {
            TileInfo ti = decode_tile<TMA_B>(p, tile);
            const int och = ti.och0 + 32 * q + lane;
            if (ti.ntaps == 0) {
                // a stride phase no tap reaches: its gradient is zero
                if (och < p.DC && half == 0) {
                    for (int e = 0; e < BN; ++e) {
                        int X, Y, n;
                        if (TMA_B) {
                            X = ti.x0 + e % p.BX;
                            Y = ti.y0 + e / p.BX;
                            n = ti.n;
                            if (X >= ti.MX || Y >= ti.MY) continue;
                        } else {
                            const long long pix = ti.p0 + e;
                            if (pix >= ti.npix) break;
                            X = (int)(pix % ti.MX);
                            const long long rest = pix / ti.MX;
                            Y = (int)(rest % ti.MY);
                            n = (int)(rest / ti.MY);
                        }
                        const long long xo = ti.rx + (long long)p.sx * X;
                        const long long yo = ti.ry + (long long)p.sy * Y;
                        p.dst[xo + p.DW * yo + plane * (och + (long long)p.DC * n)] = 0.0f;
                    }
                }
                continue;
            }
            const int b = acc_it & 1;
            if (!mbar_wait(&sm->tmem_full[b], (acc_it >> 1) & 1, abort, 2u)) break;
            tc_fence_after();
            const uint32_t taddr = tmem_base + (uint32_t)(b * BN) + ((uint32_t)(32 * q) << 16);
            if (TMA_B) {
                // 32 channels x 16 pixels at a time: TMEM -> registers -> this
                // warp's shared staging block -> 64-byte row pieces per channel
                float *stg = ep_stage + warp * EP_SLOT;
                const int orow = lane >> 2;         // 0..7: channel within a group of 8
                const int ocol = (lane & 3) * 4;    // pixel offset within the 16
                const float sc = (FP8 && och < p.DC) ? p.out_scale[och] : 1.0f;
                const float bi = (p.bias && och < p.DC) ? p.bias[och] : 0.0f;
                // scale, then the fused bias and ReLU (forward only)
                auto fin = [&](uint32_t raw) {
                    float v = sc * __uint_as_float(raw);
                    if (p.bias) v += bi;
                    if (p.relu && v < 0.0f) v = 0.0f;
                    return v;
                };
                const int osx = p.mode == 0 ? 1 : p.sx, osy = p.mode == 0 ? 1 : p.sy;
                for (int cc = half; cc < BN / 16; cc += 2) {
                    uint32_t r[16];
                    tmem_ld16(taddr + cc * 16, r);
                    tmem_ld_wait();
                    const int e0 = cc * 16;
                    if (p.tma_store) {
                        // one 64-byte row per channel, 16-byte chunks swizzled by
                        // (row >> 1) & 3 (the output map's 64-byte swizzle: conflict-
                        // free 128-bit stores); one lane stores the 32x16 block by TMA
                        // (two alternating staging buffers were measured no faster: the
                        // forward is not bound by this wait)
                        float *sbuf = stg;
                        if (lane == 0) bulk_wait_read();  // the last store has read the buffer
                        __syncwarp();
                        unsigned char *row = reinterpret_cast<unsigned char *>(sbuf) + lane * 64;
#pragma unroll
                        for (int e = 0; e < 4; ++e)
                            *reinterpret_cast<float4 *>(row + ((e ^ ((lane >> 1) & 3)) << 4)) =
                                make_float4(fin(r[4 * e]), fin(r[4 * e + 1]), fin(r[4 * e + 2]),
                                            fin(r[4 * e + 3]));
                        fence_proxy_async_smem();
                        __syncwarp();
                        if (lane == 0) {
                            tma_store_4d(&omap, smem_u32(sbuf), ti.x0 + (e0 % p.BX), ti.y0 + e0 / p.BX,
                                         ti.och0 + 32 * q, ti.n);
                            bulk_commit();
                        }
                        continue;
                    }
#pragma unroll
                    for (int e = 0; e < 4; ++e)
                        *reinterpret_cast<float4 *>(stg + lane * EP_PITCH + 4 * e) =
                            make_float4(fin(r[4 * e]), fin(r[4 * e + 1]), fin(r[4 * e + 2]),
                                        fin(r[4 * e + 3]));
                    __syncwarp();
                    // BX >= 32 keeps the 16 pixels in one row; (x, y) are
                    // coordinates in the phase grid, output (rx + osx*x, ry + osy*y)
                    const int x = ti.x0 + (e0 % p.BX) + ocol, y = ti.y0 + e0 / p.BX;
                    if (y < ti.MY && x < ti.MX) {
                        const long long xo = ti.rx + (long long)osx * x;
                        const long long yo = ti.ry + (long long)osy * y;
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const int cl = orow + 8 * i;
                            const int oc = ti.och0 + 32 * q + cl;
                            if (oc >= p.DC) continue;
                            const float4 v = *reinterpret_cast<const float4 *>(stg + cl * EP_PITCH + ocol);
                            float *d = p.dst + plane * ((long long)oc + (long long)p.DC * ti.n) + xo +
                                       (long long)p.DW * yo;
                            if (osx == 1 && vec_rows && x + 3 < ti.MX) {
                                *reinterpret_cast<float4 *>(d) = v;
                            } else {
                                d[0] = v.x;
                                if (x + 1 < ti.MX) d[osx] = v.y;
                                if (x + 2 < ti.MX) d[2 * osx] = v.z;
                                if (x + 3 < ti.MX) d[3 * osx] = v.w;
                            }
                        }
                    }
                    __syncwarp();
                }
            } else {
            for (int cc = 0; cc < BN / 16; ++cc) {
                uint32_t r[16];
                tmem_ld16(taddr + cc * 16, r);
                tmem_ld_wait();
                if (och >= p.DC) continue;
                {
                    const long long pix0 = ti.p0 + cc * 16;
                    if (pix0 >= ti.npix) continue;
                    int X = (int)(pix0 % ti.MX);
                    long long rest = pix0 / ti.MX;
                    int Y = (int)(rest % ti.MY), n = (int)(rest / ti.MY);
#pragma unroll
                    for (int e = 0; e < 16; ++e) {
                        if (pix0 + e >= ti.npix) break;
                        const long long xo = p.mode == 0 ? X : ti.rx + (long long)p.sx * X;
                        const long long yo = p.mode == 0 ? Y : ti.ry + (long long)p.sy * Y;
                        float v = (FP8 ? p.out_scale[och] : 1.0f) * __uint_as_float(r[e]);
                        if (p.bias) v += p.bias[och];
                        if (p.relu && v < 0.0f) v = 0.0f;
                        p.dst[xo + p.DW * yo + plane * (och + (long long)p.DC * n)] = v;
                        if (++X == ti.MX) {
                            X = 0;
                            if (++Y == ti.MY) {
                                Y = 0;
                                ++n;
                            }
                        }
                    }
                }
            }
            }
            tc_fence_before();
            mbar_arrive(&sm->tmem_empty[b]);
            ++acc_it;
        }
        if (TMA_B && p.tma_store && lane == 0) bulk_wait_all();  // stores done before exit
        __syncwarp();
    } else if (warp == 8) {
        // ---------------- MMA issuer
        if (lane == 0) {
            const uint32_t idesc = FP8 ? idesc_e4m3(BM, BN) : idesc_bf16(BM, BN, 0, 0);
            // descriptors: precomputed bases plus 16-byte-unit offsets (the
            // issuing thread is latency-bound on its scalar work)
            const uint64_t a0 = smem_desc(smem_u32(a_stage), 16, 1024);
            const uint64_t b0 = smem_desc(smem_u32(b_stage), 16, 1024);
            uint32_t it = 0, acc_it = 0;
            bool issued = false;
            for (int tile = blockIdx.x; tile < p.total_tiles && !*abort; tile += gridDim.x) {
                TileInfo ti = decode_tile<TMA_B>(p, tile);
                if (ti.ntaps == 0) continue;
                const int b = acc_it & 1;
                if (!mbar_wait(&sm->tmem_empty[b], ((acc_it >> 1) & 1) ^ 1, abort, 4u)) break;
                tc_fence_after();
                const uint32_t d_tmem = tmem_base + (uint32_t)(b * BN);
                bool ok = true;
                if constexpr (CG) {
                    // one stage per (channel chunk, filter column): the
                    // column's taps, each against its view of the box
                    bool first = true;
                    for (int cchunk = 0; cchunk < p.nchunk && ok; ++cchunk) {
                        for (int g = 0; g < p.cg_ngroups; ++g, ++it) {
                            const int s = it % CG_STAGES;
                            if (!mbar_wait(&sm->full[s], (it / CG_STAGES) & 1, abort, 8u)) {
                                ok = false;
                                break;
                            }
                            tc_fence_after();
                            const int nt = p.cg_begin[g + 1] - p.cg_begin[g];
                            for (int j = 0; j < nt; ++j) {
                                const uint64_t as =
                                    a0 + (uint32_t)((s * CG_STAGE_A + j * A_BYTES) >> 4);
                                const uint64_t bs =
                                    b0 + (uint32_t)((s * CG_BOX_BYTES) >> 4) +
                                    (uint32_t)(p.cg_view[g * CG_GT + j] * 8);  // rows of 128 B
#pragma unroll
                                for (int k = 0; k < 4; ++k) {
                                    mma_f16(d_tmem, as + (uint32_t)(2 * k), bs + (uint32_t)(2 * k),
                                            idesc, first ? (k != 0) : 1);
                                }
                                first = false;
                            }
                            mma_commit(&sm->empty[s]);
                            issued = true;
                        }
                    }
                    if (!ok) break;
                    mma_commit(&sm->tmem_full[b]);
                    ++acc_it;
                    continue;
                }
                const int iters = p.nchunk * ti.ntaps;
                for (int kb = 0; kb < iters; ++kb, ++it) {
                    const int s = it % STAGES;
                    if (!mbar_wait(&sm->full[s], (it / STAGES) & 1, abort, 8u)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint64_t as = a0 + (uint32_t)(s * (A_BYTES >> 4));
                    const uint64_t bs = b0 + (uint32_t)(s * (B_BYTES >> 4));
#pragma unroll
                    for (int k = 0; k < 4; ++k) {  // 4 x 32 bytes of K per stage
                        const uint64_t ad = as + (uint32_t)(2 * k);
                        const uint64_t bd = bs + (uint32_t)(2 * k);
                        if (FP8)
                            mma_f8(d_tmem, ad, bd, idesc, (kb | k) != 0);
                        else
                            mma_f16(d_tmem, ad, bd, idesc, (kb | k) != 0);
                    }
                    mma_commit(&sm->empty[s]);
                    issued = true;
                }
                if (!ok) break;
                mma_commit(&sm->tmem_full[b]);
                ++acc_it;
            }
            if (issued) {
                mma_commit(&sm->final_bar);
                unsigned n = 0;
                while (!mbar_try_wait(&sm->final_bar, 0) && ++n < kSpinLimit) {
                }
            }
        }
        __syncwarp();
    } else {
        // ---------------- TMA: weight tiles (and pixel rectangles for stride 1)
        if (lane == 0) {
            uint32_t it = 0;
            for (int tile = blockIdx.x; tile < p.total_tiles && !*abort; tile += gridDim.x) {
                TileInfo ti = decode_tile<TMA_B>(p, tile);
                if (ti.ntaps == 0) continue;
                // forward: input origin x0*s (traversal stride s in the map);
                // data gradient: the phase-grid origin x0; tap offsets from the host
                const int bx0 = p.mode == 0 ? ti.x0 * p.sx : ti.x0;
                const int by0 = p.mode == 0 ? ti.y0 * p.sy : ti.y0;
                bool stop = false;
                if constexpr (CG) {
                    for (int cchunk = 0; cchunk < p.nchunk && !stop; ++cchunk) {
                        for (int g = 0; g < p.cg_ngroups; ++g, ++it) {
                            const int s = it % CG_STAGES;
                            if (!mbar_wait(&sm->empty[s], ((it / CG_STAGES) & 1) ^ 1, abort, 16u)) {
                                stop = true;
                                break;
                            }
                            const int t0 = p.cg_begin[g], nt = p.cg_begin[g + 1] - t0;
                            mbar_arrive_expect_tx(&sm->full[s], (uint32_t)p.cg_box_bytes +
                                                                    (uint32_t)(nt * p.a_rows * 128));
                            tma_load_4d(smem_u32(b_stage + s * CG_BOX_BYTES), &xmap, &sm->full[s],
                                        cchunk * 64, bx0 + p.cg_ox[g], by0 + p.cg_oymin[g], ti.n);
                            for (int j = 0; j < nt; ++j) {
                                const int u = p.tap_u[t0 + j], v = p.tap_v[t0 + j];
                                tma_load_2d(smem_u32(a_stage + s * CG_STAGE_A + j * A_BYTES), &wmap,
                                            &sm->full[s], (u + p.fw * v) * p.SCpad + cchunk * 64,
                                            ti.och0);
                            }
                        }
                    }
                    if (stop) break;
                    continue;
                }
                for (int cchunk = 0; cchunk < p.nchunk && !stop; ++cchunk) {
                    for (int tq = ti.tap_begin; tq < ti.tap_begin + ti.ntaps; ++tq, ++it) {
                        const int s = it % STAGES;
                        if (!mbar_wait(&sm->empty[s], ((it / STAGES) & 1) ^ 1, abort, 16u)) {
                            stop = true;
                            break;
                        }
                        const int u = p.tap_u[tq], v = p.tap_v[tq];
                        mbar_arrive_expect_tx(&sm->full[s], (uint32_t)(p.a_rows * 128) +
                                                                (TMA_B ? B_BYTES : 0));
                        tma_load_2d(smem_u32(a_stage + s * A_BYTES), &wmap, &sm->full[s],
                                    (u + p.fw * v) * p.SCpad + cchunk * (FP8 ? 128 : 64), ti.och0);
                        if (TMA_B)
                            tma_load_4d(smem_u32(b_stage + s * B_BYTES), &xmap, &sm->full[s],
                                        cchunk * (FP8 ? 128 : 64), bx0 + p.tap_ox[tq], by0 + p.tap_oy[tq],
                                        ti.n);
                    }
                }
                if (stop) break;
            }
        }
        __syncwarp();
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 8) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 512);
    }
}

// ===========================================================================
// stride-1 forward and data gradient with pixels on M (strip kernel)
// ===========================================================================
// For images whose rows hold at least 128 output pixels.  A tile is SC_R
// output rows x 128 output pixels (one row segment) x all output channels
// (the MMA's N, a multiple of 16 up to 128).  For each 64-channel chunk of the
// source the producer loads one strip per source row the tile touches:
// SL = 128 + (ox_max - ox_min) pixels of 64 channels, zero outside the image
// (the convolution's padding).  Tap t of output row r reads strip
// r + oy(t) - oy_min from row ox(t) - ox_min on: its A operand (128 pixels x
// 64 channels, K-major, 128-byte swizzle) is a view into the strip, so a
// source pixel is loaded once per chunk and source row instead of once per
// tap.  The 128-byte swizzle is keyed on the shared-memory address bits, as
// the TMA wrote the strip, so a view may start at any 128-byte row.  The
// weights of one tap and chunk (N x 64, K-major) stream through their own
// ring.  MMA M=128 x N x K=16 with FP32 accumulators in TMEM (SC_R*N columns,
// double-buffered).  Every output channel is a real MMA column: nothing is
// padding when the output has 64 channels (the weights-on-M gather kernel
// pads such a data gradient to M=128).  The epilogue warps own 32 pixels
// each (their TMEM lanes) and store a channel's 32 consecutive pixels as one
// 128-byte piece.
constexpr int SC_R = 2;
constexpr int SC_MAXS = 4;                  // strips per chunk: SC_R + oy range
constexpr int SC_MAXSL = 136;               // strip pixels
constexpr int SC_STRIP = SC_MAXSL * 128;    // 17 KB, a multiple of 1024
constexpr int SC_NA = 2;                    // strip-set buffers
constexpr int SC_B_AREA = 64 * 1024;        // weight-tile ring
constexpr int SC_MAXN = 128;
constexpr int SC_MAXNB = 8;
// warp 0 TMA; warps 1 and 10 issue the MMAs of output rows 0 and 1; warps
// 2-9 epilogue.  One issuing thread needs 75-100 cycles per MMA (waits,
// fences, descriptor arithmetic), more than an N<=128 MMA takes (48-64
// cycles); two issuers, each with its own accumulator, keep the tensor pipe
// busy (measured by microbenchmark).
constexpr int SC_THREADS = 352;
constexpr int SC_MMA_WARP1 = 10;

struct StripConvParams {
    float *dst;          // ArrayFire layout (DW, DH, DC, N)
    const float *bias;   // forward: per-output-channel bias, or 0
    int relu;
    int SW, SH, SCpad, N;
    int DW, DH, DC;
    int nmma;            // MMA N (output channels rounded up to 16)
    int nchunk, ntaps, S, SL;
    int ox_min, oy_min;
    int nb;              // weight-tile buffers
    int nseg, nrg, total_tiles;
    int strip16;         // SC_STRIP in 16-byte units
    uint32_t a_off[MAX_T];  // per tap: offset of its A view within a strip set (16-byte units)
};

struct StripConvSmem {
    uint64_t a_full[SC_NA], a_empty[SC_NA];
    uint64_t b_full[SC_MAXNB], b_empty[SC_MAXNB];
    uint64_t tmem_full[2], tmem_empty[2];
    uint64_t final_bar[SC_R];
    uint32_t tmem_base;
    int abort;
};

__global__ void __launch_bounds__(SC_THREADS, 1)
    strip_conv_kernel(const __grid_constant__ StripConvParams p,
                      const __grid_constant__ CUtensorMap wmap,
                      const __grid_constant__ CUtensorMap smap) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    unsigned char *a_area = base;                                   // SC_NA x SC_MAXS strips
    unsigned char *b_area = base + SC_NA * SC_MAXS * SC_STRIP;      // weight tiles
    StripConvSmem *sm = reinterpret_cast<StripConvSmem *>(b_area + SC_B_AREA);
    volatile int *abort = &sm->abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const uint32_t b_bytes = (uint32_t)p.nmma * 128u;
    const int tiles_per_img = p.nseg * p.nrg;

    if (threadIdx.x == 0) {
        // the empty and tmem_full barriers complete when both issuers'
        // MMAs have read the stage / written the accumulator
        for (int i = 0; i < SC_NA; ++i) {
            mbar_init(&sm->a_full[i], 1);
            mbar_init(&sm->a_empty[i], SC_R);
        }
        for (int i = 0; i < p.nb; ++i) {
            mbar_init(&sm->b_full[i], 1);
            mbar_init(&sm->b_empty[i], SC_R);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&sm->tmem_full[i], SC_R);
            mbar_init(&sm->tmem_empty[i], 256);
        }
        for (int r = 0; r < SC_R; ++r) mbar_init(&sm->final_bar[r], 1);
        sm->abort = 0;
        fence_barrier_init();
    }
    if (warp == 1) tmem_alloc(&sm->tmem_base, 512);
    if (warp == 0 && lane == 0) {
        prefetch_tmap(&wmap);
        prefetch_tmap(&smap);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = sm->tmem_base;

    if (warp == 0) {
        // ---------------- TMA producer: strip sets and weight tiles
        if (lane == 0) {
            int a = 0, b = 0;
            uint32_t aph = 1, bph = 1;
            bool stop = false;
            for (int tile = blockIdx.x; tile < p.total_tiles && !stop; tile += gridDim.x) {
                const int n = tile / tiles_per_img;
                const int rem = tile - n * tiles_per_img;
                const int rg = rem / p.nseg, seg = rem - rg * p.nseg;
                const int x0 = seg * 128, y0 = rg * SC_R;
                for (int ch = 0; ch < p.nchunk && !stop; ++ch) {
                    if (!mbar_wait(&sm->a_empty[a], aph, abort, 1u)) {
                        stop = true;
                        break;
                    }
                    mbar_arrive_expect_tx(&sm->a_full[a], (uint32_t)(p.S * p.SL * 128));
                    unsigned char *set = a_area + a * (SC_MAXS * SC_STRIP);
                    for (int s = 0; s < p.S; ++s)
                        tma_load_4d(smem_u32(set + s * SC_STRIP), &smap, &sm->a_full[a], ch * 64,
                                    x0 + p.ox_min, y0 + p.oy_min + s, n);
                    if (++a == SC_NA) {
                        a = 0;
                        aph ^= 1u;
                    }
                    for (int t = 0; t < p.ntaps; ++t) {
                        if (!mbar_wait(&sm->b_empty[b], bph, abort, 2u)) {
                            stop = true;
                            break;
                        }
                        mbar_arrive_expect_tx(&sm->b_full[b], b_bytes);
                        tma_load_2d(smem_u32(b_area + b * b_bytes), &wmap, &sm->b_full[b],
                                    t * p.SCpad + ch * 64, 0);
                        if (++b == p.nb) {
                            b = 0;
                            bph ^= 1u;
                        }
                    }
                }
            }
        }
        __syncwarp();
    } else if (warp == 1 || warp == SC_MMA_WARP1) {
        // ---------------- MMA issuers, one per output row r: descriptors are
        // precomputed bases plus 16-byte-unit offsets; stage indices and
        // phases advance without division
        const int r = warp == 1 ? 0 : 1;
        if (lane == 0) {
            const uint32_t idesc = idesc_bf16(128, (uint32_t)p.nmma, 0, 0);
            const uint64_t a0 = smem_desc(smem_u32(a_area), 16, 1024);
            const uint64_t b0 = smem_desc(smem_u32(b_area), 16, 1024);
            const uint32_t set16 = (uint32_t)(SC_MAXS * SC_STRIP) >> 4;
            const uint32_t b16 = b_bytes >> 4;
            int a = 0, b = 0;
            uint32_t aph = 0, bph = 0, aoff = 0, boff = 0, acc_it = 0;
            bool issued = false, stop = false;
            for (int tile = blockIdx.x; tile < p.total_tiles && !stop; tile += gridDim.x) {
                const int acc = acc_it & 1;
                if (!mbar_wait(&sm->tmem_empty[acc], ((acc_it >> 1) & 1) ^ 1, abort, 4u)) break;
                tc_fence_after();
                const uint32_t d0 = tmem_base + (uint32_t)((acc * SC_R + r) * p.nmma);
                for (int ch = 0; ch < p.nchunk && !stop; ++ch) {
                    if (!mbar_wait(&sm->a_full[a], aph, abort, 8u)) {
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    for (int t = 0; t < p.ntaps; ++t) {
                        if (!mbar_wait(&sm->b_full[b], bph, abort, 16u)) {
                            stop = true;
                            break;
                        }
                        tc_fence_after();
                        const uint64_t ad = a0 + aoff + p.a_off[t] + (uint32_t)(r * p.strip16);
                        const uint64_t bd = b0 + boff;
#pragma unroll
                        for (int k = 0; k < 4; ++k)
                            mma_f16(d0, ad + (uint32_t)(2 * k), bd + (uint32_t)(2 * k), idesc,
                                    (ch | t | k) != 0);
                        mma_commit(&sm->b_empty[b]);
                        issued = true;
                        if (++b == p.nb) {
                            b = 0;
                            boff = 0;
                            bph ^= 1u;
                        } else {
                            boff += b16;
                        }
                    }
                    if (stop) break;
                    mma_commit(&sm->a_empty[a]);
                    if (++a == SC_NA) {
                        a = 0;
                        aoff = 0;
                        aph ^= 1u;
                    } else {
                        aoff += set16;
                    }
                }
                if (stop) break;
                mma_commit(&sm->tmem_full[acc]);
                ++acc_it;
            }
            if (issued) {
                mma_commit(&sm->final_bar[r]);
                unsigned n = 0;
                while (!mbar_try_wait(&sm->final_bar[r], 0) && ++n < kSpinLimit) {
                }
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: warp w reads TMEM lanes 32*(w % 4) ..,
        // i.e. pixels x0 + 32*(w % 4) + lane of each output row; the two
        // warps of a lane quadrant take alternate groups of 64 channels.
        // Up to four 16-column TMEM loads are in flight per wait.
        const int q = warp & 3, half = (warp - 2) >> 2;
        const long long plane = (long long)p.DW * p.DH;
        uint32_t acc_it = 0;
        for (int tile = blockIdx.x; tile < p.total_tiles && !*abort; tile += gridDim.x) {
            const int n = tile / tiles_per_img;
            const int rem = tile - n * tiles_per_img;
            const int rg = rem / p.nseg, seg = rem - rg * p.nseg;
            const int x = seg * 128 + 32 * q + lane, y0 = rg * SC_R;
            const int acc = acc_it & 1;
            if (!mbar_wait(&sm->tmem_full[acc], (acc_it >> 1) & 1, abort, 32u)) break;
            tc_fence_after();
            const uint32_t tq = tmem_base + (uint32_t)(acc * SC_R * p.nmma) + ((uint32_t)(32 * q) << 16);
            for (int r = 0; r < SC_R; ++r) {
                const int y = y0 + r;
                float *drow = p.dst + (long long)n * p.DC * plane + (long long)y * p.DW + x;
                const bool ok = y < p.DH && x < p.DW;
                for (int c0 = 64 * half; c0 < p.nmma; c0 += 128) {
                    const int ng = min(4, (p.nmma - c0) / 16);  // 16-column groups here
                    uint32_t v[4][16];
#pragma unroll
                    for (int g = 0; g < 4; ++g)
                        if (g < ng) tmem_ld16(tq + (uint32_t)(r * p.nmma + c0 + 16 * g), v[g]);
                    tmem_ld_wait();
                    if (!ok) continue;
#pragma unroll
                    for (int g = 0; g < 4; ++g) {
                        if (g >= ng) break;
#pragma unroll
                        for (int e = 0; e < 16; ++e) {
                            const int c = c0 + 16 * g + e;
                            if (c < p.DC) {
                                float val = __uint_as_float(v[g][e]);
                                if (p.bias) val += __ldg(p.bias + c);
                                if (p.relu && val < 0.0f) val = 0.0f;
                                drow[(long long)c * plane] = val;
                            }
                        }
                    }
                }
            }
            tc_fence_before();
            mbar_arrive(&sm->tmem_empty[acc]);
            ++acc_it;
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 512);
    }
}

// ===========================================================================
// stride-1 forward and data gradient by source rows (the row kernel)
// ===========================================================================
// Pixels on M, (filter row, output channel) on N.  A CTA owns one group of
// 64 output channels (ncg groups; the CTAs of a band's groups run side by
// side and share its source rows through L2) and walks bands of output rows
// (one image, one 128-pixel segment) source row by source row.  For source row r and each 64-channel
// chunk the producer loads one strip of SL = 128 + (fw-1)*dx pixels; tap
// column u's A operand (128 pixels x 64 channels, K-major, 128-byte swizzle)
// is the view ox(u) - ox_min pixel rows into it.  Tap column u's B operand
// stacks its FH filter rows' weights along N (FH blocks of 64 output
// channels), so one MMA of N = FH*64 per K step gives source row r's
// contribution to FH output rows: block j to output row r - oy_max + j.
// Each source row accumulates into a fresh TMEM buffer (two, alternating);
// MMAs that accumulate into regions overlapping the previous MMA's at another
// column offset drain the tensor pipe (measured: about 800 cycles per shift),
// while alternating disjoint regions run at the full rate.  The epilogue
// keeps FH - 1 partial output rows per pixel in registers: source row r
// completes output row r - oy_max (partial + block 0), the others shift by
// one row, and the band's last FH - 1 rows are stored after its last source
// row.  Each source pixel is loaded once per band and chunk, every MMA is
// full width (no padded M rows), and the weights stay in shared memory for
// the whole kernel.
constexpr int RC_THREADS = 320;  // warp 0 TMA, warp 1 MMA, warps 2-9 epilogue
constexpr int RC_STRIP = SC_STRIP;
constexpr int RC_DC = 64;        // output channels per block and CTA (zero rows past DC)
constexpr int RC_MAXCG = 4;      // channel groups: at most 256 output channels
constexpr int RC_MAXNS = 8;
constexpr int RC_MAXCH = 16;
constexpr int RC_MAXTAP = 48;

struct RowConvParams {
    float *dst;          // ArrayFire layout (DW, DH, DC, N)
    const float *bias;   // forward: per-output-channel bias, or 0
    int relu;
    int SW, SH, N;
    int DW, DH, DC;
    int fw, nchunk;
    int ox_min, oy_min, oy_max;
    int SL;               // strip pixels
    int nseg, ns;         // 128-pixel segments, strip buffers
    int ncg;              // 64-channel output groups (CTA b serves group b % ncg)
    long long rows;       // N * nseg * DH output rows
    int wcol[RC_MAXTAP];  // weight-map column of tap column u, block j (chunk 0), at u*FH + j
    uint32_t a_view[16];  // tap column u's A view offset in 16-byte units
};

struct RowConvSmem {
    uint64_t w_full[RC_MAXCH];
    uint64_t s_full[RC_MAXNS], s_empty[RC_MAXNS];
    uint64_t buf_full[2], buf_free[2];
    uint64_t final_bar;
    uint32_t tmem_base;
    int abort;
    float bias[RC_DC];  // forward: the group's bias per output channel (zero past DC or without one)
};

struct RowBand {
    int n, seg, y0, y1, rs, re;  // output rows [y0, y1), source rows rs..re
};

// next band of this CTA's output rows [pos, end), flattened over (image,
// segment, row); every role walks the same sequence
__device__ __forceinline__ bool row_next_band(const RowConvParams &p, long long &pos,
                                               long long end, RowBand &b) {
    if (pos >= end) return false;
    const long long col = pos / p.DH;
    b.y0 = (int)(pos - col * p.DH);
    b.y1 = (int)min((long long)p.DH, (long long)b.y0 + (end - pos));
    b.n = (int)(col / p.nseg);
    b.seg = (int)(col - (long long)b.n * p.nseg);
    b.rs = max(b.y0 + p.oy_min, 0);
    b.re = min(b.y1 - 1 + p.oy_max, p.SH - 1);
    pos += b.y1 - b.y0;
    return true;
}

template <int FH>
__global__ void __launch_bounds__(RC_THREADS, 1)
    row_conv_kernel(const __grid_constant__ RowConvParams p,
                     const __grid_constant__ CUtensorMap wmap,
                     const __grid_constant__ CUtensorMap smap) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    constexpr uint32_t kBlk = RC_DC * 128;      // one block: 64 rows of 128 bytes
    constexpr uint32_t kTile = kBlk * FH;       // tap column u, one chunk
    const uint32_t wchunk_bytes = kTile * (uint32_t)p.fw;
    unsigned char *w_area = base;  // [chunk][u][j] blocks of 8 KB
    unsigned char *s_area = base + (size_t)p.nchunk * wchunk_bytes;
    RowConvSmem *sm = reinterpret_cast<RowConvSmem *>(s_area + (size_t)p.ns * RC_STRIP);
    volatile int *abort = &sm->abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int cg = (int)(blockIdx.x % (unsigned)p.ncg);
    const long long nbands = gridDim.x / p.ncg, band = blockIdx.x / p.ncg;
    const long long r_begin = p.rows * band / nbands;
    const long long r_end = p.rows * (band + 1) / nbands;
    const int och0 = cg * RC_DC;

    if (threadIdx.x == 0) {
        for (int c = 0; c < p.nchunk; ++c) mbar_init(&sm->w_full[c], 1);
        for (int i = 0; i < p.ns; ++i) {
            mbar_init(&sm->s_full[i], 1);
            mbar_init(&sm->s_empty[i], 1);
        }
        for (int i = 0; i < 2; ++i) {
            mbar_init(&sm->buf_full[i], 1);
            mbar_init(&sm->buf_free[i], 256);
        }
        mbar_init(&sm->final_bar, 1);
        sm->abort = 0;
        fence_barrier_init();
    }
    if (threadIdx.x < RC_DC) {
        const int c = och0 + (int)threadIdx.x;
        sm->bias[threadIdx.x] = (p.bias && c < p.DC) ? p.bias[c] : 0.0f;
    }
    if (warp == 1) tmem_alloc(&sm->tmem_base, 512);
    if (warp == 0 && lane == 0) {
        prefetch_tmap(&wmap);
        prefetch_tmap(&smap);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = sm->tmem_base;

    if (warp == 0) {
        // ---------------- TMA producer: the weights once, then strips
        if (lane == 0 && r_begin < r_end) {
            for (int c = 0; c < p.nchunk; ++c) {
                mbar_arrive_expect_tx(&sm->w_full[c], wchunk_bytes);
                for (int t = 0; t < p.fw * FH; ++t)
                    tma_load_2d(smem_u32(w_area + c * wchunk_bytes + t * kBlk), &wmap, &sm->w_full[c],
                                p.wcol[t] + c * 64, och0);
            }
            int s = 0;
            uint32_t ph = 1, nload = 0;
            bool stop = false;
            long long pos = r_begin;
            RowBand b;
            while (!stop && row_next_band(p, pos, r_end, b)) {
                const int xs = b.seg * 128 + p.ox_min;
                for (int r = b.rs; r <= b.re && !stop; ++r) {
                    for (int c = 0; c < p.nchunk; ++c) {
                        if (!mbar_wait(&sm->s_empty[s], ph, abort, 1u)) {
                            stop = true;
                            break;
                        }
                        mbar_arrive_expect_tx(&sm->s_full[s], (uint32_t)p.SL * 128u);
                        tma_load_4d(smem_u32(s_area + s * RC_STRIP), &smap, &sm->s_full[s], c * 64, xs,
                                    r, b.n);
                        ++nload;
                        if (++s == p.ns) {
                            s = 0;
                            ph ^= 1u;
                        }
                    }
                }
            }
            if (stop) {
                // the CTA is unwinding: let this thread's copies land before exit
                // (bounded), the weights and the last ns strips
                const unsigned limit = g_spin_limit;
                for (int c = 0; c < p.nchunk; ++c) {
                    unsigned n = 0;
                    while (!mbar_try_wait(&sm->w_full[c], 0) && ++n < limit) {
                    }
                }
                for (uint32_t l = nload > (uint32_t)p.ns ? nload - p.ns : 0; l < nload; ++l) {
                    unsigned n = 0;
                    while (!mbar_try_wait(&sm->s_full[l % p.ns], (l / p.ns) & 1u) && ++n < limit) {
                    }
                }
            }
        }
        __syncwarp();
    } else if (warp == 1) {
        // ---------------- MMA issuer: one N = FH*64 MMA per K step into the
        // source row's buffer; descriptors are bases plus 16-byte-unit offsets
        if (lane == 0) {
            const uint64_t a0 = smem_desc(smem_u32(s_area), 16, 1024);
            const uint64_t b0 = smem_desc(smem_u32(w_area), 16, 1024);
            const uint32_t tile16 = kTile >> 4, wchunk16 = wchunk_bytes >> 4;
            const uint32_t strip16 = (uint32_t)RC_STRIP >> 4;
            constexpr uint32_t idesc = idesc_bf16(128, FH * RC_DC, 0, 0);
            int s = 0;
            uint32_t sph = 0, soff = 0, it = 0;
            bool wready = false, issued = false, stop = false;
            long long pos = r_begin;
            RowBand b;
            while (!stop && row_next_band(p, pos, r_end, b)) {
                for (int r = b.rs; r <= b.re; ++r, ++it) {
                    const uint32_t bf = it & 1u, use = it >> 1;
                    if (!mbar_wait(&sm->buf_free[bf], (use & 1u) ^ 1u, abort, 4u)) {
                        stop = true;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t d = tmem_base + bf * 256u;
                    for (int c = 0; c < p.nchunk; ++c) {
                        if (!wready && !mbar_wait(&sm->w_full[c], 0, abort, 2u)) {
                            stop = true;
                            break;
                        }
                        if (!mbar_wait(&sm->s_full[s], sph, abort, 8u)) {
                            stop = true;
                            break;
                        }
                        tc_fence_after();
                        const uint64_t as = a0 + soff;
                        const uint64_t bc = b0 + (uint32_t)c * wchunk16;
                        for (int u = 0; u < p.fw; ++u) {
                            const uint64_t au = as + p.a_view[u];
                            const uint64_t bu = bc + (uint32_t)u * tile16;
#pragma unroll
                            for (int k = 0; k < 4; ++k)
                                mma_f16(d, au + (uint32_t)(2 * k), bu + (uint32_t)(2 * k), idesc,
                                        (c | u | k) != 0);
                        }
                        mma_commit(&sm->s_empty[s]);
                        issued = true;
                        if (++s == p.ns) {
                            s = 0;
                            soff = 0;
                            sph ^= 1u;
                        } else {
                            soff += strip16;
                        }
                    }
                    if (stop) break;
                    wready = true;
                    mma_commit(&sm->buf_full[bf]);
                }
            }
            if (issued) {
                mma_commit(&sm->final_bar);
                unsigned n = 0;
                while (!mbar_try_wait(&sm->final_bar, 0) && ++n < kSpinLimit) {
                }
            }
        }
        __syncwarp();
    } else {
        // ---------------- epilogue: warp w reads TMEM lanes 32*(w % 4) .., i.e.
        // pixel seg*128 + 32*(w % 4) + lane, and channels 32*half .. +31 of
        // each block (output channels och0 + ..); partial output rows P[i]
        // (output row r - oy_max + 1 + i after source row r) stay in registers
        const int qd = warp & 3, half = (warp - 2) >> 2;
        const int cbase = 32 * half;
        const long long plane = (long long)p.DW * p.DH;
        const int nc = min(32, p.DC - och0 - cbase);  // this warp's real channels (may be <= 0)
        const bool act = p.bias != nullptr || p.relu;
        auto finish = [&](float v, int c) {
            if (act) {
                v += sm->bias[c];
                if (p.relu && v < 0.0f) v = 0.0f;
            }
            return v;
        };
        uint32_t it = 0;
        bool stop = false;
        long long pos = r_begin;
        RowBand b;
        while (!stop && row_next_band(p, pos, r_end, b)) {
            const int x = b.seg * 128 + 32 * qd + lane;
            const bool xok = x < p.DW;
            // channel cbase of this band's image at pixel x, row 0
            float *img = p.dst + ((long long)b.n * p.DC + och0 + cbase) * plane + x;
            float P[FH > 1 ? FH - 1 : 1][32];
#pragma unroll
            for (int i = 0; i < (FH > 1 ? FH - 1 : 1); ++i)
#pragma unroll
                for (int e = 0; e < 32; ++e) P[i][e] = 0.0f;
            for (int r = b.rs; r <= b.re; ++r, ++it) {
                const uint32_t bf = it & 1u, use = it >> 1;
                if (!mbar_wait(&sm->buf_full[bf], use & 1u, abort, 32u)) {
                    stop = true;
                    break;
                }
                tc_fence_after();
                const uint32_t taddr = tmem_base + bf * 256u + (uint32_t)cbase + ((uint32_t)(32 * qd) << 16);
                const int y = r - p.oy_max;
                const bool yok = xok && y >= b.y0 && y < b.y1;
                float *q = img + (long long)y * p.DW;  // advances one channel plane per value
#pragma unroll
                for (int g = 0; g < 2; ++g) {
                    uint32_t v[FH][16];
#pragma unroll
                    for (int j = 0; j < FH; ++j) tmem_ld16(taddr + (uint32_t)(j * RC_DC + 16 * g), v[j]);
                    tmem_ld_wait();
#pragma unroll
                    for (int e = 0; e < 16; ++e) {
                        const int ci = 16 * g + e;
                        float o;
                        if constexpr (FH == 1) {
                            o = __uint_as_float(v[0][e]);
                        } else {
                            o = P[0][ci] + __uint_as_float(v[0][e]);
#pragma unroll
                            for (int i = 0; i + 2 < FH; ++i) P[i][ci] = P[i + 1][ci] + __uint_as_float(v[i + 1][e]);
                            P[FH - 2][ci] = __uint_as_float(v[FH - 1][e]);
                        }
                        if (yok && ci < nc) *q = finish(o, cbase + ci);
                        q += plane;
                    }
                }
                tc_fence_before();
                mbar_arrive(&sm->buf_free[bf]);
            }
            if (stop) break;
            if constexpr (FH > 1) {
                // the band's last rows: their remaining source rows lie past the image
                // or outside the band
#pragma unroll
                for (int i = 0; i < FH - 1; ++i) {
                    const int y = b.re - p.oy_max + 1 + i;
                    if (!xok || y < b.y0 || y >= b.y1) continue;
                    float *q = img + (long long)y * p.DW;
#pragma unroll
                    for (int ci = 0; ci < 32; ++ci) {
                        if (ci < nc) *q = finish(P[i][ci], cbase + ci);
                        q += plane;
                    }
                }
            }
        }
    }

    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 512);
    }
}

// ===========================================================================
// filter gradient kernel
// ===========================================================================
constexpr int WG_STAGES = 4;
constexpr int WG_KP = 64;                      // pixels per stage (MMA K) of the cp.async path
constexpr int WG_B_GROUP = 64 * WG_KP * 2;     // cp.async path: one 64-channel group x 64 pixels
constexpr int WG_MAXG = 4;
constexpr int WG_THREADS = 256;  // warps 0-3 producers (warp 0 TMA), 4-7 epilogue, MMA in warp 4

struct WgradParams {
    const __nv_bfloat16 *x;  // [N][H][W][Cpad]
    const __nv_bfloat16 *g;  // [N][Ho][Wo][Kpad]
    float *partial;          // [splits][C*taps][K]
    int W, H, Cpad, C, N;
    int Wo, Ho, Kpad, K;  // Kpad: channels stored per pixel of G (a multiple of 64)
    int sx, sy, px, py, dx, dy, fw, fh;
    long long Q;        // cp.async path: Wo*Ho*N pixels; TMA path: pixel blocks
    long long chunk;    // pixels (cp.async) or pixel blocks (TMA) per split
    int ngroups_total;  // taps * (Cpad/64)
    int groups_per_tile;
    int n_k_tiles;
    int BX, BY, ntx, nty;  // KP-pixel rectangles (TMA path)
    // stage geometry: KP pixels per stage (64, or 128 on the TMA path: the
    // SM's copy engine costs about 400 cycles per copy whatever its size, so
    // 16 KB boxes feed twice the MMA work of 8 KB ones), nst stages, the
    // incoming-gradient tile (a_bytes) and one 64-channel signal group
    // (b_group) per stage
    int KP, nst, a_bytes, b_group;
};

template <bool TMA>
__global__ void __launch_bounds__(WG_THREADS, 1)
    wgrad_tc_kernel(const __grid_constant__ WgradParams p, const __grid_constant__ CUtensorMap gmap,
                    const __grid_constant__ CUtensorMap xmap) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    const int b_bytes = WG_MAXG * p.b_group;
    unsigned char *a_stage = base;
    unsigned char *b_stage = base + p.nst * p.a_bytes;
    Smem *sm = reinterpret_cast<Smem *>(b_stage + p.nst * b_bytes);
    volatile int *abort = &sm->abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    const int ktile = blockIdx.x % p.n_k_tiles;
    const int gtile = blockIdx.x / p.n_k_tiles;
    const int k0 = ktile * 128;
    const int g0 = gtile * p.groups_per_tile;
    const int ng = min(p.groups_per_tile, p.ngroups_total - g0);
    const long long q_begin = (long long)blockIdx.y * p.chunk;
    const long long q_end = min(p.Q, q_begin + p.chunk);
    const int nstages = TMA ? (int)(q_end - q_begin) : (int)((q_end - q_begin + p.KP - 1) / p.KP);
    const int ncols = 64 * ng;
    const int nchunk = p.Cpad / 64;

    if (threadIdx.x == 0) {
        for (int s = 0; s < p.nst; ++s) {
            mbar_init(&sm->full[s], TMA ? 1 : 128);
            mbar_init(&sm->empty[s], 1);
        }
        mbar_init(&sm->tmem_full[0], 1);
        sm->abort = 0;
        fence_barrier_init();
    }
    if (warp == 4) tmem_alloc(&sm->tmem_base, 256);
    if (TMA && warp == 0 && lane == 0) {
        prefetch_tmap(&gmap);
        prefetch_tmap(&xmap);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = sm->tmem_base;

    if (warp < 4) {
        if (TMA) {
            if (warp == 0 && lane == 0) {
                const uint32_t bytes = (uint32_t)(p.a_bytes + p.b_group * ng);
                for (int st = 0; st < nstages && !*abort; ++st) {
                    const int s = st % p.nst;
                    if (!mbar_wait(&sm->empty[s], ((st / p.nst) & 1) ^ 1, abort, 32u)) break;
                    long long blk = q_begin + st;
                    const int tx = (int)(blk % p.ntx);
                    blk /= p.ntx;
                    const int ty = (int)(blk % p.nty);
                    const int n = (int)(blk / p.nty);
                    const int x0 = tx * p.BX, y0 = ty * p.BY;
                    mbar_arrive_expect_tx(&sm->full[s], bytes);
                    const uint32_t sa = smem_u32(a_stage + s * p.a_bytes);
                    const uint32_t sb = smem_u32(b_stage + s * b_bytes);
                    tma_load_4d(sa, &gmap, &sm->full[s], k0, x0, y0, n);
                    tma_load_4d(sa + p.KP * 128, &gmap, &sm->full[s], k0 + 64, x0, y0, n);
                    for (int grp = 0; grp < ng; ++grp) {
                        const int gi = g0 + grp;
                        const int tap = gi / nchunk, cchunk = gi - tap * nchunk;
                        const int u = tap % p.fw, v = tap / p.fw;
                        tma_load_4d(sb + grp * p.b_group, &xmap, &sm->full[s], cchunk * 64,
                                    x0 * p.sx - p.px + u * p.dx, y0 * p.sy - p.py + v * p.dy, n);
                    }
                }
            }
        } else {
            // cp.async producers: thread t owns pixel row t/2 of every stage and
            // half of its chunks; the pixel is tracked incrementally
            const int t = threadIdx.x;
            const int row = t >> 1, half = t & 1;
            long long q = q_begin + row;
            int X = (int)(q % p.Wo);
            long long rest = q / p.Wo;
            int Y = (int)(rest % p.Ho), n = (int)(rest / p.Ho);
            uint32_t it = 0;
            for (int st = 0; st < nstages && !*abort; ++st, ++it) {
                const int s = it % p.nst;
                if (!mbar_wait(&sm->empty[s], ((it / p.nst) & 1) ^ 1, abort, 32u)) break;
                const uint32_t sa = smem_u32(a_stage + s * p.a_bytes);
                const uint32_t sb = smem_u32(b_stage + s * b_bytes);
                const bool qv = q < q_end;
                const uint32_t rowoff = (row >> 3) * 1024 + (row & 7) * 128;
                // A: G row (128 k = two 64-wide MN atoms); channels at or past
                // the row's stored Kpad (a multiple of 64) read as zero
                const __nv_bfloat16 *gsrc = p.g + q * p.Kpad + k0;
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int ch = half * 8 + e;  // 16-byte chunk along k
                    const int atom = ch >> 3, j = ch & 7;
                    const bool cv = qv && k0 + 8 * ch < p.Kpad;
                    cp_async_16(sa + atom * 8192 + rowoff + ((j ^ (row & 7)) << 4),
                                cv ? gsrc + 8 * ch : p.g, cv ? 16u : 0u);
                }
                // B: X rows at the shifted pixel for each (tap, channel chunk)
                for (int grp = 0; grp < ng; ++grp) {
                    const int gi = g0 + grp;
                    const int tap = gi / nchunk, cchunk = gi - tap * nchunk;
                    const int u = tap % p.fw, v = tap / p.fw;
                    const int xs = X * p.sx - p.px + u * p.dx, ys = Y * p.sy - p.py + v * p.dy;
                    const bool ok = qv && xs >= 0 && xs < p.W && ys >= 0 && ys < p.H;
                    const __nv_bfloat16 *xsrc =
                        ok ? p.x + (((long long)n * p.H + ys) * p.W + xs) * p.Cpad + cchunk * 64 : p.x;
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        const int j = half * 4 + e;
                        cp_async_16(sb + grp * WG_B_GROUP + rowoff + ((j ^ (row & 7)) << 4),
                                    ok ? xsrc + 8 * j : p.x, ok ? 16u : 0u);
                    }
                }
                cp_async_commit();
                if (it >= LAG) {
                    cp_async_wait<LAG>();
                    fence_proxy_async_smem();
                    mbar_arrive(&sm->full[(it - LAG) % p.nst]);
                }
                q += WG_KP;
                X += WG_KP;
                while (X >= p.Wo) {
                    X -= p.Wo;
                    if (++Y == p.Ho) {
                        Y = 0;
                        ++n;
                    }
                }
            }
            cp_async_wait_all();
            fence_proxy_async_smem();
            for (uint32_t k = (it >= LAG ? it - LAG : 0); k < it; ++k)
                mbar_arrive(&sm->full[k % p.nst]);
        }
    } else {
        if (warp == 4 && lane == 0) {
            // MMA: M = 128 (k), N = 64*ng, both operands MN-major; the k atoms
            // and the signal groups are KP*128 bytes apart
            const uint32_t idesc = idesc_bf16(128, (uint32_t)ncols, 1, 1);
            const uint32_t lbo = (uint32_t)p.KP * 128u;
            const int ksteps = p.KP / 16;
            for (int st = 0; st < nstages; ++st) {
                const int s = st % p.nst;
                if (!mbar_wait(&sm->full[s], (st / p.nst) & 1, abort, 64u)) break;
                tc_fence_after();
                const uint32_t sa = smem_u32(a_stage + s * p.a_bytes);
                const uint32_t sb = smem_u32(b_stage + s * b_bytes);
#pragma unroll
                for (int k = 0; k < 8; ++k) {
                    if (k >= ksteps) break;
                    const uint64_t ad = smem_desc(sa + k * 2048, lbo, 1024);
                    const uint64_t bd = smem_desc(sb + k * 2048, lbo, 1024);
                    mma_f16(tmem_base, ad, bd, idesc, (st | k) != 0);
                }
                mma_commit(&sm->empty[s]);
            }
            mma_commit(&sm->tmem_full[0]);
        }
        __syncwarp();
        // epilogue: warps 4-7 (TMEM lanes 32*(warp-4) ...); waits for the MMAs
        // even when aborting, so TMEM is never freed under them
        const int q = warp - 4;
        bool have = false;
        if (nstages > 0) {
            have = mbar_wait_sleep(&sm->tmem_full[0], 0);
            if (!have) {
                *abort = 1;
                atomicOr(&g_tc_error, 128u);
            }
        }
        tc_fence_after();
        const int k = k0 + 32 * q + lane;
        const long long rows = (long long)p.C * p.fw * p.fh;
        float *out = p.partial + (long long)blockIdx.y * rows * p.K;
        for (int cc = 0; cc < ncols / 16; ++cc) {
            uint32_t r[16];
            if (have) {
                tmem_ld16(tmem_base + cc * 16 + ((uint32_t)(32 * q) << 16), r);
                tmem_ld_wait();
            } else {
#pragma unroll
                for (int e = 0; e < 16; ++e) r[e] = 0u;
            }
            if (k >= p.K || *abort) continue;
#pragma unroll
            for (int e = 0; e < 16; ++e) {
                const int col = cc * 16 + e;
                const int gi = g0 + col / 64;
                const int tap = gi / nchunk, c = (gi - tap * nchunk) * 64 + (col & 63);
                if (c < p.C) out[((long long)c + (long long)p.C * tap) * p.K + k] = __uint_as_float(r[e]);
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 256);
    }
}

// ===========================================================================
// filter gradient, stride 1 along x: one signal strip per filter row
// ===========================================================================
// A stage is a rectangle of KP = 64 or 128 output pixels (BY rows of BX).  For
// each of its rows the producer loads one strip of BX + (nu-1)*dx signal
// pixels (64 channels each), and the nu taps u0..u0+nu-1 of filter row v read
// it at row offsets u*dx: nine shifted tiles become three strips for a 3x3
// filter.  The SM's copy engine completes about one TMA copy per 400 cycles
// whatever its size up to 18 KB (measured: 8 KB copies move 21 bytes per
// cycle, 16 KB copies 42), so a stage of 128 pixels, two 16 KB
// incoming-gradient boxes and one ~17 KB strip, feeds twice the MMA work of a
// 64-pixel stage for the same three copies.  (Tiles of two filter rows
// sharing the incoming-gradient operand were measured slower: 0.078 against
// 0.066 ms on 128x128x64x32.)  One MMA per K step covers the row's taps: B (MN-major) has
// one 64-channel N atom per tap, the atoms dx rows apart (LBO = dx * 128
// bytes, overlapping), each starting inside the strip at any 128-byte row;
// the 128-byte
// swizzle is keyed on the shared-memory address bits, as the TMA wrote the
// strip, so the base-offset field stays 0 (the parity tests cover every tap
// offset, dilation and strip width).
constexpr int WS_MAXST = 8;
constexpr int WS_SMEM = 200 * 1024;  // stage area budget

struct StripParams {
    const __nv_bfloat16 *x;  // [N][H][W][Cpad]
    const __nv_bfloat16 *g;  // [N][Ho][Wo][Kpad]
    float *partial;          // [splits][C*taps][K]
    int W, H, Cpad, C, N;
    int Wo, Ho, Kpad, K;  // Kpad: channels stored per pixel of G (a multiple of 64)
    int sy, px, py, dx, dy, fw, fh;
    int BX, BY, ntx, nty;
    int UB, nub;             // taps per tile along u, u-blocks per filter row
    int nchunk, n_k_tiles;
    int SL, strip_bytes, stage_bytes, nst;
    int KP, a_bytes;         // pixels per stage (MMA K: 64 or 128), incoming-gradient bytes per stage
    long long Q, chunk;      // pixel blocks, blocks per split
};

struct StripSmem {
    uint64_t full[WS_MAXST];
    uint64_t empty[WS_MAXST];
    uint64_t tmem_full;
    uint32_t tmem_base;
    int abort;
};

__global__ void __launch_bounds__(WG_THREADS, 1)
    wgrad_strip_kernel(const __grid_constant__ StripParams p, const __grid_constant__ CUtensorMap gmap,
                       const __grid_constant__ CUtensorMap smap) {
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    unsigned char *base = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    StripSmem *sm = reinterpret_cast<StripSmem *>(base + p.nst * p.stage_bytes);
    volatile int *abort = &sm->abort;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // tile: (k tile, u block, channel chunk, filter row)
    int t = blockIdx.x;
    const int ktile = t % p.n_k_tiles;
    t /= p.n_k_tiles;
    const int ub = t % p.nub;
    t /= p.nub;
    const int cchunk = t % p.nchunk;
    const int v = t / p.nchunk;
    const int k0 = ktile * 128;
    const int u0 = ub * p.UB;
    const int nu = min(p.UB, p.fw - u0);
    const long long q_begin = (long long)blockIdx.y * p.chunk;
    const long long q_end = min(p.Q, q_begin + p.chunk);
    const int nstages = (int)max(0LL, q_end - q_begin);

    if (threadIdx.x == 0) {
        for (int s = 0; s < p.nst; ++s) {
            mbar_init(&sm->full[s], 1);
            mbar_init(&sm->empty[s], 1);
        }
        mbar_init(&sm->tmem_full, 1);
        sm->abort = 0;
        fence_barrier_init();
    }
    if (warp == 4) tmem_alloc(&sm->tmem_base, 256);
    if (warp == 0 && lane == 0) {
        prefetch_tmap(&gmap);
        prefetch_tmap(&smap);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem_base = sm->tmem_base;

    if (warp == 0) {
        if (lane == 0) {
            const uint32_t bytes = (uint32_t)p.a_bytes + (uint32_t)(p.BY * p.SL * 128);
            // consecutive pixel blocks: (tx, ty, n) advance without division
            int tx = (int)(q_begin % p.ntx);
            const long long r0 = q_begin / p.ntx;
            int ty = (int)(r0 % p.nty), n = (int)(r0 / p.nty);
            int s = 0;
            uint32_t phase = 1;
            for (int st = 0; st < nstages && !*abort; ++st) {
                if (!mbar_wait(&sm->empty[s], phase, abort, 32u)) break;
                const int x0 = tx * p.BX, y0 = ty * p.BY;
                unsigned char *stage = base + s * p.stage_bytes;
                mbar_arrive_expect_tx(&sm->full[s], bytes);
                const uint32_t sa = smem_u32(stage);
                tma_load_4d(sa, &gmap, &sm->full[s], k0, x0, y0, n);
                tma_load_4d(sa + p.KP * 128, &gmap, &sm->full[s], k0 + 64, x0, y0, n);
                for (int j = 0; j < p.BY; ++j)
                    tma_load_4d(sa + p.a_bytes + j * p.strip_bytes, &smap, &sm->full[s], cchunk * 64,
                                x0 - p.px + u0 * p.dx, (y0 + j) * p.sy - p.py + v * p.dy, n);
                if (++s == p.nst) {
                    s = 0;
                    phase ^= 1u;
                }
                if (++tx == p.ntx) {
                    tx = 0;
                    if (++ty == p.nty) {
                        ty = 0;
                        ++n;
                    }
                }
            }
        }
        __syncwarp();
    } else if (warp >= 4) {
        if (warp == 4 && lane == 0) {
            // The issuing thread is latency-bound on its own scalar work, so
            // every descriptor is a precomputed base plus a 16-byte-unit
            // offset (the 14-bit start field holds any shared address), and
            // the stage index and barrier phase advance without division.
            // one MMA per K step covers all nu taps: B's N atoms (64 channels
            // each) are the tap-shifted views of the strip, dx rows apart
            const uint32_t idesc = idesc_bf16(128, (uint32_t)(64 * nu), 1, 1);
            const uint64_t a0 = smem_desc(smem_u32(base), (uint32_t)p.KP * 128u, 1024);
            const uint64_t b0 = smem_desc(smem_u32(base) + (uint32_t)p.a_bytes, (uint32_t)p.dx * 128u, 1024);
            const int ksteps = p.KP / 16;
            uint32_t bk[8];  // per K step: strip 16k/BX, row 16k%BX
#pragma unroll
            for (int k = 0; k < 8; ++k)
                bk[k] = (uint32_t)(((16 * k) / p.BX) * p.strip_bytes + ((16 * k) % p.BX) * 128) >> 4;
            const uint32_t stage_step = (uint32_t)p.stage_bytes >> 4;
            uint32_t soff = 0, phase = 0;
            int s = 0;
            for (int st = 0; st < nstages; ++st) {
                if (!mbar_wait(&sm->full[s], phase, abort, 64u)) break;
                tc_fence_after();
#pragma unroll
                for (int k = 0; k < 8; ++k)
                    if (k < ksteps)
                        mma_f16(tmem_base, a0 + soff + (uint32_t)k * 128u, b0 + soff + bk[k], idesc,
                                (st | k) != 0);
                mma_commit(&sm->empty[s]);
                if (++s == p.nst) {
                    s = 0;
                    soff = 0;
                    phase ^= 1u;
                } else {
                    soff += stage_step;
                }
            }
            mma_commit(&sm->tmem_full);
        }
        __syncwarp();
    }
    // ---------------- epilogue, all eight warps (warp w reads TMEM lanes
    // 32*(w % 4) .., i.e. k = k0 + 32*(w % 4) + lane, and takes every other
    // tap); waits for the MMAs even when aborting, so TMEM is never freed
    // under them.  The partial sums of one tap are 64 rows (c) of K floats:
    // with K a multiple of 4 they go through the now idle stage area, one
    // 32 KB tile [c][128 k] per tap, conflict-free shared stores, then bulk
    // copies (one per tap when K is 128, else one per row);
    // otherwise each thread stores its k column directly.
    {
        const int q = warp & 3, h = warp >> 2;
        bool have = false;
        if (nstages > 0) {
            have = mbar_wait_sleep(&sm->tmem_full, 0);
            if (!have) {
                *abort = 1;
                atomicOr(&g_tc_error, 128u);
            }
        }
        tc_fence_after();
        const int k = k0 + 32 * q + lane;
        const long long rows = (long long)p.C * p.fw * p.fh;
        float *out = p.partial + (long long)blockIdx.y * rows * p.K;
        const int ntap = nu;
        const int nrow = min(64, p.C - cchunk * 64);  // real c rows of a tap tile
        const int kcnt = min(128, p.K - k0);          // real k of a row
        const bool staged = (p.K & 3) == 0;
        const int slots = max(1, (p.nst * p.stage_bytes) / (64 * 128 * 4));
        auto tap_of = [&](int i) { return (u0 + i) + p.fw * v; };  // the tile's i-th tap
        for (int r0 = 0; r0 < ntap; r0 += slots) {
            const int rn = min(slots, ntap - r0);
            if (staged && r0 > 0) {
                if (threadIdx.x == 0) bulk_wait_read();  // the last round's copies have read the slots
                __syncthreads();
            }
            for (int i = r0 + h; i < r0 + rn; i += 2) {
                uint32_t v[4][16];
                if (have) {
#pragma unroll
                    for (int g = 0; g < 4; ++g)
                        tmem_ld16(tmem_base + (uint32_t)(i * 64 + 16 * g) + ((uint32_t)(32 * q) << 16), v[g]);
                    tmem_ld_wait();
                } else {
#pragma unroll
                    for (int g = 0; g < 4; ++g)
#pragma unroll
                        for (int e = 0; e < 16; ++e) v[g][e] = 0u;
                }
                if (*abort) continue;
                if (staged) {
                    float *tile = reinterpret_cast<float *>(base) + (size_t)(i - r0) * (64 * 128);
#pragma unroll
                    for (int g = 0; g < 4; ++g)
#pragma unroll
                        for (int e = 0; e < 16; ++e)
                            tile[(16 * g + e) * 128 + 32 * q + lane] = __uint_as_float(v[g][e]);
                } else if (k < p.K) {
                    const int tap = tap_of(i);
#pragma unroll
                    for (int g = 0; g < 4; ++g)
#pragma unroll
                        for (int e = 0; e < 16; ++e) {
                            const int c = cchunk * 64 + 16 * g + e;
                            if (c < p.C) out[((long long)c + (long long)p.C * tap) * p.K + k] = __uint_as_float(v[g][e]);
                        }
                }
            }
            if (!staged) continue;
            fence_proxy_async_smem();
            __syncthreads();
            if (threadIdx.x == 0 && !*abort) {
                for (int i = r0; i < r0 + rn; ++i) {
                    const uint32_t src = smem_u32(base) + (uint32_t)((i - r0) * 64 * 128 * 4);
                    float *dst = out + ((long long)p.C * tap_of(i) + cchunk * 64) * p.K + k0;
                    if (p.K == 128) {  // whole rows of 128 k: the tile is contiguous in the partials
                        bulk_store(dst, src, (uint32_t)(nrow * 128 * 4));
                    } else {
                        for (int c = 0; c < nrow; ++c)
                            bulk_store(dst + (long long)c * p.K, src + (uint32_t)(c * 128 * 4),
                                       (uint32_t)(kcnt * 4));
                    }
                }
                bulk_commit();
            }
        }
        if (staged && threadIdx.x == 0) bulk_wait_all();  // copies done before the CTA exits
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 4) {
        tc_fence_after();
        tmem_dealloc(tmem_base, 256);
    }
}

// ===========================================================================
// layout conversions (bandwidth-bound pre-passes)
// ===========================================================================
// f32 ArrayFire (W,H,C,N) -> bf16 [N][H][W][Cpad], channels >= C zero.
// One CTA converts a 64-pixel x 64-channel block of one image row: float4
// loads along x (256 bytes per channel row), a padded shared tile, then
// 16-byte stores of eight bf16 channels, four pixels (512 bytes) per warp.
__global__ void __launch_bounds__(256) to_nhwc_bf16_kernel(const float *__restrict__ in, int W,
                                                           int H, int C, int N, int Cpad,
                                                           __nv_bfloat16 *__restrict__ out) {
    __shared__ float tile[64][65];
    const int x0 = blockIdx.x * 64;
    const int yn = blockIdx.y;  // y + H*n
    const int y = yn % H, n = yn / H;
    const int c0 = blockIdx.z * 64;
    const long long plane = (long long)W * H;
    const int t = threadIdx.x;
    const bool vec = ((W & 3) == 0) && (x0 + 64 <= W) && ((reinterpret_cast<uintptr_t>(in) & 15) == 0);
    if (vec) {
        const int x4 = (t & 15) * 4;
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int ci = (t >> 4) + 16 * i;
            const int c = c0 + ci;
            float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
            if (c < C)
                v = __ldg(reinterpret_cast<const float4 *>(
                    in + x0 + x4 + (long long)W * y + plane * (c + (long long)C * n)));
            tile[ci][x4] = v.x;
            tile[ci][x4 + 1] = v.y;
            tile[ci][x4 + 2] = v.z;
            tile[ci][x4 + 3] = v.w;
        }
    } else {
        for (int e = t; e < 64 * 64; e += 256) {
            const int ci = e >> 6, xi = e & 63;
            const int c = c0 + ci, x = x0 + xi;
            float v = 0.f;
            if (c < C && x < W) v = in[x + (long long)W * y + plane * (c + (long long)C * n)];
            tile[ci][xi] = v;
        }
    }
    __syncthreads();
    const int lane = t & 31, warp = t >> 5;
    const int cg = lane & 7;  // eight channels
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
        const int xi = pass * 32 + warp * 4 + (lane >> 3);
        const int x = x0 + xi;
        if (x < W) {
            uint4 w;
            __nv_bfloat162 b0 = __floats2bfloat162_rn(tile[cg * 8 + 0][xi], tile[cg * 8 + 1][xi]);
            __nv_bfloat162 b1 = __floats2bfloat162_rn(tile[cg * 8 + 2][xi], tile[cg * 8 + 3][xi]);
            __nv_bfloat162 b2 = __floats2bfloat162_rn(tile[cg * 8 + 4][xi], tile[cg * 8 + 5][xi]);
            __nv_bfloat162 b3 = __floats2bfloat162_rn(tile[cg * 8 + 6][xi], tile[cg * 8 + 7][xi]);
            w.x = *reinterpret_cast<uint32_t *>(&b0);
            w.y = *reinterpret_cast<uint32_t *>(&b1);
            w.z = *reinterpret_cast<uint32_t *>(&b2);
            w.w = *reinterpret_cast<uint32_t *>(&b3);
            *reinterpret_cast<uint4 *>(out + (((long long)n * H + y) * W + x) * Cpad + c0 + cg * 8) = w;
        }
    }
}

// f32 ArrayFire (W,H,C,N) -> bf16 [N][H*W][Cpad], over the flattened pixel
// plane P = W*H (NCHW and NHWC both keep pixels in y*W + x order, so the
// conversion is a transpose of [C][P] per image, independent of W).  A block
// converts 128 pixels x 64 channels:
//   phase 1: a thread reads four pixels of two channels (two 16-byte loads;
//            eight lanes cover 128 contiguous bytes of a channel row) and
//            stores one bf16x2 word per pixel into [pixel][32 words], word
//            column c2 ^ 4*((pixel >> 2) & 7) (conflict-free for the 32
//            lanes of a warp);
//   phase 2: a thread reads one pixel's eight channels (16 bytes: the
//            swizzle keeps each aligned group of four words contiguous) and
//            stores them to the pixel's 128-byte row.
// Pixels beyond P and channels beyond C are zero.  Needs P % 4 == 0 and a
// 16-byte aligned source; to_nhwc_bf16_kernel covers the rest.
constexpr int CV_PIX = 128;
__global__ void __launch_bounds__(256) to_nhwc_flat_bf16_kernel(const float *__restrict__ in,
                                                                long long P, int C, int Cpad,
                                                                long long tiles_p,
                                                                long long ntiles,
                                                                __nv_bfloat16 *__restrict__ out) {
    __shared__ __align__(16) uint32_t tile[CV_PIX * 32];
    const int t = threadIdx.x, lane = t & 31, warp = t >> 5;
    const int nck = Cpad / 64;
    for (long long bt = blockIdx.x; bt < ntiles; bt += gridDim.x) {
        const long long ck = bt % nck;
        const long long r = bt / nck;
        const long long pt = r % tiles_p;
        const long long n = r / tiles_p;
        const long long p0 = pt * CV_PIX;
        const int c0 = (int)ck * 64;
        // phase 1: item = (c2 in 0..31, p4 in 0..31); lane -> p4 low 3 bits, c2 low 2 bits
#pragma unroll
        for (int it = 0; it < 4; ++it) {
            const int combo = warp * 4 + it;  // 0..31: (c2_hi 0..7, p4_hi 0..3)
            const int p4 = (combo & 3) * 8 + (lane & 7);
            const int c2 = (combo >> 2) * 4 + (lane >> 3);
            const int c = c0 + 2 * c2;
            const long long px = p0 + 4 * p4;
            float4 a = make_float4(0.f, 0.f, 0.f, 0.f), b = a;
            if (px < P) {
                const float *src = in + (n * C + c) * P + px;
                if (c < C) a = __ldg(reinterpret_cast<const float4 *>(src));
                if (c + 1 < C) b = __ldg(reinterpret_cast<const float4 *>(src + P));
            }
            const float av[4] = {a.x, a.y, a.z, a.w}, bv[4] = {b.x, b.y, b.z, b.w};
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int pl = 4 * p4 + i;
                __nv_bfloat162 h = __floats2bfloat162_rn(av[i], bv[i]);
                tile[pl * 32 + (c2 ^ (4 * (p4 & 7)))] = *reinterpret_cast<uint32_t *>(&h);
            }
        }
        __syncthreads();
        // phase 2: item = (pixel 0..127, 16-byte chunk j 0..7)
#pragma unroll
        for (int it = 0; it < 4; ++it) {
            const int item = it * 256 + t;
            const int pl = item >> 3, j = item & 7;
            const long long px = p0 + pl;
            if (px < P) {
                const uint4 w = *reinterpret_cast<const uint4 *>(
                    &tile[pl * 32 + 4 * (j ^ ((pl >> 2) & 7))]);
                *reinterpret_cast<uint4 *>(out + (n * P + px) * Cpad + c0 + 8 * j) = w;
            }
        }
        __syncthreads();
    }
}

// weights (fw,fh,C,K) f32 -> bf16 GEMM operand with the reference's flip:
// forward  Wt[och=k][tap*Cpad + c];  data grad Wt[och=c][tap*Kpad + k]
// with tap = u + fw*v multiplying w[fw-1-u, fh-1-v, c, k]; padded rows and
// channels are zero
__global__ void weights_bf16_kernel(const float *__restrict__ w, int fw, int fh, int C, int K,
                                    int mode, int och_pad, int in_pad,
                                    __nv_bfloat16 *__restrict__ out) {
    const long long total = (long long)och_pad * fw * fh * in_pad;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int ci = (int)(t % in_pad);
        const long long r = t / in_pad;
        const int tap = (int)(r % (fw * fh));
        const int och = (int)(r / (fw * fh));
        const int u = tap % fw, v = tap / fw;
        const int c = mode == 0 ? ci : och;
        const int k = mode == 0 ? och : ci;
        float val = 0.f;
        if (c < C && k < K) val = w[(fw - 1 - u) + fw * ((fh - 1 - v) + fh * (c + (long long)C * k))];
        out[t] = __float2bfloat16_rn(val);
    }
}

// ---- taps folded into channels ---------------------------------------------
// When C*fw*fh <= 64 (an RGB input layer, a 1x1 layer with few channels) a
// per-tap reduction would be mostly channel padding.  Folding gives each
// output pixel one 64-channel bf16 row holding every (c, u, v) its output
// reads: row[c + C*(u + fw*v)] = x[xo*sx - px + u*dx, yo*sy - py + v*dy, c, n]
// (zero outside the image), so the forward and the filter gradient become
// 1x1, stride-1 problems on the output grid.
__global__ void __launch_bounds__(256) fold_taps_bf16_kernel(
    const float *__restrict__ x, int W, int H, int C, int N, int fw, int fh, int sx, int sy,
    int px, int py, int dx, int dy, int Wo, int Ho, __nv_bfloat16 *__restrict__ out) {
    // per folded channel j: source channel and tap offset (c < 0: padding)
    __shared__ int tc[64], tdx[64], tdy[64];
    const int KC = C * fw * fh;
    if (threadIdx.x < 64) {
        const int j = threadIdx.x;
        const int tap = j / C, u = tap % fw, v = tap / fw;
        tc[j] = j < KC ? j % C : -1;
        tdx[j] = u * dx - px;
        tdy[j] = v * dy - py;
    }
    __syncthreads();
    const long long npix = (long long)Wo * Ho * N;
    const long long plane = (long long)W * H;
    const int nj8 = (KC + 7) / 8;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < npix;
         q += (long long)gridDim.x * blockDim.x) {
        const int xo = (int)(q % Wo);
        const long long r = q / Wo;
        const int yo = (int)(r % Ho);
        const int n = (int)(r / Ho);
        const float *img = x + plane * C * n;
        const int xb = xo * sx, yb = yo * sy;
        uint4 *dst = reinterpret_cast<uint4 *>(out + q * 64);
        for (int j8 = 0; j8 < 8; ++j8) {
            uint32_t wd[4] = {0u, 0u, 0u, 0u};
            if (j8 < nj8) {
#pragma unroll
                for (int e = 0; e < 4; ++e) {
                    float v2[2];
#pragma unroll
                    for (int h = 0; h < 2; ++h) {
                        const int j = j8 * 8 + e * 2 + h;
                        const int c = tc[j];
                        const int xs = xb + tdx[j], ys = yb + tdy[j];
                        v2[h] = (c >= 0 && xs >= 0 && xs < W && ys >= 0 && ys < H)
                                    ? __ldg(img + plane * c + (long long)W * ys + xs)
                                    : 0.f;
                    }
                    const __nv_bfloat162 b2 = __floats2bfloat162_rn(v2[0], v2[1]);
                    wd[e] = *reinterpret_cast<const uint32_t *>(&b2);
                }
            }
            dst[j8] = make_uint4(wd[0], wd[1], wd[2], wd[3]);
        }
    }
}

// folded filter: Wt[och][c + C*(u + fw*v)] = w[fw-1-u, fh-1-v, c, och], zero
// beyond C*fw*fh channels and K output channels; och_pad x 64 bf16
__global__ void weights_fold_bf16_kernel(const float *__restrict__ w, int fw, int fh, int C, int K,
                                         int och_pad, __nv_bfloat16 *__restrict__ out) {
    const long long total = (long long)och_pad * 64;
    const int KC = C * fw * fh;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int j = (int)(t % 64);
        const int och = (int)(t / 64);
        float val = 0.f;
        if (j < KC && och < K) {
            const int c = j % C, tap = j / C;
            const int u = tap % fw, v = tap / fw;
            val = w[(fw - 1 - u) + fw * ((fh - 1 - v) + fh * (c + (long long)C * och))];
        }
        out[t] = __float2bfloat16_rn(val);
    }
}

// ---- FP8-E4M3 operands -----------------------------------------------------
// |x| maximum over n floats, as float bits (non-negative floats order like
// their bit patterns); *out must start at 0
__global__ void amax_kernel(const float *__restrict__ x, long long n, unsigned int *out) {
    float m = 0.f;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        m = fmaxf(m, fabsf(x[i]));
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) atomicMax(out, __float_as_uint(m));
}

// per-output-channel |w| maximum of a (fw,fh,C,K) filter -> scale = amax/448
__global__ void weight_scale_kernel(const float *__restrict__ w, long long per_k, int K,
                                    float *__restrict__ scale) {
    const int k = blockIdx.x;
    if (k >= K) return;
    float m = 0.f;
    for (long long i = threadIdx.x; i < per_k; i += blockDim.x) m = fmaxf(m, fabsf(w[i + per_k * k]));
    __shared__ float red[32];
    for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, off));
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x < 32) {
        m = threadIdx.x < (blockDim.x >> 5) ? red[threadIdx.x] : 0.f;
        for (int off = 16; off > 0; off >>= 1) m = fmaxf(m, __shfl_down_sync(0xffffffffu, m, off));
        if (threadIdx.x == 0) scale[k] = m > 0.f ? m / 448.0f : 1.0f;
    }
}

// activation scale = amax/448; combined epilogue factor per output channel
__global__ void combine_scale_kernel(const unsigned int *amax_bits, const float *wscale, int K,
                                     float *act_scale, float *out_scale) {
    const float a = __uint_as_float(*amax_bits);
    const float as = a > 0.f ? a / 448.0f : 1.0f;
    if (blockIdx.x == 0 && threadIdx.x == 0) *act_scale = as;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < K; k += gridDim.x * blockDim.x)
        out_scale[k] = as * wscale[k];
}

__device__ __forceinline__ unsigned char to_e4m3(float v) {
    return (unsigned char)__nv_cvt_float_to_fp8(v, __NV_SATFINITE, __NV_E4M3);
}

// f32 ArrayFire (W,H,C,N) -> e4m3 [N][H][W][Cpad] of x / act_scale
// f32 ArrayFire planes (W*H pixels with 16-byte aligned rows, as the flat
// bf16 converter takes them) -> e4m3 [N][H][W][Cpad] scaled by 1/act_scale:
// one block converts CV_PIX pixels x 64 channels.  Phase 1: an item is four
// channels x four pixels (four float4 loads along the pixels), packed into
// one 32-bit word of four e4m3 channels per pixel, into a tile of 16 words per
// pixel whose word index is XOR-swizzled by the pixel; phase 2: 16-byte
// stores of 16 channels of one pixel.  Rounding and saturation are those of
// the per-element converter, so the bytes are the same.
__global__ void __launch_bounds__(256) to_nhwc_flat_e4m3_kernel(const float *__restrict__ in,
                                                                long long P, int C, int Cpad,
                                                                long long tiles_p, long long ntiles,
                                                                const float *act_scale,
                                                                unsigned char *__restrict__ out) {
    __shared__ __align__(16) uint32_t tile[CV_PIX * 16];
    const int t = threadIdx.x;
    const int nck = Cpad / 64;
    const float inv = 1.0f / *act_scale;
    for (long long bt = blockIdx.x; bt < ntiles; bt += gridDim.x) {
        const long long ck = bt % nck;
        const long long r = bt / nck;
        const long long pt = r % tiles_p;
        const long long n = r / tiles_p;
        const long long p0 = pt * CV_PIX;
        const int c0 = (int)ck * 64;
        // phase 1: item = (c4 in 0..15, p4 in 0..CV_PIX/4-1)
        for (int item = t; item < 16 * (CV_PIX / 4); item += 256) {
            const int c4 = item & 15, p4 = item >> 4;
            const long long px = p0 + 4 * p4;
            float4 v[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                const int c = c0 + 4 * c4 + i;
                v[i] = make_float4(0.f, 0.f, 0.f, 0.f);
                if (px < P && c < C) v[i] = __ldg(reinterpret_cast<const float4 *>(in + (n * C + c) * P + px));
            }
            const float a[4][4] = {{v[0].x, v[0].y, v[0].z, v[0].w}, {v[1].x, v[1].y, v[1].z, v[1].w},
                                   {v[2].x, v[2].y, v[2].z, v[2].w}, {v[3].x, v[3].y, v[3].z, v[3].w}};
#pragma unroll
            for (int j = 0; j < 4; ++j) {  // pixel 4*p4 + j: channels 4*c4 .. +3
                const int pl = 4 * p4 + j;
                const uint32_t w = (uint32_t)to_e4m3(a[0][j] * inv) | ((uint32_t)to_e4m3(a[1][j] * inv) << 8) |
                                   ((uint32_t)to_e4m3(a[2][j] * inv) << 16) |
                                   ((uint32_t)to_e4m3(a[3][j] * inv) << 24);
                tile[pl * 16 + (c4 ^ (pl & 15))] = w;
            }
        }
        __syncthreads();
        // phase 2: item = (pixel, 16-byte chunk j in 0..3)
        for (int item = t; item < CV_PIX * 4; item += 256) {
            const int pl = item >> 2, j = item & 3;
            const long long px = p0 + pl;
            if (px < P) {
                uint4 w;
                w.x = tile[pl * 16 + ((4 * j + 0) ^ (pl & 15))];
                w.y = tile[pl * 16 + ((4 * j + 1) ^ (pl & 15))];
                w.z = tile[pl * 16 + ((4 * j + 2) ^ (pl & 15))];
                w.w = tile[pl * 16 + ((4 * j + 3) ^ (pl & 15))];
                *reinterpret_cast<uint4 *>(out + (n * P + px) * Cpad + c0 + 16 * j) = w;
            }
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(256) to_nhwc_e4m3_kernel(const float *__restrict__ in, int W,
                                                           int H, int C, int N, int Cpad,
                                                           const float *act_scale,
                                                           unsigned char *__restrict__ out) {
    __shared__ float tile[64][65];
    const int x0 = blockIdx.x * 64;
    const int yn = blockIdx.y;
    const int y = yn % H, n = yn / H;
    const int c0 = blockIdx.z * 64;
    const long long plane = (long long)W * H;
    const int t = threadIdx.x;
    const float inv = 1.0f / *act_scale;
    for (int e = t; e < 64 * 64; e += 256) {
        const int ci = e >> 6, xi = e & 63;
        const int c = c0 + ci, x = x0 + xi;
        float v = 0.f;
        if (c < C && x < W) v = in[x + (long long)W * y + plane * (c + (long long)C * n)];
        tile[ci][xi] = v * inv;
    }
    __syncthreads();
    const int lane = t & 31, warp = t >> 5;
    const int cg = lane & 7;
#pragma unroll
    for (int pass = 0; pass < 2; ++pass) {
        const int xi = pass * 32 + warp * 4 + (lane >> 3);
        const int x = x0 + xi;
        if (x < W) {
            uint2 w;
            w.x = (uint32_t)to_e4m3(tile[cg * 8 + 0][xi]) | ((uint32_t)to_e4m3(tile[cg * 8 + 1][xi]) << 8) |
                  ((uint32_t)to_e4m3(tile[cg * 8 + 2][xi]) << 16) | ((uint32_t)to_e4m3(tile[cg * 8 + 3][xi]) << 24);
            w.y = (uint32_t)to_e4m3(tile[cg * 8 + 4][xi]) | ((uint32_t)to_e4m3(tile[cg * 8 + 5][xi]) << 8) |
                  ((uint32_t)to_e4m3(tile[cg * 8 + 6][xi]) << 16) | ((uint32_t)to_e4m3(tile[cg * 8 + 7][xi]) << 24);
            *reinterpret_cast<uint2 *>(out + (((long long)n * H + y) * W + x) * Cpad + c0 + cg * 8) = w;
        }
    }
}

// forward weights -> e4m3 Wt[k][tap*Cpad + c] of w[fw-1-u, fh-1-v, c, k] / wscale[k]
__global__ void weights_e4m3_kernel(const float *__restrict__ w, int fw, int fh, int C, int K,
                                    int och_pad, int in_pad, const float *__restrict__ wscale,
                                    unsigned char *__restrict__ out) {
    const long long total = (long long)och_pad * fw * fh * in_pad;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(t % in_pad);
        const long long r = t / in_pad;
        const int tap = (int)(r % (fw * fh));
        const int k = (int)(r / (fw * fh));
        const int u = tap % fw, v = tap / fw;
        float val = 0.f;
        if (c < C && k < K)
            val = w[(fw - 1 - u) + fw * ((fh - 1 - v) + fh * (c + (long long)C * k))] / wscale[k];
        out[t] = to_e4m3(val);
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
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiledFn>(p);
    });
    if (!fn) AFGB_THROW(AF_ERR_DRIVER, "cuTensorMapEncodeTiled is unavailable");
    return fn;
}

// 2-D tensor [rows][cols] (cols contiguous) of bf16 (esize 2) or e4m3 bytes
// (esize 1), box 128 bytes x 128 rows, 128B swizzle
static CUtensorMap make_wmap(const void *ptr, long long rows, long long cols, int esize = 2,
                             int box_rows = 128) {
    CUtensorMap m;
    cuuint64_t dims[2] = {(cuuint64_t)cols, (cuuint64_t)rows};
    cuuint64_t strides[1] = {(cuuint64_t)cols * esize};
    cuuint32_t box[2] = {(cuuint32_t)(128 / esize), (cuuint32_t)box_rows};
    cuuint32_t es[2] = {1, 1};
    CUresult r = encode_fn()(&m, esize == 2 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_UINT8,
                             2, (void *)ptr, dims, strides, box,
                             es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) AFGB_THROW(AF_ERR_INTERNAL, "cuTensorMapEncodeTiled (weights) failed");
    return m;
}

// 4-D NHWC tensor (Cpad, W, H, N) of bf16 (esize 2) or e4m3 bytes (esize 1),
// 128B swizzle, out-of-range elements read as zero.  A load brings bx x by
// pixels of 128 bytes; with traversal strides (sx, sy) those pixels are every
// sx-th along x and every sy-th along y (the box then spans bx*sx x by*sy).
static CUtensorMap make_imap(const void *ptr, int Cpad, int W, int H, int N, int bx, int by,
                             int esize = 2, int sx = 1, int sy = 1) {
    CUtensorMap m;
    cuuint64_t dims[4] = {(cuuint64_t)Cpad, (cuuint64_t)W, (cuuint64_t)H, (cuuint64_t)N};
    cuuint64_t strides[3] = {(cuuint64_t)Cpad * esize, (cuuint64_t)Cpad * esize * W,
                             (cuuint64_t)Cpad * esize * W * H};
    cuuint32_t box[4] = {(cuuint32_t)(128 / esize), (cuuint32_t)(bx * sx), (cuuint32_t)(by * sy), 1};
    cuuint32_t es[4] = {1, (cuuint32_t)sx, (cuuint32_t)sy, 1};
    CUresult r = encode_fn()(&m, esize == 2 ? CU_TENSOR_MAP_DATA_TYPE_BFLOAT16 : CU_TENSOR_MAP_DATA_TYPE_UINT8,
                             4, (void *)ptr, dims, strides, box,
                             es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) AFGB_THROW(AF_ERR_INTERNAL, "cuTensorMapEncodeTiled (image) failed");
    return m;
}

static int round_up(int v, int m) { return (v + m - 1) / m * m; }

static __nv_bfloat16 *to_nhwc(const float *src, int W, int H, int C, int N, int Cpad) {
    __nv_bfloat16 *out;
    {
        MemTag tag("bf16 channels-last copies");
        out = static_cast<__nv_bfloat16 *>(
            alloc_device((size_t)W * H * N * Cpad * sizeof(__nv_bfloat16)));
    }
    const long long P = (long long)W * H;
    if ((P & 3) == 0 && (reinterpret_cast<uintptr_t>(src) & 15) == 0) {
        const long long tiles_p = (P + CV_PIX - 1) / CV_PIX;
        const long long ntiles = tiles_p * N * (Cpad / 64);
        const unsigned grid = (unsigned)std::min<long long>(ntiles, (long long)num_sms() * 8);
        {
            KernelTimer kt("tc_convert_kernel");
            to_nhwc_flat_bf16_kernel<<<grid, 256, 0, stream()>>>(src, P, C, Cpad, tiles_p, ntiles,
                                                                 out);
        }
        count_launch();
        AFGB_POST_LAUNCH("to_nhwc_flat_bf16_kernel");
        return out;
    }
    dim3 grid((unsigned)((W + 63) / 64), (unsigned)(H * N), (unsigned)(Cpad / 64));
    {
        KernelTimer kt("tc_convert_kernel");
        to_nhwc_bf16_kernel<<<grid, 256, 0, stream()>>>(src, W, H, C, N, Cpad, out);
    }
    count_launch();
    AFGB_POST_LAUNCH("to_nhwc_bf16_kernel");
    return out;
}

// The signal in bf16 channels-last form for the tensor-core kernels.  A
// dense f32 array in library-owned memory keeps its converted copy on its
// buffer, so the forward and the filter gradient of one training step
// convert the signal once; the copy is dropped as soon as anything writes
// the buffer (or hands it out for writing), and it is reused only on the
// stream it was made on.  Other arrays are converted per call; `owned` then
// tells the caller to free the copy.
static const __nv_bfloat16 *signal_nhwc(const Array &sig, int W, int H, int C, int N, int Cpad,
                                        bool &owned) {
    Buffer *b = sig.buf.get();
    const bool cacheable = b && b->kind == BufKind::Pool && sig.type == f32 && sig.is_linear();
    owned = !cacheable;
    if (!cacheable) return to_nhwc(sig.ptr<float>(), W, H, C, N, Cpad);
    unsigned long long key = (unsigned long long)sig.offset;
    for (long long v : {(long long)W, (long long)H, (long long)C, (long long)N, (long long)Cpad})
        key = key * 0x100000001B3ull ^ (unsigned long long)v;
    key |= 1ull;  // never 0 (no copy)
    std::lock_guard<std::mutex> lk(b->derived_mu);
    if (b->derived && b->derived_key == key && b->derived_stream == stream())
        return static_cast<const __nv_bfloat16 *>(b->derived);
    __nv_bfloat16 *x = to_nhwc(sig.ptr<float>(), W, H, C, N, Cpad);
    if (b->derived) free_device(b->derived);
    b->derived = x;
    b->derived_key = key;
    b->derived_stream = stream();
    return x;
}

static bool foldable(const NNGeom &g) { return g.C * g.fw * g.fh <= 64; }

// the 1x1, stride-1 problem over the output grid that tap folding turns g into
static NNGeom folded_geometry(const NNGeom &g) {
    NNGeom f = g;
    f.W = g.Wo;
    f.H = g.Ho;
    f.C = g.C * g.fw * g.fh;
    f.fw = f.fh = 1;
    f.sx = f.sy = 1;
    f.px = f.py = 0;
    f.dx = f.dy = 1;
    return f;
}

static __nv_bfloat16 *fold_taps(const float *x, const NNGeom &g) {
    const long long npix = g.Wo * g.Ho * g.N;
    MemTag tag("bf16 channels-last copies");
    __nv_bfloat16 *out = static_cast<__nv_bfloat16 *>(alloc_device((size_t)npix * 64 * 2));
    const unsigned blocks = (unsigned)std::max(1LL, std::min<long long>((npix + 255) / 256,
                                                                        num_sms() * 16LL));
    {
        KernelTimer kt("tc_convert_kernel");
        fold_taps_bf16_kernel<<<blocks, 256, 0, stream()>>>(
            x, (int)g.W, (int)g.H, (int)g.C, (int)g.N, (int)g.fw, (int)g.fh, (int)g.sx, (int)g.sy,
            (int)g.px, (int)g.py, (int)g.dx, (int)g.dy, (int)g.Wo, (int)g.Ho, out);
    }
    count_launch();
    AFGB_POST_LAUNCH("fold_taps_bf16_kernel");
    return out;
}

// rectangle bx x by (bx*by == area, bx >= minx) covering W x H with the
// least padding; ties prefer the wider rectangle.  With traversal strides the
// box spans bx*sx x by*sy elements, at most 256 each.  False when no
// rectangle fits.
static bool pick_rect(int W, int H, int area, int minx, int &bx, int &by, int sx = 1, int sy = 1) {
    long long best = -1;
    int x = 1;  // widest power of two within the area and the box limit
    while (x * 2 <= std::min(area, 256 / sx)) x *= 2;
    bx = x;
    by = area / bx;
    for (; x >= minx; x >>= 1) {
        const int y = area / x;
        if (x * y != area) continue;
        if ((long long)y * sy > 256) break;
        const long long cover = (long long)((W + x - 1) / x) * x * ((H + y - 1) / y) * y;
        if (best < 0 || cover < best) {
            best = cover;
            bx = x;
            by = y;
        }
    }
    return best >= 0;
}

static size_t gather_smem() {
    static_assert(32 * EP_PITCH <= EP_SLOT && 32 * 16 <= EP_SLOT, "epilogue staging slot");
    return 1024 + STAGES * (A_BYTES + B_BYTES) + EP_WARPS * EP_SLOT * sizeof(float) + sizeof(Smem) +
           64;
}

// forward (mode 0) or data gradient (mode 1); fp8 (forward only): e4m3
// operands with a per-tensor activation scale and per-output-channel weight
// scales (`user_wscale`, K floats, or amax/448 computed on the device)
// `unfolded`: g is the folded geometry of *unfolded (bf16 forward only); the
// image and filter are folded from the f32 operands of *unfolded
// `img_ready`: the source image already in bf16 NHWC with its channels padded
// to a multiple of 64 (then img_f32 is not read)
static void run_gather(const NNGeom &g, int mode, const float *img_f32, const float *w_f32,
                       float *dst, bool fp8 = false, const float *user_wscale = nullptr,
                       const NNGeom *unfolded = nullptr, const __nv_bfloat16 *img_ready = nullptr,
                       const NNEpilogue *ep = nullptr) {
    const int SW = mode == 0 ? (int)g.W : (int)g.Wo;
    const int SH = mode == 0 ? (int)g.H : (int)g.Ho;
    const int SC = mode == 0 ? (int)g.C : (int)g.K;
    const int DW = mode == 0 ? (int)g.Wo : (int)g.W;
    const int DH = mode == 0 ? (int)g.Ho : (int)g.H;
    const int DC = mode == 0 ? (int)g.K : (int)g.C;
    const int CH = fp8 ? 128 : 64;  // channels per 128-byte row
    const int SCpad = round_up(SC, CH);
    const int OCpad = round_up(DC, 128);
    const int taps = (int)(g.fw * g.fh);
    // pixel operand by TMA: strided forwards through the tensor map's
    // traversal strides (at most 8); data gradients per stride phase, whose
    // operand rectangles are unit-stride in the incoming gradient
    int rbx = 0, rby = 0;
    const int tsx = mode == 0 ? (int)g.sx : 1, tsy = mode == 0 ? (int)g.sy : 1;
    const int MX0 = mode == 0 ? DW : (int)((DW + g.sx - 1) / g.sx);
    const int MY0 = mode == 0 ? DH : (int)((DH + g.sy - 1) / g.sy);
    const bool tma_b = tsx <= 8 && tsy <= 8 && pick_rect(MX0, MY0, BN, 32, rbx, rby, tsx, tsy);
    const int esize = fp8 ? 1 : 2;

    void *img = nullptr, *wt = nullptr;
    float *scales = nullptr;  // [0] activation scale, [1..K] weight scales, [K+1..2K] output factors
    unsigned int *amax = nullptr;
    if (!fp8 && unfolded) {
        img = fold_taps(img_f32, *unfolded);
        MemTag tag("weight operands");
        wt = alloc_device((size_t)OCpad * 64 * 2);
        const long long total = (long long)OCpad * 64;
        const unsigned blocks = (unsigned)std::min<long long>((total + 255) / 256, num_sms() * 8LL);
        weights_fold_bf16_kernel<<<blocks, 256, 0, stream()>>>(
            w_f32, (int)unfolded->fw, (int)unfolded->fh, (int)unfolded->C, (int)unfolded->K, OCpad,
            static_cast<__nv_bfloat16 *>(wt));
        count_launch();
        AFGB_POST_LAUNCH("weights_fold_bf16_kernel");
    } else if (!fp8) {
        img = img_ready ? const_cast<__nv_bfloat16 *>(img_ready)
                        : to_nhwc(img_f32, SW, SH, SC, (int)g.N, SCpad);
        MemTag tag("weight operands");
        wt = alloc_device((size_t)OCpad * taps * SCpad * 2);
        long long total = (long long)OCpad * taps * SCpad;
        unsigned blocks = (unsigned)std::min<long long>((total + 255) / 256, num_sms() * 8LL);
        weights_bf16_kernel<<<blocks, 256, 0, stream()>>>(w_f32, (int)g.fw, (int)g.fh, (int)g.C,
                                                          (int)g.K, mode, OCpad, SCpad,
                                                          static_cast<__nv_bfloat16 *>(wt));
        count_launch();
        AFGB_POST_LAUNCH("weights_bf16_kernel");
    } else {
        const int K = (int)g.K;
        MemTag tag("fp8 operands and scales");
        scales = static_cast<float *>(alloc_device((size_t)(2 * K + 1) * sizeof(float)));
        amax = static_cast<unsigned int *>(alloc_device(sizeof(unsigned int)));
        AFGB_CUDA(cudaMemsetAsync(amax, 0, sizeof(unsigned int), stream()));
        const long long nx = (long long)SW * SH * SC * g.N;
        amax_kernel<<<std::max(1, std::min(num_sms() * 8, (int)((nx + 255) / 256))), 256, 0, stream()>>>(
            img_f32, nx, amax);
        count_launch();
        AFGB_POST_LAUNCH("amax_kernel");
        const float *wscale = user_wscale;
        if (!wscale) {
            weight_scale_kernel<<<K, 256, 0, stream()>>>(w_f32, g.fw * g.fh * g.C, K, scales + 1);
            count_launch();
            AFGB_POST_LAUNCH("weight_scale_kernel");
            wscale = scales + 1;
        }
        combine_scale_kernel<<<(K + 255) / 256, 256, 0, stream()>>>(amax, wscale, K, scales,
                                                                  scales + 1 + K);
        count_launch();
        AFGB_POST_LAUNCH("combine_scale_kernel");
        img = alloc_device((size_t)SW * SH * g.N * SCpad);
        const long long P = (long long)SW * SH;
        if ((P & 3) == 0 && (reinterpret_cast<uintptr_t>(img_f32) & 15) == 0) {
            const long long tiles_p = (P + CV_PIX - 1) / CV_PIX;
            const long long ntiles = tiles_p * g.N * (SCpad / 64);
            const unsigned grid = (unsigned)std::min<long long>(ntiles, (long long)num_sms() * 8);
            {
                KernelTimer kt("tc_convert_kernel");
                to_nhwc_flat_e4m3_kernel<<<grid, 256, 0, stream()>>>(img_f32, P, SC, SCpad, tiles_p,
                                                                     ntiles, scales,
                                                                     static_cast<unsigned char *>(img));
            }
            count_launch();
            AFGB_POST_LAUNCH("to_nhwc_flat_e4m3_kernel");
        } else {
            dim3 cgrid((unsigned)((SW + 63) / 64), (unsigned)(SH * g.N), (unsigned)(SCpad / 64));
            {
                KernelTimer kt("tc_convert_kernel");
                to_nhwc_e4m3_kernel<<<cgrid, 256, 0, stream()>>>(img_f32, SW, SH, SC, (int)g.N, SCpad,
                                                                 scales, static_cast<unsigned char *>(img));
            }
            count_launch();
            AFGB_POST_LAUNCH("to_nhwc_e4m3_kernel");
        }
        wt = alloc_device((size_t)OCpad * taps * SCpad);
        long long total = (long long)OCpad * taps * SCpad;
        unsigned blocks = (unsigned)std::min<long long>((total + 255) / 256, num_sms() * 8LL);
        weights_e4m3_kernel<<<blocks, 256, 0, stream()>>>(w_f32, (int)g.fw, (int)g.fh, (int)g.C, K,
                                                          OCpad, SCpad, wscale,
                                                          static_cast<unsigned char *>(wt));
        count_launch();
        AFGB_POST_LAUNCH("weights_e4m3_kernel");
    }

    GatherParams p;
    std::memset(&p, 0, sizeof(p));
    p.src = static_cast<const unsigned char *>(img);
    p.dst = dst;
    p.out_scale = fp8 ? scales + 1 + g.K : nullptr;
    if (ep && mode == 0) {
        p.bias = ep->bias;
        p.relu = ep->relu;
    }
    p.SW = SW;
    p.SH = SH;
    p.SCpad = SCpad;
    p.N = (int)g.N;
    p.DW = DW;
    p.DH = DH;
    p.DC = DC;
    p.mode = mode;
    p.sx = (int)g.sx;
    p.sy = (int)g.sy;
    p.px = (int)g.px;
    p.py = (int)g.py;
    p.dx = (int)g.dx;
    p.dy = (int)g.dy;
    p.fw = (int)g.fw;
    p.nchunk = SCpad / CH;
    p.n_och_tiles = OCpad / 128;
    p.nphx = mode == 0 ? 1 : (int)g.sx;
    p.nphase = mode == 0 ? 1 : (int)(g.sx * g.sy);
    // column groups: stride 1, bf16, two or three taps per filter column
    // within a two-row span, images at least one rectangle wide
    const int cg_span = (int)((g.fh - 1) * g.dy);
    const bool cg = tma_b && !fp8 && !unfolded && g.sx == 1 && g.sy == 1 && g.fh >= 2 &&
                    g.fh <= CG_GT && cg_span <= 2 && g.fw <= MAX_G && MX0 >= CG_BX;
    if (cg) {
        rbx = CG_BX;
        rby = CG_BY;
    }
    if (tma_b) {
        p.BX = rbx;
        p.BY = rby;
    }
    int ntap = 0, ntile = 0;
    for (int ph = 0; ph < p.nphase; ++ph) {
        const int rx = ph % p.nphx, ry = ph / p.nphx;
        p.phase_tap_begin[ph] = ntap;
        p.phase_tile_begin[ph] = ntile;
        for (int v = 0; v < g.fh; ++v) {
            if (mode == 1 && (((ry + g.py - v * g.dy) % g.sy) + g.sy) % g.sy != 0) continue;
            for (int u = 0; u < g.fw; ++u) {
                if (mode == 1 && (((rx + g.px - u * g.dx) % g.sx) + g.sx) % g.sx != 0) continue;
                p.tap_u[ntap] = (short)u;
                p.tap_v[ntap] = (short)v;
                // the tap's operand offset: forward u*dx - px (input
                // pixels); data gradient (rx + px - u*dx)/sx (exact for
                // the phase's taps; gradient pixels)
                p.tap_ox[ntap] = (short)(mode == 0 ? u * g.dx - g.px : (rx + g.px - u * g.dx) / g.sx);
                p.tap_oy[ntap] = (short)(mode == 0 ? v * g.dy - g.py : (ry + g.py - v * g.dy) / g.sy);
                ++ntap;
            }
        }
        long long MX = mode == 0 ? DW : (DW - rx + g.sx - 1) / g.sx;
        long long MY = mode == 0 ? DH : (DH - ry + g.sy - 1) / g.sy;
        if (tma_b) {
            p.ph_ntx[ph] = (int)((std::max(0LL, MX) + p.BX - 1) / p.BX);
            p.ph_nty[ph] = (int)((std::max(0LL, MY) + p.BY - 1) / p.BY);
            ntile += p.n_och_tiles * p.ph_ntx[ph] * p.ph_nty[ph] * (int)g.N;
        } else {
            long long npix = std::max(0LL, MX) * std::max(0LL, MY) * g.N;
            ntile += (int)((npix + BN - 1) / BN) * p.n_och_tiles;
        }
    }
    p.phase_tap_begin[p.nphase] = ntap;
    p.phase_tile_begin[p.nphase] = ntile;
    if (cg) {
        // the one phase's taps again, filter column by filter column
        p.cg = 1;
        p.cg_ngroups = (int)g.fw;
        p.cg_box_bytes = CG_BX * (CG_BY + cg_span) * 128;
        int t = 0;
        for (int u = 0; u < g.fw; ++u) {
            p.cg_begin[u] = (short)t;
            const int ox = (int)(mode == 0 ? u * g.dx - g.px : g.px - u * g.dx);
            const int oymin = (int)(mode == 0 ? -g.py : g.py - (g.fh - 1) * g.dy);
            p.cg_ox[u] = (short)ox;
            p.cg_oymin[u] = (short)oymin;
            for (int v = 0; v < g.fh; ++v, ++t) {
                const int oy = (int)(mode == 0 ? v * g.dy - g.py : g.py - v * g.dy);
                p.tap_u[t] = (short)u;
                p.tap_v[t] = (short)v;
                p.tap_ox[t] = (short)ox;
                p.tap_oy[t] = (short)oy;
                p.cg_view[u * CG_GT + v] = (short)((oy - oymin) * CG_BX);
            }
        }
        p.cg_begin[g.fw] = (short)t;
    }
    CUtensorMap xmap;
    std::memset(&xmap, 0, sizeof(xmap));
    if (cg) xmap = make_imap(img, SCpad, SW, SH, (int)g.N, CG_BX, CG_BY + cg_span, esize, 1, 1);
    else if (tma_b) xmap = make_imap(img, SCpad, SW, SH, (int)g.N, p.BX, p.BY, esize, tsx, tsy);
    p.total_tiles = ntile;

    // epilogue by TMA stores for unit-stride outputs with 16-byte rows
    CUtensorMap omap;
    std::memset(&omap, 0, sizeof(omap));
    p.tma_store = 0;
    if (tma_b && (mode == 0 || (g.sx == 1 && g.sy == 1)) && (DW % 4) == 0 &&
        (reinterpret_cast<uintptr_t>(dst) & 15) == 0) {
        cuuint64_t odims[4] = {(cuuint64_t)DW, (cuuint64_t)DH, (cuuint64_t)DC, (cuuint64_t)g.N};
        cuuint64_t ostr[3] = {(cuuint64_t)DW * 4, (cuuint64_t)DW * DH * 4, (cuuint64_t)DW * DH * DC * 4};
        cuuint32_t obox[4] = {16, 1, 32, 1};
        cuuint32_t oes[4] = {1, 1, 1, 1};
        if (encode_fn()(&omap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, dst, odims, ostr, obox, oes,
                        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_64B,
                        CU_TENSOR_MAP_L2_PROMOTION_NONE, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS)
            p.tma_store = 1;
    }
    // at most 64 output channels: only the real half of each weight tile is loaded
    p.a_rows = (OCpad == BM && DC <= 64) ? 64 : BM;
    CUtensorMap wmap = make_wmap(wt, OCpad, (long long)taps * SCpad, esize, p.a_rows);
    const size_t smem = gather_smem();
    if (ntile > 0) {
        const int grid = std::min(ntile, num_sms());
        KernelTimer kt(fp8 ? "tc_fwd_fp8_kernel" : (mode == 0 ? "tc_fwd_kernel" : "tc_dgrad_kernel"));
#define AFGB_LAUNCH_GATHER(TB, F8)                                                               \
    do {                                                                                         \
        AFGB_CUDA(cudaFuncSetAttribute(gather_conv_kernel<TB, F8>,                               \
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
        gather_conv_kernel<TB, F8><<<grid, NUM_THREADS, smem, stream()>>>(p, wmap, xmap, omap);  \
    } while (0)
        if (cg) {
            AFGB_CUDA(cudaFuncSetAttribute(gather_conv_kernel<true, false, true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            gather_conv_kernel<true, false, true><<<grid, NUM_THREADS, smem, stream()>>>(p, wmap, xmap,
                                                                                         omap);
        } else if (tma_b && fp8) AFGB_LAUNCH_GATHER(true, true);
        else if (tma_b) AFGB_LAUNCH_GATHER(true, false);
        else if (fp8) AFGB_LAUNCH_GATHER(false, true);
        else AFGB_LAUNCH_GATHER(false, false);
#undef AFGB_LAUNCH_GATHER
        count_launch();
        AFGB_POST_LAUNCH("gather_conv_kernel");
    }
    free_device(wt);
    if (img != img_ready) free_device(img);
    if (scales) free_device(scales);
    if (amax) free_device(amax);
}

// Stride-1 forward (mode 0) or data gradient (mode 1) by the strip kernel,
// from the source already in bf16 NHWC with channels padded to 64.  False
// (nothing launched) when the shape is outside its limits: unit strides, at
// most 128 output channels, strips of at most SC_MAXSL pixels and SC_MAXS
// rows per chunk, and rows long enough that 128-pixel segments waste at most
// a quarter of the MMA rows.  The gather kernel is measured faster on the
// shapes both cover, so the strip kernel runs only when AFGB_NN_KERNEL=strip
// selects it (its parity tests run that way).
static int nn_kernel_choice();

static bool strip_conv_fits(const NNGeom &g, int mode) {
    if (nn_kernel_choice() != 2) return false;
    if (g.sx != 1 || g.sy != 1 || g.fw * g.fh > MAX_T) return false;
    const long long DW = mode == 0 ? g.Wo : g.W, DC = mode == 0 ? g.K : g.C;
    if (DC > SC_MAXN || DW < 96) return false;
    const long long nseg = (DW + 127) / 128;
    if ((nseg * 128 - DW) * 4 > nseg * 128) return false;
    if ((g.fw - 1) * g.dx > SC_MAXSL - 128) return false;
    if (SC_R + (g.fh - 1) * g.dy > SC_MAXS) return false;
    const long long SW = mode == 0 ? g.W : g.Wo, SH = mode == 0 ? g.H : g.Ho;
    return SW < (1 << 24) && SH < (1 << 24) && g.N < (1 << 24);
}

static void run_strip_conv(const NNGeom &g, int mode, const __nv_bfloat16 *img, const float *w_f32,
                           float *dst, const NNEpilogue *ep) {
    const int SW = mode == 0 ? (int)g.W : (int)g.Wo;
    const int SH = mode == 0 ? (int)g.H : (int)g.Ho;
    const int SC = mode == 0 ? (int)g.C : (int)g.K;
    const int DW = mode == 0 ? (int)g.Wo : (int)g.W;
    const int DH = mode == 0 ? (int)g.Ho : (int)g.H;
    const int DC = mode == 0 ? (int)g.K : (int)g.C;
    const int SCpad = round_up(SC, 64);
    const int OCpad = round_up(DC, 64);
    const int taps = (int)(g.fw * g.fh);
    __nv_bfloat16 *wt;
    {
        MemTag tag("weight operands");
        wt = static_cast<__nv_bfloat16 *>(alloc_device((size_t)OCpad * taps * SCpad * 2));
    }
    {
        const long long total = (long long)OCpad * taps * SCpad;
        const unsigned blocks = (unsigned)std::min<long long>((total + 255) / 256, num_sms() * 8LL);
        weights_bf16_kernel<<<blocks, 256, 0, stream()>>>(w_f32, (int)g.fw, (int)g.fh, (int)g.C,
                                                          (int)g.K, mode, OCpad, SCpad, wt);
        count_launch();
        AFGB_POST_LAUNCH("weights_bf16_kernel");
    }
    StripConvParams p;
    std::memset(&p, 0, sizeof(p));
    p.dst = dst;
    if (ep && mode == 0) {
        p.bias = ep->bias;
        p.relu = ep->relu;
    }
    p.SW = SW;
    p.SH = SH;
    p.SCpad = SCpad;
    p.N = (int)g.N;
    p.DW = DW;
    p.DH = DH;
    p.DC = DC;
    p.nmma = round_up(DC, 16);
    p.nchunk = SCpad / 64;
    p.ntaps = taps;
    // per-tap source offsets of an output pixel: forward (u*dx - px, v*dy - py),
    // data gradient (px - u*dx, py - v*dy)
    int oxs[MAX_T], oys[MAX_T];
    int oxmin = 1 << 30, oxmax = -(1 << 30), oymin = 1 << 30, oymax = -(1 << 30);
    for (int t = 0; t < taps; ++t) {
        const int u = t % (int)g.fw, v = t / (int)g.fw;
        oxs[t] = mode == 0 ? u * (int)g.dx - (int)g.px : (int)g.px - u * (int)g.dx;
        oys[t] = mode == 0 ? v * (int)g.dy - (int)g.py : (int)g.py - v * (int)g.dy;
        oxmin = std::min(oxmin, oxs[t]);
        oxmax = std::max(oxmax, oxs[t]);
        oymin = std::min(oymin, oys[t]);
        oymax = std::max(oymax, oys[t]);
    }
    p.ox_min = oxmin;
    p.oy_min = oymin;
    p.SL = 128 + (oxmax - oxmin);
    p.S = SC_R + (oymax - oymin);
    p.strip16 = SC_STRIP >> 4;
    for (int t = 0; t < taps; ++t)
        p.a_off[t] = (uint32_t)(((oys[t] - oymin) * SC_STRIP + (oxs[t] - oxmin) * 128) >> 4);
    p.nb = std::min(SC_MAXNB, SC_B_AREA / (p.nmma * 128));
    p.nseg = (DW + 127) / 128;
    p.nrg = (DH + SC_R - 1) / SC_R;
    p.total_tiles = p.nseg * p.nrg * (int)g.N;
    CUtensorMap wmap = make_wmap(wt, OCpad, (long long)taps * SCpad, 2, p.nmma);
    CUtensorMap smap = make_imap(img, SCpad, SW, SH, (int)g.N, p.SL, 1);
    const size_t smem = 1024 + (size_t)SC_NA * SC_MAXS * SC_STRIP + SC_B_AREA +
                        sizeof(StripConvSmem) + 64;
    if (p.total_tiles > 0) {
        const int grid = std::min(p.total_tiles, num_sms());
        KernelTimer kt(mode == 0 ? "tc_fwd_kernel" : "tc_dgrad_kernel");
        AFGB_CUDA(cudaFuncSetAttribute(strip_conv_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
        strip_conv_kernel<<<grid, SC_THREADS, smem, stream()>>>(p, wmap, smap);
        count_launch();
        AFGB_POST_LAUNCH("strip_conv_kernel");
    }
    free_device(wt);
}

// Which stride-1 kernel serves a bf16 forward or data gradient: the row
// kernel where its limits hold, unless AFGB_NN_KERNEL names "gather" or
// "strip" (read once per process; the parity tests of the other kernels run
// that way).
static int nn_kernel_choice() {
    static const int v = [] {
        const char *e = std::getenv("AFGB_NN_KERNEL");
        if (e && std::strcmp(e, "gather") == 0) return 1;
        if (e && std::strcmp(e, "strip") == 0) return 2;
        return 0;
    }();
    return v;
}

static size_t smem_optin() {
    static const size_t v = [] {
        int s = 0;
        AFGB_CUDA(cudaDeviceGetAttribute(&s, cudaDevAttrMaxSharedMemoryPerBlockOptin, device()));
        return (size_t)s;
    }();
    return v;
}

// The row kernel's plan for g (mode 0 forward, 1 data gradient); false when
// its limits do not hold: unit strides and unit vertical dilation, filters at
// most three rows high, at most 256 output channels, rows long enough that
// 128-pixel segments waste at most a quarter of the MMA rows, strips of at
// most RC_STRIP / 128 pixels, every output row reached by some source row
// (py <= fh - 1), and the weights plus two strips within one CTA's shared
// memory.
static bool row_conv_plan(const NNGeom &g, int mode, RowConvParams &p, size_t &smem) {
    if (nn_kernel_choice() != 0) return false;
    if (g.sx != 1 || g.sy != 1 || g.dy != 1) return false;
    if (g.fh > 3 || g.fw > 16 || g.fw * g.fh > RC_MAXTAP || g.py > g.fh - 1) return false;
    const long long SW = mode == 0 ? g.W : g.Wo, SH = mode == 0 ? g.H : g.Ho;
    const long long DW = mode == 0 ? g.Wo : g.W, DH = mode == 0 ? g.Ho : g.H;
    const long long SC = mode == 0 ? g.C : g.K, DC = mode == 0 ? g.K : g.C;
    if (DW < 96 || DC > RC_DC * RC_MAXCG || SW >= (1 << 24) || SH >= (1 << 24) || g.N >= (1 << 24))
        return false;
    const long long nseg = (DW + 127) / 128;
    if ((nseg * 128 - DW) * 4 > nseg * 128) return false;
    if ((g.fw - 1) * g.dx > RC_STRIP / 128 - 128) return false;
    const int SCpad = round_up((int)SC, 64);
    const int nchunk = SCpad / 64;
    if (nchunk > RC_MAXCH) return false;
    const size_t wbytes = (size_t)nchunk * g.fw * g.fh * RC_DC * 128;
    const size_t fixed = 1024 + wbytes + sizeof(RowConvSmem) + 64;
    if (fixed + 2 * (size_t)RC_STRIP > smem_optin()) return false;
    std::memset(&p, 0, sizeof(p));
    p.ns = (int)std::min<size_t>(RC_MAXNS, (smem_optin() - fixed) / RC_STRIP);
    smem = fixed + (size_t)p.ns * RC_STRIP;
    p.SW = (int)SW;
    p.SH = (int)SH;
    p.N = (int)g.N;
    p.DW = (int)DW;
    p.DH = (int)DH;
    p.DC = (int)DC;
    p.fw = (int)g.fw;
    p.nchunk = nchunk;
    p.nseg = (int)nseg;
    p.ncg = (int)((DC + RC_DC - 1) / RC_DC);
    p.rows = g.N * nseg * DH;
    // source offsets of an output pixel: forward (u*dx - px, v - py), data
    // gradient (px - u*dx, py - v); block j of a tap column holds filter row
    // v_j, the one whose offset is oy_max - j
    int oxmin = 1 << 30, oxmax = -(1 << 30);
    for (int u = 0; u < g.fw; ++u) {
        const int ox = mode == 0 ? u * (int)g.dx - (int)g.px : (int)g.px - u * (int)g.dx;
        oxmin = std::min(oxmin, ox);
        oxmax = std::max(oxmax, ox);
    }
    p.ox_min = oxmin;
    p.SL = 128 + (oxmax - oxmin);
    p.oy_min = mode == 0 ? -(int)g.py : (int)g.py - (int)(g.fh - 1);
    p.oy_max = p.oy_min + (int)(g.fh - 1);
    for (int u = 0; u < g.fw; ++u) {
        const int ox = mode == 0 ? u * (int)g.dx - (int)g.px : (int)g.px - u * (int)g.dx;
        p.a_view[u] = (uint32_t)(((ox - oxmin) * 128) >> 4);
        for (int j = 0; j < g.fh; ++j) {
            const int v = mode == 0 ? (int)(g.fh - 1) - j : j;
            p.wcol[u * g.fh + j] = (u + (int)g.fw * v) * SCpad;
        }
    }
    return true;
}

// Stride-1 forward (mode 0) or data gradient (mode 1) by the row kernel from
// the source already in bf16 NHWC with channels padded to 64; false (nothing
// launched) when row_conv_plan rejects the shape.
static bool run_row_conv(const NNGeom &g, int mode, const __nv_bfloat16 *img, const float *w_f32,
                          float *dst, const NNEpilogue *ep) {
    RowConvParams p;
    size_t smem = 0;
    if (!row_conv_plan(g, mode, p, smem)) return false;
    const int SC = mode == 0 ? (int)g.C : (int)g.K;
    const int DC = p.DC;
    const int SCpad = round_up(SC, 64);
    const int OCpad = round_up(DC, 64);
    const int taps = (int)(g.fw * g.fh);
    __nv_bfloat16 *wt;
    {
        MemTag tag("weight operands");
        wt = static_cast<__nv_bfloat16 *>(alloc_device((size_t)OCpad * taps * SCpad * 2));
    }
    {
        const long long total = (long long)OCpad * taps * SCpad;
        const unsigned blocks = (unsigned)std::min<long long>((total + 255) / 256, num_sms() * 8LL);
        weights_bf16_kernel<<<blocks, 256, 0, stream()>>>(w_f32, (int)g.fw, (int)g.fh, (int)g.C,
                                                          (int)g.K, mode, OCpad, SCpad, wt);
        count_launch();
        AFGB_POST_LAUNCH("weights_bf16_kernel");
    }
    p.dst = dst;
    if (ep && mode == 0) {
        p.bias = ep->bias;
        p.relu = ep->relu;
    }
    CUtensorMap wmap = make_wmap(wt, OCpad, (long long)taps * SCpad, 2, RC_DC);
    CUtensorMap smap = make_imap(img, SCpad, p.SW, p.SH, (int)g.N, p.SL, 1);
    if (p.rows > 0) {
        // bands of at least 8 rows (each band loads fh - 1 extra source rows),
        // one CTA per band and channel group
        const long long nbands = std::max(1LL, std::min<long long>(num_sms() / p.ncg, p.rows / 8));
        const int grid = (int)(nbands * p.ncg);
        KernelTimer kt(mode == 0 ? "tc_fwd_kernel" : "tc_dgrad_kernel");
        KernelTimer kr("tc_row_kernel");  // which stride-1 kernel ran, for the tests
#define AFGB_LAUNCH_ROW(FH)                                                                  \
    do {                                                                                     \
        AFGB_CUDA(cudaFuncSetAttribute(row_conv_kernel<FH>,                                 \
                                       cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem)); \
        row_conv_kernel<FH><<<grid, RC_THREADS, smem, stream()>>>(p, wmap, smap);           \
    } while (0)
        if (g.fh == 1) AFGB_LAUNCH_ROW(1);
        else if (g.fh == 2) AFGB_LAUNCH_ROW(2);
        else AFGB_LAUNCH_ROW(3);
#undef AFGB_LAUNCH_ROW
        count_launch();
        AFGB_POST_LAUNCH("row_conv_kernel");
    }
    free_device(wt);
    return true;
}

// the gather kernel's limits: phases and taps fit the parameter block,
// 32-bit pixel coordinates
static bool gather_fits(const NNGeom &g, int mode) {
    if (g.fw * g.fh > MAX_T) return false;
    // per-tap operand offsets are 16-bit
    if ((g.fw - 1) * g.dx + g.px >= 32768 || (g.fh - 1) * g.dy + g.py >= 32768) return false;
    if (mode == 1 && g.sx * g.sy > MAX_PH) return false;
    if (g.W > (1 << 24) || g.H > (1 << 24) || g.N > (1 << 24)) return false;
    return true;
}

}  // namespace tc

using namespace tc;

void tc_set_wait_limit(unsigned int polls) {
    const unsigned int v = polls ? polls : kSpinLimit;
    AFGB_CUDA(cudaMemcpyToSymbol(g_spin_limit, &v, sizeof(v)));
}

unsigned int tc_take_error() {
    unsigned int v = 0, zero = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(v)) != cudaSuccess) return 0;
    if (v) (void)cudaMemcpyToSymbol(g_tc_error, &zero, sizeof(zero));
    return v;
}

bool tc_forward(const NNGeom &g, const Array &sig, const Array &filt, Array &out,
                afgb_precision prec, const Array *scales, const NNEpilogue *ep) {
    if (sig.type != f32 || !gather_fits(g, 0)) return false;
    if (prec == AFGB_PRECISION_FP8_E4M3) {
        run_gather(g, 0, sig.ptr<float>(), filt.ptr<float>(), out.ptr<float>(), true,
                   scales ? scales->ptr<float>() : nullptr, nullptr, nullptr, ep);
        return true;
    }
    if (prec != AFGB_PRECISION_BF16) return false;
    if (foldable(g)) {
        const NNGeom f = folded_geometry(g);
        run_gather(f, 0, sig.ptr<float>(), filt.ptr<float>(), out.ptr<float>(), false, nullptr, &g,
                   nullptr, ep);
        return true;
    }
    bool owned = false;
    const __nv_bfloat16 *x = signal_nhwc(sig, (int)g.W, (int)g.H, (int)g.C, (int)g.N,
                                         round_up((int)g.C, 64), owned);
    if (run_row_conv(g, 0, x, filt.ptr<float>(), out.ptr<float>(), ep)) {
    } else if (strip_conv_fits(g, 0)) {
        run_strip_conv(g, 0, x, filt.ptr<float>(), out.ptr<float>(), ep);
    } else {
        run_gather(g, 0, nullptr, filt.ptr<float>(), out.ptr<float>(), false, nullptr, nullptr, x,
                   ep);
    }
    if (owned) free_device(const_cast<__nv_bfloat16 *>(x));
    return true;
}

bool tc_data_grad(const NNGeom &g, const Array &grad, const Array &filt, Array &dx) {
    if (grad.type != f32 || !gather_fits(g, 1)) return false;
    RowConvParams rp;
    size_t rsm = 0;
    if (row_conv_plan(g, 1, rp, rsm) || strip_conv_fits(g, 1)) {
        const int Kp = round_up((int)g.K, 64);
        __nv_bfloat16 *gg = to_nhwc(grad.ptr<float>(), (int)g.Wo, (int)g.Ho, (int)g.K, (int)g.N, Kp);
        if (!run_row_conv(g, 1, gg, filt.ptr<float>(), dx.ptr<float>(), nullptr))
            run_strip_conv(g, 1, gg, filt.ptr<float>(), dx.ptr<float>(), nullptr);
        free_device(gg);
        return true;
    }
    run_gather(g, 1, grad.ptr<float>(), filt.ptr<float>(), dx.ptr<float>());
    return true;
}

// the strip kernel (stride 1 along x); false when its shape limits do not hold
static bool run_wgrad_strip(const NNGeom &g, const __nv_bfloat16 *x, const __nv_bfloat16 *gg,
                            int Cpad, int Kpad, const NNGeom &g0, float *dw) {
    // one-tap-wide filters give the strip kernel an N of only 64; the tile
    // kernel groups up to four 64-channel groups into one N=256 MMA instead
    if (g.sx != 1 || g.sy > 8 || g.fw * g.fh > 64 || g.fw < 2) return false;
    StripParams p;
    std::memset(&p, 0, sizeof(p));
    // stages of 128 pixels where the rows allow: every TMA copy costs about
    // 400 cycles of the SM's copy engine whatever its size (measured, up to
    // 18 KB), so fewer, larger copies per MMA cycle
    p.KP = 128;
    if (!pick_rect((int)g.Wo, (int)g.Ho, 128, 64, p.BX, p.BY)) {
        p.KP = 64;
        if (!pick_rect((int)g.Wo, (int)g.Ho, 64, 16, p.BX, p.BY)) return false;
    }
    p.a_bytes = 2 * p.KP * 128;
    p.nub = (int)((g.fw + 3) / 4);
    p.UB = (int)((g.fw + p.nub - 1) / p.nub);
    p.SL = p.BX + (p.UB - 1) * (int)g.dx;
    if (p.SL > 256) return false;
    p.strip_bytes = (p.SL * 128 + 1023) / 1024 * 1024;
    p.stage_bytes = p.a_bytes + p.BY * p.strip_bytes;
    p.nst = std::min(WS_MAXST, WS_SMEM / p.stage_bytes);
    if (p.nst < 2) return false;
    p.x = x;
    p.g = gg;
    p.W = (int)g.W;
    p.H = (int)g.H;
    p.Cpad = Cpad;
    p.C = (int)g.C;
    p.N = (int)g.N;
    p.Wo = (int)g.Wo;
    p.Ho = (int)g.Ho;
    p.Kpad = Kpad;
    p.K = (int)g.K;
    p.sy = (int)g.sy;
    p.px = (int)g.px;
    p.py = (int)g.py;
    p.dx = (int)g.dx;
    p.dy = (int)g.dy;
    p.fw = (int)g.fw;
    p.fh = (int)g.fh;
    p.nchunk = Cpad / 64;
    p.n_k_tiles = round_up((int)g.K, 128) / 128;  // past Kpad the G map reads zeros
    p.ntx = ((int)g.Wo + p.BX - 1) / p.BX;
    p.nty = ((int)g.Ho + p.BY - 1) / p.BY;
    p.Q = (long long)p.ntx * p.nty * g.N;
    CUtensorMap gmap = make_imap(gg, Kpad, (int)g.Wo, (int)g.Ho, (int)g.N, p.BX, p.BY);
    // strips: SL pixels of one row (box {64 channels, SL, 1, 1}), every sy-th row
    CUtensorMap smap = make_imap(x, Cpad, (int)g.W, (int)g.H, (int)g.N, p.SL, 1);
    const long long ntiles = (long long)p.n_k_tiles * p.nub * p.nchunk * g.fh;
    // one wave of CTAs (one fits an SM): two waves of half the pixels each
    // were measured slower (0.065 against 0.057 ms on 128x128x64x32), with
    // twice the partial sums to reduce
    const long long target = (long long)num_sms();
    long long splits = std::max(1LL, target / std::max(1LL, ntiles));
    long long chunk = std::max<long long>(16, (p.Q + splits - 1) / splits);
    splits = (p.Q + chunk - 1) / chunk;
    p.chunk = chunk;
    const long long rows = g.C * g.fw * g.fh;
    float *partial;
    {
        MemTag tag("split-K partial sums");
        partial = static_cast<float *>(alloc_device((size_t)(splits * rows * g.K) * sizeof(float)));
    }
    p.partial = partial;
    const size_t smem = 1024 + (size_t)p.nst * p.stage_bytes + sizeof(StripSmem) + 64;
    {
        KernelTimer kt("tc_wgrad_kernel");
        AFGB_CUDA(cudaFuncSetAttribute(wgrad_strip_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem));
        wgrad_strip_kernel<<<dim3((unsigned)ntiles, (unsigned)splits), WG_THREADS, smem, stream()>>>(
            p, gmap, smap);
    }
    count_launch();
    AFGB_POST_LAUNCH("wgrad_strip_kernel");
    reduce_filter_partials(g0, partial, (int)splits, dw);
    free_device(partial);
    return true;
}

// filter gradient from the incoming gradient already in bf16 NHWC, its
// channels padded to Kpad (a multiple of 64; the 128-row k tiles read the
// channels past it as zeros)
static void filter_grad_from(const NNGeom &g0, const __nv_bfloat16 *gg, int Kpad, const Array &sig,
                             Array &dw) {
    // folded taps: the signal operand is the folded image and the problem is
    // 1x1 on the output grid; its partial rows c + C*tap are the unfolded ones
    const bool fold = foldable(g0);
    const NNGeom g = fold ? folded_geometry(g0) : g0;
    const int Cpad = round_up((int)g.C, 64);
    bool owned = true;
    const __nv_bfloat16 *x =
        fold ? fold_taps(sig.ptr<float>(), g0)
             : signal_nhwc(sig, (int)g.W, (int)g.H, (int)g.C, (int)g.N, Cpad, owned);
    auto release = [&] {
        if (owned) free_device(const_cast<__nv_bfloat16 *>(x));
    };
    if (!fold && run_wgrad_strip(g, x, gg, Cpad, Kpad, g0, dw.ptr<float>())) {
        release();
        return;
    }
    WgradParams p;
    std::memset(&p, 0, sizeof(p));
    p.x = x;
    p.g = gg;
    p.W = (int)g.W;
    p.H = (int)g.H;
    p.Cpad = Cpad;
    p.C = (int)g.C;
    p.N = (int)g.N;
    p.Wo = (int)g.Wo;
    p.Ho = (int)g.Ho;
    p.Kpad = Kpad;
    p.K = (int)g.K;
    p.sx = (int)g.sx;
    p.sy = (int)g.sy;
    p.px = (int)g.px;
    p.py = (int)g.py;
    p.dx = (int)g.dx;
    p.dy = (int)g.dy;
    p.fw = (int)g.fw;
    p.fh = (int)g.fh;
    p.ngroups_total = (int)(g.fw * g.fh) * (Cpad / 64);
    // groups per tile: fewest tiles, then an even split
    int best = 4, best_tiles = 1 << 30;
    for (int gp = 4; gp >= 1; --gp) {
        const int tiles = (p.ngroups_total + gp - 1) / gp;
        if (tiles < best_tiles) {
            best_tiles = tiles;
            best = gp;
        }
    }
    for (int gp = 4; gp >= 1; --gp) {
        if (p.ngroups_total % gp == 0 && (p.ngroups_total / gp) <= best_tiles) {
            best = gp;
            break;
        }
    }
    p.groups_per_tile = best;
    p.n_k_tiles = round_up((int)g.K, 128) / 128;  // past Kpad the G loads read zeros
    // 128- (else 64-) pixel rectangles by TMA, two (four) stages; the signal
    // map walks every s-th pixel (traversal strides up to 8); otherwise the
    // cp.async row gather of 64-pixel stages
    int rbx = 0, rby = 0;
    p.KP = 128;
    bool tma = g.sx <= 8 && g.sy <= 8 &&
               pick_rect((int)g.Wo, (int)g.Ho, 128, 8, rbx, rby, (int)g.sx, (int)g.sy);
    if (!tma) {
        p.KP = WG_KP;
        tma = g.sx <= 8 && g.sy <= 8 &&
              pick_rect((int)g.Wo, (int)g.Ho, WG_KP, 8, rbx, rby, (int)g.sx, (int)g.sy);
    }
    p.nst = p.KP == 128 ? 2 : WG_STAGES;
    p.a_bytes = 2 * p.KP * 128;
    p.b_group = p.KP * 128;
    CUtensorMap gmap, xmap;
    std::memset(&gmap, 0, sizeof(gmap));
    std::memset(&xmap, 0, sizeof(xmap));
    long long units;  // pixel blocks (TMA) or pixels (cp.async)
    if (tma) {
        p.BX = rbx;
        p.BY = rby;
        p.ntx = ((int)g.Wo + p.BX - 1) / p.BX;
        p.nty = ((int)g.Ho + p.BY - 1) / p.BY;
        units = (long long)p.ntx * p.nty * g.N;
        gmap = make_imap(gg, Kpad, (int)g.Wo, (int)g.Ho, (int)g.N, p.BX, p.BY);
        xmap = make_imap(x, Cpad, (int)g.W, (int)g.H, (int)g.N, p.BX, p.BY, 2, (int)g.sx, (int)g.sy);
    } else {
        units = g.Wo * g.Ho * g.N;
    }
    p.Q = units;
    const long long ntiles = (long long)p.n_k_tiles * ((p.ngroups_total + best - 1) / best);
    // one wave of CTAs (two waves were measured slower: 0.106 against 0.087 ms
    // on 56x56x256x64 with a 1x1 filter, 0.076 against 0.053 ms on the 5x5
    // stride-2 backward shape)
    const long long target = (long long)num_sms();
    long long splits = std::max(1LL, target / std::max(1LL, ntiles));
    long long chunk = (units + splits - 1) / splits;
    if (tma) {
        chunk = std::max<long long>(16, chunk);
    } else {
        chunk = std::max<long long>(1024, (chunk + WG_KP - 1) / WG_KP * WG_KP);
    }
    splits = (units + chunk - 1) / chunk;
    p.chunk = chunk;
    const long long rows = g.C * g.fw * g.fh;
    float *partial;
    {
        MemTag tag("split-K partial sums");
        partial = static_cast<float *>(alloc_device((size_t)(splits * rows * g.K) * sizeof(float)));
    }
    p.partial = partial;
    const size_t smem = 1024 + (size_t)p.nst * (p.a_bytes + WG_MAXG * p.b_group) + sizeof(Smem) + 64;
    {
        KernelTimer kt("tc_wgrad_kernel");
        if (tma) {
            AFGB_CUDA(cudaFuncSetAttribute(wgrad_tc_kernel<true>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            wgrad_tc_kernel<true><<<dim3((unsigned)ntiles, (unsigned)splits), WG_THREADS, smem,
                                    stream()>>>(p, gmap, xmap);
        } else {
            AFGB_CUDA(cudaFuncSetAttribute(wgrad_tc_kernel<false>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
            wgrad_tc_kernel<false><<<dim3((unsigned)ntiles, (unsigned)splits), WG_THREADS, smem,
                                     stream()>>>(p, gmap, xmap);
        }
    }
    count_launch();
    AFGB_POST_LAUNCH("wgrad_tc_kernel");
    // fixed-order compensated reduction over splits, flipped into (fw,fh,C,K)
    reduce_filter_partials(g0, partial, (int)splits, dw.ptr<float>());
    free_device(partial);
    release();
}

bool tc_filter_grad(const NNGeom &g, const Array &grad, const Array &sig, Array &dw) {
    if (grad.type != f32) return false;
    const int Kpad = round_up((int)g.K, 64);
    __nv_bfloat16 *gg = to_nhwc(grad.ptr<float>(), (int)g.Wo, (int)g.Ho, (int)g.K, (int)g.N, Kpad);
    filter_grad_from(g, gg, Kpad, sig, dw);
    free_device(gg);
    return true;
}

// data and filter gradients sharing one bf16 copy of the incoming gradient
// (channels padded to 64); false (nothing done) when the data-gradient kernel
// does not cover the shape
bool tc_data_filter_grads(const NNGeom &g, const Array &grad, const Array &sig, const Array &filt,
                          Array &dx, Array &dw) {
    if (grad.type != f32 || !gather_fits(g, 1)) return false;
    const int Kpad = round_up((int)g.K, 64);
    __nv_bfloat16 *gg = to_nhwc(grad.ptr<float>(), (int)g.Wo, (int)g.Ho, (int)g.K, (int)g.N, Kpad);
    if (run_row_conv(g, 1, gg, filt.ptr<float>(), dx.ptr<float>(), nullptr)) {
    } else if (strip_conv_fits(g, 1)) {
        run_strip_conv(g, 1, gg, filt.ptr<float>(), dx.ptr<float>(), nullptr);
    } else {
        run_gather(g, 1, nullptr, filt.ptr<float>(), dx.ptr<float>(), false, nullptr, nullptr, gg);
    }
    filter_grad_from(g, gg, Kpad, sig, dw);
    free_device(gg);
    return true;
}

}  // namespace afgb
