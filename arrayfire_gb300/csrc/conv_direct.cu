// Direct small-filter convolutions (af_convolve1/2/3, af_convolve2_sep) for
// sm_103a.
//
// Reference behaviour: src/backend/cpu/kernel/convolve.hpp (the loop order
// that defines the rounding) and src/backend/cuda/kernel/convolve*.cuh (the
// reference's GPU kernels, which launch once per filter batch with the filter
// in constant memory).  Design here:
//   * one launch covers every batch slice (NONE/LHS/RHS/SAME) — the batch
//     index comes from blockIdx.z, filters are read per slice;
//   * the hot 2-D shapes (3x3, 5x5, 7x7 on f32 and 8-bit inputs) use a
//     register-blocked tile kernel: a 64x64 output tile per CTA, the haloed
//     input tile staged once in shared memory, each thread producing a 4x4
//     block from 128-bit shared loads and taps held in registers;
//   * the separable convolution is fused: column pass and row pass run in
//     one CTA and the intermediate image never leaves shared memory (the
//     reference writes a full-size temporary between two launches,
//     src/backend/cuda/convolve.cpp:76-80);
//   * every other dtype/shape uses a generic one-thread-per-output kernel
//     with the same arithmetic.
// The accumulation order is the reference's: taps of the outer dimension
// outside, dim-0 taps inside, ascending, starting from zero.
#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include <algorithm>
#include <cstdint>
#include <cstring>
#include <mutex>
#include <type_traits>

#include "conv_common.cuh"
#include "conv_direct.hpp"
#include "conv_params.cuh"
#include "conv_tma.hpp"

namespace afgb {

// ---------------------------------------------------------------------------
// generic kernel: one output per thread, any rank/dtype/stride
// (one2one_{1,2,3}d, src/backend/cpu/kernel/convolve.hpp:19-130)
// ---------------------------------------------------------------------------
template <typename T, bool EXACT>
__global__ void conv_generic_kernel(DirectParams p, long long slice) {
    using A = typename AccOf<T>::type;
    const T *sig = static_cast<const T *>(p.sig);
    const A *filt = static_cast<const A *>(p.filt);
    T *out = static_cast<T *>(p.out);
    const long long total = slice * p.nbatch;
    const long long f0 = p.fd[0];
    const long long f1 = p.rank >= 2 ? p.fd[1] : 1;
    const long long f2 = p.rank >= 3 ? p.fd[2] : 1;
    const long long c0 = p.expand ? 0 : f0 / 2;
    const long long c1 = p.expand ? 0 : f1 / 2;
    const long long c2 = p.expand ? 0 : f2 / 2;
    const long long o0 = p.od[0];
    const long long o1 = p.rank >= 2 ? p.od[1] : 1;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        long long b = t / slice;
        long long e = t - b * slice;
        long long i = e % o0;
        long long j = (e / o0) % o1;
        long long k = e / (o0 * o1);
        BatchOff bo = batch_offsets(p, b);
        const T *in = sig + bo.in;
        const A *w = filt + bo.filt;
        A acc = acc_zero<A>();
        for (long long wk = 0; wk < f2; ++wk) {
            long long kIdx = k + c2 - wk;
            bool kv = (p.rank < 3) || (kIdx >= 0 && kIdx < p.sd[2]);
            for (long long wj = 0; wj < f1; ++wj) {
                long long jIdx = j + c1 - wj;
                bool jv = (p.rank < 2) || (jIdx >= 0 && jIdx < p.sd[1]);
                for (long long wi = 0; wi < f0; ++wi) {
                    long long iIdx = i + c0 - wi;
                    T s{};
                    if (kv && jv && iIdx >= 0 && iIdx < p.sd[0]) {
                        long long off = iIdx * p.ss[0];
                        if (p.rank >= 2) off += jIdx * p.ss[1];
                        if (p.rank >= 3) off += kIdx * p.ss[2];
                        s = in[off];
                    }
                    A fv = w[wi * p.fs[0] + (p.rank >= 2 ? wj * p.fs[1] : 0) +
                             (p.rank >= 3 ? wk * p.fs[2] : 0)];
                    acc = mac<EXACT>(acc, to_acc(s, A{}), fv);
                }
            }
        }
        long long ooff = bo.out + i * p.os[0];
        if (p.rank >= 2) ooff += j * p.os[1];
        if (p.rank >= 3) ooff += k * p.os[2];
        out[ooff] = from_acc_any(acc, T{});
    }
}

// ---------------------------------------------------------------------------
// fast 2-D tile kernel
// ---------------------------------------------------------------------------
constexpr int T2_BX = 64;
constexpr int T2_BY = 64;
constexpr int T2_THREADS = 256;

template <typename T>
__device__ __forceinline__ float load_as_float(const T *p) {
    return to_acc(__ldg(p), 0.0f);
}
template <>
__device__ __forceinline__ float load_as_float<float>(const float *p) {
    return __ldg(p);
}

// Stage a TH x TW input window (origin ox, oy; zero outside the signal) into
// a shared tile of pitch PITCH floats.  f32 uses 4-byte cp.async with zero
// fill, so every load of the tile is in flight at once; other types load
// through registers in a division-free 2-D loop.
template <typename T>
__device__ __forceinline__ void stage_tile(float *tile, int PITCH, int TH, int TW, const T *in,
                                           long long ox, long long oy, long long sd0,
                                           long long sd1, long long ss0, long long ss1) {
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nwarps = blockDim.x >> 5;
    if constexpr (sizeof(T) == 4 && !IsInt<T>::value) {
        const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(tile));
        for (int r = warp; r < TH; r += nwarps) {
            const long long gy = oy + r;
            const bool rv = gy >= 0 && gy < sd1;
            for (int c = lane; c < TW; c += 32) {
                const long long gx = ox + c;
                const bool v = rv && gx >= 0 && gx < sd0;
                const T *src = v ? in + gx * ss0 + gy * ss1 : in;
                asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(
                                 sbase + 4u * (uint32_t)(r * PITCH + c)),
                             "l"(src), "r"(v ? 4u : 0u)
                             : "memory");
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    } else {
        for (int r = warp; r < TH; r += nwarps) {
            const long long gy = oy + r;
            const bool rv = gy >= 0 && gy < sd1;
#pragma unroll 4
            for (int c = lane; c < TW; c += 32) {
                const long long gx = ox + c;
                float v = 0.0f;
                if (rv && gx >= 0 && gx < sd0) v = load_as_float<T>(in + gx * ss0 + gy * ss1);
                tile[r * PITCH + c] = v;
            }
        }
    }
}

template <typename T>
__device__ __forceinline__ void store4(T *dst, const float *v, bool vec_ok) {
    if (vec_ok) {
        if constexpr (sizeof(T) == 4 && !IsInt<T>::value) {
            *reinterpret_cast<float4 *>(dst) = make_float4(v[0], v[1], v[2], v[3]);
            return;
        } else if constexpr (sizeof(T) == 1) {
            uint32_t w = (uint32_t)(uint8_t)from_acc<T>(v[0]) |
                         ((uint32_t)(uint8_t)from_acc<T>(v[1]) << 8) |
                         ((uint32_t)(uint8_t)from_acc<T>(v[2]) << 16) |
                         ((uint32_t)(uint8_t)from_acc<T>(v[3]) << 24);
            *reinterpret_cast<uint32_t *>(dst) = w;
            return;
        }
    }
#pragma unroll
    for (int c = 0; c < 4; ++c) dst[c] = from_acc_any(v[c], T{});
}

// T in {float, uint8_t, int8_t}; taps are float.  F0 x F1 filter.
template <typename T, int F0, int F1, bool EXACT>
__global__ void __launch_bounds__(T2_THREADS) conv2_tile_kernel(DirectParams p) {
    constexpr int TW = T2_BX + F0 - 1;
    constexpr int TH = T2_BY + F1 - 1;
    constexpr int PITCH = ((TW + 3) / 4) * 4;
    constexpr int WIN = 4 + F0 - 1;
    constexpr int WIN4 = (WIN + 3) / 4;
    __shared__ __align__(16) float tile[TH * PITCH];

    const long long b = blockIdx.z;
    BatchOff bo = batch_offsets(p, b);
    const T *in = static_cast<const T *>(p.sig) + bo.in;
    const float *w = static_cast<const float *>(p.filt) + bo.filt;
    T *out = static_cast<T *>(p.out) + bo.out;

    const long long i0 = (long long)blockIdx.x * T2_BX;
    const long long j0 = (long long)blockIdx.y * T2_BY;
    const int ci = p.expand ? 0 : F0 / 2;
    const int cj = p.expand ? 0 : F1 / 2;
    const long long ox = i0 + ci - (F0 - 1);
    const long long oy = j0 + cj - (F1 - 1);
    const long long sd0 = p.sd[0], sd1 = p.sd[1];
    const long long ss0 = p.ss[0], ss1 = p.ss[1];

    // stage the haloed input tile (zero outside the signal)
    stage_tile<T>(tile, PITCH, TH, TW, in, ox, oy, sd0, sd1, ss0, ss1);
    float wr[F0 * F1];
#pragma unroll
    for (int fj = 0; fj < F1; ++fj)
#pragma unroll
        for (int fi = 0; fi < F0; ++fi) wr[fj * F0 + fi] = __ldg(w + fi * p.fs[0] + fj * p.fs[1]);
    __syncthreads();

    const int tx = threadIdx.x & 15;
    const int ty = threadIdx.x >> 4;
    float acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = 0.0f;

    // walk input rows bottom-up so each output sees its dim-1 taps in
    // ascending order (fj = rr + F1 - 1 - q), dim-0 taps ascending inside
#pragma unroll
    for (int q = 3 + F1 - 1; q >= 0; --q) {
        float v[WIN4 * 4];
        const float *row = tile + (4 * ty + q) * PITCH + 4 * tx;
#pragma unroll
        for (int u = 0; u < WIN4; ++u) {
            float4 t4 = *reinterpret_cast<const float4 *>(row + 4 * u);
            v[4 * u + 0] = t4.x;
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
                        acc[rr][cc] = mac<EXACT>(acc[rr][cc], v[cc + F0 - 1 - fi], wv);
                }
            }
        }
    }

    const long long od0 = p.od[0], od1 = p.od[1];
    const long long x = i0 + 4 * tx;
    const bool vec_ok = (x + 3 < od0) && (p.os[0] == 1) &&
                        ((reinterpret_cast<uintptr_t>(out) % (4 * sizeof(T))) == 0) &&
                        ((p.os[1] % 4) == 0) && ((x % 4) == 0);
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) {
        long long y = j0 + 4 * ty + rr;
        if (y >= od1) break;
        T *dst = out + y * p.os[1] + x * p.os[0];
        if (vec_ok) {
            store4<T>(dst, acc[rr], true);
        } else {
#pragma unroll
            for (int cc = 0; cc < 4; ++cc)
                if (x + cc < od0) dst[cc * p.os[0]] = from_acc_any(acc[rr][cc], T{});
        }
    }
}

// ---------------------------------------------------------------------------
// 3-D tile kernel (f32): output block 64 (x) x 8 (y) x 8 (z) per CTA; each
// thread produces 4 consecutive x for one y and 4 consecutive z.  Input
// planes are walked from high z to low so every output sees its dim-2 taps
// in ascending order, dim-1 taps ascending inside, dim-0 taps innermost —
// the reference's order (src/backend/cpu/kernel/convolve.hpp:77-130).
// ---------------------------------------------------------------------------
constexpr int T3_BX = 64, T3_BY = 8, T3_BZ = 8, T3_THREADS = 256;

template <int F0, int F1, int F2, bool EXACT>
__global__ void __launch_bounds__(T3_THREADS) conv3_tile_kernel(DirectParams p) {
    constexpr int TW = T3_BX + F0 - 1;
    constexpr int TH = T3_BY + F1 - 1;
    constexpr int TD = T3_BZ + F2 - 1;
    constexpr int PITCH = ((TW + 3) / 4) * 4;
    constexpr int WIN = 4 + F0 - 1;
    constexpr int WIN4 = (WIN + 3) / 4;
    __shared__ __align__(16) float tile[TD * TH * PITCH];

    const long long b = blockIdx.z / ((p.od[2] + T3_BZ - 1) / T3_BZ);
    const long long zt = blockIdx.z - b * ((p.od[2] + T3_BZ - 1) / T3_BZ);
    BatchOff bo = batch_offsets(p, b);
    const float *in = static_cast<const float *>(p.sig) + bo.in;
    const float *w = static_cast<const float *>(p.filt) + bo.filt;
    float *out = static_cast<float *>(p.out) + bo.out;

    const long long i0 = (long long)blockIdx.x * T3_BX;
    const long long j0 = (long long)blockIdx.y * T3_BY;
    const long long k0 = zt * T3_BZ;
    const int ci = p.expand ? 0 : F0 / 2, cj = p.expand ? 0 : F1 / 2, ck = p.expand ? 0 : F2 / 2;
    const long long ox = i0 + ci - (F0 - 1), oy = j0 + cj - (F1 - 1), oz = k0 + ck - (F2 - 1);

    // stage (TD*TH) rows of TW floats with 4-byte cp.async, zero outside
    {
        const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
        const uint32_t sbase = static_cast<uint32_t>(__cvta_generic_to_shared(tile));
        for (int r = warp; r < TD * TH; r += T3_THREADS / 32) {
            const int rz = r / TH, ry = r - rz * TH;
            const long long gy = oy + ry, gz = oz + rz;
            const bool rv = gy >= 0 && gy < p.sd[1] && gz >= 0 && gz < p.sd[2];
            for (int c = lane; c < TW; c += 32) {
                const long long gx = ox + c;
                const bool v = rv && gx >= 0 && gx < p.sd[0];
                const float *src = v ? in + gx * p.ss[0] + gy * p.ss[1] + gz * p.ss[2] : in;
                asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(
                                 sbase + 4u * (uint32_t)(r * PITCH + c)),
                             "l"(src), "r"(v ? 4u : 0u)
                             : "memory");
            }
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
    }
    float wr[F0 * F1 * F2];
#pragma unroll
    for (int fk = 0; fk < F2; ++fk)
#pragma unroll
        for (int fj = 0; fj < F1; ++fj)
#pragma unroll
            for (int fi = 0; fi < F0; ++fi)
                wr[(fk * F1 + fj) * F0 + fi] = __ldg(w + fi * p.fs[0] + fj * p.fs[1] + fk * p.fs[2]);
    __syncthreads();

    const int tx = threadIdx.x & 15;
    const int ty = (threadIdx.x >> 4) & 7;
    const int tz = threadIdx.x >> 7;  // 0..1, four z each
    float acc[4][4];  // [z][x]
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[a][c] = 0.0f;

#pragma unroll
    for (int q = 3 + F2 - 1; q >= 0; --q) {        // input plane (relative), high to low
#pragma unroll
        for (int fj = 0; fj < F1; ++fj) {          // dim-1 tap, ascending
            float v[WIN4 * 4];
            const float *row = tile + ((4 * tz + q) * TH + (ty + F1 - 1 - fj)) * PITCH + 4 * tx;
#pragma unroll
            for (int u = 0; u < WIN4; ++u) {
                float4 t4 = *reinterpret_cast<const float4 *>(row + 4 * u);
                v[4 * u] = t4.x;
                v[4 * u + 1] = t4.y;
                v[4 * u + 2] = t4.z;
                v[4 * u + 3] = t4.w;
            }
#pragma unroll
            for (int rz = 0; rz < 4; ++rz) {
                const int fk = rz + F2 - 1 - q;
                if (fk >= 0 && fk < F2) {
#pragma unroll
                    for (int fi = 0; fi < F0; ++fi) {
                        const float wv = wr[(fk * F1 + fj) * F0 + fi];
#pragma unroll
                        for (int cc = 0; cc < 4; ++cc)
                            acc[rz][cc] = mac<EXACT>(acc[rz][cc], v[cc + F0 - 1 - fi], wv);
                    }
                }
            }
        }
    }
    const long long x = i0 + 4 * tx, y = j0 + ty;
    if (y >= p.od[1]) return;
    const bool vec_ok = (x + 3 < p.od[0]) && (p.os[0] == 1) &&
                        ((reinterpret_cast<uintptr_t>(out) & 15) == 0) && ((p.os[1] & 3) == 0) &&
                        ((p.os[2] & 3) == 0);
#pragma unroll
    for (int rz = 0; rz < 4; ++rz) {
        const long long z = k0 + 4 * tz + rz;
        if (z >= p.od[2]) break;
        float *dst = out + x + y * p.os[1] + z * p.os[2];
        if (vec_ok) {
            *reinterpret_cast<float4 *>(dst) = make_float4(acc[rz][0], acc[rz][1], acc[rz][2], acc[rz][3]);
        } else {
#pragma unroll
            for (int cc = 0; cc < 4; ++cc)
                if (x + cc < p.od[0]) dst[cc] = acc[rz][cc];
        }
    }
}

// ---------------------------------------------------------------------------
// fused separable kernel (f32 and 8-bit inputs)
// ---------------------------------------------------------------------------
constexpr int SP_BX = 64;
constexpr int SP_BY = 64;
constexpr int SP_THREADS = 256;

struct SepParams {
    const void *sig;
    const float *cf;
    const float *rf;
    void *out;
    int cflen, rflen;
    int expand;
    long long sd[4], ss[4];
    long long od[4], os[4];
    long long tw;  // width of the intermediate image (reference temp dims[0])
};

// tap as the reference's separable kernel sees it: converted to the input
// type (src/backend/cpu/kernel/convolve.hpp:233), then back to float for the
// exact integer arithmetic
template <typename T>
__device__ __forceinline__ float sep_tap(float f) {
    if constexpr (IsInt<T>::value) return (float)from_acc<T>(f);
    return f;
}
template <typename T>
__device__ __forceinline__ float sep_round(float a) {
    if constexpr (IsInt<T>::value) return (float)from_acc<T>(a);
    return a;
}

// CFL/RFL: compile-time filter lengths (0 = runtime, bounded by 31)
template <typename T, int CFL, int RFL, bool EXACT>
__global__ void __launch_bounds__(SP_THREADS) sep_fused_kernel(SepParams p) {
    constexpr int CMAX = CFL ? CFL : 31;
    constexpr int RMAX = RFL ? RFL : 31;
    const int cfl = CFL ? CFL : p.cflen;
    const int rfl = RFL ? RFL : p.rflen;
    const int TW = SP_BX + cfl - 1;
    const int TH = SP_BY + rfl - 1;
    const int PITCH = ((SP_BX + CMAX - 1 + 3) / 4) * 4;
    extern __shared__ __align__(16) float smem[];
    float *tile = smem;                           // TH x PITCH input values
    float *temp = smem + (SP_BY + RMAX - 1) * PITCH;  // TH x SP_BX intermediate
    __shared__ float ctap[32], rtap[32];

    const long long b = blockIdx.z;
    const long long b2 = b % p.sd[2];
    const long long b3 = b / p.sd[2];
    const T *in = static_cast<const T *>(p.sig) + b2 * p.ss[2] + b3 * p.ss[3];
    T *out = static_cast<T *>(p.out) + b2 * p.os[2] + b3 * p.os[3];

    const long long i0 = (long long)blockIdx.x * SP_BX;
    const long long j0 = (long long)blockIdx.y * SP_BY;
    const int cc0 = p.expand ? 0 : cfl / 2;
    const int cr0 = p.expand ? 0 : rfl / 2;
    const long long ox = i0 + cc0 - (cfl - 1);
    const long long oy = j0 + cr0 - (rfl - 1);
    const long long sd0 = p.sd[0], sd1 = p.sd[1];

    if (threadIdx.x < 32) {
        ctap[threadIdx.x] = threadIdx.x < cfl ? sep_tap<T>(p.cf[threadIdx.x]) : 0.0f;
        rtap[threadIdx.x] = threadIdx.x < rfl ? sep_tap<T>(p.rf[threadIdx.x]) : 0.0f;
    }
    stage_tile<T>(tile, PITCH, TH, TW, in, ox, oy, sd0, sd1, p.ss[0], p.ss[1]);
    __syncthreads();

    // pass 1 (dim 0): temp[r][x] = IN( sum_f tile[r][x + cfl-1-f] * c[f] ),
    // 8 consecutive x per work item; rows outside the signal are zero
    // (isCJValid in the reference's second pass)
    constexpr int W1 = 8 + CMAX - 1;
    constexpr int W1V = (W1 + 3) / 4;
    for (int it = threadIdx.x; it < TH * (SP_BX / 8); it += SP_THREADS) {
        const int r = it / (SP_BX / 8);
        const int g = it - r * (SP_BX / 8);
        const long long gy = oy + r;
        float a[8];
#pragma unroll
        for (int e = 0; e < 8; ++e) a[e] = 0.0f;
        if (gy >= 0 && gy < sd1) {
            float v[W1V * 4];
            const float *row = tile + r * PITCH + 8 * g;
#pragma unroll
            for (int u = 0; u < W1V; ++u) {
                if (4 * u < 8 + cfl - 1) {
                    float4 t4 = *reinterpret_cast<const float4 *>(row + 4 * u);
                    v[4 * u] = t4.x;
                    v[4 * u + 1] = t4.y;
                    v[4 * u + 2] = t4.z;
                    v[4 * u + 3] = t4.w;
                } else {
                    v[4 * u] = v[4 * u + 1] = v[4 * u + 2] = v[4 * u + 3] = 0.0f;
                }
            }
#pragma unroll
            for (int f = 0; f < CMAX; ++f) {
                if (f < cfl) {
                    const float wv = ctap[f];
#pragma unroll
                    for (int e = 0; e < 8; ++e) {
                        // window index e + cfl-1-f, resolved at compile time
                        // when CFL is fixed
                        a[e] = mac<EXACT>(a[e], v[e + (CFL ? CFL - 1 - f : 0) +
                                                   (CFL ? 0 : cfl - 1 - f)],
                                          wv);
                    }
                }
            }
#pragma unroll
            for (int e = 0; e < 8; ++e) a[e] = sep_round<T>(a[e]);
        }
        float *trow = temp + r * SP_BX + 8 * g;
        *reinterpret_cast<float4 *>(trow) = make_float4(a[0], a[1], a[2], a[3]);
        *reinterpret_cast<float4 *>(trow + 4) = make_float4(a[4], a[5], a[6], a[7]);
    }
    __syncthreads();

    // pass 2 (dim 1): out[x][y] = IN( sum_g temp[y + rfl-1-g][x] * r[g] ),
    // 4 x 4 outputs per thread, temp rows walked bottom-up
    const int tx = threadIdx.x & 15;
    const int ty = threadIdx.x >> 4;
    float acc[4][4];
#pragma unroll
    for (int r = 0; r < 4; ++r)
#pragma unroll
        for (int c = 0; c < 4; ++c) acc[r][c] = 0.0f;
#pragma unroll
    for (int q = 3 + RMAX - 1; q >= 0; --q) {
        if (q < 3 + rfl) {
            float4 t4 = *reinterpret_cast<const float4 *>(temp + (4 * ty + q) * SP_BX + 4 * tx);
            const float v[4] = {t4.x, t4.y, t4.z, t4.w};
#pragma unroll
            for (int rr = 0; rr < 4; ++rr) {
                const int g = rr + rfl - 1 - q;
                if (g >= 0 && g < rfl) {
                    const float wv = rtap[g];
#pragma unroll
                    for (int cc = 0; cc < 4; ++cc) acc[rr][cc] = mac<EXACT>(acc[rr][cc], v[cc], wv);
                }
            }
        }
    }
    const long long od0 = p.od[0], od1 = p.od[1];
    const long long x = i0 + 4 * tx;
    const bool vec_ok = (x + 3 < od0) && (p.os[0] == 1) &&
                        ((reinterpret_cast<uintptr_t>(out) % (4 * sizeof(T))) == 0) &&
                        ((p.os[1] % 4) == 0);
#pragma unroll
    for (int rr = 0; rr < 4; ++rr) {
        long long y = j0 + 4 * ty + rr;
        if (y >= od1) break;
        T *dst = out + y * p.os[1] + x * p.os[0];
        if (vec_ok) {
            store4<T>(dst, acc[rr], true);
        } else {
#pragma unroll
            for (int cc = 0; cc < 4; ++cc)
                if (x + cc < od0) dst[cc * p.os[0]] = from_acc_any(acc[rr][cc], T{});
        }
    }
}

// ---------------------------------------------------------------------------
// generic separable passes (every other dtype): one 1-D pass per launch
// through a temporary, exactly as the reference CPU backend's two calls
// (src/backend/cpu/kernel/convolve.hpp:213-255)
// ---------------------------------------------------------------------------
template <typename T, typename A, bool EXACT, int DIM>
__global__ void sep_pass_kernel(const T *in, long long id0, long long id1, long long is0,
                                long long is1, long long is2, long long is3, const A *filt,
                                int flen, T *out, long long od0, long long od1, long long os1,
                                long long os2, long long os3, long long n2, long long n3,
                                int expand) {
    const long long total = od0 * od1 * n2 * n3;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        long long i = t % od0;
        long long j = (t / od0) % od1;
        long long bb = t / (od0 * od1);
        long long b2 = bb % n2, b3 = bb / n2;
        const T *src = in + b2 * is2 + b3 * is3;
        long long ci = i + (DIM == 0 ? (expand ? 0 : flen / 2) : 0);
        long long cj = j + (DIM == 1 ? (expand ? 0 : flen / 2) : 0);
        A acc = acc_zero<A>();
        for (int f = 0; f < flen; ++f) {
            long long ii = DIM == 0 ? ci - f : ci;
            long long jj = DIM == 1 ? cj - f : cj;
            T s{};
            if (ii >= 0 && ii < id0 && jj >= 0 && jj < id1) s = src[ii * is0 + jj * is1];
            if constexpr (IsInt<T>::value) {
                T fv = from_acc<T>(filt[f]);
                acc = __fadd_rn(acc, int_prod(s, fv));
            } else {
                acc = mac<EXACT>(acc, to_acc(s, A{}), filt[f]);
            }
        }
        out[b2 * os2 + b3 * os3 + j * os1 + i] = from_acc_any(acc, T{});
    }
}

// ---------------------------------------------------------------------------
// casts and copies
// ---------------------------------------------------------------------------
template <typename F> __device__ __forceinline__ double real_of(F v) { return (double)v; }
__device__ __forceinline__ double real_of(__half v) { return (double)__half2float(v); }
__device__ __forceinline__ double mag_of(cf32 v) { return (double)hypotf(v.x, v.y); }
__device__ __forceinline__ double mag_of(cf64 v) { return hypot(v.x, v.y); }

// b8 target: char(v != 0) (src/backend/cpu/cast.hpp:140-155)
struct BoolByte {
    signed char v;
};

template <typename F, typename To> struct CastOp {
    __device__ static To run(F v) {
        if constexpr (std::is_same<To, BoolByte>::value) {
            if constexpr (std::is_same<F, __half>::value) return BoolByte{(signed char)(__half2float(v) != 0.f)};
            else return BoolByte{(signed char)(v != F(0))};
        } else if constexpr (std::is_integral<To>::value) {
            // C conversion: truncation toward zero for floating sources
            if constexpr (std::is_same<F, __half>::value) return (To)__half2float(v);
            else return (To)v;
        } else if constexpr (std::is_same<To, float>::value) {
            if constexpr (std::is_same<F, __half>::value) return __half2float(v);
            else return (float)v;
        } else if constexpr (std::is_same<To, double>::value) {
            if constexpr (std::is_same<F, __half>::value) return (double)__half2float(v);
            else return (double)v;
        } else if constexpr (std::is_same<To, cf32>::value) {
            if constexpr (std::is_same<F, __half>::value) return cf32{__half2float(v), 0.f};
            else return cf32{(float)v, 0.f};
        } else {
            if constexpr (std::is_same<F, __half>::value) return cf64{(double)__half2float(v), 0.0};
            else return cf64{(double)v, 0.0};
        }
    }
};
template <typename To> struct CastOp<cf32, To> {
    __device__ static To run(cf32 v) {
        if constexpr (std::is_same<To, BoolByte>::value) return BoolByte{(signed char)(v.x != 0.f || v.y != 0.f)};
        else if constexpr (std::is_same<To, cf32>::value) return v;
        else if constexpr (std::is_same<To, cf64>::value) return cf64{(double)v.x, (double)v.y};
        else return (To)mag_of(v);
    }
};
template <typename To> struct CastOp<cf64, To> {
    __device__ static To run(cf64 v) {
        if constexpr (std::is_same<To, BoolByte>::value) return BoolByte{(signed char)(v.x != 0.0 || v.y != 0.0)};
        else if constexpr (std::is_same<To, cf64>::value) return v;
        else if constexpr (std::is_same<To, cf32>::value) return cf32{(float)v.x, (float)v.y};
        else return (To)mag_of(v);
    }
};

template <typename F, typename To>
__global__ void cast_kernel(const F *in, long long d0, long long d1, long long d2,
                            long long s0, long long s1, long long s2, long long s3, To *out,
                            long long total) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        long long i = t % d0, j = (t / d0) % d1, k = (t / (d0 * d1)) % d2, l = t / (d0 * d1 * d2);
        out[t] = CastOp<F, To>::run(in[i * s0 + j * s1 + k * s2 + l * s3]);
    }
}

template <int BYTES> struct Blob {
    unsigned char b[BYTES];
};
template <int BYTES>
__global__ void dense_copy_kernel(const Blob<BYTES> *in, long long d0, long long d1, long long d2,
                                  long long s0, long long s1, long long s2, long long s3,
                                  Blob<BYTES> *out, long long total) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        long long i = t % d0, j = (t / d0) % d1, k = (t / (d0 * d1)) % d2, l = t / (d0 * d1 * d2);
        out[t] = in[i * s0 + j * s1 + k * s2 + l * s3];
    }
}

template <typename T, typename A>
__global__ void sep_scalar_kernel(const T *in, long long d0, long long d1, long long d2,
                                  long long s0, long long s1, long long s2, long long s3,
                                  const A *cf, const A *rf, T *out, long long total) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        long long i = t % d0, j = (t / d0) % d1, k = (t / (d0 * d1)) % d2, l = t / (d0 * d1 * d2);
        A s = to_acc(in[i * s0 + j * s1 + k * s2 + l * s3], A{});
        A f;
        if constexpr (std::is_same<A, cf32>::value) {
            cf32 c = cf[0], r = rf[0];
            f = cf32{__fsub_rn(__fmul_rn(c.x, r.x), __fmul_rn(c.y, r.y)),
                     __fadd_rn(__fmul_rn(c.x, r.y), __fmul_rn(c.y, r.x))};
            A prod = cf32{__fsub_rn(__fmul_rn(s.x, f.x), __fmul_rn(s.y, f.y)),
                          __fadd_rn(__fmul_rn(s.x, f.y), __fmul_rn(s.y, f.x))};
            out[t] = prod;
        } else if constexpr (std::is_same<A, cf64>::value) {
            cf64 c = cf[0], r = rf[0];
            f = cf64{__dsub_rn(__dmul_rn(c.x, r.x), __dmul_rn(c.y, r.y)),
                     __dadd_rn(__dmul_rn(c.x, r.y), __dmul_rn(c.y, r.x))};
            A prod = cf64{__dsub_rn(__dmul_rn(s.x, f.x), __dmul_rn(s.y, f.y)),
                          __dadd_rn(__dmul_rn(s.x, f.y), __dmul_rn(s.y, f.x))};
            out[t] = prod;
        } else if constexpr (std::is_same<A, double>::value) {
            out[t] = __dmul_rn(s, __dmul_rn(cf[0], rf[0]));
        } else {
            out[t] = from_acc_any(__fmul_rn(s, __fmul_rn(cf[0], rf[0])), T{});
        }
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
static unsigned grid_for(long long total, int threads) {
    long long blocks = (total + threads - 1) / threads;
    long long cap = (long long)num_sms() * 32;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (unsigned)blocks;
}

#define AFGB_DISPATCH_ALL(dt, FN)                       \
    switch (dt) {                                       \
        case f32: FN(float); break;                     \
        case f64: FN(double); break;                    \
        case c32: FN(cf32); break;                      \
        case c64: FN(cf64); break;                      \
        case b8: FN(int8_t); break;                     \
        case s8: FN(int8_t); break;                     \
        case u8: FN(uint8_t); break;                    \
        case s16: FN(int16_t); break;                   \
        case u16: FN(uint16_t); break;                  \
        case s32: FN(int32_t); break;                   \
        case u32: FN(uint32_t); break;                  \
        case s64: FN(long long); break;                 \
        case u64: FN(unsigned long long); break;        \
        default: AFGB_TYPE_ERROR(1, dt);                \
    }

static DirectParams make_params(const Array &sig, const Array &filt, Array &out, int kind,
                                int rank, bool expand) {
    DirectParams p;
    std::memset(&p, 0, sizeof(p));
    p.sig = sig.data();
    p.filt = filt.data();
    p.out = out.data();
    p.rank = rank;
    p.expand = expand ? 1 : 0;
    for (int i = 0; i < 4; ++i) {
        p.sd[i] = sig.dims[i];
        p.ss[i] = sig.strides[i];
        p.od[i] = out.dims[i];
        p.os[i] = out.strides[i];
        p.fd[i] = filt.dims[i];
        p.fs[i] = filt.strides[i];
        p.batch[i] = 1;
    }
    // batch steps per kind (src/backend/cpu/kernel/convolve.hpp:160-180)
    for (int i = 1; i < 4; ++i) {
        switch (kind) {
            case BATCH_LHS:
                p.out_step[i] = out.strides[i];
                p.in_step[i] = sig.strides[i];
                if (i >= rank) p.batch[i] = sig.dims[i];
                break;
            case BATCH_SAME:
                p.out_step[i] = out.strides[i];
                p.in_step[i] = sig.strides[i];
                p.filt_step[i] = filt.strides[i];
                if (i >= rank) p.batch[i] = sig.dims[i];
                break;
            case BATCH_RHS:
                p.out_step[i] = out.strides[i];
                p.filt_step[i] = filt.strides[i];
                if (i >= rank) p.batch[i] = filt.dims[i];
                break;
            default: break;
        }
    }
    p.nbatch = p.batch[1] * p.batch[2] * p.batch[3];
    return p;
}

template <typename T, int F0, int F1, bool EXACT>
static void run_tile2(const DirectParams &p) {
    dim3 grid((unsigned)((p.od[0] + T2_BX - 1) / T2_BX), (unsigned)((p.od[1] + T2_BY - 1) / T2_BY),
              (unsigned)p.nbatch);
    {
        KernelTimer kt("conv2_tile_kernel");
        conv2_tile_kernel<T, F0, F1, EXACT><<<grid, T2_THREADS, 0, stream()>>>(p);
    }
    count_launch();
    AFGB_POST_LAUNCH("conv2_tile_kernel");
}

template <typename T, bool EXACT>
static bool try_tile2(const DirectParams &p) {
    const long long f0 = p.fd[0], f1 = p.fd[1];
    if (p.nbatch > 65535) return false;
    if (f0 == 3 && f1 == 3) { run_tile2<T, 3, 3, EXACT>(p); return true; }
    if (f0 == 5 && f1 == 5) { run_tile2<T, 5, 5, EXACT>(p); return true; }
    if (f0 == 7 && f1 == 7) { run_tile2<T, 7, 7, EXACT>(p); return true; }
    return false;
}

// ---- 1-D, f32: a block stages C1_BX outputs' worth of input (zero outside
// the signal, as the reference's loop reads zeros there) and the taps in
// shared memory; thread t computes outputs t + 256r, taps in the reference's
// order (wi = 0..f0-1), one shared load and one multiply-add per tap
constexpr int C1_BX = 4096;

template <bool EXACT>
__global__ void __launch_bounds__(256) conv1_tile_kernel(DirectParams p, long long ntx) {
    extern __shared__ float c1_smem[];
    const int f0 = (int)p.fd[0];
    const int span = C1_BX + f0 - 1;
    float *tin = c1_smem;
    float *tw = c1_smem + span;
    const float *sig = static_cast<const float *>(p.sig);
    const float *filt = static_cast<const float *>(p.filt);
    float *out = static_cast<float *>(p.out);
    const long long c0 = p.expand ? 0 : f0 / 2;
    for (long long blk = blockIdx.x; blk < ntx * p.nbatch; blk += gridDim.x) {
        const long long b = blk / ntx, tx = blk - b * ntx;
        const BatchOff bo = batch_offsets(p, b);
        const long long x0 = tx * C1_BX;
        const long long lo = x0 + c0 - (f0 - 1);  // input index of tin[0]
        __syncthreads();                          // the previous tile's readers are done
        for (int e = threadIdx.x; e < span; e += blockDim.x) {
            const long long ii = lo + e;
            tin[e] = (ii >= 0 && ii < p.sd[0]) ? sig[bo.in + ii * p.ss[0]] : 0.0f;
        }
        for (int e = threadIdx.x; e < f0; e += blockDim.x) tw[e] = filt[bo.filt + e * p.fs[0]];
        __syncthreads();
        float acc[C1_BX / 256];
#pragma unroll
        for (int r = 0; r < C1_BX / 256; ++r) acc[r] = 0.0f;
        // output li reads input index li + c0 - wi, i.e. tin[li + f0 - 1 - wi]
        for (int wi = 0; wi < f0; ++wi) {
            const float w = tw[wi];
#pragma unroll
            for (int r = 0; r < C1_BX / 256; ++r)
                acc[r] = mac<EXACT>(acc[r], tin[threadIdx.x + 256 * r + f0 - 1 - wi], w);
        }
#pragma unroll
        for (int r = 0; r < C1_BX / 256; ++r) {
            const long long i = x0 + threadIdx.x + 256 * r;
            if (i < p.od[0]) out[bo.out + i * p.os[0]] = acc[r];
        }
    }
}

// ---- 1-D, f32, unit-stride signal and output rows: persistent blocks walk
// tiles of C1P_T outputs through a C1P_NST-stage ring filled by 16-byte
// cp.async copies (zero-filled outside the signal).  Thread t owns outputs
// 32t .. 32t+31 of a tile and slides a register window over the input: the
// taps run in chunks of eight, each chunk loading 40 inputs with ten 128-bit
// shared loads for 256 multiply-adds (with 16 outputs per thread, half of
// the instructions were not FMAs).
//
// The copy grid is aligned to the absolute address, so a tile's staged span
// starts `mis` (0..3) elements before its first needed input.  Chunk k of
// the padded tap range [0, 8M) holds tap wi = W_hi - k with
// W_hi = F - 1 + mis, which makes every thread's window start on a 16-byte
// boundary; k outside [mis, W_hi] is no tap and is skipped (never multiplied
// by zero, so an inf or NaN next to the window cannot leak in).
// Shared layout: 32-float groups at a pitch of 36 floats (nine 16-byte
// words), so eight lanes reading 128 bits at the same offset of consecutive
// groups hit eight different bank quads.
constexpr int C1P_OPT = 32;   // outputs per thread
constexpr int C1P_THREADS = 128;
constexpr int C1P_T = C1P_OPT * C1P_THREADS;
constexpr int C1P_NST = 2;
static_assert(C1P_NST >= 2, "the ring issues the next tile after the barrier that frees its stage");
constexpr int C1P_MAXF = 129;
constexpr int C1P_GP = 36;    // group pitch (floats)
// the last thread's window of the last chunk ends at element
// 32*127 + 8*(M-1) + 39 with M <= (C1P_MAXF + 2) / 8 + 1
constexpr int C1P_GROUPS = (C1P_OPT * (C1P_THREADS - 1) + 8 * ((C1P_MAXF + 2) / 8) + 40 + 31) / 32;
constexpr int C1P_STAGE = C1P_GROUPS * C1P_GP;                    // floats
constexpr int C1P_WMAX = 8 * ((C1P_MAXF + 2) / 8 + 1);            // padded taps
// taps staged with each tile (reversed and zero-padded for its `mis`)
constexpr size_t C1P_SMEM = (size_t)C1P_NST * C1P_STAGE * 4 + (size_t)C1P_NST * C1P_WMAX * 4;
// staged element e of a tile (e >= 0)
__device__ __forceinline__ int c1p_at(int e) { return (e >> 5) * C1P_GP + (e & 31); }

// one tap into shared memory, or zero when bytes == 0
__device__ __forceinline__ void c1p_copy4(float *dst, const float *src, int bytes) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;" ::"r"(
                     (unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void c1p_copy16(float *dst, const float *src, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(
                     (unsigned)__cvta_generic_to_shared(dst)),
                 "l"(src), "r"(bytes)
                 : "memory");
}

// one chunk of eight taps for the 32 outputs of a thread.  gb points at the
// thread's first group for this chunk; PH (0..3) is the chunk's window
// start within it, 8 PH floats.  wk holds the chunk's eight taps; k0 is the
// chunk's first padded tap index and [klo, khi] the real taps.
template <int PH>
__device__ __forceinline__ void c1p_window(float (&win)[40], const float *gb) {
#pragma unroll
    for (int q = 0; q < 10; ++q) {
        const int o = 8 * PH + 4 * q;
        const float4 v = *reinterpret_cast<const float4 *>(gb + (o >> 5) * C1P_GP + (o & 31));
        win[4 * q] = v.x;
        win[4 * q + 1] = v.y;
        win[4 * q + 2] = v.z;
        win[4 * q + 3] = v.w;
    }
}

// fused mode: one fused multiply-add per tap and output from the register
// window
template <int PH, bool FULL>
__device__ __forceinline__ void c1p_chunk_fused(float (&acc)[C1P_OPT], const float *gb, const float *wk,
                                                int k0, int klo, int khi) {
    float win[40];
    c1p_window<PH>(win, gb);
    const float4 wa = *reinterpret_cast<const float4 *>(wk);
    const float4 wb = *reinterpret_cast<const float4 *>(wk + 4);
    const float w[8] = {wa.x, wa.y, wa.z, wa.w, wb.x, wb.y, wb.z, wb.w};
#pragma unroll
    for (int r = 0; r < 8; ++r) {
        if (FULL || (k0 + r >= klo && k0 + r <= khi)) {
#pragma unroll
            for (int j = 0; j < C1P_OPT; ++j) acc[j] = __fmaf_rn(win[j + r], w[r], acc[j]);
        }
    }
}

// exact mode: taps in ascending wi, i.e. descending k, each product and sum
// rounded separately
template <int PH, bool FULL>
__device__ __forceinline__ void c1p_chunk_exact(float (&acc)[C1P_OPT], const float *gb, const float *wk,
                                                int k0, int klo, int khi) {
    float win[40];
    c1p_window<PH>(win, gb);
#pragma unroll
    for (int r = 7; r >= 0; --r) {
        if (FULL || (k0 + r >= klo && k0 + r <= khi)) {
            const float w = wk[r];
#pragma unroll
            for (int j = 0; j < C1P_OPT; ++j) acc[j] = mac<true>(acc[j], win[j + r], w);
        }
    }
}

// chunk m of a thread's window, dispatched on its phase and on whether all
// eight of its taps are real
template <bool EXACT>
__device__ __forceinline__ void c1p_chunk(float (&acc)[C1P_OPT], const float *st, const float *wbuf,
                                          int m, int mis, int whi) {
    const float *gb = st + (threadIdx.x + (m >> 2)) * C1P_GP;
    const float *wk = wbuf + 8 * m;
    const bool full = 8 * m >= mis && 8 * m + 7 <= whi;
#define C1P_CASE(PH)                                                                          \
    case PH:                                                                                  \
        if (EXACT) {                                                                          \
            if (full) c1p_chunk_exact<PH, true>(acc, gb, wk, 8 * m, mis, whi);                \
            else c1p_chunk_exact<PH, false>(acc, gb, wk, 8 * m, mis, whi);                    \
        } else {                                                                              \
            if (full) c1p_chunk_fused<PH, true>(acc, gb, wk, 8 * m, mis, whi);                \
            else c1p_chunk_fused<PH, false>(acc, gb, wk, 8 * m, mis, whi);                    \
        }                                                                                     \
        break;
    switch (m & 3) {
        C1P_CASE(0)
        C1P_CASE(1)
        C1P_CASE(2)
        C1P_CASE(3)
    }
#undef C1P_CASE
}

template <bool EXACT>
__global__ void __launch_bounds__(C1P_THREADS, 4)
    conv1_pipe_kernel(const DirectParams p, long long ntx, long long ntiles) {
    extern __shared__ __align__(16) float c1p_smem[];
    float *wring = c1p_smem + C1P_NST * C1P_STAGE;  // C1P_NST x C1P_WMAX staged taps
    const int F = (int)p.fd[0];
    const long long len = p.sd[0], od = p.od[0];
    const long long c0 = p.expand ? 0 : F / 2;
    const float *sig = static_cast<const float *>(p.sig);
    const float *filt = static_cast<const float *>(p.filt);
    float *out = static_cast<float *>(p.out);
    const int tid = threadIdx.x;

    // the tile's batch slice, first output and staging misalignment,
    // decoded with 32-bit divisions (the launcher keeps tile counts and
    // batch extents below 2^31) when the tile is issued, and kept in shared
    // memory for the iteration that computes it
    struct Tile {
        BatchOff bo;
        long long x0, lo;
        int mis;
    };
    __shared__ Tile tinfo[C1P_NST];
    const unsigned untx = (unsigned)ntx, nb1 = (unsigned)p.batch[1], nb2 = (unsigned)p.batch[2];
    auto decode = [&](long long tile) {
        Tile t;
        const unsigned b = (unsigned)tile / untx;
        t.x0 = (long long)((unsigned)tile - b * untx) * C1P_T;
        const unsigned r = b / nb1, b1 = b - r * nb1, b3 = r / nb2, b2 = r - b3 * nb2;
        t.bo.in = b1 * p.in_step[1] + b2 * p.in_step[2] + b3 * p.in_step[3];
        t.bo.out = b1 * p.out_step[1] + b2 * p.out_step[2] + b3 * p.out_step[3];
        t.bo.filt = b1 * p.filt_step[1] + b2 * p.filt_step[2] + b3 * p.filt_step[3];
        const long long first = t.x0 + c0 - (F - 1);  // first input index any output reads
        const long long abs_first = (long long)(reinterpret_cast<uintptr_t>(sig + t.bo.in) >> 2) + first;
        t.mis = (int)(abs_first & 3);
        t.lo = first - t.mis;  // signal index of staged element 0 (16-byte aligned address)
        return t;
    };
    auto issue = [&](long long tile, int buf) {
        const Tile t = decode(tile);
        if (tid == 0) tinfo[buf] = t;
        const float *sp = sig + t.bo.in;
        const long long nout = min((long long)C1P_T, od - t.x0);
        const int nch = (int)((t.mis + nout + F - 1 + 3) / 4);
        float *st = c1p_smem + buf * C1P_STAGE;
        for (int c = tid; c < nch; c += C1P_THREADS) {
            const long long ci = t.lo + 4LL * c;
            int bytes = 0;
            const float *src = sp;
            if (ci < len && ci + 4 > 0) {
                bytes = (int)min(4LL, len - ci) * 4;
                src = sp + ci;  // up to 3 elements before the slice: zeroed after landing
            }
            c1p_copy16(st + c1p_at(4 * c), src, bytes);
        }
        // the tile's taps, reversed from W_hi = F - 1 + mis and zero outside
        // [0, F), arrive with the same copy group: no global load waits at
        // the barrier that opens the tile
        const int whi = F - 1 + t.mis;
        const int nw = 8 * (whi / 8 + 1);
        float *wb = wring + buf * C1P_WMAX;
        const float *fp = filt + t.bo.filt;
        for (int kk = tid; kk < nw; kk += C1P_THREADS) {
            const int wi = whi - kk;
            const bool in = wi >= 0 && wi < F;
            c1p_copy4(wb + kk, in ? fp + (long long)wi * p.fs[0] : fp, in ? 4 : 0);
        }
    };

#pragma unroll 1
    for (int i = 0; i < C1P_NST - 1; ++i) {
        const long long t = blockIdx.x + (long long)i * gridDim.x;
        if (t < ntiles) issue(t, i);
        asm volatile("cp.async.commit_group;" ::: "memory");
    }
    long long k = 0;
#pragma unroll 1
    for (long long tile = blockIdx.x; tile < ntiles; tile += gridDim.x, ++k) {
        const int buf = (int)(k % C1P_NST);
        // this thread's copies of this tile have landed (the later tiles'
        // groups may still be in flight); after the barrier every thread's
        // have, and every thread is done with the previous tile, whose
        // stage and record the next issue overwrites: one barrier per tile
        asm volatile("cp.async.wait_group %0;" ::"n"(C1P_NST - 2) : "memory");
        __syncthreads();
        const long long ahead = tile + (long long)(C1P_NST - 1) * gridDim.x;
        if (ahead < ntiles) issue(ahead, (int)((k + C1P_NST - 1) % C1P_NST));
        asm volatile("cp.async.commit_group;" ::: "memory");
        // tinfo[buf] was written when this tile was issued, before this
        // iteration's barrier
        const Tile t = tinfo[buf];
        const int whi = F - 1 + t.mis;
        const int M = whi / 8 + 1;
        const float *wbuf = wring + buf * C1P_WMAX;
        float *st = c1p_smem + buf * C1P_STAGE;
        if (t.lo < 0) {  // staged elements before the signal start read as zero
            const int nz = (int)min(-t.lo, (long long)C1P_GROUPS * 32);
            for (int e = tid; e < nz; e += C1P_THREADS) st[c1p_at(e)] = 0.0f;
            __syncthreads();
        }
        const long long i0 = t.x0 + (long long)C1P_OPT * tid;
        float res[C1P_OPT];
#pragma unroll
        for (int j = 0; j < C1P_OPT; ++j) res[j] = 0.0f;
        if (EXACT) {
#pragma unroll 1
            for (int m = M - 1; m >= 0; --m) c1p_chunk<true>(res, st, wbuf, m, t.mis, whi);
        } else {
#pragma unroll 1
            for (int m = 0; m < M; ++m) c1p_chunk<false>(res, st, wbuf, m, t.mis, whi);
        }
        if (i0 < od) {
            float *op = out + t.bo.out + i0;
            if (i0 + C1P_OPT - 1 < od && (reinterpret_cast<uintptr_t>(op) & 15) == 0) {
#pragma unroll
                for (int q = 0; q < C1P_OPT / 4; ++q)
                    reinterpret_cast<float4 *>(op)[q] =
                        make_float4(res[4 * q], res[4 * q + 1], res[4 * q + 2], res[4 * q + 3]);
            } else {
#pragma unroll
                for (int j = 0; j < C1P_OPT; ++j)
                    if (i0 + j < od) op[j] = res[j];
            }
        }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
}

static bool try_conv1_pipe(const DirectParams &p, bool exact) {
    if (p.ss[0] != 1 || p.os[0] != 1) return false;
    const long long ntx = (p.od[0] + C1P_T - 1) / C1P_T;
    const long long ntiles = ntx * p.nbatch;
    if (ntiles <= 0 || ntiles >= (1LL << 31) || p.batch[1] >= (1LL << 31) ||
        p.batch[2] >= (1LL << 31))
        return false;
    static int per_sm[2] = {0, 0};
    static std::once_flag once[2];
    std::call_once(once[exact ? 1 : 0], [&] {
        auto fn = exact ? conv1_pipe_kernel<true> : conv1_pipe_kernel<false>;
        AFGB_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)C1P_SMEM));
        int n = 0;
        AFGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, C1P_THREADS, C1P_SMEM));
        per_sm[exact ? 1 : 0] = std::max(1, n);
    });
    const unsigned grid = (unsigned)std::min<long long>(
        ntiles, (long long)num_sms() * per_sm[exact ? 1 : 0]);
    {
        KernelTimer kt("conv1_pipe_kernel");
        if (exact)
            conv1_pipe_kernel<true><<<grid, C1P_THREADS, C1P_SMEM, stream()>>>(p, ntx, ntiles);
        else
            conv1_pipe_kernel<false><<<grid, C1P_THREADS, C1P_SMEM, stream()>>>(p, ntx, ntiles);
    }
    count_launch();
    AFGB_POST_LAUNCH("conv1_pipe_kernel");
    return true;
}

// f32 1-D convolutions (filters up to 129 taps: the spatial limit)
static bool try_conv1_tile(const DirectParams &p, bool exact) {
    if (p.rank != 1 || p.nbatch <= 0 || p.fd[0] < 1 || p.fd[0] > 129) return false;
    if (try_conv1_pipe(p, exact)) return true;
    const long long ntx = (p.od[0] + C1_BX - 1) / C1_BX;
    if (ntx * p.nbatch <= 0) return false;
    const size_t smem = (size_t)(C1_BX + 2 * p.fd[0]) * sizeof(float);
    const unsigned grid = (unsigned)std::min<long long>(ntx * p.nbatch, (long long)num_sms() * 8);
    {
        KernelTimer kt("conv1_tile_kernel");
        if (exact)
            conv1_tile_kernel<true><<<grid, 256, smem, stream()>>>(p, ntx);
        else
            conv1_tile_kernel<false><<<grid, 256, smem, stream()>>>(p, ntx);
    }
    count_launch();
    AFGB_POST_LAUNCH("conv1_tile_kernel");
    return true;
}

template <typename T>
static void run_generic(const DirectParams &p, bool exact) {
    long long slice = p.od[0];
    if (p.rank >= 2) slice *= p.od[1];
    if (p.rank >= 3) slice *= p.od[2];
    long long total = slice * p.nbatch;
    if (total == 0) return;
    unsigned g = grid_for(total, 256);
    {
        KernelTimer kt("conv_generic_kernel");
        if (exact || IsInt<T>::value)
            conv_generic_kernel<T, true><<<g, 256, 0, stream()>>>(p, slice);
        else
            conv_generic_kernel<T, false><<<g, 256, 0, stream()>>>(p, slice);
    }
    count_launch();
    AFGB_POST_LAUNCH("conv_generic_kernel");
}

void launch_convolve_nd(const Array &sig, const Array &filt, Array &out, int kind, int rank,
                        bool expand) {
    if (out.elements() == 0) return;
    DirectParams p = make_params(sig, filt, out, kind, rank, expand);
    const bool exact = exact_fp();
    if (rank == 2 && p.nbatch > 0 && dtma::tma_convolve2(p, sig.type, exact)) return;
    if (rank == 2) {
        bool done = false;
        switch (sig.type) {
            case f32: done = exact ? try_tile2<float, true>(p) : try_tile2<float, false>(p); break;
            case u8: done = try_tile2<uint8_t, true>(p); break;
            case s8:
            case b8: done = try_tile2<int8_t, true>(p); break;
            default: break;
        }
        if (done) return;
    }
    if (rank == 1 && sig.type == f32 && try_conv1_tile(p, exact)) return;
    if (rank == 3 && sig.type == f32 && p.nbatch > 0 && dtma::tma_convolve3(p, exact)) return;
    if (rank == 3 && sig.type == f32 && p.fd[0] == 3 && p.fd[1] == 3 && p.fd[2] == 3) {
        const long long nz = (p.od[2] + T3_BZ - 1) / T3_BZ;
        if (p.nbatch * nz <= 65535 && (p.od[1] + T3_BY - 1) / T3_BY <= 65535) {
            dim3 grid((unsigned)((p.od[0] + T3_BX - 1) / T3_BX),
                      (unsigned)((p.od[1] + T3_BY - 1) / T3_BY), (unsigned)(p.nbatch * nz));
            KernelTimer kt("conv3_tile_kernel");
            if (exact)
                conv3_tile_kernel<3, 3, 3, true><<<grid, T3_THREADS, 0, stream()>>>(p);
            else
                conv3_tile_kernel<3, 3, 3, false><<<grid, T3_THREADS, 0, stream()>>>(p);
            count_launch();
            AFGB_POST_LAUNCH("conv3_tile_kernel");
            return;
        }
    }
#define AFGB_RUN_GENERIC(T) run_generic<T>(p, exact)
    AFGB_DISPATCH_ALL(sig.type, AFGB_RUN_GENERIC);
#undef AFGB_RUN_GENERIC
}

// ---- separable
template <typename T, int CFL, int RFL, bool EXACT>
static void run_sep_fused(const SepParams &p, long long nb) {
    constexpr int CMAX = CFL ? CFL : 31;
    constexpr int RMAX = RFL ? RFL : 31;
    const int PITCH = ((SP_BX + CMAX - 1 + 3) / 4) * 4;
    size_t smem = (size_t)(SP_BY + RMAX - 1) * PITCH * 4 + (size_t)(SP_BY + RMAX - 1) * SP_BX * 4;
    auto kfn = sep_fused_kernel<T, CFL, RFL, EXACT>;
    AFGB_CUDA(cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    dim3 grid((unsigned)((p.od[0] + SP_BX - 1) / SP_BX), (unsigned)((p.od[1] + SP_BY - 1) / SP_BY),
              (unsigned)nb);
    {
        KernelTimer kt("sep_fused_kernel");
        kfn<<<grid, SP_THREADS, smem, stream()>>>(p);
    }
    count_launch();
    AFGB_POST_LAUNCH("sep_fused_kernel");
}

template <typename T, bool EXACT>
static void sep_fused_dispatch(const SepParams &p, long long nb) {
    if (p.cflen == 15 && p.rflen == 15) run_sep_fused<T, 15, 15, EXACT>(p, nb);
    else run_sep_fused<T, 0, 0, EXACT>(p, nb);
}

template <typename T>
static void run_sep_generic(const Array &sig, const Array &cfilt, const Array &rfilt, Array &out,
                            bool expand) {
    using A = typename AccOf<T>::type;
    const bool exact = exact_fp();
    const long long cfl = cfilt.elements(), rfl = rfilt.elements();
    const long long n2 = sig.dims[2], n3 = sig.dims[3];
    long long tw = sig.dims[0] + (expand ? cfl - 1 : 0);
    long long th = sig.dims[1];
    size_t tbytes = (size_t)(tw * th * n2 * n3) * sizeof(T);
    T *temp;
    {
        MemTag tag("separable intermediates");
        temp = static_cast<T *>(alloc_device(tbytes));
    }
    long long total1 = tw * th * n2 * n3;
    long long total2 = out.elements();
    const T *in = sig.ptr<T>();
    const A *cf = cfilt.ptr<A>();
    const A *rf = rfilt.ptr<A>();
    if (total1 > 0) {
        auto k0 = exact ? sep_pass_kernel<T, A, true, 0> : sep_pass_kernel<T, A, false, 0>;
        k0<<<grid_for(total1, 256), 256, 0, stream()>>>(
            in, sig.dims[0], sig.dims[1], sig.strides[0], sig.strides[1], sig.strides[2],
            sig.strides[3], cf, (int)cfl, temp, tw, th, tw, tw * th, tw * th * n2, n2, n3,
            expand ? 1 : 0);
        count_launch();
        AFGB_POST_LAUNCH("sep_pass_kernel<0>");
    }
    if (total2 > 0) {
        auto k1 = exact ? sep_pass_kernel<T, A, true, 1> : sep_pass_kernel<T, A, false, 1>;
        k1<<<grid_for(total2, 256), 256, 0, stream()>>>(
            temp, tw, th, 1, tw, tw * th, tw * th * n2, rf, (int)rfl, out.ptr<T>(), out.dims[0],
            out.dims[1], out.strides[1], out.strides[2], out.strides[3], n2, n3, expand ? 1 : 0);
        count_launch();
        AFGB_POST_LAUNCH("sep_pass_kernel<1>");
    }
    free_device(temp);
}

void launch_convolve2_sep(const Array &sig, const Array &cfilt, const Array &rfilt, Array &out,
                          bool expand) {
    if (out.elements() == 0) return;
    const long long cfl = cfilt.elements(), rfl = rfilt.elements();
    const long long nb = sig.dims[2] * sig.dims[3];
    const af_dtype t = sig.type;
    const bool fused_type = (t == f32 || t == u8 || t == s8 || t == b8);
    if (fused_type && dtma::tma_convolve2_sep(sig, cfilt.ptr<float>(), rfilt.ptr<float>(), (int)cfl,
                                              (int)rfl, out, expand, exact_fp()))
        return;
    if (fused_type && nb <= 65535 && cfl <= 31 && rfl <= 31) {
        SepParams p;
        std::memset(&p, 0, sizeof(p));
        p.sig = sig.data();
        p.cf = cfilt.ptr<float>();
        p.rf = rfilt.ptr<float>();
        p.out = out.data();
        p.cflen = (int)cfl;
        p.rflen = (int)rfl;
        p.expand = expand ? 1 : 0;
        for (int i = 0; i < 4; ++i) {
            p.sd[i] = sig.dims[i];
            p.ss[i] = sig.strides[i];
            p.od[i] = out.dims[i];
            p.os[i] = out.strides[i];
        }
        p.tw = sig.dims[0] + (expand ? cfl - 1 : 0);
        // 8-bit inputs: taps become integers, every product and partial sum
        // is an integer below 2^24, so fused multiply-add is exact
        switch (t) {
            case f32:
                if (exact_fp()) sep_fused_dispatch<float, true>(p, nb);
                else sep_fused_dispatch<float, false>(p, nb);
                return;
            case u8: sep_fused_dispatch<uint8_t, false>(p, nb); return;
            default: sep_fused_dispatch<int8_t, false>(p, nb); return;
        }
    }
#define AFGB_RUN_SEP(T) run_sep_generic<T>(sig, cfilt, rfilt, out, expand)
    AFGB_DISPATCH_ALL(t, AFGB_RUN_SEP);
#undef AFGB_RUN_SEP
}

// ---- casts
template <typename F, typename To>
static void run_cast(const Array &in, Array &out) {
    long long total = in.elements();
    if (!total) return;
    cast_kernel<F, To><<<grid_for(total, 256), 256, 0, stream()>>>(
        in.ptr<F>(), in.dims[0], in.dims[1], in.dims[2], in.strides[0], in.strides[1],
        in.strides[2], in.strides[3], out.ptr<To>(), total);
    count_launch();
    AFGB_POST_LAUNCH("cast_kernel");
}

template <typename To>
static void cast_from(const Array &in, Array &out) {
    switch (in.type) {
        case f32: run_cast<float, To>(in, out); break;
        case f64: run_cast<double, To>(in, out); break;
        case c32: run_cast<cf32, To>(in, out); break;
        case c64: run_cast<cf64, To>(in, out); break;
        case b8:
        case s8: run_cast<int8_t, To>(in, out); break;
        case u8: run_cast<uint8_t, To>(in, out); break;
        case s16: run_cast<int16_t, To>(in, out); break;
        case u16: run_cast<uint16_t, To>(in, out); break;
        case s32: run_cast<int32_t, To>(in, out); break;
        case u32: run_cast<uint32_t, To>(in, out); break;
        case s64: run_cast<long long, To>(in, out); break;
        case u64: run_cast<unsigned long long, To>(in, out); break;
        case f16: run_cast<__half, To>(in, out); break;
    }
}

Array make_dense(const Array &in) {
    Array out = *create_array(in.type, in.dims);
    long long total = in.elements();
    if (!total) return out;
    size_t es = dtype_size(in.type);
#define AFGB_COPY(B)                                                                         \
    dense_copy_kernel<B><<<grid_for(total, 256), 256, 0, stream()>>>(                        \
        static_cast<const Blob<B> *>(in.data()), in.dims[0], in.dims[1], in.dims[2],         \
        in.strides[0], in.strides[1], in.strides[2], in.strides[3],                          \
        static_cast<Blob<B> *>(out.data()), total)
    switch (es) {
        case 1: AFGB_COPY(1); break;
        case 2: AFGB_COPY(2); break;
        case 4: AFGB_COPY(4); break;
        case 8: AFGB_COPY(8); break;
        default: AFGB_COPY(16); break;
    }
#undef AFGB_COPY
    count_launch();
    AFGB_POST_LAUNCH("dense_copy_kernel");
    return out;
}

Array cast_array(const Array &in, af_dtype to) {
    if (in.type == to) return in.is_linear() ? in : make_dense(in);
    Array out = *create_array(to, in.dims);
    switch (to) {
        case f32: cast_from<float>(in, out); break;
        case f64: cast_from<double>(in, out); break;
        case c32: cast_from<cf32>(in, out); break;
        case c64: cast_from<cf64>(in, out); break;
        case s32: cast_from<int32_t>(in, out); break;
        case u32: cast_from<uint32_t>(in, out); break;
        case s64: cast_from<long long>(in, out); break;
        case u64: cast_from<unsigned long long>(in, out); break;
        case s16: cast_from<int16_t>(in, out); break;
        case u16: cast_from<uint16_t>(in, out); break;
        case s8: cast_from<int8_t>(in, out); break;
        case u8: cast_from<uint8_t>(in, out); break;
        case b8: cast_from<BoolByte>(in, out); break;
        default: AFGB_TYPE_ERROR(1, to);
    }
    return out;
}

void launch_sep_scalar(const Array &sig, const Array &cfilt, const Array &rfilt, Array &out) {
    long long total = sig.elements();
    if (!total) return;
#define AFGB_SCALAR(T)                                                                          \
    {                                                                                           \
        using A = typename AccOf<T>::type;                                                      \
        sep_scalar_kernel<T, A><<<grid_for(total, 256), 256, 0, stream()>>>(                    \
            sig.ptr<T>(), sig.dims[0], sig.dims[1], sig.dims[2], sig.strides[0], sig.strides[1], \
            sig.strides[2], sig.strides[3], cfilt.ptr<A>(), rfilt.ptr<A>(), out.ptr<T>(), total); \
    }
    AFGB_DISPATCH_ALL(sig.type, AFGB_SCALAR);
#undef AFGB_SCALAR
    count_launch();
    AFGB_POST_LAUNCH("sep_scalar_kernel");
}

}  // namespace afgb
