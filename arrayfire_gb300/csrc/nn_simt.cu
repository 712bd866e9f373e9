// Plain CUDA-core NN convolution: forward, data gradient, filter gradient,
// bias gradient — the FP32 (and f64/f16) form of af_convolve2_nn and
// af_convolve2_gradient_nn.
//
// The reference materialises the unwrapped patches (unwrap + reorder +
// flip + GEMM, src/backend/cpu/convolve.cpp:123-243 and
// src/backend/cuda/convolveNN.cpp:175-407); here every operand is gathered
// straight from the image inside the GEMM (implicit GEMM), so nothing of size
// fw*fh*C*Wo*Ho*N is ever written.
//
//   forward      D[pixel][k]  = sum_{tap,c} X[pixel*s - p + tap*d][c] * W'[tap][c][k]
//   data grad    split by stride phase (x' mod sx, y' mod sy): inside one
//                phase the transposed convolution is a stride-1 gather with a
//                per-phase tap list, so no zero-stuffed products are computed
//   filter grad  R[tap,c][k] = sum_{pixel} X[pixel*s - p + tap*d][c] * G[pixel][k]
//                split-K over pixels, partials combined in a fixed order with
//                Neumaier compensation (deterministic, FP32 only)
//   bias grad    db[k] = sum_{pixel} G[pixel][k], same compensated scheme
#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <mutex>
#include <string>
#include <type_traits>
#include <vector>

#include "nn_conv.hpp"

namespace afgb {

template <typename T> struct NNAcc { using type = float; };
template <> struct NNAcc<double> { using type = double; };

template <typename A, typename T> __device__ __forceinline__ A ld_acc(const T *p) { return (A)*p; }
template <> __device__ __forceinline__ float ld_acc<float, __half>(const __half *p) {
    return __half2float(*p);
}
template <typename T, typename A> __device__ __forceinline__ T st_conv(A v) { return (T)v; }
template <> __device__ __forceinline__ __half st_conv<__half, float>(float v) {
    return __float2half_rn(v);
}

constexpr int MAX_TAPS = 1024;

// ---------------------------------------------------------------------------
// filter re-layout (small): forward wants B[tap][c][k], data grad B[tap][k][c],
// both with the reference's flip applied (tap (u,v) multiplies
// w[fw-1-u, fh-1-v]).  tap = u + fw*v.
// ---------------------------------------------------------------------------
template <typename T, typename A>
__global__ void filter_relayout_kernel(const T *w, long long fw, long long fh, long long C,
                                       long long K, A *out, int kc_order) {
    long long total = fw * fh * C * K;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        // t indexes the output
        long long tap, c, k;
        if (kc_order == 0) {  // [tap][c][k]
            k = t % K;
            c = (t / K) % C;
            tap = t / (K * C);
        } else {  // [tap][k][c]
            c = t % C;
            k = (t / C) % K;
            tap = t / (K * C);
        }
        long long u = tap % fw, v = tap / fw;
        long long src = (fw - 1 - u) + fw * ((fh - 1 - v) + fh * (c + C * k));
        out[t] = ld_acc<A, T>(w + src);
    }
}

// ---------------------------------------------------------------------------
// gather implicit GEMM (forward and phase-split data gradient)
// ---------------------------------------------------------------------------
template <typename T>
struct GatherParams {
    const T *A;  // source image (SW,SH,SC,N)
    long long SW, SH, SC;
    const typename NNAcc<T>::type *B;  // [fw*fh][SC][NC]
    T *D;                              // destination image (DW,DH,NC,N)
    long long DW, DH, NC, N;
    int fw, fh, sx, sy, px, py, dx, dy;
    int mode;  // 0 forward, 1 data gradient
};

constexpr int GB_K = 8, GB_THREADS = 256;

// Tiles of TM pixels x TN output channels (128 x 128, or 256 x 64 when the
// output has at most 64 channels, which would leave half of a 128-wide tile
// empty), 8 x 8 accumulators per thread, the K loop in steps of GB_K
// channels of one tap with double-buffered shared tiles and one step of
// register prefetch.  The tap and channel step advance incrementally.
template <typename T, int TM, int TN>
__global__ void __launch_bounds__(GB_THREADS) igemm_gather_kernel(GatherParams<T> p) {
    static_assert(TM * TN == 64 * GB_THREADS && TM % 32 == 0 && TN % 32 == 0, "tile shape");
    using A_t = typename NNAcc<T>::type;
    constexpr int HM = TM / 2, HN = TN / 2;
    constexpr int NA = TM / 32, ASTEP = GB_THREADS / TM;  // A loads per thread, their channel step
    constexpr int NB = TN / 32, BSTEP = GB_THREADS / TN;
    __shared__ __align__(16) A_t As[2][GB_K][TM];
    __shared__ __align__(16) A_t Bs[2][GB_K][TN];
    __shared__ short tap_u[MAX_TAPS], tap_v[MAX_TAPS];
    __shared__ int s_ntaps;

    const int tid = threadIdx.x;
    const int nphx = p.mode ? p.sx : 1;
    const int rx = blockIdx.z % nphx;
    const int ry = blockIdx.z / nphx;
    const long long MX = p.mode ? (p.DW - rx + p.sx - 1) / p.sx : p.DW;
    const long long MY = p.mode ? (p.DH - ry + p.sy - 1) / p.sy : p.DH;
    if (MX <= 0 || MY <= 0) return;
    const long long Mp = MX * MY * p.N;
    const long long m0 = (long long)blockIdx.x * TM;
    if (m0 >= Mp) return;
    const long long n0 = (long long)blockIdx.y * TN;

    if (tid == 0) {
        int cnt = 0;
        for (int v = 0; v < p.fh; ++v) {
            if (p.mode && ((((ry + p.py - v * p.dy) % p.sy) + p.sy) % p.sy) != 0) continue;
            for (int u = 0; u < p.fw; ++u) {
                if (p.mode && ((((rx + p.px - u * p.dx) % p.sx) + p.sx) % p.sx) != 0) continue;
                tap_u[cnt] = (short)u;
                tap_v[cnt] = (short)v;
                ++cnt;
            }
        }
        s_ntaps = cnt;
    }
    __syncthreads();
    const int ntaps = s_ntaps;
    const long long nch = (p.SC + GB_K - 1) / GB_K;
    const long long iters = (long long)ntaps * nch;

    // A-load role: one pixel, NA channel slots ASTEP apart
    const int am = tid % TM;
    const int akk = tid / TM;
    const long long mA = m0 + am;
    const bool mvalid = mA < Mp;
    long long AX = 0, AY = 0, An = 0;
    if (mvalid) {
        AX = mA % MX;
        AY = (mA / MX) % MY;
        An = mA / (MX * MY);
    }
    const long long SWH = p.SW * p.SH;
    const T *Abase = p.A + An * SWH * p.SC;
    // B-load role
    const int bn = tid % TN;
    const int bkk = tid / TN;
    const bool nvalid = (n0 + bn) < p.NC;

    A_t ra[NA], rb[NB];
    int lt = 0;        // tap of the next load
    long long lc0 = 0; // its first channel
    auto load_tile = [&]() {
        const int u = tap_u[lt], v = tap_v[lt];
        long long xs, ys;
        if (p.mode == 0) {
            xs = AX * p.sx + (long long)u * p.dx - p.px;
            ys = AY * p.sy + (long long)v * p.dy - p.py;
        } else {
            xs = AX + (rx + p.px - (long long)u * p.dx) / p.sx;
            ys = AY + (ry + p.py - (long long)v * p.dy) / p.sy;
        }
        const bool ok = mvalid && xs >= 0 && xs < p.SW && ys >= 0 && ys < p.SH;
        const T *src = Abase + xs + p.SW * ys;
        const long long tapidx = u + (long long)p.fw * v;
#pragma unroll
        for (int j = 0; j < NA; ++j) {
            const long long c = lc0 + akk + ASTEP * j;
            ra[j] = (ok && c < p.SC) ? ld_acc<A_t, T>(src + c * SWH) : (A_t)0;
        }
#pragma unroll
        for (int j = 0; j < NB; ++j) {
            const long long cb = lc0 + bkk + BSTEP * j;
            rb[j] = (nvalid && cb < p.SC) ? p.B[(tapidx * p.SC + cb) * p.NC + n0 + bn] : (A_t)0;
        }
        lc0 += GB_K;
        if (lc0 >= p.SC) {
            lc0 = 0;
            ++lt;
        }
    };
    auto store_tile = [&](int buf) {
#pragma unroll
        for (int j = 0; j < NA; ++j) As[buf][akk + ASTEP * j][am] = ra[j];
#pragma unroll
        for (int j = 0; j < NB; ++j) Bs[buf][bkk + BSTEP * j][bn] = rb[j];
    };

    const int tm = tid % (TM / 8), tn = tid / (TM / 8);
    A_t acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = (A_t)0;

    if (iters > 0) {
        load_tile();
        store_tile(0);
        __syncthreads();
        int cur = 0;
        for (long long it = 0; it < iters; ++it) {
            if (it + 1 < iters) load_tile();
#pragma unroll
            for (int kk = 0; kk < GB_K; ++kk) {
                A_t a[8], b[8];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    a[i] = As[cur][kk][4 * tm + i];
                    a[4 + i] = As[cur][kk][HM + 4 * tm + i];
                    b[i] = Bs[cur][kk][4 * tn + i];
                    b[4 + i] = Bs[cur][kk][HN + 4 * tn + i];
                }
#pragma unroll
                for (int i = 0; i < 8; ++i)
#pragma unroll
                    for (int j = 0; j < 8; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
            }
            if (it + 1 < iters) store_tile(cur ^ 1);
            __syncthreads();
            cur ^= 1;
        }
    }

    const int aox = p.mode ? p.sx : 1, aoy = p.mode ? p.sy : 1;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const long long m = m0 + (i < 4 ? 4 * tm + i : HM + 4 * tm + i - 4);
        if (m >= Mp) continue;
        const long long X = m % MX, Y = (m / MX) % MY, n = m / (MX * MY);
        const long long dxp = rx + aox * X, dyp = ry + aoy * Y;
        T *dst = p.D + dxp + p.DW * (dyp + p.DH * p.NC * n);
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const long long nc = n0 + (j < 4 ? 4 * tn + j : HN + 4 * tn + j - 4);
            if (nc < p.NC) dst[p.DW * p.DH * nc] = st_conv<T, A_t>(acc[i][j]);
        }
    }
}

// ---------------------------------------------------------------------------
// filter gradient: split-K implicit GEMM over output pixels
// ---------------------------------------------------------------------------
template <typename T>
struct WgradParams {
    const T *X;  // (W,H,C,N)
    long long W, H, C, N;
    const T *G;  // (Wo,Ho,K,N)
    long long Wo, Ho, K;
    int fw, fh, sx, sy, px, py, dx, dy;
    long long rows;   // fw*fh*C, row r = c + C*tap
    long long Q;      // Wo*Ho*N
    long long chunk;  // pixels per split (multiple of WG_K)
    typename NNAcc<T>::type *partial;  // [splits][rows][K]
};

constexpr int WG_M = 128, WG_N = 128, WG_K = 32, WG_THREADS = 256;
// shared tile pitch: a warp stores one row of 32 pixels (lanes) at stride
// WG_P, so a pitch of 128 would put all 32 lanes on one bank; 132 keeps the
// compute loop's 16-byte reads aligned and spreads the stores over 8 banks
constexpr int WG_P = WG_M + 4;

template <typename T>
__global__ void __launch_bounds__(WG_THREADS) wgrad_kernel(WgradParams<T> p) {
    using A_t = typename NNAcc<T>::type;
    extern __shared__ __align__(16) unsigned char wg_smem[];
    A_t *As = reinterpret_cast<A_t *>(wg_smem);       // [WG_K][WG_P]
    A_t *Bs = As + WG_K * WG_P;                         // [WG_K][WG_P]
    long long *row_off = reinterpret_cast<long long *>(Bs + WG_K * WG_P);
    int *row_x = reinterpret_cast<int *>(row_off + WG_M);
    int *row_y = row_x + WG_M;

    const int tid = threadIdx.x;
    const long long r0 = (long long)blockIdx.x * WG_M;
    const long long n0 = (long long)blockIdx.y * WG_N;
    const long long q_begin = (long long)blockIdx.z * p.chunk;
    const long long q_end = min(p.Q, q_begin + p.chunk);
    const long long WH = p.W * p.H;

    if (tid < WG_M) {
        long long r = r0 + tid;
        if (r < p.rows) {
            long long c = r % p.C, tap = r / p.C;
            long long u = tap % p.fw, v = tap / p.fw;
            row_off[tid] = c * WH;
            row_x[tid] = (int)(u * p.dx - p.px);
            row_y[tid] = (int)(v * p.dy - p.py);
        } else {
            row_off[tid] = -1;
            row_x[tid] = 0;
            row_y[tid] = 0;
        }
    }
    __syncthreads();

    const int aq = tid & 31, ar = tid >> 5;  // A: pixel lane, 16 rows ar+8j
    const int bq = tid & 31, bk = tid >> 5;  // B: pixel lane, 16 k's bk+8j
    const long long WoHo = p.Wo * p.Ho;
    // pixel tracking for q = q_begin + step*32 + lane
    long long q = q_begin + aq;
    long long qx = q % p.Wo, qy = (q / p.Wo) % p.Ho, qn = q / WoHo;

    A_t ra[16], rb[16];
    auto load = [&]() {
        const bool qv = q < q_end;
        const long long xs0 = qx * p.sx, ys0 = qy * p.sy;
        const T *xb = p.X + qn * WH * p.C;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const int rr = ar + 8 * j;
            const long long off = row_off[rr];
            const long long xs = xs0 + row_x[rr], ys = ys0 + row_y[rr];
            const bool ok = qv && off >= 0 && xs >= 0 && xs < p.W && ys >= 0 && ys < p.H;
            ra[j] = ok ? ld_acc<A_t, T>(xb + off + xs + p.W * ys) : (A_t)0;
        }
        const T *gb = p.G + qx + p.Wo * qy + WoHo * p.K * qn;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            const long long k = n0 + bk + 8 * j;
            rb[j] = (qv && k < p.K) ? ld_acc<A_t, T>(gb + WoHo * k) : (A_t)0;
        }
    };
    auto advance = [&]() {
        q += WG_K;
        qx += WG_K;
        while (qx >= p.Wo) {
            qx -= p.Wo;
            if (++qy == p.Ho) {
                qy = 0;
                ++qn;
            }
        }
    };
    auto store = [&]() {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
            As[aq * WG_P + ar + 8 * j] = ra[j];
            Bs[bq * WG_P + bk + 8 * j] = rb[j];
        }
    };

    const int tm = tid & 15, tn = tid >> 4;
    A_t acc[8][8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = (A_t)0;

    const long long steps = (q_end - q_begin + WG_K - 1) / WG_K;
    if (steps > 0) load();
    for (long long s = 0; s < steps; ++s) {
        __syncthreads();
        store();
        __syncthreads();
        if (s + 1 < steps) {
            advance();
            load();
        }
#pragma unroll 8
        for (int kk = 0; kk < WG_K; ++kk) {
            A_t a[8], b[8];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                a[i] = As[kk * WG_P + 4 * tm + i];
                a[4 + i] = As[kk * WG_P + 64 + 4 * tm + i];
                b[i] = Bs[kk * WG_P + 4 * tn + i];
                b[4 + i] = Bs[kk * WG_P + 64 + 4 * tn + i];
            }
#pragma unroll
            for (int i = 0; i < 8; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fma(a[i], b[j], acc[i][j]);
        }
    }

    A_t *out = p.partial + (long long)blockIdx.z * p.rows * p.K;
#pragma unroll
    for (int i = 0; i < 8; ++i) {
        const long long r = r0 + (i < 4 ? 4 * tm + i : 64 + 4 * tm + i - 4);
        if (r >= p.rows) continue;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const long long k = n0 + (j < 4 ? 4 * tn + j : 64 + 4 * tn + j - 4);
            if (k < p.K) out[r * p.K + k] = acc[i][j];
        }
    }
}

__device__ __forceinline__ float abs_of(float v) { return fabsf(v); }
__device__ __forceinline__ double abs_of(double v) { return fabs(v); }

// s + v into the running sum s with its Neumaier compensation comp
template <typename A>
__device__ __forceinline__ void neumaier_add(A &s, A &comp, A v) {
    const A tsum = s + v;
    if (abs_of(s) >= abs_of(v)) comp += (s - tsum) + v;
    else comp += (v - tsum) + s;
    s = tsum;
}

// Split-K partial sums -> the filter gradient with the reference's flip into
// dW (fw,fh,C,K): R[c + C*tap][k] -> dW[fw-1-u, fh-1-v, c, k].  One thread
// per output sums the splits in split order with Neumaier compensation; the
// loads of eight splits are issued before any of them is summed, so their
// latencies overlap.  The order is fixed, so results are bit-reproducible.
template <typename T, typename A>
__global__ void __launch_bounds__(256) wgrad_reduce_kernel(const A *partial, int splits,
                                                           long long rows, long long K,
                                                           long long C, long long fw,
                                                           long long fh, T *dw) {
    const long long total = rows * K;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        A s = 0, comp = 0;
        int z = 0;
        for (; z + 8 <= splits; z += 8) {
            A v[8];
#pragma unroll
            for (int i = 0; i < 8; ++i) v[i] = partial[(long long)(z + i) * total + t];
#pragma unroll
            for (int i = 0; i < 8; ++i) neumaier_add(s, comp, v[i]);
        }
        for (; z < splits; ++z) neumaier_add(s, comp, partial[(long long)z * total + t]);
        const A res = s + comp;
        const long long r = t / K, k = t % K;
        const long long c = r % C, tap = r / C;
        const long long u = tap % fw, v = tap / fw;
        dw[(fw - 1 - u) + fw * ((fh - 1 - v) + fh * (c + C * k))] = st_conv<T, A>(res);
    }
}

__global__ void reduce_partials_kernel(const float *partial, int splits, long long total,
                                       float *out) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        float s = 0.f, comp = 0.f;
        for (int z = 0; z < splits; ++z) {
            float v = partial[(long long)z * total + t];
            float tsum = s + v;
            if (fabsf(s) >= fabsf(v)) comp += (s - tsum) + v;
            else comp += (v - tsum) + s;
            s = tsum;
        }
        out[t] = s + comp;
    }
}

// ---------------------------------------------------------------------------
// bias gradient: db[k] = sum over Wo*Ho*N of g[.,.,k,.]
// stage 1: CTA (k, chunk) -> compensated partial; stage 2: compensated sum
// of partials per k in chunk order.  Both orders are fixed by the launch
// shape, so the result is bit-reproducible.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

template <typename T>
__global__ void bias_stage1_kernel(const T *g, long long WoHo, long long K, long long N,
                                   long long chunk, float *partial, int nchunks) {
    const long long k = blockIdx.y;
    const long long total = WoHo * N;
    const long long beg = (long long)blockIdx.x * chunk;
    const long long end = min(total, beg + chunk);
    float s = 0.f, c = 0.f;
    for (long long i = beg + threadIdx.x; i < end; i += blockDim.x) {
        long long n = i / WoHo, pix = i - n * WoHo;
        float v = ld_acc<float, T>(g + pix + WoHo * (k + K * n));
        float t, e;
        two_sum(s, v, t, e);
        s = t;
        c += e;
    }
    // fixed-shape tree: warp shuffles then shared memory
    for (int off = 16; off > 0; off >>= 1) {
        float so = __shfl_down_sync(0xffffffffu, s, off);
        float co = __shfl_down_sync(0xffffffffu, c, off);
        float t, e;
        two_sum(s, so, t, e);
        s = t;
        c = c + co + e;
    }
    __shared__ float ws[32], wc[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) {
        ws[warp] = s;
        wc[warp] = c;
    }
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
        s = lane < nw ? ws[lane] : 0.f;
        c = lane < nw ? wc[lane] : 0.f;
        for (int off = 16; off > 0; off >>= 1) {
            float so = __shfl_down_sync(0xffffffffu, s, off);
            float co = __shfl_down_sync(0xffffffffu, c, off);
            float t, e;
            two_sum(s, so, t, e);
            s = t;
            c = c + co + e;
        }
        if (lane == 0) partial[k * nchunks + blockIdx.x] = s + c;
    }
}

template <typename T>
__global__ void bias_stage2_kernel(const float *partial, int nchunks, long long K, T *db) {
    long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= K) return;
    float s = 0.f, c = 0.f;
    for (int i = 0; i < nchunks; ++i) {
        float t, e;
        two_sum(s, partial[k * nchunks + i], t, e);
        s = t;
        c += e;
    }
    db[k] = st_conv<T, float>(s + c);
}

template <>
__global__ void bias_stage2_kernel<double>(const float *partial, int nchunks, long long K,
                                           double *db) {
    long long k = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (k >= K) return;
    float s = 0.f, c = 0.f;
    for (int i = 0; i < nchunks; ++i) {
        float t, e;
        two_sum(s, partial[k * nchunks + i], t, e);
        s = t;
        c += e;
    }
    db[k] = (double)s + (double)c;
}

// ---------------------------------------------------------------------------
// host launchers
// ---------------------------------------------------------------------------
static unsigned grid_cap(long long total, int threads) {
    long long b = (total + threads - 1) / threads;
    long long cap = (long long)num_sms() * 16;
    return (unsigned)std::max(1LL, std::min(b, cap));
}

template <typename T>
static void gather_run(const NNGeom &g, int mode, const T *A, long long SW, long long SH,
                       long long SC, T *D, long long DW, long long DH, long long NC,
                       const T *w) {
    using A_t = typename NNAcc<T>::type;
    if (g.fw * g.fh > MAX_TAPS) AFGB_THROW(AF_ERR_NOT_SUPPORTED, "filter has more than 1024 taps");
    const long long nw = g.fw * g.fh * g.C * g.K;
    MemTag tag("weight operands");
    A_t *B = static_cast<A_t *>(alloc_device((size_t)nw * sizeof(A_t)));
    filter_relayout_kernel<T, A_t><<<grid_cap(nw, 256), 256, 0, stream()>>>(
        w, g.fw, g.fh, g.C, g.K, B, mode == 0 ? 0 : 1);
    count_launch();
    AFGB_POST_LAUNCH("filter_relayout_kernel");

    GatherParams<T> p;
    std::memset(&p, 0, sizeof(p));
    p.A = A;
    p.SW = SW;
    p.SH = SH;
    p.SC = SC;
    p.B = B;
    p.D = D;
    p.DW = DW;
    p.DH = DH;
    p.NC = NC;
    p.N = g.N;
    p.fw = (int)g.fw;
    p.fh = (int)g.fh;
    p.sx = (int)g.sx;
    p.sy = (int)g.sy;
    p.px = (int)g.px;
    p.py = (int)g.py;
    p.dx = (int)g.dx;
    p.dy = (int)g.dy;
    p.mode = mode;
    long long maxM;
    unsigned phases;
    if (mode == 0) {
        maxM = DW * DH * g.N;
        phases = 1;
    } else {
        maxM = ((DW + g.sx - 1) / g.sx) * ((DH + g.sy - 1) / g.sy) * g.N;
        phases = (unsigned)(g.sx * g.sy);
    }
    // 256-pixel x 64-channel tiles when the output has at most 64 channels
    const bool narrow = NC <= 64;
    const long long TMl = narrow ? 256 : 128, TNl = narrow ? 64 : 128;
    dim3 grid((unsigned)((maxM + TMl - 1) / TMl), (unsigned)((NC + TNl - 1) / TNl), phases);
    if (maxM > 0 && NC > 0) {
        KernelTimer kt(mode == 0 ? "simt_fwd_kernel" : "simt_dgrad_kernel");
        if (narrow)
            igemm_gather_kernel<T, 256, 64><<<grid, GB_THREADS, 0, stream()>>>(p);
        else
            igemm_gather_kernel<T, 128, 128><<<grid, GB_THREADS, 0, stream()>>>(p);
        count_launch();
        AFGB_POST_LAUNCH("igemm_gather_kernel");
    }
    free_device(B);
}

template <typename T>
static void simt_forward_t(const NNGeom &g, const Array &sig, const Array &filt, Array &out) {
    gather_run<T>(g, 0, sig.ptr<T>(), g.W, g.H, g.C, out.ptr<T>(), g.Wo, g.Ho, g.K, filt.ptr<T>());
}
template <typename T>
static void simt_dgrad_t(const NNGeom &g, const Array &grad, const Array &filt, Array &dx) {
    gather_run<T>(g, 1, grad.ptr<T>(), g.Wo, g.Ho, g.K, dx.ptr<T>(), g.W, g.H, g.C, filt.ptr<T>());
}

template <typename T>
static void simt_wgrad_t(const NNGeom &g, const Array &grad, const Array &sig, Array &dw) {
    using A_t = typename NNAcc<T>::type;
    WgradParams<T> p;
    std::memset(&p, 0, sizeof(p));
    p.X = sig.ptr<T>();
    p.W = g.W;
    p.H = g.H;
    p.C = g.C;
    p.N = g.N;
    p.G = grad.ptr<T>();
    p.Wo = g.Wo;
    p.Ho = g.Ho;
    p.K = g.K;
    p.fw = (int)g.fw;
    p.fh = (int)g.fh;
    p.sx = (int)g.sx;
    p.sy = (int)g.sy;
    p.px = (int)g.px;
    p.py = (int)g.py;
    p.dx = (int)g.dx;
    p.dy = (int)g.dy;
    p.rows = g.fw * g.fh * g.C;
    p.Q = g.Wo * g.Ho * g.N;
    const long long mt = (p.rows + WG_M - 1) / WG_M, nt = (g.K + WG_N - 1) / WG_N;
    long long target = (long long)num_sms() * 2;
    long long splits = std::max(1LL, target / std::max(1LL, mt * nt));
    long long chunk = (p.Q + splits - 1) / splits;
    chunk = ((chunk + WG_K - 1) / WG_K) * WG_K;
    if (chunk < 512) chunk = 512;
    splits = std::max(1LL, (p.Q + chunk - 1) / chunk);
    p.chunk = chunk;
    const long long total = p.rows * g.K;
    if (total == 0) return;
    A_t *partial;
    {
        MemTag tag("split-K partial sums");
        partial = static_cast<A_t *>(alloc_device((size_t)(splits * total) * sizeof(A_t)));
    }
    p.partial = partial;
    size_t smem = (size_t)(2 * WG_K * WG_P) * sizeof(A_t) + WG_M * (8 + 4 + 4);
    AFGB_CUDA(cudaFuncSetAttribute(wgrad_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    if (p.Q > 0) {
        dim3 grid((unsigned)mt, (unsigned)nt, (unsigned)splits);
        KernelTimer kt("simt_wgrad_kernel");
        wgrad_kernel<T><<<grid, WG_THREADS, smem, stream()>>>(p);
        count_launch();
        AFGB_POST_LAUNCH("wgrad_kernel");
    } else {
        AFGB_CUDA(cudaMemsetAsync(partial, 0, (size_t)(splits * total) * sizeof(A_t), stream()));
    }
    wgrad_reduce_kernel<T, A_t><<<grid_cap(total, 256), 256, 0, stream()>>>(
        partial, (int)splits, p.rows, g.K, g.C, g.fw, g.fh, dw.ptr<T>());
    count_launch();
    AFGB_POST_LAUNCH("wgrad_reduce_kernel");
    free_device(partial);
}

#define AFGB_NN_DISPATCH(t, FN, ...)                                  \
    switch (t) {                                                      \
        case f32: FN<float>(__VA_ARGS__); break;                      \
        case f64: FN<double>(__VA_ARGS__); break;                     \
        case f16: FN<__half>(__VA_ARGS__); break;                     \
        default: AFGB_TYPE_ERROR(1, t);                               \
    }

void simt_forward(const NNGeom &g, const Array &sig, const Array &filt, Array &out) {
    if (out.elements() == 0) return;
    AFGB_NN_DISPATCH(sig.type, simt_forward_t, g, sig, filt, out);
}
void simt_data_grad(const NNGeom &g, const Array &grad, const Array &filt, Array &dx) {
    if (dx.elements() == 0) return;
    AFGB_NN_DISPATCH(grad.type, simt_dgrad_t, g, grad, filt, dx);
}
void simt_filter_grad(const NNGeom &g, const Array &grad, const Array &sig, Array &dw) {
    if (dw.elements() == 0) return;
    AFGB_NN_DISPATCH(grad.type, simt_wgrad_t, g, grad, sig, dw);
}

void reduce_partials(const float *partials, int splits, long long rows, long long cols,
                     float *out) {
    long long total = rows * cols;
    if (!total) return;
    reduce_partials_kernel<<<grid_cap(total, 256), 256, 0, stream()>>>(partials, splits, total, out);
    count_launch();
    AFGB_POST_LAUNCH("reduce_partials_kernel");
}

void reduce_filter_partials(const NNGeom &g, const float *partials, int splits, float *dw) {
    const long long rows = g.fw * g.fh * g.C;
    const long long total = rows * g.K;
    if (!total) return;
    {
        KernelTimer kt("wgrad_reduce_kernel");
        wgrad_reduce_kernel<float, float><<<grid_cap(total, 256), 256, 0, stream()>>>(
            partials, splits, rows, g.K, g.C, g.fw, g.fh, dw);
    }
    count_launch();
    AFGB_POST_LAUNCH("wgrad_reduce_kernel");
}

template <typename T>
static void bias_t(const NNGeom &g, const Array &grad, Array &db) {
    const long long WoHo = g.Wo * g.Ho;
    const long long total = WoHo * g.N;
    const long long chunk = 16384;
    const int nchunks = (int)std::max(1LL, (total + chunk - 1) / chunk);
    float *partial;
    {
        MemTag tag("split-K partial sums");
        partial = static_cast<float *>(alloc_device((size_t)nchunks * g.K * sizeof(float)));
    }
    dim3 grid1((unsigned)nchunks, (unsigned)g.K);
    bias_stage1_kernel<T><<<grid1, 256, 0, stream()>>>(grad.ptr<T>(), WoHo, g.K, g.N, chunk,
                                                        partial, nchunks);
    count_launch();
    AFGB_POST_LAUNCH("bias_stage1_kernel");
    bias_stage2_kernel<T><<<(unsigned)((g.K + 127) / 128), 128, 0, stream()>>>(partial, nchunks,
                                                                               g.K, db.ptr<T>());
    count_launch();
    AFGB_POST_LAUNCH("bias_stage2_kernel");
    free_device(partial);
}

void nn_bias_grad(const NNGeom &g, const Array &grad, Array &db) {
    if (db.elements() == 0) return;
    AFGB_NN_DISPATCH(grad.type, bias_t, g, grad, db);
}

// ---------------------------------------------------------------------------
// filter gradient without device allocation (afgb_convolve2_filter_grad_noalloc)
//
// Same kernels as the FP32 filter gradient above, but the split-K partial
// sums live in a fixed file-scope device array instead of memory obtained
// from the stream-ordered pool, so the call allocates nothing.  The array
// exists once per GPU that loads this library and stays until exit; every
// call shares it.
// ---------------------------------------------------------------------------
constexpr long long kNoAllocScratchFloats = 2LL * 1024 * 1024;  // 8 MiB
static __device__ __align__(256) float g_noalloc_scratch[kNoAllocScratchFloats];

// device address of g_noalloc_scratch, looked up once per device with that
// device current (the host-side symbol is only a stand-in for it)
static float *noalloc_scratch_ptr(int dev) {
    static std::mutex mu;
    static float *ptrs[64] = {nullptr};
    if (dev < 0 || dev >= 64) AFGB_THROW(AF_ERR_DEVICE, "device ordinal out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (!ptrs[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p) {
            (void)cudaGetLastError();
            AFGB_THROW(AF_ERR_RUNTIME, std::string("cudaGetSymbolAddress of the no-allocation "
                                                   "scratch failed: ") + cudaGetErrorString(e));
        }
        ptrs[dev] = static_cast<float *>(p);
    }
    return ptrs[dev];
}

// the launch error of the kernel just enqueued: the caller clears the
// thread's error state (cudaGetLastError) right before the launch, so an
// earlier, unrelated non-sticky error is not reported against this call
static void noalloc_check_launch(const char *what) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess)
        AFGB_THROW(AF_ERR_RUNTIME, std::string("kernel launch failed: ") + what + ": " +
                                       cudaGetErrorString(e));
}

static void filter_grad_noalloc(const NNGeom &g, const float *grad, const float *sig, float *dw,
                                cudaStream_t st) {
    WgradParams<float> p;
    std::memset(&p, 0, sizeof(p));
    p.X = sig;
    p.W = g.W;
    p.H = g.H;
    p.C = g.C;
    p.N = g.N;
    p.G = grad;
    p.Wo = g.Wo;
    p.Ho = g.Ho;
    p.K = g.K;
    p.fw = (int)g.fw;
    p.fh = (int)g.fh;
    p.sx = (int)g.sx;
    p.sy = (int)g.sy;
    p.px = (int)g.px;
    p.py = (int)g.py;
    p.dx = (int)g.dx;
    p.dy = (int)g.dy;
    p.rows = g.fw * g.fh * g.C;
    p.Q = g.Wo * g.Ho * g.N;
    const long long total = p.rows * g.K;
    if (total == 0) return;
    if (total > kNoAllocScratchFloats) {
        AFGB_THROW(AF_ERR_SIZE, "the filter gradient needs " + std::to_string(total) +
                                    " floats of scratch; the no-allocation entry point holds at "
                                    "most " + std::to_string(kNoAllocScratchFloats));
    }
    int dev = device();
    float *scratch = noalloc_scratch_ptr(dev);
    int sms = 0;
    AFGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const long long mt = (p.rows + WG_M - 1) / WG_M, nt = (g.K + WG_N - 1) / WG_N;
    const long long cap = kNoAllocScratchFloats / total;  // splits that fit
    long long splits = std::max(1LL, std::min(cap, (long long)sms * 2 / std::max(1LL, mt * nt)));
    long long chunk = (p.Q + splits - 1) / splits;
    chunk = ((chunk + WG_K - 1) / WG_K) * WG_K;
    if (chunk < 512) chunk = 512;
    splits = std::max(1LL, (p.Q + chunk - 1) / chunk);
    if (splits > cap) {  // the 512-pixel floor can only lower splits; keep the cap explicit
        chunk = ((p.Q + cap - 1) / cap + WG_K - 1) / WG_K * WG_K;
        splits = std::max(1LL, (p.Q + chunk - 1) / chunk);
    }
    p.chunk = chunk;
    p.partial = scratch;
    const size_t smem = (size_t)(2 * WG_K * WG_P) * sizeof(float) + WG_M * (8 + 4 + 4);
    AFGB_CUDA(cudaFuncSetAttribute(wgrad_kernel<float>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   (int)smem));
    // p.Q > 0: the entry point rejects empty signals and output grids.  Every
    // split writes its whole rows x K slice, so the scratch left by an
    // earlier call needs no clearing.
    (void)cudaGetLastError();
    wgrad_kernel<float><<<dim3((unsigned)mt, (unsigned)nt, (unsigned)splits), WG_THREADS, smem,
                          st>>>(p);
    count_launch();
    noalloc_check_launch("wgrad_kernel");
    // the reduce grid from the SM count read above (grid_cap would go through
    // the library's per-device state, which creates its streams on first use)
    const unsigned rgrid =
        (unsigned)std::max(1LL, std::min((total + 255) / 256, (long long)sms * 16));
    (void)cudaGetLastError();
    wgrad_reduce_kernel<float, float><<<rgrid, 256, 0, st>>>(
        scratch, (int)splits, p.rows, g.K, g.C, g.fw, g.fh, dw);
    count_launch();
    noalloc_check_launch("wgrad_reduce_kernel");
}

// ---------------------------------------------------------------------------
// precision routing
// ---------------------------------------------------------------------------
// out = act(out + bias[k]) over (Wo, Ho, K, N): the epilogue of the SIMT
// forward, which does not fuse it
__global__ void bias_act_kernel(float *out, long long plane, long long K, long long total,
                                const float *bias, int relu) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        float v = out[t];
        if (bias) v += bias[(t / plane) % K];
        if (relu && v < 0.0f) v = 0.0f;
        out[t] = v;
    }
}

void nn_forward(const NNGeom &g, const Array &sig, const Array &filt, Array &out,
                afgb_precision prec, const Array *scales, const NNEpilogue *ep) {
    if (prec == AFGB_PRECISION_FP32) {
        simt_forward(g, sig, filt, out);
        const long long total = out.elements();
        if (ep && (ep->bias || ep->relu) && total) {
            if (out.type != f32) AFGB_THROW(AF_ERR_TYPE, "fused epilogues take f32 arrays");
            const unsigned blocks =
                (unsigned)std::min<long long>((total + 255) / 256, (long long)num_sms() * 32);
            bias_act_kernel<<<blocks, 256, 0, stream()>>>(out.ptr<float>(), g.Wo * g.Ho, g.K,
                                                          total, ep->bias, ep->relu);
            count_launch();
            AFGB_POST_LAUNCH("bias_act_kernel");
        }
        return;
    }
    if (out.elements() == 0) return;
    if (!tc_forward(g, sig, filt, out, prec, scales, ep))
        AFGB_THROW(AF_ERR_NOT_SUPPORTED, "tensor-core forward does not cover this shape");
}

void nn_data_grad(const NNGeom &g, const Array &grad, const Array &filt, Array &dx,
                  afgb_precision prec) {
    if (prec == AFGB_PRECISION_FP32) return simt_data_grad(g, grad, filt, dx);
    if (prec == AFGB_PRECISION_FP8_E4M3)
        AFGB_THROW(AF_ERR_NOT_SUPPORTED, "FP8 is provided for the forward pass only");
    if (dx.elements() == 0) return;
    if (!tc_data_grad(g, grad, filt, dx))
        AFGB_THROW(AF_ERR_NOT_SUPPORTED, "tensor-core data gradient does not cover this shape");
}

void nn_filter_grad(const NNGeom &g, const Array &grad, const Array &sig, Array &dw,
                    afgb_precision prec) {
    if (prec == AFGB_PRECISION_FP32) return simt_filter_grad(g, grad, sig, dw);
    if (prec == AFGB_PRECISION_FP8_E4M3)
        AFGB_THROW(AF_ERR_NOT_SUPPORTED, "FP8 is provided for the forward pass only");
    if (dw.elements() == 0) return;
    if (!tc_filter_grad(g, grad, sig, dw))
        AFGB_THROW(AF_ERR_NOT_SUPPORTED, "tensor-core filter gradient does not cover this shape");
}

void nn_gradients(const NNGeom &g, const Array &grad, const Array &sig, const Array &filt,
                  Array *dx, Array *dw, Array *db, afgb_precision prec) {
    if (dx && dw && prec == AFGB_PRECISION_BF16 && dx->elements() > 0 && dw->elements() > 0 &&
        tc_data_filter_grads(g, grad, sig, filt, *dx, *dw)) {
        dx = dw = nullptr;
    }
    if (dx) nn_data_grad(g, grad, filt, *dx, prec);
    if (dw) nn_filter_grad(g, grad, sig, *dw, prec);
    if (db) nn_bias_grad(g, grad, *db);
}

}  // namespace afgb

extern "C" af_err afgb_convolve2_filter_grad_noalloc(
    float *filter_grad, const float *incoming_gradient, const float *signal,
    const dim_t *signal_dims, const dim_t *filter_dims, const dim_t *strides,
    const dim_t *paddings, const dim_t *dilations, void *stream) {
    using namespace afgb;
    AFGB_TRY
    AFGB_ARG_ASSERT(0, filter_grad != nullptr);
    AFGB_ARG_ASSERT(1, incoming_gradient != nullptr);
    AFGB_ARG_ASSERT(2, signal != nullptr);
    AFGB_ARG_ASSERT(3, signal_dims != nullptr && filter_dims != nullptr);
    AFGB_ARG_ASSERT(5, strides != nullptr && paddings != nullptr && dilations != nullptr);
    for (int i = 0; i < 4; ++i) {
        AFGB_DIM_ASSERT(3, signal_dims[i] > 0);
        AFGB_DIM_ASSERT(4, filter_dims[i] > 0);
    }
    AFGB_DIM_ASSERT(4, signal_dims[2] == filter_dims[2]);
    AFGB_ARG_ASSERT(5, strides[0] > 0 && strides[1] > 0);
    AFGB_ARG_ASSERT(6, paddings[0] >= 0 && paddings[1] >= 0);
    AFGB_ARG_ASSERT(7, dilations[0] > 0 && dilations[1] > 0);
    NNGeom g;
    std::memset(&g, 0, sizeof(g));
    g.W = signal_dims[0];
    g.H = signal_dims[1];
    g.C = signal_dims[2];
    g.N = signal_dims[3];
    g.fw = filter_dims[0];
    g.fh = filter_dims[1];
    g.K = filter_dims[3];
    g.sx = strides[0];
    g.sy = strides[1];
    g.px = paddings[0];
    g.py = paddings[1];
    g.dx = dilations[0];
    g.dy = dilations[1];
    g.Wo = 1 + (g.W + 2 * g.px - (((g.fw - 1) * g.dx) + 1)) / g.sx;
    g.Ho = 1 + (g.H + 2 * g.py - (((g.fh - 1) * g.dy) + 1)) / g.sy;
    AFGB_DIM_ASSERT(3, g.Wo > 0 && g.Ho > 0);
    cudaStream_t st = stream ? static_cast<cudaStream_t>(stream) : afgb::stream();
    filter_grad_noalloc(g, incoming_gradient, signal, filter_grad, st);
    AFGB_CATCHALL
}
