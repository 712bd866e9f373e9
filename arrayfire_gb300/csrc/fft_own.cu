// The transforms of the frequency-domain convolution: mixed-radix (8, 4, 2, 9, 3)
// Stockham FFTs in shared memory, for lengths 2^a 3^b (the sizes the
// convolution pads to).
//
//  * fft_real_forward: each contiguous real row of even length n0 = 2h is
//    read as h complex values z[j] = x[2j] + i x[2j+1], transformed (length
//    h), and split into the n0/2 + 1 bins of the real transform:
//    X[k] = (Z[k] + conj Z[h-k]) / 2 - i e^{-2 pi i k / n0} (Z[k] - conj Z[h-k]) / 2;
//  * fft_real_inverse: the reverse, Z'[k] = (X[k] + conj X[h-k]) +
//    i e^{+2 pi i k / n0} (X[k] - conj X[h-k]), an inverse length-h transform,
//    and the real row read back from its real and imaginary parts;
//  * fft_axis: complex transforms along one axis of a (inner, n, outer)
//    layout, P neighbouring pencils per block so that each row of the
//    gather reads P consecutive elements.
// One block holds its pencils in shared memory as two buffers; stage s of
// radix r reads x[j + q n/r] (q < r), multiplies by the twiddles
// w^(q k), k = j mod Ns, does the radix-r butterfly and writes
// y[(j - k) r + k + q Ns] (Ns = product of the earlier radices), then the
// buffers swap.  Twiddles come from per-stage tables computed in double on
// the host: stage s holds w^(q k) = e^{-2 pi i q k / (R Ns)} at
// [(q - 1) Ns + k], so the lanes of a warp (consecutive k) read consecutive
// entries (a single table e^{-2 pi i j / L} read at q k L / (R Ns) put the
// lanes of the late stages up to 16 entries apart, 16-way bank conflicts);
// the stages' tables add up to L - 1 entries.  Transforms are unnormalised
// (forward e^{-...}, inverse e^{+...}), as the convolution's output pass
// divides by the size.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <mutex>
#include <vector>

#include "afgb_internal.hpp"
#include "conv_common.cuh"
#include "fft_own.hpp"

namespace afgb {

namespace {

// elements one buffer of n values takes (see sp): whole 16-element rows,
// and at least the former one-slot-per-32 padding's size
__host__ __device__ __forceinline__ int fft_padded(int n) {
    const int rows = (n + 15) & ~15, padded = n + (n >> 5) + 1;
    return rows > padded ? rows : padded;
}

template <typename C> struct ScalarT { using type = float; };
template <> struct ScalarT<cf64> { using type = double; };

template <typename C> __device__ __forceinline__ C cadd(C a, C b) { return C{a.x + b.x, a.y + b.y}; }
template <typename C> __device__ __forceinline__ C csub(C a, C b) { return C{a.x - b.x, a.y - b.y}; }
template <typename C> __device__ __forceinline__ C cmulc(C a, C b) {
    return C{a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x};
}
template <typename C> __device__ __forceinline__ C cconj(C a) { return C{a.x, -a.y}; }
// i * a
template <typename C> __device__ __forceinline__ C cmuli(C a) { return C{-a.y, a.x}; }

// small DFTs in registers, forward (e^{-2 pi i q k / R}) or inverse (e^{+...});
// v is transformed in place, natural order in and out
template <typename C, bool INV>
__device__ __forceinline__ void dft2(C &a, C &b) {
    const C t = a;
    a = cadd(t, b);
    b = csub(t, b);
}

template <typename C, bool INV>
__device__ __forceinline__ void dft3(C &a, C &b, C &c) {
    using S = typename ScalarT<C>::type;
    const S h = S(0.86602540378443864676);  // sqrt(3) / 2
    const C s = cadd(b, c);
    const C m = C{a.x - S(0.5) * s.x, a.y - S(0.5) * s.y};
    const C d = csub(b, c);
    const C id = C{-h * d.y, h * d.x};  // i (sqrt(3)/2) (b - c)
    a = cadd(a, s);
    b = INV ? cadd(m, id) : csub(m, id);
    c = INV ? csub(m, id) : cadd(m, id);
}

template <typename C, bool INV>
__device__ __forceinline__ void dft4(C &a, C &b, C &c, C &d) {
    const C t0 = cadd(a, c), t1 = csub(a, c);
    const C t2 = cadd(b, d), t3 = csub(b, d);
    const C it3 = cmuli(t3);
    a = cadd(t0, t2);
    c = csub(t0, t2);
    b = INV ? cadd(t1, it3) : csub(t1, it3);
    d = INV ? csub(t1, it3) : cadd(t1, it3);
}

// multiply by e^{sign 2 pi i num / den} with constants (cos, sin of the
// forward angle -2 pi num / den)
template <typename C, bool INV>
__device__ __forceinline__ C rot(C v, double cr, double si) {
    using S = typename ScalarT<C>::type;
    const S c = S(cr), s = INV ? S(-si) : S(si);
    return C{v.x * c - v.y * s, v.x * s + v.y * c};
}

template <typename C, int R, bool INV>
__device__ __forceinline__ void small_dft(C (&v)[R]) {
    if constexpr (R == 2) {
        dft2<C, INV>(v[0], v[1]);
    } else if constexpr (R == 3) {
        dft3<C, INV>(v[0], v[1], v[2]);
    } else if constexpr (R == 4) {
        dft4<C, INV>(v[0], v[1], v[2], v[3]);
    } else if constexpr (R == 8) {
        // decimation in frequency: a_q = v_q + v_{q+4}, b_q = (v_q - v_{q+4}) w8^q,
        // X_{2k} = DFT4(a)_k, X_{2k+1} = DFT4(b)_k
        const double r2 = 0.70710678118654752440;
        C a[4], b[4];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            a[q] = cadd(v[q], v[q + 4]);
            b[q] = csub(v[q], v[q + 4]);
        }
        b[1] = rot<C, INV>(b[1], r2, -r2);
        b[2] = INV ? cmuli(b[2]) : C{b[2].y, -b[2].x};
        b[3] = rot<C, INV>(b[3], -r2, -r2);
        dft4<C, INV>(a[0], a[1], a[2], a[3]);
        dft4<C, INV>(b[0], b[1], b[2], b[3]);
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            v[2 * k] = a[k];
            v[2 * k + 1] = b[k];
        }
    } else {  // 9: DFT3 over v_{q+3t}, twiddles w9^(q k1), DFT3 over q
        const double c1 = 0.76604444311897803520, s1 = 0.64278760968653932632;  // 2 pi / 9
        const double c2 = 0.17364817766693034885, s2 = 0.98480775301220805936;  // 4 pi / 9
        const double c4 = -0.93969262078590838405, s4 = 0.34202014332566873304;  // 8 pi / 9
        C u[3][3];
#pragma unroll
        for (int q = 0; q < 3; ++q) {
            u[q][0] = v[q];
            u[q][1] = v[q + 3];
            u[q][2] = v[q + 6];
            dft3<C, INV>(u[q][0], u[q][1], u[q][2]);
        }
        u[1][1] = rot<C, INV>(u[1][1], c1, -s1);
        u[1][2] = rot<C, INV>(u[1][2], c2, -s2);
        u[2][1] = rot<C, INV>(u[2][1], c2, -s2);
        u[2][2] = rot<C, INV>(u[2][2], c4, -s4);
#pragma unroll
        for (int k1 = 0; k1 < 3; ++k1) {
            dft3<C, INV>(u[0][k1], u[1][k1], u[2][k1]);
            v[k1] = u[0][k1];
            v[k1 + 3] = u[1][k1];
            v[k1 + 6] = u[2][k1];
        }
    }
}

__device__ __forceinline__ int fft_div(int v, const FftDiv &f) {
    return (int)((__umulhi((unsigned)v, f.m) + (unsigned)v) >> f.s);
}

// shared-memory position of element i: the 16 complex values of each
// 128-byte row permuted by XOR with the row number, so the Stockham writes
// of the early stages (runs of Ns values R Ns apart) spread over the banks
// while consecutive elements stay one 128-byte row apart (9.02 against 9.12 ms
// per 64 x 2048^2 call with one spare slot after every 32 elements)
__device__ __forceinline__ int sp(int i) { return (i & ~15) | ((i ^ (i >> 4)) & 15); }

// one Stockham stage of radix R over `npen` pencils of length n
template <typename C, int R, bool INV>
__device__ __forceinline__ void fft_stage(const C *__restrict__ x, C *__restrict__ y, int n,
                                          int npen, int Ns, const FftDiv &mdiv,
                                          const FftDiv &nsdiv, const C *__restrict__ tw) {
    const int m = n / R;
    for (int idx = threadIdx.x; idx < npen * m; idx += blockDim.x) {
        const int pen = fft_div(idx, mdiv), j = idx - pen * m;
        const int k = j - fft_div(j, nsdiv) * Ns;
        const int xi = pen * n + j;
        C v[R];
#pragma unroll
        for (int q = 0; q < R; ++q) v[q] = x[sp(xi + q * m)];
        if (Ns > 1) {
#pragma unroll
            for (int q = 1; q < R; ++q) {
                const C w = tw[(q - 1) * Ns + k];
                v[q] = cmulc(v[q], INV ? cconj(w) : w);
            }
        }
        small_dft<C, R, INV>(v);
        const int yo = pen * n + (j - k) * R + k;
#pragma unroll
        for (int q = 0; q < R; ++q) y[sp(yo + q * Ns)] = v[q];
    }
}

// the transform of `npen` pencils of length n held at x[sp(p n + t)]; returns
// the buffer (x or y) that holds the result.  Every thread of the block calls
// it.
template <typename C>
__device__ C *smem_fft(C *x, C *y, int n, int npen, const FftPlan &pl, const C *tw, bool inverse) {
    int Ns = 1;
    for (int s = 0; s < pl.nst; ++s) {
        const int r = pl.rad[s];
#define AFGB_FFT_STAGE(RR)                                                                        \
    (inverse ? fft_stage<C, RR, true>(x, y, n, npen, Ns, pl.mdiv[s], pl.nsdiv[s], tw + pl.twoff[s]) \
             : fft_stage<C, RR, false>(x, y, n, npen, Ns, pl.mdiv[s], pl.nsdiv[s], tw + pl.twoff[s]))
        switch (r) {
            case 8: AFGB_FFT_STAGE(8); break;
            case 9: AFGB_FFT_STAGE(9); break;
            case 4: AFGB_FFT_STAGE(4); break;
            case 3: AFGB_FFT_STAGE(3); break;
            default: AFGB_FFT_STAGE(2); break;
        }
#undef AFGB_FFT_STAGE
        __syncthreads();
        C *t = x;
        x = y;
        y = t;
        Ns *= r;
    }
    return x;
}

// P consecutive rows per block (their complex views are one contiguous run)
template <typename R, typename C>
__global__ void __launch_bounds__(512) fft_r2c_rows_kernel(const R *__restrict__ in, C *__restrict__ out, int h,
                                    long long rows, int P, FftPlan pl, const C *__restrict__ tw_h,
                                    const C *__restrict__ tw_n) {
    using S = typename ScalarT<C>::type;
    extern __shared__ __align__(16) unsigned char fft_smem[];
    C *x = reinterpret_cast<C *>(fft_smem), *y = x + fft_padded(P * h);
    C *tws = y + fft_padded(P * h);  // the stage twiddles, copied once per block
    for (int j = threadIdx.x; j < h; j += blockDim.x) tws[j] = tw_h[j];
    for (long long row0 = (long long)blockIdx.x * P; row0 < rows; row0 += (long long)gridDim.x * P) {
        const int np = (int)min((long long)P, rows - row0);
        const C *src = reinterpret_cast<const C *>(in + row0 * 2LL * h);
        for (int j = threadIdx.x; j < np * h; j += blockDim.x) x[sp(j)] = src[j];
        __syncthreads();
        const C *Z = smem_fft<C>(x, y, h, np, pl, tws, false);
        for (int e = threadIdx.x; e < np * (h + 1); e += blockDim.x) {
            const int r = e / (h + 1), k = e - r * (h + 1);
            const C zk = Z[sp(r * h + (k == h ? 0 : k))];
            const C zc = cconj(Z[sp(r * h + (k == 0 ? 0 : h - k))]);
            const C ev = C{S(0.5) * (zk.x + zc.x), S(0.5) * (zk.y + zc.y)};
            const C d = csub(zk, zc);
            const C o = C{S(0.5) * d.y, S(-0.5) * d.x};  // (zk - zc) / (2i)
            out[row0 * (h + 1) + e] = cadd(ev, cmulc(tw_n[k], o));
        }
        __syncthreads();
    }
}

template <typename R, typename C>
__global__ void __launch_bounds__(512) fft_c2r_rows_kernel(const C *__restrict__ in, R *__restrict__ out, int h,
                                    long long rows, int P, FftPlan pl, const C *__restrict__ tw_h,
                                    const C *__restrict__ tw_n) {
    extern __shared__ __align__(16) unsigned char fft_smem[];
    C *x = reinterpret_cast<C *>(fft_smem), *y = x + fft_padded(P * h);
    C *tws = y + fft_padded(P * h);
    for (int j = threadIdx.x; j < h; j += blockDim.x) tws[j] = tw_h[j];
    for (long long row0 = (long long)blockIdx.x * P; row0 < rows; row0 += (long long)gridDim.x * P) {
        const int np = (int)min((long long)P, rows - row0);
        for (int e = threadIdx.x; e < np * h; e += blockDim.x) {
            const int r = e / h, k = e - r * h;
            const C *src = in + (row0 + r) * (long long)(h + 1);
            const C a = src[k], b = cconj(src[h - k]);
            const C t = cmulc(csub(a, b), cconj(tw_n[k]));
            x[sp(e)] = cadd(cadd(a, b), cmuli(t));
        }
        __syncthreads();
        const C *Z = smem_fft<C>(x, y, h, np, pl, tws, true);
        C *dst = reinterpret_cast<C *>(out + row0 * 2LL * h);
        for (int j = threadIdx.x; j < np * h; j += blockDim.x) dst[j] = Z[sp(j)];
        __syncthreads();
    }
}

// element (o, t, i) of the layout at (o n + t) inner + i
template <typename C>
__global__ void __launch_bounds__(512) fft_axis_kernel(C *__restrict__ data, int n, long long inner, long long outer,
                                int P, FftPlan pl, const C *__restrict__ tw, int inverse) {
    extern __shared__ __align__(16) unsigned char fft_smem[];
    C *x = reinterpret_cast<C *>(fft_smem), *y = x + fft_padded(P * n);
    C *tws = y + fft_padded(P * n);
    for (int j = threadIdx.x; j < n; j += blockDim.x) tws[j] = tw[j];
    const long long groups = (inner + P - 1) / P;
    for (long long g = blockIdx.x; g < outer * groups; g += gridDim.x) {
        const long long o = g / groups;
        const long long i0 = (g - o * groups) * P;
        const int np = (int)min((long long)P, inner - i0);
        C *base = data + o * (long long)n * inner + i0;
        for (int e = threadIdx.x; e < n * P; e += blockDim.x) {
            const int t = e / P, p = e - t * P;
            if (p < np) x[sp(p * n + t)] = base[(long long)t * inner + p];
        }
        __syncthreads();
        const C *Z = smem_fft<C>(x, y, n, np, pl, tws, inverse != 0);
        for (int e = threadIdx.x; e < n * P; e += blockDim.x) {
            const int t = e / P, p = e - t * P;
            if (p < np) base[(long long)t * inner + p] = Z[sp(p * n + t)];
        }
        __syncthreads();
    }
}

constexpr size_t kSmemCap = 220 * 1024;  // two padded buffers and the twiddles
constexpr size_t kRowSmem = 48 * 1024;    // rows kernels: several blocks per SM
// axis kernel: at least four neighbouring pencils (32-byte runs of the
// strided gather) when they fit the cap
constexpr int kAxisMinP = 4;
constexpr size_t kAxisSmem = 96 * 1024;

FftDiv make_div(unsigned d) {
    unsigned l = 0;
    while ((1ull << l) < d) ++l;
    const unsigned long long m = ((1ull << 32) * ((1ull << l) - d)) / d + 1;
    return FftDiv{d, (unsigned)m, l};
}

FftPlan make_plan(long long n) {
    FftPlan pl{};
    pl.n = (int)n;
    long long m = n;
    while (m % 8 == 0) {
        pl.rad[pl.nst++] = 8;
        m /= 8;
    }
    while (m % 4 == 0) {
        pl.rad[pl.nst++] = 4;
        m /= 4;
    }
    while (m % 2 == 0) {
        pl.rad[pl.nst++] = 2;
        m /= 2;
    }
    while (m % 9 == 0) {
        pl.rad[pl.nst++] = 9;
        m /= 9;
    }
    while (m % 3 == 0) {
        pl.rad[pl.nst++] = 3;
        m /= 3;
    }
    unsigned ns = 1;
    int off = 0;
    for (int s = 0; s < pl.nst; ++s) {
        pl.mdiv[s] = make_div((unsigned)(n / pl.rad[s]));
        pl.nsdiv[s] = make_div(ns);
        pl.twoff[s] = off;
        if (ns > 1) off += (pl.rad[s] - 1) * (int)ns;
        ns *= (unsigned)pl.rad[s];
    }
    return pl;
}

// the per-stage twiddle tables of make_plan(L)'s stages, in double on the
// host, kept per length and type; L entries (the stages use L - 1)
std::mutex g_stw_mu;
std::map<std::tuple<int, long long, int>, void *> g_stw;

template <typename C>
const C *stage_twiddles(long long L) {
    using S = typename ScalarT<C>::type;
    const auto key = std::make_tuple(device(), L, (int)sizeof(C));
    std::lock_guard<std::mutex> lk(g_stw_mu);
    auto it = g_stw.find(key);
    if (it != g_stw.end()) return static_cast<const C *>(it->second);
    const FftPlan pl = make_plan(L);
    std::vector<C> h((size_t)L, C{(S)0, (S)0});
    const double pi = 3.14159265358979323846264338327950288;
    long long ns = 1;
    for (int s = 0; s < pl.nst; ++s) {
        const int R = pl.rad[s];
        if (ns > 1)
            for (int q = 1; q < R; ++q)
                for (long long k = 0; k < ns; ++k) {
                    const double a = -2.0 * pi * (double)(q * k) / (double)(R * ns);
                    h[(size_t)(pl.twoff[s] + (q - 1) * ns + k)] = C{(S)std::cos(a), (S)std::sin(a)};
                }
        ns *= R;
    }
    void *d = nullptr;
    AFGB_CUDA(cudaMalloc(&d, (size_t)L * sizeof(C)));  // held for the process
    AFGB_CUDA(cudaMemcpy(d, h.data(), (size_t)L * sizeof(C), cudaMemcpyHostToDevice));
    g_stw[key] = d;
    return static_cast<const C *>(d);
}

// e^{-2 pi i j / L}, j < L, in double on the host, kept per length and type
std::mutex g_tw_mu;
std::map<std::tuple<int, long long, int>, void *> g_tw;

template <typename C>
const C *twiddles(long long L) {
    using S = typename ScalarT<C>::type;
    const auto key = std::make_tuple(device(), L, (int)sizeof(C));
    std::lock_guard<std::mutex> lk(g_tw_mu);
    auto it = g_tw.find(key);
    if (it != g_tw.end()) return static_cast<const C *>(it->second);
    std::vector<C> h((size_t)L);
    const double pi = 3.14159265358979323846264338327950288;
    for (long long j = 0; j < L; ++j) {
        const double a = -2.0 * pi * (double)j / (double)L;
        h[(size_t)j] = C{(S)std::cos(a), (S)std::sin(a)};
    }
    void *d = nullptr;
    AFGB_CUDA(cudaMalloc(&d, (size_t)L * sizeof(C)));  // held for the process
    AFGB_CUDA(cudaMemcpy(d, h.data(), (size_t)L * sizeof(C), cudaMemcpyHostToDevice));
    g_tw[key] = d;
    return static_cast<const C *>(d);
}

unsigned fft_grid(long long units) {
    return (unsigned)std::max(1LL, std::min(units, (long long)num_sms() * 8));
}

int fft_threads(long long n) { return n >= 2048 ? 512 : (n >= 256 ? 256 : 128); }

int rows_per_block(long long h, size_t csize, long long rows) {
    const size_t per = 2 * (size_t)h * csize;
    long long P = std::max<long long>(1, (long long)(kRowSmem / per));
    return (int)std::min<long long>(std::min<long long>(P, 16), std::max<long long>(rows, 1));
}

}  // namespace

bool fft_own_len_ok(long long n, bool real_rows, size_t csize) {
    if (n < 1) return false;
    long long m = n;
    if (real_rows) {
        if (m & 1) return false;
        m /= 2;
    }
    const long long len = m;
    while (m % 2 == 0) m /= 2;
    while (m % 3 == 0) m /= 3;
    return m == 1 && (2 * (size_t)fft_padded((int)std::min<long long>(len, 1 << 20)) + len) * csize <= kSmemCap;
}

template <typename R, typename C>
void fft_real_forward(const R *in, C *out, long long n0, long long rows) {
    if (rows <= 0) return;
    const int h = (int)(n0 / 2);
    const FftPlan pl = make_plan(h);
    const int P = rows_per_block(h, sizeof(C), rows);
    const size_t smem = (2 * (size_t)fft_padded(P * h) + h) * sizeof(C);
    auto k = fft_r2c_rows_kernel<R, C>;
    AFGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const C *twh = stage_twiddles<C>(h), *twn = twiddles<C>(n0);
    {
        KernelTimer kt("fft_r2c_rows_kernel");
        k<<<fft_grid((rows + P - 1) / P), fft_threads((long long)P * h), smem, stream()>>>(
            in, out, h, rows, P, pl, twh, twn);
    }
    count_launch();
    AFGB_POST_LAUNCH("fft_r2c_rows_kernel");
}

template <typename R, typename C>
void fft_real_inverse(const C *in, R *out, long long n0, long long rows) {
    if (rows <= 0) return;
    const int h = (int)(n0 / 2);
    const FftPlan pl = make_plan(h);
    const int P = rows_per_block(h, sizeof(C), rows);
    const size_t smem = (2 * (size_t)fft_padded(P * h) + h) * sizeof(C);
    auto k = fft_c2r_rows_kernel<R, C>;
    AFGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const C *twh = stage_twiddles<C>(h), *twn = twiddles<C>(n0);
    {
        KernelTimer kt("fft_c2r_rows_kernel");
        k<<<fft_grid((rows + P - 1) / P), fft_threads((long long)P * h), smem, stream()>>>(
            in, out, h, rows, P, pl, twh, twn);
    }
    count_launch();
    AFGB_POST_LAUNCH("fft_c2r_rows_kernel");
}

template <typename C>
void fft_axis(C *data, long long n, long long inner, long long outer, bool inverse) {
    if (n <= 1 || inner <= 0 || outer <= 0) return;
    const FftPlan pl = make_plan(n);
    // neighbouring pencils per block: rows of the gather read P consecutive
    // elements; at least one pencil, within the shared-memory cap
    const size_t per = 2 * (size_t)n * sizeof(C);
    int P = (int)std::max<size_t>(1, std::min<size_t>(16, kRowSmem / per));
    // at least kAxisMinP neighbouring pencils (32-byte runs) while two
    // blocks still fit an SM
    if (P < kAxisMinP)
        P = (int)std::max<size_t>(1, std::min<size_t>(kAxisMinP, kAxisSmem / per));
    P = (int)std::min<long long>(P, inner);
    while (P > 1 && (2 * (size_t)fft_padded(P * (int)n) + n) * sizeof(C) > kSmemCap) --P;
    const size_t smem = (2 * (size_t)fft_padded(P * (int)n) + n) * sizeof(C);
    auto k = fft_axis_kernel<C>;
    AFGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    const long long units = outer * ((inner + P - 1) / P);
    const C *tw = stage_twiddles<C>(n);
    {
        KernelTimer kt("fft_axis_kernel");
        k<<<fft_grid(units), fft_threads(n * P), smem, stream()>>>(data, (int)n, inner, outer, P,
                                                                  pl, tw, inverse ? 1 : 0);
    }
    count_launch();
    AFGB_POST_LAUNCH("fft_axis_kernel");
}

template void fft_real_forward<float, cf32>(const float *, cf32 *, long long, long long);
template void fft_real_forward<double, cf64>(const double *, cf64 *, long long, long long);
template void fft_real_inverse<float, cf32>(const cf32 *, float *, long long, long long);
template void fft_real_inverse<double, cf64>(const cf64 *, double *, long long, long long);
template void fft_axis<cf32>(cf32 *, long long, long long, long long, bool);
template void fft_axis<cf64>(cf64 *, long long, long long, long long, bool);

}  // namespace afgb
