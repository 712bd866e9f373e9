// af_harris: the Harris corner detector built around the separable
// convolution (src/api/c/harris.cpp:42-95; CPU backend
// src/backend/cpu/harris.cpp:28-144 with the kernels of
// src/backend/cpu/kernel/gradient.hpp:18-80 and
// src/backend/cpu/kernel/harris.hpp:18-118).
//
// Device pipeline; for f32 and f64 images the corners, their order and their
// scores are identical to the reference CPU backend's:
//  1. harris_products_kernel: the gradient along both dimensions (central
//     differences halved, one-sided differences at the edges) and the three
//     products ix*ix, ix*iy, iy*iy, written as the three planes of one
//     (d0, d1, 3) array, each operation rounded separately;
//  2. the window (a box of 1/len when sigma < 0.5, else the sampled
//     Gaussian) over the three planes as one batched separable convolution
//     (launch_convolve2_sep) in the reference's rounding order;
//  3. harris_response_kernel: det - k * tr^2 on [border, d - border) in both
//     dimensions, border = len/2 + 1;
//  4. nms_count_kernel / nms_scan_kernel / nms_scatter_kernel: strict maxima
//     of their 8 neighbours (the reference's std::max chain) that reach the
//     minimum response, on [border + 1, d - border - 1), compacted in
//     column-major scan order: each block owns a contiguous range of pixels,
//     the block totals are scanned, then each block writes its corners at its
//     offset in order (ballot + warp prefix); at most 20% of the pixels are
//     kept, the total found is counted in full;
//  5. with max_corners > 0 and more corners found: one radix sort (CUB's
//     DeviceRadixSort) of 64-bit keys (descending score, list position),
//     which is the reference's stable descending sort, and a gather of the
//     first max_corners.
// The host reads the number of corners once (after step 4's scan) to size
// the outputs, as the reference does.
#include <cuda_runtime.h>

#include <cub/device/device_radix_sort.cuh>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <vector>

#include "afgb_internal.hpp"
#include "conv_common.cuh"
#include "conv_direct.hpp"

namespace afgb {

namespace {

constexpr int NMS_THREADS = 256;
constexpr int NMS_ITEMS = 16;
constexpr long long NMS_CHUNK = (long long)NMS_THREADS * NMS_ITEMS;

template <typename T>
__global__ void harris_products_kernel(const T *in, long long d0, long long d1, T *out) {
    const long long n = d0 * d1;
    const T half = T(0.5);
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const long long i = t % d0, j = t / d0;
        // grad0 (along dim0) is iy, grad1 (along dim1) is ix; the edge
        // factor 1 leaves the difference as it is
        T gy, gx;
        if (i == 0) gy = r_sub(in[t + 1], in[t]);
        else if (i == d0 - 1) gy = r_sub(in[t], in[t - 1]);
        else gy = r_mul(half, r_sub(in[t + 1], in[t - 1]));
        if (j == 0) gx = r_sub(in[t + d0], in[t]);
        else if (j == d1 - 1) gx = r_sub(in[t], in[t - d0]);
        else gx = r_mul(half, r_sub(in[t + d0], in[t - d0]));
        out[t] = r_mul(gx, gx);
        out[n + t] = r_mul(gx, gy);
        out[2 * n + t] = r_mul(gy, gy);
    }
}

// k is the float k_thr in the image type (a double image promotes it)
template <typename T>
__global__ void harris_response_kernel(const T *win, long long d0, long long d1, long long border,
                                       T k, T *resp) {
    const long long n = d0 * d1;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const long long i = t % d0, j = t / d0;
        T v = T(0);
        if (i >= border && i < d0 - border && j >= border && j < d1 - border) {
            const T xx = win[t], xy = win[n + t], yy = win[2 * n + t];
            const T tr = r_add(xx, yy);
            const T det = r_sub(r_mul(xx, yy), r_mul(xy, xy));
            v = r_sub(det, r_mul(k, r_mul(tr, tr)));
        }
        resp[t] = v;
    }
}

// std::max(a, b) as the reference's chain evaluates it
template <typename T>
__device__ __forceinline__ T ref_max(T a, T b) { return (a < b) ? b : a; }

// whether pixel t is a corner; its response in *v
template <typename T>
__device__ __forceinline__ bool is_corner(const T *resp, long long t, long long n, long long d0,
                                          long long d1, long long r, T minr, T *v) {
    if (t >= n) return false;
    const long long y = t % d0, x = t / d0;
    if (y < r || y >= d0 - r || x < r || x >= d1 - r) return false;
    const T c = resp[t];
    T m = ref_max(resp[t - d0 - 1], resp[t - 1]);
    m = ref_max(m, resp[t + d0 - 1]);
    m = ref_max(m, resp[t - d0]);
    m = ref_max(m, resp[t + d0]);
    m = ref_max(m, resp[t - d0 + 1]);
    m = ref_max(m, resp[t + 1]);
    m = ref_max(m, resp[t + d0 + 1]);
    *v = c;
    return c > m && c >= minr;
}

__device__ __forceinline__ unsigned long long block_sum(unsigned long long v,
                                                        unsigned long long *sh) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (lane == 0) sh[w] = v;
    __syncthreads();
    unsigned long long s = 0;
    if (threadIdx.x == 0)
        for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += sh[i];
    return s;
}

template <typename T>
__global__ void __launch_bounds__(NMS_THREADS)
    nms_count_kernel(const T *resp, long long d0, long long d1, long long r, T minr,
                     unsigned *counts) {
    __shared__ unsigned long long sh[NMS_THREADS / 32];
    const long long n = d0 * d1;
    const long long base = blockIdx.x * NMS_CHUNK;
    unsigned c = 0;
    T v;
#pragma unroll 4
    for (int it = 0; it < NMS_ITEMS; ++it)
        c += is_corner(resp, base + it * NMS_THREADS + threadIdx.x, n, d0, d1, r, minr, &v) ? 1u
                                                                                         : 0u;
    const unsigned long long s = block_sum(c, sh);
    if (threadIdx.x == 0) counts[blockIdx.x] = (unsigned)s;
}

// exclusive scan of the block counts (one block of 1024 threads); the grand
// total into *found
__global__ void __launch_bounds__(1024)
    nms_scan_kernel(const unsigned *counts, long long nblocks, unsigned long long *offsets,
                    unsigned long long *found) {
    __shared__ unsigned long long warp_tot[32];
    __shared__ unsigned long long carry;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (long long b0 = 0; b0 < nblocks; b0 += 1024) {
        const long long b = b0 + threadIdx.x;
        const unsigned long long v = b < nblocks ? counts[b] : 0ull;
        unsigned long long inc = v;
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned long long u = __shfl_up_sync(0xffffffffu, inc, o);
            if (lane >= o) inc += u;
        }
        if (lane == 31) warp_tot[w] = inc;
        __syncthreads();
        unsigned long long before = 0;
        for (int i = 0; i < w; ++i) before += warp_tot[i];
        const unsigned long long c0 = carry;
        if (b < nblocks) offsets[b] = c0 + before + inc - v;
        __syncthreads();
        if (threadIdx.x == 1023) carry = c0 + before + inc;
        __syncthreads();
    }
    if (threadIdx.x == 0) *found = carry;
}

// the corners of each block at its offset, in scan order.  Positions below
// `lim` are written: straight into the outputs, or (keys != nullptr) into the
// candidate lists with their sort keys
template <typename T>
__global__ void __launch_bounds__(NMS_THREADS)
    nms_scatter_kernel(const T *resp, long long d0, long long d1, long long r, T minr,
                       const unsigned long long *offsets, long long lim, float *xo, float *yo,
                       float *so, unsigned long long *keys) {
    __shared__ unsigned warp_cnt[NMS_THREADS / 32];
    const long long n = d0 * d1;
    const long long base = blockIdx.x * NMS_CHUNK;
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    unsigned long long pos0 = offsets[blockIdx.x];
    for (int it = 0; it < NMS_ITEMS; ++it) {
        const long long t = base + it * NMS_THREADS + threadIdx.x;
        T v = T(0);
        const bool hit = is_corner(resp, t, n, d0, d1, r, minr, &v);
        const unsigned mask = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) warp_cnt[w] = __popc(mask);
        __syncthreads();
        unsigned before = 0, total = 0;
#pragma unroll
        for (int i = 0; i < NMS_THREADS / 32; ++i) {
            const unsigned c = warp_cnt[i];
            before += i < w ? c : 0u;
            total += c;
        }
        if (hit) {
            const unsigned long long pos =
                pos0 + before + __popc(mask & ((1u << lane) - 1u));
            if ((long long)pos < lim) {
                const float s = (float)v;
                xo[pos] = (float)(t / d0);
                yo[pos] = (float)(t % d0);
                so[pos] = s;
                if (keys) {
                    // ascending keys = descending scores, ties by position;
                    // -0 and +0 compare equal in the reference's sort
                    unsigned u = __float_as_uint(s == 0.f ? 0.f : s);
                    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
                    keys[pos] = ((unsigned long long)(~u) << 32) | (unsigned long long)pos;
                }
            }
        }
        pos0 += total;
        __syncthreads();
    }
}

__global__ void keep_corners_kernel(const unsigned long long *sorted, long long nout,
                                    const float *xs, const float *ys, const float *ss, float *xo,
                                    float *yo, float *so) {
    for (long long f = blockIdx.x * (long long)blockDim.x + threadIdx.x; f < nout;
         f += (long long)gridDim.x * blockDim.x) {
        const unsigned p = (unsigned)(sorted[f] & 0xffffffffull);
        xo[f] = xs[p];
        yo[f] = ys[p];
        so[f] = ss[p];
    }
}

__global__ void fill_f32_kernel(float *p, long long n, float v) {
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x)
        p[i] = v;
}

unsigned grid_of(long long total, int threads) {
    const long long b = (total + threads - 1) / threads;
    return (unsigned)std::max(1LL, std::min(b, (long long)num_sms() * 32));
}

// The window of src/backend/cpu/harris.cpp:38-47: a box of 1/len, or
// gaussian1D (src/backend/cpu/utility.hpp:35-49): each tap evaluated in
// double, stored in T, summed in T in order, then divided by the sum in T.
template <typename T>
std::vector<T> harris_window(unsigned len, float sigma) {
    std::vector<T> f(len);
    if (sigma < 0.5f) {
        for (unsigned i = 0; i < len; i++) f[i] = static_cast<T>(1) / (len);
        return f;
    }
    const double pi = 3.14159265358979323846264338327950288;
    const double s = sigma;
    T sum = (T)0;
    for (int i = 0; i < (int)len; i++) {
        const int x = i - ((int)len - 1) / 2;
        const T el = 1. / std::sqrt(2 * pi * s * s) * std::exp(-((x * x) / (2 * (s * s))));
        f[i] = el;
        sum += el;
    }
    for (unsigned k = 0; k < len; k++) f[k] /= sum;
    return f;
}

Array new_f32(long long n) {
    const dim_t d[4] = {(dim_t)n, 1, 1, 1};
    return *create_array(f32, d);
}

template <typename T>
void harris_t(const Array &img, unsigned max_corners, float min_response, float sigma,
              unsigned filter_len, float k_thr, HarrisOut &res) {
    const long long d0 = img.dims[0], d1 = img.dims[1], n = d0 * d1;
    const long long border = filter_len / 2 + 1, r = border + 1;
    const unsigned corner_lim = static_cast<unsigned>(n * 0.2f);
    res.n = 0;
    // no pixel has the full neighbourhood: the reference's loops are empty
    if (d0 <= 2 * r || d1 <= 2 * r || corner_lim == 0) return;
    const Array src = img.is_linear() ? img : make_dense(img);

    // 1. gradient products as the planes of one (d0, d1, 3) array
    const dim_t pd[4] = {(dim_t)d0, (dim_t)d1, 3, 1};
    Array prod, win;
    {
        MemTag tag("corner-detector intermediates");
        prod = *create_array(img.type, pd);
        win = *create_array(img.type, pd);
    }
    harris_products_kernel<T><<<grid_of(n, 256), 256, 0, stream()>>>(src.ptr<T>(), d0, d1,
                                                                     prod.ptr<T>());
    count_launch();
    AFGB_POST_LAUNCH("harris_products_kernel");

    // 2. the window over the three planes, in the reference's rounding order
    {
        const std::vector<T> h = harris_window<T>(filter_len, sigma);
        const dim_t fd[4] = {(dim_t)filter_len, 1, 1, 1};
        Array filt;
        {
            MemTag tag("corner-detector intermediates");
            filt = *create_array(img.type, fd);
        }
        AFGB_CUDA(cudaMemcpyAsync(filt.data(), h.data(), h.size() * sizeof(T),
                                  cudaMemcpyHostToDevice, stream()));
        ExactScope exact;
        launch_convolve2_sep(prod, filt, filt, win, false);
    }

    // 3. responses (into the first product plane, no longer needed)
    T *resp = prod.ptr<T>();
    harris_response_kernel<T><<<grid_of(n, 256), 256, 0, stream()>>>(
        win.ptr<T>(), d0, d1, border, (T)k_thr, resp);
    count_launch();
    AFGB_POST_LAUNCH("harris_response_kernel");

    // 4. maxima, counted per block, scanned, then compacted in scan order
    const unsigned min_r = (max_corners > 0) ? 0U : static_cast<unsigned>(min_response);
    const T minr = (T)(float)min_r;
    const long long nblocks = (n + NMS_CHUNK - 1) / NMS_CHUNK;
    unsigned *counts;
    unsigned long long *offsets;
    {
        MemTag tag("corner-detector intermediates");
        counts = static_cast<unsigned *>(alloc_device((size_t)nblocks * sizeof(unsigned)));
        offsets = static_cast<unsigned long long *>(
            alloc_device((size_t)(nblocks + 1) * sizeof(unsigned long long)));
    }
    nms_count_kernel<T><<<(unsigned)nblocks, NMS_THREADS, 0, stream()>>>(resp, d0, d1, r, minr,
                                                                        counts);
    count_launch();
    AFGB_POST_LAUNCH("nms_count_kernel");
    nms_scan_kernel<<<1, 1024, 0, stream()>>>(counts, nblocks, offsets, offsets + nblocks);
    count_launch();
    AFGB_POST_LAUNCH("nms_scan_kernel");
    unsigned long long found = 0;
    AFGB_CUDA(cudaMemcpyAsync(&found, offsets + nblocks, sizeof(found), cudaMemcpyDeviceToHost,
                              stream()));
    AFGB_CUDA(cudaStreamSynchronize(stream()));
    check_device_errors();

    const unsigned long long cap = (max_corners > 0) ? max_corners : corner_lim;
    const long long nout = (long long)std::min<unsigned long long>(found, cap);
    if (nout > 0) {
        res.x = new_f32(nout);
        res.y = new_f32(nout);
        res.score = new_f32(nout);
        const bool sort = max_corners > 0 && found > (unsigned long long)nout;
        if (!sort) {
            nms_scatter_kernel<T><<<(unsigned)nblocks, NMS_THREADS, 0, stream()>>>(
                resp, d0, d1, r, minr, offsets, nout, res.x.ptr<float>(), res.y.ptr<float>(),
                res.score.ptr<float>(), nullptr);
            count_launch();
            AFGB_POST_LAUNCH("nms_scatter_kernel");
        } else {
            // the candidates the reference keeps (at most corner_lim), sorted
            const long long m = (long long)std::min<unsigned long long>(found, corner_lim);
            float *xs, *ys, *ss;
            unsigned long long *keys, *sorted;
            size_t tmp_bytes = 0;
            AFGB_CUDA(cub::DeviceRadixSort::SortKeys(nullptr, tmp_bytes,
                                                     (const unsigned long long *)nullptr,
                                                     (unsigned long long *)nullptr, (int)m, 0, 64,
                                                     stream()));
            void *tmp;
            {
                MemTag tag("corner-detector intermediates");
                xs = static_cast<float *>(alloc_device((size_t)m * sizeof(float)));
                ys = static_cast<float *>(alloc_device((size_t)m * sizeof(float)));
                ss = static_cast<float *>(alloc_device((size_t)m * sizeof(float)));
                keys = static_cast<unsigned long long *>(alloc_device((size_t)m * 8));
                sorted = static_cast<unsigned long long *>(alloc_device((size_t)m * 8));
                tmp = alloc_device(std::max<size_t>(tmp_bytes, 16));
            }
            nms_scatter_kernel<T><<<(unsigned)nblocks, NMS_THREADS, 0, stream()>>>(
                resp, d0, d1, r, minr, offsets, m, xs, ys, ss, keys);
            count_launch();
            AFGB_POST_LAUNCH("nms_scatter_kernel");
            AFGB_CUDA(cub::DeviceRadixSort::SortKeys(tmp, tmp_bytes,
                                                     (const unsigned long long *)keys, sorted,
                                                     (int)m, 0, 64, stream()));
            count_launch();
            AFGB_POST_LAUNCH("DeviceRadixSort::SortKeys");
            keep_corners_kernel<<<grid_of(nout, 256), 256, 0, stream()>>>(
                sorted, nout, xs, ys, ss, res.x.ptr<float>(), res.y.ptr<float>(),
                res.score.ptr<float>());
            count_launch();
            AFGB_POST_LAUNCH("keep_corners_kernel");
            free_device(tmp);
            free_device(sorted);
            free_device(keys);
            free_device(ss);
            free_device(ys);
            free_device(xs);
        }
        res.orientation = new_f32(nout);
        res.size = new_f32(nout);
        AFGB_CUDA(cudaMemsetAsync(res.orientation.data(), 0, (size_t)nout * sizeof(float), stream()));
        fill_f32_kernel<<<grid_of(nout, 256), 256, 0, stream()>>>(res.size.ptr<float>(), nout, 1.f);
        count_launch();
        AFGB_POST_LAUNCH("fill_f32_kernel");
    }
    free_device(offsets);
    free_device(counts);
    res.n = nout;
}

}  // namespace

void harris_corners(const Array &img, unsigned max_corners, float min_response, float sigma,
                    unsigned filter_len, float k_thr, HarrisOut &out) {
    if (img.type == f64)
        harris_t<double>(img, max_corners, min_response, sigma, filter_len, k_thr, out);
    else
        harris_t<float>(img, max_corners, min_response, sigma, filter_len, k_thr, out);
}

}  // namespace afgb
