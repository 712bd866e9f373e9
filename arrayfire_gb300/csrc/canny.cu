// af_canny: Canny edges built around the separable convolution and the Sobel
// derivatives (src/api/c/canny.cpp:196-285; CPU kernels
// src/backend/cpu/kernel/canny.hpp and src/backend/cpu/canny.cpp).
//
// Device pipeline; the 0/1 edge map is identical to the reference CPU
// backend's for every accepted type:
//  1. the image in float (cast_array) smoothed by the 5-tap separable filter
//     (launch_convolve2_sep, in the reference's rounding order), then the 3x3
//     Sobel derivatives (sobel_3x3);
//  2. canny_mag_kernel: |gx| + |gy|, or sqrt(gx^2 + gy^2);
//  3. canny_nms_kernel: non-maximum suppression on the interior of each
//     slice, the magnitude interpolated along the gradient direction with
//     every operation rounded as the reference's loop rounds it;
//  4. canny_minmax_kernel: the maximum and minimum over all slices (the
//     values are non-negative, so their bit patterns order like the values);
//  5. thresholds, one byte per pixel (bit 0 strong, bit 1 weak):
//     manual -- (s - min) / (max - min) against the two ratios; Otsu --
//     canny_hist_kernel (one histogram of floor(max) bins per slice),
//     canny_otsu_kernel (one block per slice: the prefix sums in the
//     reference's sequential order by one thread, then the between-class
//     variance of every split and its first maximum by the block), then
//     canny_classify_otsu_kernel;
//  6. hysteresis as connected components: weak pixels are joined with their
//     weak neighbours (the reference's linear offsets t +- 1, t +- d0,
//     t +- d0 +- 1) by a lock-free union-find (atomicMin linking, roots only
//     decrease, so every loop ends); each seed -- a strong pixel whose linear
//     index lies in the range the reference's seed scan visits -- marks the
//     components of its weak neighbours; an edge is a seed or a weak pixel
//     of a marked component.
// The host reads the maximum and minimum once (step 4), as the reference
// does.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>

#include "afgb_internal.hpp"
#include "conv_common.cuh"
#include "conv_direct.hpp"

namespace afgb {

namespace {

constexpr uint8_t kStrong = 1, kWeak = 2;

__global__ void canny_mag_kernel(const float *gx, const float *gy, long long n, int isf,
                                 float *mag) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const float x = gx[t], y = gy[t];
        mag[t] = isf ? __fadd_rn(fabsf(x), fabsf(y))
                     : __fsqrt_rn(__fadd_rn(__fmul_rn(x, x), __fmul_rn(y, y)));
    }
}

// src/backend/cpu/kernel/canny.hpp:18-116 for the pixel at linear offset t of
// a slice (d0 x d1), 1 <= row <= d0-2, 1 <= column <= d1-2
__device__ __forceinline__ float nms_pixel(const float *mag, const float *dX, const float *dY,
                                           long long t, long long d0) {
    const float curr = mag[t];
    if (curr == 0) return 0.f;
    const float se = mag[t + d0 + 1], nw = mag[t - d0 - 1];
    const float ea = mag[t + 1], we = mag[t - 1];
    const float ne = mag[t - d0 + 1], sw = mag[t + d0 - 1];
    const float no = mag[t - d0], so = mag[t + d0];
    const float dx = dX[t], dy = dY[t];
    float a1, a2, b1, b2, alpha;
    if (dx >= 0) {
        if (dy >= 0) {
            const bool g = __fsub_rn(dx, dy) >= 0;
            a1 = g ? ea : so;
            a2 = g ? we : no;
            b1 = se;
            b2 = nw;
            alpha = g ? __fdiv_rn(dy, dx) : __fdiv_rn(dx, dy);
        } else {
            const bool g = __fadd_rn(dx, dy) >= 0;
            a1 = g ? ea : no;
            a2 = g ? we : so;
            b1 = ne;
            b2 = sw;
            alpha = g ? __fdiv_rn(-dy, dx) : __fdiv_rn(dx, -dy);
        }
    } else {
        if (dy >= 0) {
            const bool g = __fadd_rn(dx, dy) >= 0;
            a1 = g ? so : we;
            a2 = g ? no : ea;
            b1 = sw;
            b2 = ne;
            alpha = g ? __fdiv_rn(-dx, dy) : __fdiv_rn(dy, -dx);
        } else {
            const bool g = __fadd_rn(-dx, dy) >= 0;
            a1 = g ? we : no;
            a2 = g ? ea : so;
            b1 = nw;
            b2 = se;
            alpha = g ? __fdiv_rn(dy, dx) : __fdiv_rn(dx, dy);
        }
    }
    const float oma = __fsub_rn(1.0f, alpha);
    const float mag1 = __fadd_rn(__fmul_rn(oma, a1), __fmul_rn(alpha, b1));
    const float mag2 = __fadd_rn(__fmul_rn(oma, a2), __fmul_rn(alpha, b2));
    return (curr > mag1 && curr > mag2) ? curr : 0.f;
}

__global__ void canny_nms_kernel(const float *mag, const float *gx, const float *gy, long long d0,
                                 long long d1, long long n, float *sup) {
    const long long plane = d0 * d1;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const long long l = t % plane;
        const long long i = l % d0, j = l / d0;
        float v = 0.f;
        if (i >= 1 && i <= d0 - 2 && j >= 1 && j <= d1 - 2) v = nms_pixel(mag, gx, gy, t, d0);
        sup[t] = v;
    }
}

// mm[0] = bits of the maximum, mm[1] = bits of the minimum (values >= 0)
__global__ void canny_minmax_kernel(const float *sup, long long n, unsigned *mm) {
    unsigned hi = 0u, lo = 0x7f800000u;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const unsigned b = __float_as_uint(sup[t]);
        hi = max(hi, b);
        lo = min(lo, b);
    }
    for (int o = 16; o > 0; o >>= 1) {
        hi = max(hi, __shfl_down_sync(0xffffffffu, hi, o));
        lo = min(lo, __shfl_down_sync(0xffffffffu, lo, o));
    }
    if ((threadIdx.x & 31) == 0) {
        atomicMax(&mm[0], hi);
        atomicMin(&mm[1], lo);
    }
}

__global__ void canny_classify_manual_kernel(const float *sup, long long n, float minv, float denom,
                                             float t1, float t2, uint8_t *cls) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const float g = __fdiv_rn(__fsub_rn(sup[t], minv), denom);
        cls[t] = (g >= t2 ? kStrong : 0) | ((g >= t1 && g < t2) ? kWeak : 0);
    }
}

// kernel::histogram<float, true> (src/backend/cpu/kernel/histogram.hpp:18-45)
// of each slice: bin = (int)((v - 0) / step) clamped to [0, nb-1].  The lanes
// of a warp that hit the same bin (most pixels of a suppressed image are 0)
// add their count with one atomic.
__global__ void canny_hist_kernel(const float *sup, long long plane, long long n, unsigned nb,
                                  float step, unsigned *hist) {
    const int lane = threadIdx.x & 31;
    for (long long t0 = (blockIdx.x * (long long)blockDim.x + threadIdx.x) - lane; t0 < n;
         t0 += (long long)gridDim.x * blockDim.x) {
        const long long t = t0 + lane;
        unsigned long long key = ~0ull;
        if (t < n) {
            int bin = (int)__fdiv_rn(__fsub_rn(sup[t], 0.f), step);
            bin = max(bin, 0);
            bin = min(bin, (int)(nb - 1));
            key = (unsigned long long)(t / plane) * nb + (unsigned)bin;
        }
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        if (key != ~0ull && lane == __ffs(peers) - 1) atomicAdd(&hist[key], (unsigned)__popc(peers));
    }
}

// otsuThreshold (src/api/c/canny.cpp:81-141) for slice blockIdx.x: thread 0
// forms the prefix sums in the reference's order (scan and reduce add each
// element to the running value); then every split b < nb-1 gets its
// between-class variance and the block takes the first maximum, NaN skipped
// (ireduce<af_max_t>, src/backend/cpu/kernel/ireduce.hpp:47-63).  T2 = that
// split, T1 = T2 * t1.
__global__ void __launch_bounds__(256)
    canny_otsu_kernel(const unsigned *hist, unsigned nb, float total, float t1, float *cum,
                      float *cprod, float *thr) {
    const unsigned *h = hist + (long long)blockIdx.x * nb;
    float *cs = cum + (long long)blockIdx.x * nb;
    float *cp = cprod + (long long)blockIdx.x * nb;
    __shared__ float ws;
    __shared__ float best_v[256];
    __shared__ unsigned best_i[256];
    if (threadIdx.x == 0) {
        float c = 0.f, p = 0.f;
        for (unsigned b = 0; b < nb; ++b) {
            const float f = __fdiv_rn((float)h[b], total);
            c = __fadd_rn(f, c);
            cs[b] = c;
            p = __fadd_rn(__fmul_rn((float)b, f), p);
            cp[b] = p;
        }
        ws = p;
    }
    __syncthreads();
    float bv = -INFINITY;
    unsigned bi = 0xffffffffu;
    for (unsigned b = threadIdx.x; b + 1 < nb; b += blockDim.x) {
        const float qL = cs[b];
        const float qH = __fsub_rn(1.0f, qL);
        const float muL = __fdiv_rn(cp[b], qL);
        const float muH = __fdiv_rn(__fsub_rn(ws, cp[b]), qH);
        const float diff = __fsub_rn(muL, muH);
        float s = __fmul_rn(__fmul_rn(diff, diff), __fmul_rn(qL, __fsub_rn(1.0f, qL)));
        if (s != s) s = -INFINITY;
        if (bi == 0xffffffffu || s > bv) {  // splits arrive in increasing order
            bv = s;
            bi = b;
        }
    }
    best_v[threadIdx.x] = bv;
    best_i[threadIdx.x] = bi;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) {
            const float ov = best_v[threadIdx.x + w];
            const unsigned oi = best_i[threadIdx.x + w];
            const float mv = best_v[threadIdx.x];
            const unsigned mi = best_i[threadIdx.x];
            if (oi != 0xffffffffu &&
                (mi == 0xffffffffu || ov > mv || (ov == mv && oi < mi))) {
                best_v[threadIdx.x] = ov;
                best_i[threadIdx.x] = oi;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        const unsigned loc = best_i[0] == 0xffffffffu ? 0u : best_i[0];
        const float T2 = (float)loc;
        thr[2 * blockIdx.x] = __fmul_rn(T2, t1);
        thr[2 * blockIdx.x + 1] = T2;
    }
}

__global__ void canny_classify_otsu_kernel(const float *sup, long long plane, long long n,
                                           const float *thr, uint8_t *cls) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const long long z = t / plane;
        const float T1 = thr[2 * z], T2 = thr[2 * z + 1];
        const float s = sup[t];
        cls[t] = (s >= T2 ? kStrong : 0) | ((s >= T1 && s < T2) ? kWeak : 0);
    }
}

__device__ __forceinline__ int uf_find(const int *parent, int x) {
    int p = *((const volatile int *)&parent[x]);
    while (p != x) {
        x = p;
        p = *((const volatile int *)&parent[x]);
    }
    return x;
}

// join the sets of a and b: the larger root is linked under the smaller one;
// a root only ever decreases, so the loop ends
__device__ __forceinline__ void uf_union(int *parent, int a, int b) {
    for (;;) {
        a = uf_find(parent, a);
        b = uf_find(parent, b);
        if (a == b) return;
        if (a < b) {
            const int t = a;
            a = b;
            b = t;
        }
        const int old = atomicMin(&parent[a], b);
        if (old == a) return;
        a = old;
    }
}

__global__ void canny_uf_init_kernel(int *parent, long long n) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        parent[t] = (int)t;
}

// each weak pixel joins its weak neighbours at the four backward offsets
// (the forward ones are the backward ones of those neighbours); neighbours
// outside the slice are skipped
__global__ void canny_uf_merge_kernel(const uint8_t *cls, long long d0, long long plane,
                                      long long n, int *parent) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        if (!(cls[t] & kWeak)) continue;
        const long long l = t % plane;
        const long long offs[4] = {-1, -d0 - 1, -d0, -d0 + 1};
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            const long long u = l + offs[k];
            if (u >= 0 && u < plane && (cls[t - l + u] & kWeak))
                uf_union(parent, (int)t, (int)(t - l + u));
        }
    }
}

__global__ void canny_uf_flatten_kernel(const uint8_t *cls, long long n, int *parent) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        if (cls[t] & kWeak) parent[t] = uf_find(parent, (int)t);
}

// seeds: strong pixels at slice-local linear indices [d0+1, d0+(d0-1)(d1-1)]
// (src/backend/cpu/kernel/canny.hpp:158-178 advances its index d0-1 times per
// column, so its scan covers exactly this range)
__device__ __forceinline__ bool is_seed(const uint8_t *cls, long long t, long long l, long long d0,
                                        long long d1) {
    return (cls[t] & kStrong) && l >= d0 + 1 && l <= d0 + (d0 - 1) * (d1 - 1);
}

__global__ void canny_mark_kernel(const uint8_t *cls, const int *parent, long long d0,
                                  long long d1, long long n, uint8_t *on) {
    const long long plane = d0 * d1;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const long long l = t % plane;
        if (!is_seed(cls, t, l, d0, d1)) continue;
        const long long offs[8] = {-d0 - 1, -d0, -d0 + 1, -1, 1, d0 - 1, d0, d0 + 1};
#pragma unroll
        for (int k = 0; k < 8; ++k) {
            const long long u = l + offs[k];
            if (u >= 0 && u < plane && (cls[t - l + u] & kWeak)) on[parent[t - l + u]] = 1;
        }
    }
}

__global__ void canny_edges_kernel(const uint8_t *cls, const int *parent, const uint8_t *on,
                                   long long d0, long long d1, long long n, int8_t *out) {
    const long long plane = d0 * d1;
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x) {
        const long long l = t % plane;
        int8_t e = 0;
        if (is_seed(cls, t, l, d0, d1)) e = 1;
        else if ((cls[t] & kWeak) && on[parent[t]]) e = 1;
        out[t] = e;
    }
}

unsigned grid_of(long long total, int threads) {
    const long long b = (total + threads - 1) / threads;
    return (unsigned)std::max(1LL, std::min(b, (long long)num_sms() * 32));
}

}  // namespace

Array canny_edges(const Array &img, bool otsu, float t1, float t2, bool is_fast) {
    const long long d0 = img.dims[0], d1 = img.dims[1];
    const long long plane = d0 * d1, nslices = img.dims[2] * img.dims[3];
    const long long n = plane * nslices;
    if (n > 0x7fffffffLL)
        AFGB_THROW(AF_ERR_NOT_SUPPORTED, "af_canny: more than 2^31 - 1 pixels");
    Array out = *create_array(b8, img.dims);
    if (n == 0) return out;

    // 1. float image, smoothed, derivatives
    const Array fimg = img.type == f32 ? (img.is_linear() ? img : make_dense(img)) : cast_array(img, f32);
    Array smt, gx, gy, mag, sup;
    {
        MemTag tag("edge-detector intermediates");
        smt = *create_array(f32, img.dims);
        gx = *create_array(f32, img.dims);
        gy = *create_array(f32, img.dims);
    }
    {
        static const float taps[5] = {-0.11021f, -0.23691f, -0.30576f, -0.23691f, -0.11021f};
        const dim_t fd[4] = {5, 1, 1, 1};
        Array filt = *create_array(f32, fd);
        AFGB_CUDA(cudaMemcpyAsync(filt.data(), taps, sizeof(taps), cudaMemcpyHostToDevice, stream()));
        ExactScope exact;
        launch_convolve2_sep(fimg, filt, filt, smt, false);
    }
    sobel_3x3(smt, gx, gy);

    // 2-3. magnitude, suppression (into smt and a new plane)
    mag = smt;  // the smoothed image is no longer needed
    canny_mag_kernel<<<grid_of(n, 256), 256, 0, stream()>>>(gx.ptr<float>(), gy.ptr<float>(), n,
                                                            is_fast ? 1 : 0, mag.ptr<float>());
    count_launch();
    AFGB_POST_LAUNCH("canny_mag_kernel");
    {
        MemTag tag("edge-detector intermediates");
        sup = *create_array(f32, img.dims);
    }
    canny_nms_kernel<<<grid_of(n, 256), 256, 0, stream()>>>(mag.ptr<float>(), gx.ptr<float>(),
                                                            gy.ptr<float>(), d0, d1, n,
                                                            sup.ptr<float>());
    count_launch();
    AFGB_POST_LAUNCH("canny_nms_kernel");

    // 4. maximum and minimum
    unsigned *mm = static_cast<unsigned *>(alloc_device(2 * sizeof(unsigned)));
    const unsigned init[2] = {0u, 0x7f800000u};
    AFGB_CUDA(cudaMemcpyAsync(mm, init, sizeof(init), cudaMemcpyHostToDevice, stream()));
    canny_minmax_kernel<<<grid_of(n, 256), 256, 0, stream()>>>(sup.ptr<float>(), n, mm);
    count_launch();
    AFGB_POST_LAUNCH("canny_minmax_kernel");
    unsigned host_mm[2];
    AFGB_CUDA(cudaMemcpyAsync(host_mm, mm, sizeof(host_mm), cudaMemcpyDeviceToHost, stream()));
    AFGB_CUDA(cudaStreamSynchronize(stream()));
    free_device(mm);
    float maxv, minv;
    std::memcpy(&maxv, &host_mm[0], 4);
    std::memcpy(&minv, &host_mm[1], 4);

    // 5. strong / weak classes (gx's buffer, no longer needed, holds them)
    uint8_t *cls = gx.ptr<uint8_t>();
    if (!otsu) {
        const float denom = maxv - minv;
        canny_classify_manual_kernel<<<grid_of(n, 256), 256, 0, stream()>>>(
            sup.ptr<float>(), n, minv, denom, t1, t2, cls);
        count_launch();
        AFGB_POST_LAUNCH("canny_classify_manual_kernel");
    } else {
        const unsigned nb = static_cast<unsigned>(maxv);
        // the reference's histogram and variance loop need two bins; below
        // that it indexes outside its arrays
        if (nb < 2)
            AFGB_THROW(AF_ERR_NOT_SUPPORTED,
                       "af_canny: the Otsu threshold needs a gradient maximum of at least 2");
        const float step = (float)(((double)maxv - 0.0) / (double)(float)nb);
        unsigned *hist;
        float *cum, *cprod, *thr;
        {
            MemTag tag("edge-detector intermediates");
            hist = static_cast<unsigned *>(alloc_device((size_t)nb * nslices * sizeof(unsigned)));
            cum = static_cast<float *>(alloc_device((size_t)nb * nslices * sizeof(float)));
            cprod = static_cast<float *>(alloc_device((size_t)nb * nslices * sizeof(float)));
            thr = static_cast<float *>(alloc_device((size_t)2 * nslices * sizeof(float)));
        }
        AFGB_CUDA(cudaMemsetAsync(hist, 0, (size_t)nb * nslices * sizeof(unsigned), stream()));
        canny_hist_kernel<<<grid_of(n, 256), 256, 0, stream()>>>(sup.ptr<float>(), plane, n, nb,
                                                                 step, hist);
        count_launch();
        AFGB_POST_LAUNCH("canny_hist_kernel");
        canny_otsu_kernel<<<(unsigned)nslices, 256, 0, stream()>>>(hist, nb, (float)plane, t1, cum,
                                                                  cprod, thr);
        count_launch();
        AFGB_POST_LAUNCH("canny_otsu_kernel");
        canny_classify_otsu_kernel<<<grid_of(n, 256), 256, 0, stream()>>>(sup.ptr<float>(), plane,
                                                                          n, thr, cls);
        count_launch();
        AFGB_POST_LAUNCH("canny_classify_otsu_kernel");
        free_device(thr);
        free_device(cprod);
        free_device(cum);
        free_device(hist);
    }

    // 6. hysteresis: components of weak pixels (labels in gy's buffer; the
    // marks in the suppressed plane's)
    int *parent = gy.ptr<int>();
    uint8_t *on = sup.ptr<uint8_t>();
    canny_uf_init_kernel<<<grid_of(n, 256), 256, 0, stream()>>>(parent, n);
    count_launch();
    AFGB_POST_LAUNCH("canny_uf_init_kernel");
    canny_uf_merge_kernel<<<grid_of(n, 256), 256, 0, stream()>>>(cls, d0, plane, n, parent);
    count_launch();
    AFGB_POST_LAUNCH("canny_uf_merge_kernel");
    canny_uf_flatten_kernel<<<grid_of(n, 256), 256, 0, stream()>>>(cls, n, parent);
    count_launch();
    AFGB_POST_LAUNCH("canny_uf_flatten_kernel");
    AFGB_CUDA(cudaMemsetAsync(on, 0, (size_t)n, stream()));
    canny_mark_kernel<<<grid_of(n, 256), 256, 0, stream()>>>(cls, parent, d0, d1, n, on);
    count_launch();
    AFGB_POST_LAUNCH("canny_mark_kernel");
    canny_edges_kernel<<<grid_of(n, 256), 256, 0, stream()>>>(cls, parent, on, d0, d1, n,
                                                              out.ptr<int8_t>());
    count_launch();
    AFGB_POST_LAUNCH("canny_edges_kernel");
    return out;
}

}  // namespace afgb
