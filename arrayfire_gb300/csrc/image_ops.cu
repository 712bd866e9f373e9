// Image-processing callers around the convolution path: af_gaussian_kernel
// (src/api/c/gaussian_kernel.cpp:29-99), af_dog (src/api/c/dog.cpp:30-85)
// and af_sobel_operator (src/api/c/sobel.cpp:30-87, CPU kernel
// src/backend/cpu/kernel/sobel.hpp:19-75).
//
// * gaussian_kernel: one block evaluates exp(-(((j - (cols-1)/2) / sc)^2 +
//   ((i - (rows-1)/2) / sr)^2) / 2) in float with the reference's operation
//   order (sc = sigma_c, or cols/4 when sigma_c <= 0; likewise sr), sums it and
//   normalises to unit sum;
// * dog: the input in the accumulator type convolved (direct kernels,
//   DEFAULT mode, NONE or LHS batch) with the (2r1+1)^2 and (2r2+1)^2
//   Gaussians, then subtracted -- one launch per convolution, one for the
//   difference;
// * sobel: 3x3 derivative stencils with reflect-101 borders, one thread per
//   pixel, each operation rounded separately in the reference's order (so
//   float results match the reference CPU kernel bit for bit).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "afgb_internal.hpp"
#include "conv_common.cuh"
#include "conv_direct.hpp"

namespace afgb {

namespace {

__global__ void gaussian_kernel_kernel(float *out, int rows, int cols, float rc, float cc,
                                       float sr, float sc) {
    __shared__ float part[256];
    const long long n = (long long)rows * cols;
    float local = 0.f;
    for (long long t = threadIdx.x; t < n; t += blockDim.x) {
        const int i = (int)(t % rows), j = (int)(t / rows);
        float tmp = 0.f;
        if (cols > 1) {
            float w = __fsub_rn((float)j, cc);
            w = __fdiv_rn(w, sc);
            w = __fmul_rn(w, w);
            tmp = __fadd_rn(w, tmp);
        }
        if (rows > 1) {
            float w = __fsub_rn((float)i, rc);
            w = __fdiv_rn(w, sr);
            w = __fmul_rn(w, w);
            tmp = __fadd_rn(w, tmp);
        }
        tmp = __fmul_rn(0.5f, tmp);
        tmp = __fsub_rn(0.f, tmp);
        tmp = expf(tmp);
        out[t] = tmp;
        local = __fadd_rn(local, tmp);
    }
    part[threadIdx.x] = local;
    __syncthreads();
    for (int w = blockDim.x / 2; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) part[threadIdx.x] = __fadd_rn(part[threadIdx.x], part[threadIdx.x + w]);
        __syncthreads();
    }
    const float norm = part[0];
    for (long long t = threadIdx.x; t < n; t += blockDim.x) out[t] = __fdiv_rn(out[t], norm);
}

// reflect-101 index |end - |end - idx|| (sobel.hpp:26-28); a size-1 dim
// reflects onto its only element
__device__ __forceinline__ long long reflect101(long long idx, long long end) {
    if (end == 0) return 0;
    const long long a = end - idx;
    return llabs(end - (a < 0 ? -a : a));
}

template <typename Ti, typename To>
__global__ void sobel_kernel(const Ti *__restrict__ in, To *__restrict__ dx, To *__restrict__ dy,
                             long long d0, long long d1, long long total) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < total;
         t += (long long)gridDim.x * blockDim.x) {
        const long long i = t % d0, r = t / d0, j = r % d1, s = r / d1;
        const Ti *p = in + s * d0 * d1;
        const long long im = reflect101(i - 1, d0 - 1), ip = reflect101(i + 1, d0 - 1);
        const long long jm = reflect101(j - 1, d1 - 1), jp = reflect101(j + 1, d1 - 1);
        const To NW = (To)p[jm * d0 + im], SW = (To)p[jm * d0 + ip];
        const To NE = (To)p[jp * d0 + im], SE = (To)p[jp * d0 + ip];
        const To N = (To)p[j * d0 + im], S = (To)p[j * d0 + ip];
        const To W = (To)p[jm * d0 + i], E = (To)p[jp * d0 + i];
        const To two = (To)2;
        // dx = SW + SE - (NW + NE) + 2 * (S - N); dy = NE + SE - (NW + SW) + 2 * (E - W)
        dx[t] = r_add(r_sub(r_add(SW, SE), r_add(NW, NE)), r_mul(two, r_sub(S, N)));
        dy[t] = r_add(r_sub(r_add(NE, SE), r_add(NW, SW)), r_mul(two, r_sub(E, W)));
    }
}

template <typename T>
__global__ void sub_inplace_kernel(T *a, const T *b, long long n) {
    for (long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x; t < n;
         t += (long long)gridDim.x * blockDim.x)
        a[t] = r_sub(a[t], b[t]);
}

unsigned grid_of(long long n) {
    return (unsigned)std::min<long long>(std::max<long long>((n + 255) / 256, 1),
                                         (long long)num_sms() * 32);
}

template <typename Ti, typename To>
void run_sobel(const Array &in, Array &dx, Array &dy) {
    const long long total = in.elements();
    if (total == 0) return;
    sobel_kernel<Ti, To><<<grid_of(total), 256, 0, stream()>>>(
        in.ptr<Ti>(), dx.ptr<To>(), dy.ptr<To>(), in.dims[0], in.dims[1], total);
    count_launch();
    AFGB_POST_LAUNCH("sobel_kernel");
}

}  // namespace

Array gaussian_kernel(int rows, int cols, double sigma_r, double sigma_c) {
    const dim_t d[4] = {rows, cols, 1, 1};
    Array out = *create_array(f32, d);
    if ((long long)rows * cols == 0) return out;
    const float rc = (float)((double)(rows - 1) / 2.0), cc = (float)((double)(cols - 1) / 2.0);
    const float sr = (float)(sigma_r > 0 ? sigma_r : 0.25 * rows);
    const float sc = (float)(sigma_c > 0 ? sigma_c : 0.25 * cols);
    gaussian_kernel_kernel<<<1, 256, 0, stream()>>>(out.ptr<float>(), rows, cols, rc, cc, sr, sc);
    count_launch();
    AFGB_POST_LAUNCH("gaussian_kernel_kernel");
    return out;
}

Array dog(const Array &in, int radius1, int radius2) {
    const af_dtype acc = in.type == f64 ? f64 : f32;
    Array g1 = cast_array(gaussian_kernel(2 * radius1 + 1, 2 * radius1 + 1, 0.0, 0.0), acc);
    Array g2 = cast_array(gaussian_kernel(2 * radius2 + 1, 2 * radius2 + 1, 0.0, 0.0), acc);
    Array x = cast_array(in, acc);
    const int kind = in.dims[2] > 1 ? BATCH_LHS : BATCH_NONE;
    Array s1 = *create_array(acc, in.dims);
    Array s2 = *create_array(acc, in.dims);
    launch_convolve_nd(x, g1, s1, kind, 2, false);
    launch_convolve_nd(x, g2, s2, kind, 2, false);
    const long long n = s1.elements();
    if (n) {
        if (acc == f64)
            sub_inplace_kernel<double><<<grid_of(n), 256, 0, stream()>>>(s1.ptr<double>(),
                                                                          s2.ptr<double>(), n);
        else
            sub_inplace_kernel<float><<<grid_of(n), 256, 0, stream()>>>(s1.ptr<float>(),
                                                                         s2.ptr<float>(), n);
        count_launch();
        AFGB_POST_LAUNCH("sub_inplace_kernel");
    }
    return s1;
}

void sobel_3x3(const Array &img, Array &dx, Array &dy) {
    Array in = img.is_linear() ? img : make_dense(img);
    switch (in.type) {
        case f32: run_sobel<float, float>(in, dx, dy); break;
        case f64: run_sobel<double, double>(in, dx, dy); break;
        case s32: run_sobel<int, int>(in, dx, dy); break;
        case u32: run_sobel<unsigned, int>(in, dx, dy); break;
        case s16: run_sobel<short, int>(in, dx, dy); break;
        case u16: run_sobel<unsigned short, int>(in, dx, dy); break;
        case b8:
        case s8: run_sobel<signed char, int>(in, dx, dy); break;
        case u8: run_sobel<unsigned char, int>(in, dx, dy); break;
        default: AFGB_TYPE_ERROR(1, in.type);
    }
}

}  // namespace afgb
