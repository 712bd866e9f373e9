// Kernel parameter blocks shared by the direct-convolution translation units.
#pragma once

#include "conv_common.cuh"

namespace afgb {

// One direct convolution: signal, filter and output views plus the per-batch
// steps of src/backend/cpu/kernel/convolve.hpp:147-180.
struct DirectParams {
    const void *sig;
    const void *filt;
    void *out;
    int rank;
    int expand;
    long long sd[4], ss[4];
    long long od[4], os[4];
    long long fd[4], fs[4];
    long long in_step[4], out_step[4], filt_step[4];
    long long batch[4];
    long long nbatch;
};

struct BatchOff {
    long long in, out, filt;
};

__device__ __forceinline__ BatchOff batch_offsets(const DirectParams &p, long long b) {
    long long b1 = b % p.batch[1];
    long long r = b / p.batch[1];
    long long b2 = r % p.batch[2];
    long long b3 = r / p.batch[2];
    BatchOff o;
    o.in = b1 * p.in_step[1] + b2 * p.in_step[2] + b3 * p.in_step[3];
    o.out = b1 * p.out_step[1] + b2 * p.out_step[2] + b3 * p.out_step[3];
    o.filt = b1 * p.filt_step[1] + b2 * p.filt_step[2] + b3 * p.filt_step[3];
    return o;
}


// The fused separable kernel on dense images (TMA path)
struct SepTmaParams {
    const float *cf, *rf;  // taps (float; converted to the input type in-kernel)
    void *out;
    long long od0, od1, out_slice;
    long long sd1;  // signal height (rows outside it read as zero in the row pass)
    long long tiles_x, tiles_y, ntiles;
};

}  // namespace afgb
