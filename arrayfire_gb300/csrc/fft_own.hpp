// Transforms of the frequency-domain convolution (fft_own.cu): mixed-radix
// Stockham FFTs for lengths 2^a 3^b, unnormalised.
#pragma once

#include <cstddef>

namespace afgb {

struct FftDiv {
    unsigned d, m, s;  // n / d == (umulhi(n, m) + n) >> s for n < 2^31
};
struct FftPlan {
    int n, nst;
    int rad[32];         // radices (8, 4, 2, 9, 3) in stage order
    FftDiv mdiv[32];     // n / radix of each stage
    FftDiv nsdiv[32];    // product of the earlier radices of each stage
    int twoff[32];       // offset of each stage's twiddles in the plan's table
};

// whether a length runs on these kernels: 2^a 3^b (an even real row length
// whose half is 2^a 3^b when real_rows) whose two shared-memory buffers of
// `csize`-byte complex values fit one block
bool fft_own_len_ok(long long n, bool real_rows, size_t csize);

// rows contiguous real rows of even length n0 -> rows x (n0/2 + 1) bins
template <typename R, typename C>
void fft_real_forward(const R *in, C *out, long long n0, long long rows);
// the inverse: rows x (n0/2 + 1) Hermitian bins -> rows real rows of n0
template <typename R, typename C>
void fft_real_inverse(const C *in, R *out, long long n0, long long rows);
// complex transforms of length n along the middle axis of an
// (inner, n, outer) layout (inner fastest), in place
template <typename C>
void fft_axis(C *data, long long n, long long inner, long long outer, bool inverse);

}  // namespace afgb
