// Element types, accumulation rules and conversions of the direct
// convolutions, written once for every kernel.
//
// The arithmetic rules follow the reference CPU backend
// (src/backend/cpu/kernel/convolve.hpp):
//   * every integer input accumulates in float (accT table in
//     src/api/c/convolve.cpp:172-206); f64 in double, complex in complex;
//   * one2one_{1,2,3}d: `accum += AccT(s_val * fptr[f])` — the signal value is
//     converted to AccT, multiplied, rounded, then added (no fused multiply-add
//     in the reference build);
//   * the separable kernel converts the *tap* to the input type first
//     (`InT f_val = fptr[f]`, convolve.hpp:233) and multiplies in the input
//     type's C++ arithmetic (integer promotion for narrow types);
//   * the result is written back as `InT(accum)`.  C++ leaves an out-of-range
//     float->integer conversion undefined; this library defines it as
//     truncation toward zero, saturated to the type's range, NaN -> 0.
#pragma once

#include <cuda_runtime.h>
#include <cuda_fp16.h>

#include <cstdint>

namespace afgb {

struct cf32 {
    float x, y;
};
struct cf64 {
    double x, y;
};

// accumulator type for each input type
template <typename T> struct AccOf { using type = float; };
template <> struct AccOf<double> { using type = double; };
template <> struct AccOf<cf32> { using type = cf32; };
template <> struct AccOf<cf64> { using type = cf64; };

template <typename T> struct IsInt { static constexpr bool value = true; };
template <> struct IsInt<float> { static constexpr bool value = false; };
template <> struct IsInt<double> { static constexpr bool value = false; };
template <> struct IsInt<cf32> { static constexpr bool value = false; };
template <> struct IsInt<cf64> { static constexpr bool value = false; };

// ---- value -> accumulator conversion (the usual arithmetic conversions)
__device__ __forceinline__ float to_acc(float v, float) { return v; }
__device__ __forceinline__ double to_acc(double v, double) { return v; }
__device__ __forceinline__ cf32 to_acc(cf32 v, cf32) { return v; }
__device__ __forceinline__ cf64 to_acc(cf64 v, cf64) { return v; }
__device__ __forceinline__ float to_acc(uint8_t v, float) { return (float)v; }
__device__ __forceinline__ float to_acc(int8_t v, float) { return (float)v; }
__device__ __forceinline__ float to_acc(uint16_t v, float) { return (float)v; }
__device__ __forceinline__ float to_acc(int16_t v, float) { return (float)v; }
__device__ __forceinline__ float to_acc(int32_t v, float) { return __int2float_rn(v); }
__device__ __forceinline__ float to_acc(uint32_t v, float) { return __uint2float_rn(v); }
__device__ __forceinline__ float to_acc(long long v, float) { return __ll2float_rn(v); }
__device__ __forceinline__ float to_acc(unsigned long long v, float) { return __ull2float_rn(v); }

// separately rounded arithmetic for floating types, plain for integers
template <typename T> __device__ __forceinline__ T r_add(T a, T b) { return a + b; }
template <typename T> __device__ __forceinline__ T r_sub(T a, T b) { return a - b; }
template <typename T> __device__ __forceinline__ T r_mul(T a, T b) { return a * b; }
template <> __device__ __forceinline__ float r_add(float a, float b) { return __fadd_rn(a, b); }
template <> __device__ __forceinline__ float r_sub(float a, float b) { return __fsub_rn(a, b); }
template <> __device__ __forceinline__ float r_mul(float a, float b) { return __fmul_rn(a, b); }
template <> __device__ __forceinline__ double r_add(double a, double b) { return __dadd_rn(a, b); }
template <> __device__ __forceinline__ double r_sub(double a, double b) { return __dsub_rn(a, b); }
template <> __device__ __forceinline__ double r_mul(double a, double b) { return __dmul_rn(a, b); }

// ---- accumulate one product: acc + fl(s*f), either exactly in the
// reference's order (separate rounding of product and sum) or fused.
template <bool EXACT>
__device__ __forceinline__ float mac(float acc, float s, float f) {
    if (EXACT) return __fadd_rn(acc, __fmul_rn(s, f));
    return __fmaf_rn(s, f, acc);
}
template <bool EXACT>
__device__ __forceinline__ double mac(double acc, double s, double f) {
    if (EXACT) return __dadd_rn(acc, __dmul_rn(s, f));
    return __fma_rn(s, f, acc);
}
// complex: (a+bi)(c+di) = (ac-bd) + (ad+bc)i, each product and sum rounded
// (the finite-value branch of GCC's complex multiply).
template <bool EXACT>
__device__ __forceinline__ cf32 mac(cf32 acc, cf32 s, cf32 f) {
    float re = __fsub_rn(__fmul_rn(s.x, f.x), __fmul_rn(s.y, f.y));
    float im = __fadd_rn(__fmul_rn(s.x, f.y), __fmul_rn(s.y, f.x));
    return cf32{__fadd_rn(acc.x, re), __fadd_rn(acc.y, im)};
}
template <bool EXACT>
__device__ __forceinline__ cf64 mac(cf64 acc, cf64 s, cf64 f) {
    double re = __dsub_rn(__dmul_rn(s.x, f.x), __dmul_rn(s.y, f.y));
    double im = __dadd_rn(__dmul_rn(s.x, f.y), __dmul_rn(s.y, f.x));
    return cf64{__dadd_rn(acc.x, re), __dadd_rn(acc.y, im)};
}

template <typename A> __device__ __forceinline__ A acc_zero();
template <> __device__ __forceinline__ float acc_zero<float>() { return 0.0f; }
template <> __device__ __forceinline__ double acc_zero<double>() { return 0.0; }
template <> __device__ __forceinline__ cf32 acc_zero<cf32>() { return cf32{0.f, 0.f}; }
template <> __device__ __forceinline__ cf64 acc_zero<cf64>() { return cf64{0.0, 0.0}; }

// ---- accumulator -> output type
template <typename T> __device__ __forceinline__ T from_acc(float a);
template <> __device__ __forceinline__ float from_acc<float>(float a) { return a; }

// truncate toward zero and saturate in single precision (the bounds of the
// 8/16-bit types are exact floats); NaN -> 0
__device__ __forceinline__ float trunc_sat_f(float a, float lo, float hi) {
    if (a != a) return 0.0f;
    return fminf(fmaxf(truncf(a), lo), hi);
}
template <> __device__ __forceinline__ uint8_t from_acc<uint8_t>(float a) {
    return (uint8_t)trunc_sat_f(a, 0.0f, 255.0f);
}
template <> __device__ __forceinline__ int8_t from_acc<int8_t>(float a) {
    return (int8_t)trunc_sat_f(a, -128.0f, 127.0f);
}
template <> __device__ __forceinline__ uint16_t from_acc<uint16_t>(float a) {
    return (uint16_t)trunc_sat_f(a, 0.0f, 65535.0f);
}
template <> __device__ __forceinline__ int16_t from_acc<int16_t>(float a) {
    return (int16_t)trunc_sat_f(a, -32768.0f, 32767.0f);
}
// 32-bit: cvt.rzi saturates to the destination range; NaN -> 0
template <> __device__ __forceinline__ int32_t from_acc<int32_t>(float a) {
    return (a != a) ? 0 : __float2int_rz(a);
}
template <> __device__ __forceinline__ uint32_t from_acc<uint32_t>(float a) {
    return (a != a) ? 0u : __float2uint_rz(a);
}
template <> __device__ __forceinline__ long long from_acc<long long>(float a) {
    if (a != a) return 0;
    if (a >= 9223372036854775807.0f) return 9223372036854775807LL;
    if (a <= -9223372036854775808.0f) return (-9223372036854775807LL - 1);
    return (long long)a;  // cvt.rzi, in range
}
template <> __device__ __forceinline__ unsigned long long from_acc<unsigned long long>(float a) {
    if (a != a || a <= 0.0f) return 0ull;
    if (a >= 18446744073709551615.0f) return 18446744073709551615ull;
    return (unsigned long long)a;
}
template <typename T> __device__ __forceinline__ T from_acc_d(double a);
template <> __device__ __forceinline__ double from_acc_d<double>(double a) { return a; }
__device__ __forceinline__ double from_acc_any(double a, double) { return a; }
__device__ __forceinline__ cf32 from_acc_any(cf32 a, cf32) { return a; }
__device__ __forceinline__ cf64 from_acc_any(cf64 a, cf64) { return a; }
template <typename T>
__device__ __forceinline__ T from_acc_any(float a, T) { return from_acc<T>(a); }

// ---- accumulator -> input type for taps (separable kernel, CPU semantics)
template <typename T> __device__ __forceinline__ T tap_to_input(float f) { return from_acc<T>(f); }

// ---- C++ integer multiply in the promoted type, then converted to float
// (`AccT(s_val * f_val)` with both operands of the input type).  Signed
// overflow is undefined in C++; this library wraps modulo 2^32 / 2^64.
__device__ __forceinline__ float int_prod(uint8_t a, uint8_t b) { return (float)((int)a * (int)b); }
__device__ __forceinline__ float int_prod(int8_t a, int8_t b) { return (float)((int)a * (int)b); }
__device__ __forceinline__ float int_prod(uint16_t a, uint16_t b) {
    return __int2float_rn((int)((unsigned)a * (unsigned)b));
}
__device__ __forceinline__ float int_prod(int16_t a, int16_t b) { return __int2float_rn((int)a * (int)b); }
__device__ __forceinline__ float int_prod(int32_t a, int32_t b) {
    return __int2float_rn((int32_t)((uint32_t)a * (uint32_t)b));
}
__device__ __forceinline__ float int_prod(uint32_t a, uint32_t b) { return __uint2float_rn(a * b); }
__device__ __forceinline__ float int_prod(long long a, long long b) {
    return __ll2float_rn((long long)((unsigned long long)a * (unsigned long long)b));
}
__device__ __forceinline__ float int_prod(unsigned long long a, unsigned long long b) {
    return __ull2float_rn(a * b);
}

// n / d for 0 <= n < 2^31 by multiply-high (Granlund and Montgomery,
// "Division by invariant integers using multiplication", PLDI 1994, with
// l = ceil(log2 d) and m = floor(2^32 (2^l - d) / d) + 1: q = (mulhi(n, m) + n) >> l;
// n < 2^31 keeps the sum within 32 bits)
struct FastDiv {
    uint32_t d, m, s;
};
inline FastDiv make_fastdiv(uint32_t d) {
    uint32_t l = 0;
    while ((1ull << l) < d) ++l;
    const uint64_t m = ((1ull << 32) * ((1ull << l) - d)) / d + 1;
    return FastDiv{d, (uint32_t)m, l};
}
__device__ __forceinline__ uint32_t fdiv(uint32_t n, const FastDiv &f) {
    return (__umulhi(n, f.m) + n) >> f.s;
}

}  // namespace afgb
