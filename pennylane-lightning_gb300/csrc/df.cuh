// Double-float ("df") arithmetic: a value is hi + lo with two floats,
// |lo| <= ulp(hi) / 2, about 48 significant bits.
//
// Why: GB300 executes FP64 at 1/64 of its FP32 rate (measured 0.63 T DFMA/s
// against 34 T FFMA/s), so complex128 gate arithmetic is FP64-bound.  The
// fused complex128 passes instead run on the FP32 pipe in df arithmetic,
// built from the error-free transformations TwoSum (Knuth) and TwoProd with
// FMA (the Dekker / Shewchuk / QD-library constructions); the per-operation
// relative error is about 2^-47, far inside the 1e-12 parity tolerance
// after thousands of gates.  Conversions between double and df are also
// slow on GB300 (f64<->f32 converts run at FP64 rate), so a double is split
// with integer operations and a register stays in df form between the
// passes of one program; only its first pass reads doubles and only its last
// pass writes them.
//
// Range: |value| < 2^128.  Values below 2^-126 in magnitude become 0, and
// the low part is dropped below 2^-74 (absolute errors far below the
// tolerance of normalised states); larger magnitudes and infinities become
// +-infinity, and NaN stays NaN.
#pragma once

#include "plgb_common.cuh"

#include <type_traits>

namespace plgb {

struct df {
    float hi, lo;
    df() = default; // trivial: df can live in __shared__ arrays
    __host__ __device__ constexpr df(float h) : hi(h), lo(0.f) {}
    __host__ __device__ constexpr df(float h, float l) : hi(h), lo(l) {}
    // exact split up to the last 5 of 53 bits (device: one f64 conversion
    // each; meant for per-tile constants, not per-amplitude values)
    __host__ __device__ explicit df(double x) {
        hi = static_cast<float>(x);
        lo = static_cast<float>(x - static_cast<double>(hi));
    }
    __host__ __device__ explicit operator double() const {
        return static_cast<double>(hi) + static_cast<double>(lo);
    }
};

#if defined(__CUDACC__)
__device__ __forceinline__ df df_quick_two_sum(float a, float b) { // |a| >= |b|
    const float s = __fadd_rn(a, b);
    return df{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ df df_two_sum(float a, float b) {
    const float s = __fadd_rn(a, b);
    const float bb = __fsub_rn(s, a);
    return df{s, __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb))};
}
__device__ __forceinline__ df operator+(df a, df b) {
    const df s = df_two_sum(a.hi, b.hi);
    return df_quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, b.lo)));
}
__device__ __forceinline__ df operator-(df a) { return df{-a.hi, -a.lo}; }
__device__ __forceinline__ df operator-(df a, df b) { return a + (-b); }
__device__ __forceinline__ df operator*(df a, df b) {
    const float p = __fmul_rn(a.hi, b.hi);
    float e = __fmaf_rn(a.hi, b.hi, -p);
    e = __fmaf_rn(a.hi, b.lo, e);
    e = __fmaf_rn(a.lo, b.hi, e);
    return df_quick_two_sum(p, e);
}
__device__ __forceinline__ bool operator==(df a, df b) { return a.hi == b.hi && a.lo == b.lo; }
// a + b * c with one renormalisation: the product's error terms go straight
// into the low sum (15 FP32 instructions instead of 18 for * then +).
__device__ __forceinline__ df df_fma(df a, df b, df c) {
    const float p = __fmul_rn(b.hi, c.hi);
    float e = __fmaf_rn(b.hi, c.hi, -p);
    e = __fmaf_rn(b.hi, c.lo, e);
    e = __fmaf_rn(b.lo, c.hi, e);
    const df s = df_two_sum(a.hi, p);
    return df_quick_two_sum(s.hi, __fadd_rn(s.lo, __fadd_rn(a.lo, e)));
}
// complex products and acc + a * b as chains of df_fma
__device__ __forceinline__ cx<df> operator*(cx<df> a, cx<df> b) {
    return cx<df>{df_fma(a.x * b.x, -a.y, b.y), df_fma(a.x * b.y, a.y, b.x)};
}
__device__ __forceinline__ cx<df> cfma(cx<df> a, cx<df> b, cx<df> acc) {
    return cx<df>{df_fma(df_fma(acc.x, a.x, b.x), -a.y, b.y), df_fma(df_fma(acc.y, a.x, b.y), a.y, b.x)};
}

// double -> df with integer operations only (no f64 instruction)
__device__ __forceinline__ df df_from_bits(double x) {
    const unsigned long long u = static_cast<unsigned long long>(__double_as_longlong(x));
    const unsigned hw = static_cast<unsigned>(u >> 32), lw = static_cast<unsigned>(u);
    const unsigned sign = hw & 0x80000000u;
    const int e = static_cast<int>((hw >> 20) & 0x7ffu);
    if (e < 897) { // below the float normal range (or zero)
        return df{0.f, 0.f};
    }
    if (e > 1150) { // |x| >= 2^128 (beyond the float range), infinity or NaN
        const bool nan = e == 2047 && ((hw & 0xfffffu) | lw) != 0u;
        return df{__int_as_float(static_cast<int>(nan ? 0x7fc00000u : (sign | 0x7f800000u))), 0.f};
    }
    // hi: the top 24 significant bits, truncated
    const unsigned m23 = ((hw & 0xfffffu) << 3) | (lw >> 29);
    const float hi = __int_as_float(static_cast<int>(sign | (static_cast<unsigned>(e - 896) << 23) | m23));
    // lo: the remaining 29 bits times 2^(e - 1075), same sign
    float lo = 0.f;
    if (e >= 949) {
        const unsigned r = lw & 0x1fffffffu;
        const float scale = __int_as_float(static_cast<int>(sign | (static_cast<unsigned>(e - 948) << 23)));
        lo = __fmul_rn(__uint2float_rn(r), scale);
    }
    return df_quick_two_sum(hi, lo);
}
__device__ __forceinline__ double df_to_double(df v) {
    return __dadd_rn(static_cast<double>(v.hi), static_cast<double>(v.lo));
}

// Register <-> memory formats: complex64 / complex128 registers compute in
// their own type; a df register reads doubles (first pass of a program) or
// df, and writes df or doubles (last pass).
template <class T, class S> __device__ __forceinline__ cx<T> ld_conv(const cx<S> &v) {
    if constexpr (std::is_same_v<T, df> && std::is_same_v<S, double>) {
        return cx<df>{df_from_bits(v.x), df_from_bits(v.y)};
    } else {
        return v;
    }
}
template <class S, class T> __device__ __forceinline__ cx<S> st_conv(const cx<T> &v) {
    if constexpr (std::is_same_v<T, df> && std::is_same_v<S, double>) {
        return cx<double>{df_to_double(v.x), df_to_double(v.y)};
    } else {
        return v;
    }
}
// a per-pass double constant in the register's type
template <class T> __device__ __forceinline__ T from_double(double x) {
    if constexpr (std::is_same_v<T, df>) {
        return df(x);
    } else {
        return static_cast<T>(x);
    }
}
#endif

} // namespace plgb
