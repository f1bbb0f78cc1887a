// Double-float (FP32 pair) arithmetic for device code: about 48 significant bits on the
// FP32 pipe, which on GB300 issues 64 times the FP64 rate (Dekker 1971; TwoSum / TwoProd
// via FMA).  Shared by the block SVD kernels.
#pragma once

#include <cuda_runtime.h>

namespace tn {
namespace dfa {

struct __align__(8) df2 {
    float hi, lo;
};
__device__ __forceinline__ df2 fast_two_sum(float a, float b) {
    const float s = a + b;
    return df2{s, b - (s - a)};
}
__device__ __forceinline__ df2 df_add(df2 a, df2 b) {
    const float s = a.hi + b.hi;
    const float bb = s - a.hi;
    float e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    return fast_two_sum(s, e);
}
__device__ __forceinline__ df2 df_neg(df2 a) { return df2{-a.hi, -a.lo}; }
__device__ __forceinline__ df2 df_mul(df2 a, df2 b) {
    const float p = a.hi * b.hi;
    float e = fmaf(a.hi, b.hi, -p);
    e = fmaf(a.hi, b.lo, e);
    e = fmaf(a.lo, b.hi, e);
    return fast_two_sum(p, e);
}
__device__ __forceinline__ df2 df_fma(df2 a, df2 b, df2 c) { return df_add(df_mul(a, b), c); }
__device__ __forceinline__ df2 df_shfl_xor(df2 a, int o) {
    return df2{__shfl_xor_sync(0xffffffffu, a.hi, o), __shfl_xor_sync(0xffffffffu, a.lo, o)};
}
// x * 2^k for an exact power of two (no rounding)
__device__ __forceinline__ df2 df_ldexp(df2 a, int k) { return df2{ldexpf(a.hi, k), ldexpf(a.lo, k)}; }
__device__ __forceinline__ df2 df_from_double(double x) {
    const float h = __double2float_rn(x);
    return df2{h, __double2float_rn(x - double(h))};
}
__device__ __forceinline__ double df_to_double(df2 a) { return double(a.hi) + double(a.lo); }
// 1 / sqrt(u) in double-float: FP32 estimate + one Newton step.  u y0 is formed before the
// second factor y0 so that no intermediate leaves the FP32 range for tiny u (y0^2 would
// overflow below u ~ 1e-38).
__device__ __forceinline__ df2 df_rsqrt(df2 u) {
    const df2 y0{rsqrtf(u.hi), 0.f};
    const df2 e = df_add(df2{1.f, 0.f}, df_neg(df_mul(df_mul(u, y0), y0)));
    return df_add(y0, df_mul(df_mul(y0, e), df2{0.5f, 0.f}));
}

__device__ __forceinline__ df2 df_recip(df2 b) {
    const df2 y0{1.f / b.hi, 0.f};
    const df2 e = df_add(df2{1.f, 0.f}, df_neg(df_mul(b, y0)));
    return df_add(y0, df_mul(y0, e));
}
__device__ __forceinline__ df2 df_sqrt(df2 x) {
    if (!(x.hi > 0.f)) return df2{0.f, 0.f};
    return df_mul(x, df_rsqrt(x));
}

}  // namespace dfa
}  // namespace tn
