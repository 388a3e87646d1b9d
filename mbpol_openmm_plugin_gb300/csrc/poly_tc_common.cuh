// Device helpers shared by the two tensor-core kernels of the three-body
// polynomial (poly_tc.cu: mma.sync; poly_tc5.cu: tcgen05).
#pragma once

namespace mbpol {
namespace {

// double-float accumulation: (s.x + s.y) += a * b (TwoProd by FMA, TwoSum)
__device__ __forceinline__ void df_fma(float2& s, float a, float b) {
    const float p = __fmul_rn(a, b);
    const float pe = __fmaf_rn(a, b, -p);
    const float t = __fadd_rn(s.x, p);
    const float bb = __fsub_rn(t, s.x);
    const float e = __fadd_rn(__fsub_rn(s.x, __fsub_rn(t, bb)), __fsub_rn(p, bb));
    s.x = t;
    s.y = __fadd_rn(s.y, __fadd_rn(e, pe));
}

__device__ __forceinline__ void df_add(float2& s, float2 v) {
    const float t = __fadd_rn(s.x, v.x);
    const float bb = __fsub_rn(t, s.x);
    const float e = __fadd_rn(__fsub_rn(s.x, __fsub_rn(t, bb)), __fsub_rn(v.x, bb));
    s.x = t;
    s.y = __fadd_rn(s.y, __fadd_rn(e, v.y));
}

// per-unit exponent e: inputs up to m times the sampled bounds give
// |y'| <= 2^12 max(1, m)^2; scaled by 2^-e they stay below 2^15
__device__ __forceinline__ int unit_exp(float m) {
    if (!(m > 1.f)) return 0;
    if (!(m < 1e30f)) return 100;
    return max(0, 2 * ilogbf(m) - 1);
}

// 2^k as a float for k in [-126, 127]
__device__ __forceinline__ float exp2i(int k) {
    k = max(-126, min(127, k));
    return __int_as_float((k + 127) << 23);
}

}  // namespace
}  // namespace mbpol
