// Double-float (unevaluated FP32 pair) arithmetic for the polynomial
// variables: products, sums, square root and exponential to ~1e-14 relative
// on the FP32 pipe (FP64 arithmetic runs at a small fraction of the FP32
// rate on this part).  __host__ __device__ so that the same code can be
// checked against libm on the host.
#pragma once
#include <cmath>

#ifdef __CUDACC__
#define DFM_HD __host__ __device__ __forceinline__
#else
#define DFM_HD inline
#endif

namespace mbpol {
namespace dfm {

struct df {
    float h, l;
};

DFM_HD df two_sum(float a, float b) {
    const float s = a + b;
    const float bb = s - a;
    return {s, (a - (s - bb)) + (b - bb)};
}
DFM_HD df fast_two_sum(float a, float b) {  // |a| >= |b|
    const float s = a + b;
    return {s, b - (s - a)};
}
DFM_HD df add(df a, df b) {
    df s = two_sum(a.h, b.h);
    s.l += a.l + b.l;
    return fast_two_sum(s.h, s.l);
}
DFM_HD df mul(df a, df b) {
    const float p = a.h * b.h;
    float e = std::fma(a.h, b.h, -p);
    e = std::fma(a.h, b.l, e);
    e = std::fma(a.l, b.h, e);
    return fast_two_sum(p, e);
}
DFM_HD df mulf(df a, float b) {
    const float p = a.h * b;
    float e = std::fma(a.h, b, -p);
    e = std::fma(a.l, b, e);
    return fast_two_sum(p, e);
}
DFM_HD df sub(df a, df b) { return add(a, df{-b.h, -b.l}); }
// 1/a: one Newton step on the FP32 reciprocal with the residual in double-float
DFM_HD df recip(df a) {
    const float y = 1.f / a.h;
    const float e = std::fma(-a.h, y, 1.f) - a.l * y;
    return fast_two_sum(y, y * e);
}
// FP64 value -> double-float (host/device conversion of a double)
DFM_HD df from_double(double v) {
    const float h = (float)v;
    return {h, (float)(v - (double)h)};
}
// sqrt of a positive double-float: one Newton step on sqrtf with the
// residual formed exactly (Karp & Markstein)
DFM_HD df sqrt_df(df a) {
    const float y = std::sqrt(a.h);
    const float yy = y * y;
    const float r = std::fma(-y, y, a.h);  // a.h - y^2 exactly (to rounding of the sum)
    const float resid = (r + (yy - yy)) + a.l;
    return fast_two_sum(y, resid / (2.f * y));
}
// |a - b| of two double-float 3-vectors
DFM_HD df dist(const df (&a)[3], const df (&b)[3]) {
    const df x = sub(a[0], b[0]), y = sub(a[1], b[1]), z = sub(a[2], b[2]);
    return sqrt_df(add(add(mul(x, x), mul(y, y)), mul(z, z)));
}
// exp of a double-float argument, |a| < 80: a = n ln2 + f, |f| <= ln2/2,
// exp(f) by its Taylor series to degree 13 in double-float (Horner), then
// the exact scaling by 2^n.
DFM_HD df exp_df(df a) {
    const float n = std::nearbyint(a.h * 1.4426950408889634f);
    // ln2 in three parts (Cody & Waite); hi has 9 trailing zero bits, so
    // n * hi is exact for |n| < 512
    const float ln2_hi = 0.693145751953125f;
    const float ln2_mid = 1.428606765330187e-06f;
    const float ln2_lo = 5.495603971894525e-14f;
    const float t = a.h - n * ln2_hi;  // exact (Sterbenz)
    df f = two_sum(t, a.l);
    const float pm = -n * ln2_mid;
    f = add(f, df{pm, std::fma(-n, ln2_mid, -pm) - n * ln2_lo});
    // 1/k! as double-float constants (hi, lo), k = 13 .. 0
    const float ch[14] = {1.6059044372074283e-10f, 2.0876755879584152e-09f, 2.5052107943679403e-08f, 2.755731998149713e-07f, 2.7557318844628753e-06f, 2.4801587642286904e-05f, 0.00019841270113829523f, 0.0013888889225199819f, 0.008333333767950535f, 0.0416666679084301f, 0.1666666716337204f, 0.5f, 1.0f, 1.0f};
    const float cl[14] = {-5.352526511562726e-18f, 1.1082839809204342e-16f, 4.4176230446483665e-16f, -7.575112209051195e-15f, 3.793571224297229e-14f, -3.40699609366682e-13f, -2.725596874933456e-12f, -3.3631094437103215e-11f, -4.34617203337595e-10f, -1.2417634698280722e-09f, -4.967053879312289e-09f, 0.0f, 0.0f, 0.0f};
    df p = {ch[0], cl[0]};
    for (int k = 1; k < 14; ++k) {
        p = mul(p, f);
        p = add(p, df{ch[k], cl[k]});
    }
    return {std::ldexp(p.h, (int)n), std::ldexp(p.l, (int)n)};
}

}  // namespace dfm
}  // namespace mbpol
