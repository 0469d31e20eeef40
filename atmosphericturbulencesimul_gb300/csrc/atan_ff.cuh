// atan_ff.cuh -- atan2 of two floats, rounded to float, in FP32 arithmetic
// only.  The science unwrap takes the angle of each bin's phasor sum as
// (float)atan2((double)im, (double)re) (AtmosphericTurbulence.c computes the
// bin peaks in double); on GB300 a double atan2 per bin keeps the FP64 pipe
// of the SM busy for the whole unwrap.  Here the angle is evaluated in
// float-float (pairs hi + lo of floats, about 46 significant bits) and
// rounded once at the end, so the float result equals the correctly rounded
// angle except when the exact angle lies within about 2^-46 (relative) of a
// midpoint between two floats.
//
// Method: table-driven argument reduction (P. T. P. Tang, "Table-lookup
// algorithms for elementary functions and their error analysis", ARITH 10,
// 1991) with the arctan addition formula: with q = min(|x|,|y|) /
// max(|x|,|y|) in [0, 1] and the nearest table point c = k / 1024,
//     atan(q) = atan(c) + atan(u),  u = (q - c) / (1 + q c),  |u| <= 2^-11,
// and atan(u) = u - u^3/3 + u^5/5 (the next term is below 2^-56 |u|).  The
// table holds atan(k / 1024), k = 0..1024, as float-float pairs computed on
// the host in double.  The quadrant follows from pi/2 - angle (|y| > |x|),
// pi - angle (x < 0) and the sign of y.
//
// Host-compilable so that the CPU emulation checks it against the double
// atan2; every rounding step is an explicit intrinsic on the device so that
// no multiply is contracted into an add of an error-free transformation.
#pragma once
#include "fft_core.cuh"

namespace atmwfs {

constexpr int kAtanTabN = 1024;  // table points k / 1024, k = 0 .. 1024

constexpr double kPiD = 3.14159265358979323846;
constexpr float kPiH = (float)kPiD;
constexpr float kPiL = (float)(kPiD - (double)kPiH);
constexpr float kPi2H = (float)(kPiD / 2);
constexpr float kPi2L = (float)(kPiD / 2 - (double)kPi2H);

AW_HD float ff_add(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fadd_rn(a, b);
#else
    return a + b;
#endif
}
AW_HD float ff_sub(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fsub_rn(a, b);
#else
    return a - b;
#endif
}
AW_HD float ff_mul(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fmul_rn(a, b);
#else
    return a * b;
#endif
}
AW_HD float ff_div(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fdiv_rn(a, b);
#else
    return a / b;
#endif
}
AW_HD float ff_fma(float a, float b, float c)
{
#if defined(__CUDA_ARCH__)
    return __fmaf_rn(a, b, c);
#else
    return std::fma(a, b, c);
#endif
}

AW_HD bool ff_signbit(float v)
{
#if defined(__CUDA_ARCH__)
    return (__float_as_uint(v) >> 31) != 0;
#else
    return std::signbit(v);
#endif
}
AW_HD float ff_rint(float v)
{
#if defined(__CUDA_ARCH__)
    return rintf(v);
#else
    return std::rint(v);
#endif
}
// the double function, for infinities and NaN only
AW_HD float atan2_via_double(float y, float x)
{
#if defined(__CUDA_ARCH__)
    return (float)atan2((double)y, (double)x);
#else
    return (float)std::atan2((double)y, (double)x);
#endif
}

// s + e = a + b exactly (Knuth's two-sum)
AW_HD void ff_two_sum(float a, float b, float& s, float& e)
{
    s = ff_add(a, b);
    const float bp = ff_sub(s, a);
    e = ff_add(ff_sub(a, ff_sub(s, bp)), ff_sub(b, bp));
}

// s + e = a + b exactly when |a| >= |b| (Dekker's fast two-sum)
AW_HD void ff_fast_two_sum(float a, float b, float& s, float& e)
{
    s = ff_add(a, b);
    e = ff_sub(b, ff_sub(s, a));
}

// (ah + al) - (bh + bl), normalised
AW_HD void ff_sub2(float ah, float al, float bh, float bl, float& rh, float& rl)
{
    float s, e;
    ff_two_sum(ah, -bh, s, e);
    e = ff_add(e, ff_sub(al, bl));
    ff_fast_two_sum(s, e, rh, rl);
}

// atan(k / 1024) as (hi, lo) floats, k = 0 .. 1024 (host, double atan)
inline void atan_table_host(float2* tab)
{
    for (int k = 0; k <= kAtanTabN; k++) {
        const double t = std::atan((double)k / kAtanTabN);
        const float h = (float)t;
        tab[k] = make_float2(h, (float)(t - (double)h));
    }
}

// atan2(y, x) rounded to float; tab from atan_table_host.  Signed zeros and
// the axes follow atan2; infinities and NaN take the double function.
AW_HD float atan2_ff(float y, float x, const float2* tab)
{
    const float ax = ff_signbit(x) ? -x : x, ay = ff_signbit(y) ? -y : y;
    if (!(ax <= 3.4028234663852886e38f && ay <= 3.4028234663852886e38f)) return atan2_via_double(y, x);
    if (ax == 0.0f && ay == 0.0f) {
        const float r = ff_signbit(x) ? kPiH : 0.0f;
        return ff_signbit(y) ? -r : r;
    }
    const bool swap = ay > ax;
    const float num = swap ? ax : ay, den = swap ? ay : ax;
    // q = num / den = qh + ql (the remainder of a rounded quotient is exact)
    const float qh = ff_div(num, den);
    float th = qh, tl = 0.0f;
    if (qh >= 9.094947e-13f) {  // 2^-40; below it atan(q) rounds as q (q^3/3 < 2^-80 q)
        const float ql = ff_div(ff_fma(-qh, den, num), den);
        // nearest table point c = k / 1024; qh - c is exact (Sterbenz)
        const int k = (int)ff_rint(ff_mul(qh, (float)kAtanTabN));
        const float c = ff_mul((float)k, 1.0f / kAtanTabN);
        float nh, nl;
        ff_two_sum(ff_sub(qh, c), ql, nh, nl);
        // 1 + q c = mh + ml
        const float p = ff_mul(qh, c);
        const float pe = ff_fma(qh, c, -p);
        float mh, me;
        ff_two_sum(1.0f, p, mh, me);
        const float ml = ff_add(me, ff_add(pe, ff_mul(ql, c)));
        // u = (nh + nl) / (mh + ml) = uh + ul
        const float uh = ff_div(nh, mh);
        const float t = ff_fma(-uh, mh, nh);
        const float ul = ff_div(ff_sub(ff_add(t, nl), ff_mul(uh, ml)), mh);
        // atan(u) - u = u^3 (-1/3 + u^2/5) - u^2 ul  (to 2^-46 |u|)
        const float u2 = ff_mul(uh, uh);
        const float corr = ff_sub(ff_mul(ff_mul(uh, u2), ff_fma(u2, 0.2f, -1.0f / 3.0f)), ff_mul(u2, ul));
        const float2 T = tab[k];
        ff_two_sum(T.x, uh, th, tl);
        tl = ff_add(tl, ff_add(T.y, ff_add(ul, corr)));
        ff_fast_two_sum(th, tl, th, tl);
    }
    if (swap) ff_sub2(kPi2H, kPi2L, th, tl, th, tl);
    if (x < 0.0f) ff_sub2(kPiH, kPiL, th, tl, th, tl);
    const float r = ff_add(th, tl);
    return ff_signbit(y) ? -r : r;
}

}  // namespace atmwfs
