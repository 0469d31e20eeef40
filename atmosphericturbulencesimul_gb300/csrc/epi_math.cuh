// epi_math.cuh -- angle and magnitude of the propagated field in the output
// epilogue of the last pass (the reference's atan2 / sqrt of the cropped
// complex amplitude, AtmosphericTurbulence.c:3418-3476), at a few FP32
// instructions per pixel.
//
// The output bar is far looser than the last bit: a phase error of 1e-7 rad
// is 3.5e-5 nm of OPD at 2.2 um, against frames that agree with the FP64
// oracle to about 2e-4 nm.  So the epilogue evaluates
//   * the angle by octant reduction and one odd polynomial:
//       with a = max(|x|, |y|), b = min(|x|, |y|), the octant angle atan(b/a)
//       in [0, pi/4] is atan(s) with s = b / a when b <= tan(pi/8) a, else
//       pi/4 + atan(s) with s = (b - a) / (b + a) (the arctan subtraction
//       formula), so |s| <= tan(pi/8) either way and one reciprocal serves
//       both; then pi/2 - angle (|y| > |x|), pi - angle (x < 0) and the sign
//       of y give the quadrant;
//       atan(s) = s + s^3 P(s^2) with P of degree 3, its coefficients a
//       least-squares fit of (atan(s) - s) / s^3 weighted by s^3 on 4,000
//       Chebyshev nodes of s^2 in [0, tan^2(pi/8)], computed in double and
//       rounded to float (largest error of the polynomial in float
//       arithmetic 2.2e-8 rad on that interval; the CPU emulation checks the
//       whole function against the double atan2);
//   * the magnitude with the approximate square root (relative error a few
//     units in the last place).
// Host-compilable for the CPU emulation.
#pragma once
#include "fft_core.cuh"

namespace atmwfs {

AW_HD float fdiv_approx(float a, float b)
{
#if defined(__CUDA_ARCH__)
    return __fdividef(a, b);
#else
    return a / b;
#endif
}

AW_HD float sqrt_approx(float q)
{
#if defined(__CUDA_ARCH__)
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(q));
    return r;
#else
    return sqrtf(q);
#endif
}

// atan2(y, x) for the output phase; atan2(+-0, +0) = +-0 and atan2(+-0, x < 0)
// = +-pi as the library function.
AW_HD float atan2_out(float y, float x)
{
    const float ax = fabsf(x), ay = fabsf(y);
    const float a = fmaxf(ax, ay), b = fminf(ax, ay);
    const bool hi = b > 0.414213562373095049f * a;
    const float num = hi ? b - a : b;
    const float den = hi ? b + a : a;
    const float s = den > 0.0f ? fdiv_approx(num, den) : 0.0f;
    const float u = s * s;
    float p = fmaf(u, 0.07882428169250488f, -0.13817109167575836f);
    p = fmaf(u, p, 0.19971036911010742f);
    p = fmaf(u, p, -0.3333272635936737f);
    float ang = fmaf(s * u, p, s);
    if (hi) ang += 0.785398163397448310f;
    if (ay > ax) ang = 1.57079632679489662f - ang;
    if (x < 0.0f) ang = 3.14159265358979324f - ang;
    return copysignf(ang, y);
}

}  // namespace atmwfs
