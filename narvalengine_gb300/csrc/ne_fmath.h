// Portable single-precision elementary functions with identical results on the
// host (g++, -ffp-contract=off) and on sm_103a (nvcc, -fmad=false, IEEE div/sqrt).
//
// The reference renderer calls libm (std::log, std::sin, std::cos, std::acos,
// std::pow) inside its integrator (utils/Math.h:454,503-506, core/Microfacet.cpp:44-49,
// core/BSDF.h:155, materials/Medium.h:110-111, materials/GridMedia.cpp:56,82).
// CUDA's and glibc's versions of those functions round differently, so a CPU
// restatement and the GPU kernels that called them would draw different
// directions for the same random numbers and paths would diverge. Both sides
// therefore call these functions instead. Each one is built only from IEEE
// +, -, *, / and sqrt, so the same source produces the same bits on both sides as
// long as no multiply-add is contracted.
//
// Methods (all from the published literature, coefficients derived here):
//  * log: x = 2^k m, m in [sqrt(1/2), sqrt(2)); log(m) = 2 atanh(s), s = (m-1)/(m+1),
//    odd Taylor series of atanh (5 terms; |s| <= 0.1716); k ln2 added with a two-part
//    Cody-Waite constant (Cody & Waite, "Software Manual for the Elementary Functions", 1980).
//  * exp: k = round(x/ln2), r = x - k ln2 (two-part constant), Taylor series of e^r to r^7,
//    scaled by 2^k through the exponent field.
//  * sin/cos: k = round(x 2/pi), r = x - k pi/2 with a three-part Cody-Waite constant,
//    Taylor series of sin (to r^9) and cos (to r^10) on |r| <= pi/4, quadrant selected by k.
//    Accurate for |x| < 2^12 pi/2, which covers every angle the integrator forms.
//  * acos: acos(x) = pi/2 - asin(x) for |x| <= 1/2, 2 asin(sqrt((1-x)/2)) above,
//    pi - 2 asin(sqrt((1+x)/2)) below; asin by its Taylor series (10 terms, |y| <= 1/2).
//  * atan2: atan on [0, 1] (the larger magnitude divides the smaller; pi/2 - atan above 1),
//    reduced past tan(pi/12) by atan(t) = pi/6 + atan((t sqrt3 - 1)/(t + sqrt3)), then the odd
//    Taylor series of atan (7 terms, |r| <= tan(pi/12)); quadrants and signed zeros as C99.
//  * pow(x, 5): ((x x)(x x)) x.
// Measured accuracy against a double-precision libm is checked by the test suite.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define NE_HD __host__ __device__ __forceinline__
#else
#define NE_HD inline
#include <string.h>
#include <math.h>
#endif

namespace nefm {

NE_HD uint32_t f2u(float f) {
#if defined(__CUDA_ARCH__)
  return __float_as_uint(f);
#else
  uint32_t u; memcpy(&u, &f, 4); return u;
#endif
}
NE_HD float u2f(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __uint_as_float(u);
#else
  float f; memcpy(&f, &u, 4); return f;
#endif
}
NE_HD float fsqrt(float x) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(x);
#else
  return sqrtf(x);
#endif
}
NE_HD float ffloor(float x) {
#if defined(__CUDA_ARCH__)
  return floorf(x);
#else
  return floorf(x);
#endif
}
// Round to nearest integer (ties away from zero) as a float, exact for |x| < 2^23.
NE_HD float fround(float x) {
  float a = x < 0.0f ? -x : x;
  float r = ffloor(a + 0.5f);
  return x < 0.0f ? -r : r;
}
NE_HD bool isnan_(float x) { return x != x; }
NE_HD bool isinf_(float x) { return (f2u(x) & 0x7fffffffu) == 0x7f800000u; }

constexpr float kPi = 0x1.921fb6p+1f;
constexpr float kPiO2 = 0x1.921fb6p+0f;
constexpr float kTwoOverPi = 0x1.45f306p-1f;
constexpr float kPiO2_1 = 0x1.92p+0f;       // 10 significant bits
constexpr float kPiO2_2 = 0x1.fb4p-12f;     // next 12 bits
constexpr float kPiO2_3 = 0x1.4442d2p-24f;  // remainder
constexpr float kLn2Hi = 0x1.62ep-1f;       // 12 significant bits
constexpr float kLn2Lo = 0x1.0bfbe8p-15f;
constexpr float kInvLn2 = 0x1.715476p+0f;
constexpr float kSqrt2 = 0x1.6a09e6p+0f;

// log(x 2^-k0) for a positive, normal, finite x.
NE_HD float log_normal(float x, int k) {
  uint32_t ix = f2u(x);
  k += (int)((ix >> 23) & 0xffu) - 127;
  float m = u2f((ix & 0x007fffffu) | 0x3f800000u);  // [1, 2)
  if (m > kSqrt2) { m = m * 0.5f; k += 1; }
  float f = m - 1.0f;
  float s = f / (2.0f + f);
  float z = s * s;
  // atanh series: 2 atanh(s) = 2s + s z (2/3 + 2/5 z + 2/7 z^2 + 2/9 z^3 + 2/11 z^4)
  float R = z * (0x1.555556p-1f + z * (0x1.99999ap-2f + z * (0x1.24924ap-2f + z * (0x1.c71c72p-3f + z * 0x1.745d18p-3f))));
  // 2s = f - s f, so log(1+f) = f - s (f - R)
  float lg = f - s * (f - R);
  float fk = (float)k;
  return (fk * kLn2Hi + (lg + fk * kLn2Lo));
}

// Natural logarithm.
NE_HD float log(float x) {
  if (isnan_(x) || x < 0.0f) return u2f(0x7fc00000u);
  if (x == 0.0f) return -u2f(0x7f800000u);
  if (isinf_(x)) return x;
  if (f2u(x) < 0x00800000u) return log_normal(x * 33554432.0f, -25);  // subnormal: scale up by 2^25
  return log_normal(x, 0);
}

// log(1 - u) for a uniform draw u = k 2^-24 (the tracking steps): 1 - u lies in [2^-24, 1],
// positive and normal, so this is log without its special cases, with the same result.
NE_HD float log1m_draw(float u) { return log_normal(1 - u, 0); }

// Exponential.
NE_HD float exp(float x) {
  if (isnan_(x)) return x;
  if (x > 88.72283f) return u2f(0x7f800000u);
  if (x < -103.97208f) return 0.0f;
  float kf = fround(x * kInvLn2);
  int k = (int)kf;
  float r = (x - kf * kLn2Hi) - kf * kLn2Lo;
  // Taylor series of e^r to r^7 (|r| <= 0.35)
  float p = 1.0f + r * (1.0f + r * (0.5f + r * (0x1.555556p-3f + r * (0x1.555556p-5f + r * (0x1.111112p-7f + r * (0x1.6c16c2p-10f + r * 0x1.a01a02p-13f))))));
  // p * 2^k, split so that subnormal results round once
  if (k > 127) { p = p * 2.0f; k -= 1; }
  if (k < -126) {
    p = p * u2f((uint32_t)(k + 126 + 127) << 23);
    return p * u2f(0x00800000u);  // 2^-126
  }
  return p * u2f((uint32_t)(k + 127) << 23);
}

NE_HD float sin_poly(float r) {
  float z = r * r;
  // r - r^3/3! + r^5/5! - r^7/7! + r^9/9!
  return r + r * z * (-0x1.555556p-3f + z * (0x1.111112p-7f + z * (-0x1.a01a02p-13f + z * 0x1.71de3ap-19f)));
}
NE_HD float cos_poly(float r) {
  float z = r * r;
  // 1 - z/2 + z^2/4! - z^3/6! + z^4/8! - z^5/10!
  return 1.0f - 0.5f * z + z * z * (0x1.555556p-5f + z * (-0x1.6c16c2p-10f + z * (0x1.a01a02p-16f - z * 0x1.27e4fcp-22f)));
}
NE_HD float reduce_pio2(float x, int* q) {
  float kf = fround(x * kTwoOverPi);
  *q = (int)kf;
  return ((x - kf * kPiO2_1) - kf * kPiO2_2) - kf * kPiO2_3;
}
NE_HD float sin(float x) {
  if (isnan_(x) || isinf_(x)) return u2f(0x7fc00000u);
  int q;
  float r = reduce_pio2(x, &q);
  switch (q & 3) {
    case 0: return sin_poly(r);
    case 1: return cos_poly(r);
    case 2: return -sin_poly(r);
    default: return -cos_poly(r);
  }
}
NE_HD float cos(float x) {
  if (isnan_(x) || isinf_(x)) return u2f(0x7fc00000u);
  int q;
  float r = reduce_pio2(x, &q);
  switch (q & 3) {
    case 0: return cos_poly(r);
    case 1: return -sin_poly(r);
    case 2: return -cos_poly(r);
    default: return sin_poly(r);
  }
}

// asin on |y| <= 1/2 by its Taylor series (c_n = (2n)! / (4^n (n!)^2 (2n+1))).
NE_HD float asin_small(float y) {
  float z = y * y;
  float p = 0x1.555556p-3f + z * (0x1.333334p-4f + z * (0x1.6db6dcp-5f + z * (0x1.f1c71cp-6f + z * (0x1.6e8ba2p-6f +
            z * (0x1.1c4ec4p-6f + z * (0x1.c9999ap-7f + z * (0x1.7a8788p-7f + z * (0x1.3fde50p-7f + z * 0x1.12ef3cp-7f))))))));
  return y + y * z * p;
}
NE_HD float acos(float x) {
  if (isnan_(x) || x > 1.0f || x < -1.0f) return u2f(0x7fc00000u);
  if (x <= 0.5f && x >= -0.5f) return kPiO2 - asin_small(x);
  if (x > 0.5f) {
    float y = fsqrt((1.0f - x) * 0.5f);
    return 2.0f * asin_small(y);
  }
  float y = fsqrt((1.0f + x) * 0.5f);
  return kPi - 2.0f * asin_small(y);
}

// atan on |r| <= tan(pi/12) by its Taylor series r - r^3/3 + r^5/5 - ... - r^11/11 + r^13/13.
NE_HD float atan_small(float r) {
  float z = r * r;
  float p = -0x1.555556p-2f + z * (0x1.99999ap-3f + z * (-0x1.24924ap-3f + z * (0x1.c71c72p-4f +
            z * (-0x1.745d18p-4f + z * 0x1.3b13b2p-4f))));
  return r + r * z * p;
}
// atan on [0, 1].
NE_HD float atan01(float t) {
  if (t <= 0x1.126146p-2f) return atan_small(t);  // tan(pi/12)
  const float sqrt3 = 0x1.bb67aep+0f;
  float r = (t * sqrt3 - 1.0f) / (t + sqrt3);
  return 0x1.0c1524p-1f + atan_small(r);  // pi/6 + atan(r)
}
NE_HD bool signbit_(float x) { return (f2u(x) >> 31) != 0; }
// atan2(y, x) in [-pi, pi].
NE_HD float atan2(float y, float x) {
  if (isnan_(x) || isnan_(y)) return u2f(0x7fc00000u);
  float ax = x < 0.0f ? -x : x, ay = y < 0.0f ? -y : y;
  float a;
  if (isinf_(ax) && isinf_(ay)) {
    a = 0x1.921fb6p-1f;  // pi/4
  } else if (isinf_(ay) || (ax == 0.0f && ay != 0.0f)) {
    a = kPiO2;
  } else if (isinf_(ax) || ay == 0.0f) {
    a = 0.0f;
  } else if (ay <= ax) {
    a = atan01(ay / ax);
  } else {
    a = kPiO2 - atan01(ax / ay);
  }
  if (signbit_(x)) a = kPi - a;
  return signbit_(y) ? -a : a;
}

NE_HD float pow5(float x) {
  float x2 = x * x;
  return (x2 * x2) * x;
}

}  // namespace nefm
