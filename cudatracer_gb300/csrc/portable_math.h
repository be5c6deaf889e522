// Reproducible single-precision sin, cos, atan2 and acos.
//
// Every function here is a fixed sequence of IEEE-754 binary32 operations that
// round correctly on every conforming platform (add, subtract, multiply,
// divide, square root and fused multiply-add, each written as an explicit
// round-to-nearest call so that no compiler contracts or reorders them). The
// same source therefore gives the same bits in a CUDA kernel and in host C++:
// the exact-math shading kernels and the CPU oracle both use it, which is what
// makes exact-math frames bit-identical between the GPU and the oracle without
// any double-precision arithmetic (binary64 runs at a small fraction of the
// binary32 rate on this GPU).
//
// Methods (textbook mathematics, nothing taken from a vendor library):
//   sin/cos  Cody & Waite argument reduction, x = k (pi/2) + r, with pi/2
//            split into three 12-bit parts (k * part exact for |k| < 2^12) and
//            a 24-bit tail; Taylor series of sin to r^11 and of cos to r^12 on
//            |r| <= pi/4 (truncation below 1e-11), Horner form with fused
//            multiply-adds; quadrant from k mod 4.
//   atan2    reduction to atan(t), t = min(|x|,|y|) / max(|x|,|y|) in [0, 1];
//            for t > 2 - sqrt(3) the identity atan(t) = pi/6 + atan((sqrt(3) t
//            - 1) / (sqrt(3) + t)) brings the argument into [-0.268, 0.268];
//            Taylor series of atan to t^19 (truncation below 1e-13); the
//            octant is restored with pi/2 and pi carried as two floats.
//   acos     acos(x) = atan2(sqrt((1 - x)(1 + x)), x).
// Accuracy against correctly rounded values (tests/test_portable_math.py):
// sin/cos within 2 ulp on [0, 2 pi], atan2 and acos within 3 ulp; domain of
// sin/cos: |x| <= 1024 (the shading kernels pass angles in [0, 2 pi)).
#pragma once

#include <stdint.h>

#include <cmath>
#include <cstring>

#if defined(__CUDACC__)
#define CT_PM_FN __host__ __device__ __forceinline__
#else
#define CT_PM_FN inline
#endif

namespace ct {
namespace pm {

CT_PM_FN float add(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fadd_rn(a, b);
#else
  volatile float r = a + b;  // no contraction or reassociation across this point
  return r;
#endif
}
CT_PM_FN float sub(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fsub_rn(a, b);
#else
  volatile float r = a - b;
  return r;
#endif
}
CT_PM_FN float mul(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fmul_rn(a, b);
#else
  volatile float r = a * b;
  return r;
#endif
}
CT_PM_FN float div(float a, float b) {
#if defined(__CUDA_ARCH__)
  return __fdiv_rn(a, b);
#else
  volatile float r = a / b;
  return r;
#endif
}
CT_PM_FN float fma(float a, float b, float c) {
#if defined(__CUDA_ARCH__)
  return __fmaf_rn(a, b, c);
#else
  return std::fmaf(a, b, c);
#endif
}
CT_PM_FN float sqrt(float a) {
#if defined(__CUDA_ARCH__)
  return __fsqrt_rn(a);
#else
  return std::sqrt(a);
#endif
}
CT_PM_FN uint32_t bits(float f) {
#if defined(__CUDA_ARCH__)
  return (uint32_t)__float_as_int(f);
#else
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
#endif
}
CT_PM_FN float from_bits(uint32_t u) {
#if defined(__CUDA_ARCH__)
  return __int_as_float((int)u);
#else
  float f;
  std::memcpy(&f, &u, 4);
  return f;
#endif
}
CT_PM_FN float fabs_(float a) { return from_bits(bits(a) & 0x7fffffffu); }
CT_PM_FN float copysign_(float a, float s) { return from_bits((bits(a) & 0x7fffffffu) | (bits(s) & 0x80000000u)); }
CT_PM_FN bool is_nan(float a) { return (bits(a) & 0x7fffffffu) > 0x7f800000u; }
CT_PM_FN float quiet_nan() { return from_bits(0x7fc00000u); }

// nearest integer of a float of magnitude < 2^22 (ties away from zero), as a float
CT_PM_FN float round_int(float a) {
  const float h = copysign_(0.5f, a);
  const float t = add(a, h);
  // truncate toward zero: clear the fraction bits of t
  const uint32_t u = bits(t);
  const int e = (int)((u >> 23) & 0xff) - 127;
  if (e < 0) return copysign_(0.0f, a);
  if (e >= 23) return t;
  return from_bits(u & ~((1u << (23 - e)) - 1u));
}

// sin and cos of x (|x| <= 1024).
CT_PM_FN void sincos(float x, float* s_out, float* c_out) {
  // pi/2 = P1 + P2 + P3 + P4 (P1..P3 with 12 significant bits)
  const float P1 = 0x1.922p+0f, P2 = -0x1.2aep-18f, P3 = -0x1.deap-31f, P4 = 0x1.184698p-44f;
  const float k = round_int(mul(x, 0x1.45f306p-1f));  // x * 2/pi
  float r = sub(x, mul(k, P1));
  r = sub(r, mul(k, P2));
  r = sub(r, mul(k, P3));
  r = sub(r, mul(k, P4));
  const float z = mul(r, r);
  // sin(r) = r + r^3 (s3 + z (s5 + z (s7 + z (s9 + z s11))))
  float ps = fma(z, -0x1.ae6456p-26f, 0x1.71de3ap-19f);
  ps = fma(z, ps, -0x1.a01a02p-13f);
  ps = fma(z, ps, 0x1.111112p-7f);
  ps = fma(z, ps, -0x1.555556p-3f);
  const float sr = fma(mul(r, z), ps, r);
  // cos(r) = 1 + z (c2 + z (c4 + z (c6 + z (c8 + z (c10 + z c12)))))
  float pc = fma(z, 0x1.1eed8ep-29f, -0x1.27e4fcp-22f);
  pc = fma(z, pc, 0x1.a01a02p-16f);
  pc = fma(z, pc, -0x1.6c16c2p-10f);
  pc = fma(z, pc, 0x1.555556p-5f);
  pc = fma(z, pc, -0.5f);
  const float cr = fma(z, pc, 1.0f);
  const int q = (int)k & 3;  // two's complement: k mod 4 also for negative k
  float s, c;
  if (q == 0) s = sr, c = cr;
  else if (q == 1) s = cr, c = -sr;
  else if (q == 2) s = -sr, c = -cr;
  else s = -cr, c = sr;
  *s_out = s;
  *c_out = c;
}
CT_PM_FN float sin(float x) {
  float s, c;
  sincos(x, &s, &c);
  return s;
}
CT_PM_FN float cos(float x) {
  float s, c;
  sincos(x, &s, &c);
  return c;
}

// atan(t) for t in [0, 1]
CT_PM_FN float atan01(float t) {
  const float kLow = 0x1.126146p-2f;  // 2 - sqrt(3), rounded down
  float u = t, base_hi = 0.0f, base_lo = 0.0f;
  if (t > kLow) {
    // (sqrt(3) t - 1) / (sqrt(3) + t), sqrt(3) = S_HI + S_LO
    const float num = fma(t, 0x1.bb67aep+0f, -1.0f);
    const float num2 = fma(t, 0x1.0b0996p-25f, num);
    u = div(num2, add(0x1.bb67aep+0f, t));
    base_hi = 0x1.0c1524p-1f;  // pi/6
    base_lo = -0x1.f4a326p-27f;
  }
  const float z = mul(u, u);
  float p = fma(z, -0x1.af286cp-5f, 0x1.e1e1e2p-5f);
  p = fma(z, p, -0x1.111112p-4f);
  p = fma(z, p, 0x1.3b13b2p-4f);
  p = fma(z, p, -0x1.745d18p-4f);
  p = fma(z, p, 0x1.c71c72p-4f);
  p = fma(z, p, -0x1.24924ap-3f);
  p = fma(z, p, 0x1.99999ap-3f);
  p = fma(z, p, -0x1.555556p-2f);
  const float a = fma(mul(u, z), p, add(u, base_lo));
  return add(base_hi, a);
}

// atan2(y, x) with the C library's conventions for signed zeros and infinities.
CT_PM_FN float atan2(float y, float x) {
  if (is_nan(x) || is_nan(y)) return add(x, y);
  const float ax = fabs_(x), ay = fabs_(y);
  const bool x_neg = (bits(x) & 0x80000000u) != 0;
  const float PIO2_HI = 0x1.921fb6p+0f, PIO2_LO = -0x1.777a5cp-25f;
  const float PI_HI = 0x1.921fb6p+1f, PI_LO = -0x1.777a5cp-24f;
  float a;
  if (ay == 0.0f) {
    a = x_neg ? PI_HI : 0.0f;
  } else if (ax == 0.0f) {
    a = PIO2_HI;
  } else {
    const float inf = from_bits(0x7f800000u);
    const bool steep = ay > ax;
    const float mn = steep ? ax : ay, mxv = steep ? ay : ax;
    float t;
    if (mxv == inf) t = mn == inf ? 1.0f : 0.0f;
    else t = div(mn, mxv);
    a = atan01(t);
    if (steep) a = add(sub(PIO2_HI, a), PIO2_LO);
    if (x_neg) a = add(sub(PI_HI, a), PI_LO);
  }
  return copysign_(a, y);
}

// acos(x); NaN outside [-1, 1].
CT_PM_FN float acos(float x) {
  if (!(fabs_(x) <= 1.0f)) return quiet_nan();
  const float s = sqrt(mul(sub(1.0f, x), add(1.0f, x)));
  return atan2(s, x);
}

}  // namespace pm
}  // namespace ct
