/*
 * Portable stand-in for the eight SSE intrinsics the reference's AABB
 * (BVH/AABB.h) uses, so its host BVH builder also compiles on aarch64 hosts.
 * Only placed on the include path when the compiler is not targeting x86.
 *
 * TEST INFRASTRUCTURE ONLY (oracle). Semantics follow the SSE definitions:
 *   MINPS(a, b) = a < b ? a : b   (second operand on NaN or equal)
 *   MAXPS(a, b) = a > b ? a : b
 *   _mm_set_ps(e3, e2, e1, e0) puts e0 in lane 0; _mm_setr_ps is lane order.
 * All arithmetic is lane-wise IEEE single precision, like the SSE originals.
 */
#pragma once
#if defined(__x86_64__) || defined(__i386__)
#error "portable immintrin.h must not shadow the real header on x86"
#endif

typedef float __m128 __attribute__((vector_size(16), aligned(16)));

static inline __m128 ct__lanes(float a, float b, float c, float d) {
  __m128 r;
  r[0] = a; r[1] = b; r[2] = c; r[3] = d;
  return r;
}
static inline __m128 _mm_set_ps(float e3, float e2, float e1, float e0) { return ct__lanes(e0, e1, e2, e3); }
static inline __m128 _mm_setr_ps(float e0, float e1, float e2, float e3) { return ct__lanes(e0, e1, e2, e3); }
static inline __m128 _mm_set_ps1(float x) { return ct__lanes(x, x, x, x); }
static inline __m128 _mm_add_ps(__m128 a, __m128 b) {
  __m128 r;
  for (int i = 0; i < 4; i++) r[i] = a[i] + b[i];
  return r;
}
static inline __m128 _mm_sub_ps(__m128 a, __m128 b) {
  __m128 r;
  for (int i = 0; i < 4; i++) r[i] = a[i] - b[i];
  return r;
}
static inline __m128 _mm_mul_ps(__m128 a, __m128 b) {
  __m128 r;
  for (int i = 0; i < 4; i++) r[i] = a[i] * b[i];
  return r;
}
static inline __m128 _mm_min_ps(__m128 a, __m128 b) {
  __m128 r;
  for (int i = 0; i < 4; i++) r[i] = a[i] < b[i] ? a[i] : b[i];
  return r;
}
static inline __m128 _mm_max_ps(__m128 a, __m128 b) {
  __m128 r;
  for (int i = 0; i < 4; i++) r[i] = a[i] > b[i] ? a[i] : b[i];
  return r;
}
