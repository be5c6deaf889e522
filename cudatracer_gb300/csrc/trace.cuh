// Device BVH traversal: closest hit and any hit over the quad tree.
//
// Arithmetic is written with round-to-nearest intrinsics so no multiply-add is
// ever fused, whatever the translation unit's -fmad setting: every slab and
// Moller-Trumbore quantity is computed with the same IEEE single-precision
// operations, in the same order, as the reference's glm code
// (src/BVH/MBVHNode.cuh:69-110, src/Core/Triangle.cuh:13-44), which is what
// makes closest-hit primitive ids and t bit-exact against it.
#pragma once

#include "ct_internal.h"
#include "vmath.cuh"

namespace ct {

__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }
// gmin / gmax (vmath.cuh) are glm::min / glm::max: (y < x) ? y : x and (x < y) ? y : x.

template <typename T>
__device__ __forceinline__ T sel4(T a, T b, T c, T d, int i) {
  return i == 0 ? a : (i == 1 ? b : (i == 2 ? c : d));
}

// One child's slab interval, reference order: x, then y, then z.
__device__ __forceinline__ void slab(float bminx, float bmaxx, float bminy, float bmaxy, float bminz, float bmaxz,
                                     float ox, float oy, float oz, float ix, float iy, float iz, float& tmin,
                                     float& tmax) {
  float t1 = fmul(fsub(bminx, ox), ix), t2 = fmul(fsub(bmaxx, ox), ix);
  tmin = gmin(t1, t2);
  tmax = gmax(t1, t2);
  t1 = fmul(fsub(bminy, oy), iy);
  t2 = fmul(fsub(bmaxy, oy), iy);
  tmin = gmax(tmin, gmin(t1, t2));
  tmax = gmin(tmax, gmax(t1, t2));
  t1 = fmul(fsub(bminz, oz), iz);
  t2 = fmul(fsub(bmaxz, oz), iz);
  tmin = gmax(tmin, gmin(t1, t2));
  tmax = gmin(tmax, gmax(t1, t2));
}

// Moller-Trumbore with the reference's absolute epsilon. Returns the new t
// through `t` when the hit is closer (t' > eps && t > t').
__device__ __forceinline__ bool tri_test(const float4 a, const float4 e1v, const float4 e2v, float ox, float oy,
                                         float oz, float dx, float dy, float dz, float eps, float& t) {
  const float e1x = e1v.x, e1y = e1v.y, e1z = e1v.z;
  const float e2x = e2v.x, e2y = e2v.y, e2z = e2v.z;
  // h = cross(dir, edge2)
  const float hx = fsub(fmul(dy, e2z), fmul(e2y, dz));
  const float hy = fsub(fmul(dz, e2x), fmul(e2z, dx));
  const float hz = fsub(fmul(dx, e2y), fmul(e2x, dy));
  const float det = fadd(fadd(fmul(e1x, hx), fmul(e1y, hy)), fmul(e1z, hz));
  if (det > -eps && det < eps) return false;
  const float f = __frcp_rn(det);
  const float sx = fsub(ox, a.x), sy = fsub(oy, a.y), sz = fsub(oz, a.z);
  const float u = fmul(f, fadd(fadd(fmul(sx, hx), fmul(sy, hy)), fmul(sz, hz)));
  if (u < 0.0f || u > 1.0f) return false;
  // q = cross(s, edge1)
  const float qx = fsub(fmul(sy, e1z), fmul(e1y, sz));
  const float qy = fsub(fmul(sz, e1x), fmul(e1z, sx));
  const float qz = fsub(fmul(sx, e1y), fmul(e1x, sy));
  const float v = fmul(f, fadd(fadd(fmul(dx, qx), fmul(dy, qy)), fmul(dz, qz)));
  if (v < 0.0f || fadd(u, v) > 1.0f) return false;
  const float tt = fmul(f, fadd(fadd(fmul(e2x, qx), fmul(e2y, qy)), fmul(e2z, qz)));
  if (tt > eps && t > tt) {
    t = tt;
    return true;
  }
  return false;
}

// Traverse one ray. ANY = stop at the first hit (traverseMBVHShadow semantics:
// nodes culled against maxDist, triangles accepted below it).
// `stack` points at this thread's column of a [entries][stride] shared array.
// Returns false if the stack limit was reached (the ray's result is dropped).
template <bool ANY>
__device__ __forceinline__ bool traverse(const DevBVH& b, float ox, float oy, float oz, float dx, float dy, float dz,
                                         float eps, float& t, int& hit, int* stack, int stride) {
  const float ix = __frcp_rn(dx), iy = __frcp_rn(dy), iz = __frcp_rn(dz);
  const int limit = b.stack_entries;
  int sp = 0;
  int ref = 0;  // root: inner node 0 (the reference's todo[0] = {0, -1})
  while (true) {
    if (ref >= 0) {
      const QNodeDev* n = b.nodes + ref;
      const float4 nx0 = __ldg(&n->bminx), nx1 = __ldg(&n->bmaxx);
      const float4 ny0 = __ldg(&n->bminy), ny1 = __ldg(&n->bmaxy);
      const float4 nz0 = __ldg(&n->bminz), nz1 = __ldg(&n->bmaxz);
      const int4 ch = __ldg(&n->child);
      float tn0, tn1, tn2, tn3, tf0, tf1, tf2, tf3;
      slab(nx0.x, nx1.x, ny0.x, ny1.x, nz0.x, nz1.x, ox, oy, oz, ix, iy, iz, tn0, tf0);
      slab(nx0.y, nx1.y, ny0.y, ny1.y, nz0.y, nz1.y, ox, oy, oz, ix, iy, iz, tn1, tf1);
      slab(nx0.z, nx1.z, ny0.z, ny1.z, nz0.z, nz1.z, ox, oy, oz, ix, iy, iz, tn2, tf2);
      slab(nx0.w, nx1.w, ny0.w, ny1.w, nz0.w, nz1.w, ox, oy, oz, ix, iy, iz, tn3, tf3);
      // child id in the low two bits of tmin (MBVHNode.cuh:91-94)
      float p0 = __int_as_float((__float_as_int(tn0) & ~3) | 0);
      float p1 = __int_as_float((__float_as_int(tn1) & ~3) | 1);
      float p2 = __int_as_float((__float_as_int(tn2) & ~3) | 2);
      float p3 = __int_as_float((__float_as_int(tn3) & ~3) | 3);
      const bool r0 = tf0 > 0.0f && p0 <= tf0 && p0 < t;
      const bool r1 = tf1 > 0.0f && p1 <= tf1 && p1 < t;
      const bool r2 = tf2 > 0.0f && p2 <= tf2 && p2 < t;
      const bool r3 = tf3 > 0.0f && p3 <= tf3 && p3 < t;
      // the reference's 5-exchange network, last pair (2,3) (MBVHNode.cuh:98-107)
      float s;
      if (p0 > p1) s = p0, p0 = p1, p1 = s;
      if (p2 > p3) s = p2, p2 = p3, p3 = s;
      if (p0 > p2) s = p0, p0 = p2, p2 = s;
      if (p1 > p3) s = p1, p1 = p3, p3 = s;
      if (p2 > p3) s = p2, p2 = p3, p3 = s;
      // push far to near (i = 3..0); the nearest stays in a register
      int held = kEmptyChild;
      bool have = false;
#pragma unroll
      for (int i = 3; i >= 0; i--) {
        const float pi = sel4(p0, p1, p2, p3, i);
        const int c = __float_as_int(pi) & 3;
        const bool ri = sel4(r0, r1, r2, r3, c);
        const int cr = sel4(ch.x, ch.y, ch.z, ch.w, c);
        if (ri && cr != kEmptyChild) {
          if (have) {
            if (sp >= limit) return false;
            stack[sp * stride] = held;
            sp++;
          }
          held = cr;
          have = true;
        }
      }
      if (have) {
        ref = held;
        continue;
      }
    } else {
      const uint32_t u = (uint32_t)ref;
      const uint32_t first = u & b.first_mask;
      const uint32_t cnt = (u >> b.leaf_shift) & b.count_mask;
      const float4* tp = b.tris + 3 * (size_t)first;
      for (uint32_t i = 0; i < cnt; i++) {
        const float4 a = __ldg(tp + 3 * i), e1 = __ldg(tp + 3 * i + 1), e2 = __ldg(tp + 3 * i + 2);
        if (tri_test(a, e1, e2, ox, oy, oz, dx, dy, dz, eps, t)) {
          hit = __float_as_int(a.w);
          if (ANY) return true;
        }
      }
    }
    if (sp == 0) break;
    sp--;
    ref = stack[sp * stride];
  }
  return true;
}

}  // namespace ct
