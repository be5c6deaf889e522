// Device BVH traversal: closest hit and any hit over the quad tree.
//
// Arithmetic is written with round-to-nearest intrinsics so no multiply-add is
// ever fused, whatever the translation unit's -fmad setting: every slab and
// Moller-Trumbore quantity is computed with the same IEEE single-precision
// operations, in the same order, as the reference's glm code
// (src/BVH/MBVHNode.cuh:69-110, src/Core/Triangle.cuh:13-44), which is what
// makes closest-hit primitive ids and t bit-exact against it.
//
// Min/max: glm::min(x,y) = y < x ? y : x and glm::max(x,y) = x < y ? y : x.
// With FASTMM the hardware min/max is used instead; the two agree except when
// a slab term is NaN (a zero direction component with the origin exactly on a
// bounding plane) or when two zeros of opposite sign meet (an origin on two
// planes). The fast-math render path uses FASTMM; exact paths never do.
// FASTMM traversal also computes each slab plane with one fused multiply-add
// and, for closest hit, visits hit children in true distance order
// (inner_step_sorted) instead of the reference's partial order network: the
// same nearest hit up to exact ties and the rounding of box distances, fewer
// instructions per node.
#pragma once

#include "ct_internal.h"
#include "vmath.cuh"

namespace ct {

__device__ __forceinline__ float fsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ float fadd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ float fmul(float a, float b) { return __fmul_rn(a, b); }

template <bool FASTMM>
__device__ __forceinline__ float mn(float x, float y) {
  return FASTMM ? fminf(x, y) : gmin(x, y);
}
template <bool FASTMM>
__device__ __forceinline__ float mx(float x, float y) {
  return FASTMM ? fmaxf(x, y) : gmax(x, y);
}

template <typename T>
__device__ __forceinline__ T sel4(T a, T b, T c, T d, int i) {
  return i == 0 ? a : (i == 1 ? b : (i == 2 ? c : d));
}

// One child's slab interval, reference order: x, then y, then z.
template <bool FASTMM>
__device__ __forceinline__ void slab(float bminx, float bmaxx, float bminy, float bmaxy, float bminz, float bmaxz,
                                     float ox, float oy, float oz, float ix, float iy, float iz, float& tmin,
                                     float& tmax) {
  float t1 = fmul(fsub(bminx, ox), ix), t2 = fmul(fsub(bmaxx, ox), ix);
  tmin = mn<FASTMM>(t1, t2);
  tmax = mx<FASTMM>(t1, t2);
  t1 = fmul(fsub(bminy, oy), iy);
  t2 = fmul(fsub(bmaxy, oy), iy);
  tmin = mx<FASTMM>(tmin, mn<FASTMM>(t1, t2));
  tmax = mn<FASTMM>(tmax, mx<FASTMM>(t1, t2));
  t1 = fmul(fsub(bminz, oz), iz);
  t2 = fmul(fsub(bmaxz, oz), iz);
  tmin = mx<FASTMM>(tmin, mn<FASTMM>(t1, t2));
  tmax = mn<FASTMM>(tmax, mx<FASTMM>(t1, t2));
}

// Fast-math slab: one fused multiply-add per plane, b * inv + (-o * inv). A
// zero direction component makes that axis NaN, which the hardware min/max
// drop: the axis then culls nothing (more boxes visited, never a hit lost).
__device__ __forceinline__ void slab_fma(float bminx, float bmaxx, float bminy, float bmaxy, float bminz,
                                         float bmaxz, float nox, float noy, float noz, float ix, float iy, float iz,
                                         float& tmin, float& tmax) {
  const float x1 = fmaf(bminx, ix, nox), x2 = fmaf(bmaxx, ix, nox);
  const float y1 = fmaf(bminy, iy, noy), y2 = fmaf(bmaxy, iy, noy);
  const float z1 = fmaf(bminz, iz, noz), z2 = fmaf(bmaxz, iz, noz);
  tmin = fmaxf(fmaxf(fminf(x1, x2), fminf(y1, y2)), fminf(z1, z2));
  tmax = fminf(fminf(fmaxf(x1, x2), fmaxf(y1, y2)), fmaxf(z1, z2));
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

// Per-ray traversal state.
struct RayState {
  float ox, oy, oz, dx, dy, dz, ix, iy, iz, t;
  float nox, noy, noz;  // -o * inv, read by the fast-math slab only
  int hit, sp, ref;
};

__device__ __forceinline__ void ray_begin(RayState& r, float4 o, float4 d, float t0) {
  r.ox = o.x, r.oy = o.y, r.oz = o.z, r.dx = d.x, r.dy = d.y, r.dz = d.z;
  r.ix = __frcp_rn(d.x), r.iy = __frcp_rn(d.y), r.iz = __frcp_rn(d.z);
  r.nox = -o.x * r.ix, r.noy = -o.y * r.iy, r.noz = -o.z * r.iz;
  r.t = t0;
  r.hit = -1;
  r.sp = 0;
  r.ref = 0;  // root: inner node 0 (the reference's todo[0] = {0, -1})
}

enum StepResult { kContinue = 0, kDone = 1, kOverflow = 2 };

// The four child intervals of a node in fast math.
__device__ __forceinline__ void fast_slab4(const float4& nx0, const float4& nx1, const float4& ny0, const float4& ny1,
                                           const float4& nz0, const float4& nz1, const RayState& r, float& tn0,
                                           float& tn1, float& tn2, float& tn3, float& tf0, float& tf1, float& tf2,
                                           float& tf3) {
  slab_fma(nx0.x, nx1.x, ny0.x, ny1.x, nz0.x, nz1.x, r.nox, r.noy, r.noz, r.ix, r.iy, r.iz, tn0, tf0);
  slab_fma(nx0.y, nx1.y, ny0.y, ny1.y, nz0.y, nz1.y, r.nox, r.noy, r.noz, r.ix, r.iy, r.iz, tn1, tf1);
  slab_fma(nx0.z, nx1.z, ny0.z, ny1.z, nz0.z, nz1.z, r.nox, r.noy, r.noz, r.ix, r.iy, r.iz, tn2, tf2);
  slab_fma(nx0.w, nx1.w, ny0.w, ny1.w, nz0.w, nz1.w, r.nox, r.noy, r.noz, r.ix, r.iy, r.iz, tn3, tf3);
}

// Compare-and-swap of (distance, child) pairs: the nearer pair goes first.
__device__ __forceinline__ void cas_pair(float& ka, int& ca, float& kb, int& cb) {
  const bool sw = kb < ka;
  const float k = sw ? kb : ka;
  const int c = sw ? cb : ca;
  kb = sw ? ka : kb;
  cb = sw ? ca : cb;
  ka = k;
  ca = c;
}

// Fast-math closest-hit node step: the hit children in true distance order (a
// full 4-sort of (tmin, child) pairs, misses last as +inf), nearest visited
// next and the others pushed far to near with predicated stores. Frames in
// fast math do not reproduce the reference's visiting order, only its nearest
// hit, which no order changes beyond exact ties.
__device__ __forceinline__ StepResult inner_step_sorted(const DevBVH& b, RayState& r, int* stack, int stride,
                                                        int limit) {
  const QNodeDev* n = b.nodes + r.ref;
  const float4 nx0 = __ldg(&n->bminx), nx1 = __ldg(&n->bmaxx);
  const float4 ny0 = __ldg(&n->bminy), ny1 = __ldg(&n->bmaxy);
  const float4 nz0 = __ldg(&n->bminz), nz1 = __ldg(&n->bmaxz);
  const int4 ch = __ldg(&n->child);
  float tn0, tn1, tn2, tn3, tf0, tf1, tf2, tf3;
  fast_slab4(nx0, nx1, ny0, ny1, nz0, nz1, r, tn0, tn1, tn2, tn3, tf0, tf1, tf2, tf3);
  const float t = r.t, inf = __int_as_float(0x7f800000);
  const bool h0 = tf0 > 0.0f && tn0 <= tf0 && tn0 < t && ch.x != kEmptyChild;
  const bool h1 = tf1 > 0.0f && tn1 <= tf1 && tn1 < t && ch.y != kEmptyChild;
  const bool h2 = tf2 > 0.0f && tn2 <= tf2 && tn2 < t && ch.z != kEmptyChild;
  const bool h3 = tf3 > 0.0f && tn3 <= tf3 && tn3 < t && ch.w != kEmptyChild;
  const int cnt = (int)h0 + (int)h1 + (int)h2 + (int)h3;
  if (cnt == 0) {
    if (r.sp == 0) return kDone;
    r.ref = stack[--r.sp * stride];
    return kContinue;
  }
  float k0 = h0 ? tn0 : inf, k1 = h1 ? tn1 : inf, k2 = h2 ? tn2 : inf, k3 = h3 ? tn3 : inf;
  int c0 = ch.x, c1 = ch.y, c2 = ch.z, c3 = ch.w;
  if (cnt > 1) {
    cas_pair(k0, c0, k1, c1);
    cas_pair(k2, c2, k3, c3);
    cas_pair(k0, c0, k2, c2);
    cas_pair(k1, c1, k3, c3);
    cas_pair(k1, c1, k2, c2);
    if (r.sp + cnt - 1 > limit) return kOverflow;
    if (cnt > 3) stack[r.sp++ * stride] = c3;
    if (cnt > 2) stack[r.sp++ * stride] = c2;
    stack[r.sp++ * stride] = c1;
  } else {
    c0 = h0 ? ch.x : (h1 ? ch.y : (h2 ? ch.z : ch.w));
  }
  r.ref = c0;
  return kContinue;
}

// Visit the inner node r.ref: slab-test the four children (MBVHNode.cuh:69-110),
// then continue with the nearest hit child and push the others far to near
// (:153-161). With zero or one child hit the order network cannot matter, so
// it is skipped; with two or more it runs over all four packed tmin values,
// exactly as the reference's does.
template <bool FASTMM>
__device__ __forceinline__ StepResult inner_step(const DevBVH& b, RayState& r, int* stack, int stride, int limit) {
  const QNodeDev* n = b.nodes + r.ref;
  const float4 nx0 = __ldg(&n->bminx), nx1 = __ldg(&n->bmaxx);
  const float4 ny0 = __ldg(&n->bminy), ny1 = __ldg(&n->bmaxy);
  const float4 nz0 = __ldg(&n->bminz), nz1 = __ldg(&n->bmaxz);
  const int4 ch = __ldg(&n->child);
  float tn0, tn1, tn2, tn3, tf0, tf1, tf2, tf3;
  slab<FASTMM>(nx0.x, nx1.x, ny0.x, ny1.x, nz0.x, nz1.x, r.ox, r.oy, r.oz, r.ix, r.iy, r.iz, tn0, tf0);
  slab<FASTMM>(nx0.y, nx1.y, ny0.y, ny1.y, nz0.y, nz1.y, r.ox, r.oy, r.oz, r.ix, r.iy, r.iz, tn1, tf1);
  slab<FASTMM>(nx0.z, nx1.z, ny0.z, ny1.z, nz0.z, nz1.z, r.ox, r.oy, r.oz, r.ix, r.iy, r.iz, tn2, tf2);
  slab<FASTMM>(nx0.w, nx1.w, ny0.w, ny1.w, nz0.w, nz1.w, r.ox, r.oy, r.oz, r.ix, r.iy, r.iz, tn3, tf3);
  // child id in the low two bits of tmin (MBVHNode.cuh:91-94)
  float p0 = __int_as_float((__float_as_int(tn0) & ~3) | 0);
  float p1 = __int_as_float((__float_as_int(tn1) & ~3) | 1);
  float p2 = __int_as_float((__float_as_int(tn2) & ~3) | 2);
  float p3 = __int_as_float((__float_as_int(tn3) & ~3) | 3);
  const float t = r.t;
  // hit mask by child slot (MBVHNode.cuh:96); empty slots are never pushed
  const unsigned vm = ((tf0 > 0.0f && p0 <= tf0 && p0 < t && ch.x != kEmptyChild) ? 1u : 0u) |
                      ((tf1 > 0.0f && p1 <= tf1 && p1 < t && ch.y != kEmptyChild) ? 2u : 0u) |
                      ((tf2 > 0.0f && p2 <= tf2 && p2 < t && ch.z != kEmptyChild) ? 4u : 0u) |
                      ((tf3 > 0.0f && p3 <= tf3 && p3 < t && ch.w != kEmptyChild) ? 8u : 0u);
  if (vm == 0) {
    if (r.sp == 0) return kDone;
    r.ref = stack[--r.sp * stride];
    return kContinue;
  }
  if ((vm & (vm - 1)) == 0) {
    r.ref = vm == 1 ? ch.x : (vm == 2 ? ch.y : (vm == 4 ? ch.z : ch.w));
    return kContinue;
  }
  // the reference's 5-exchange network, last pair (2,3) (MBVHNode.cuh:98-107)
  float s;
  if (p0 > p1) s = p0, p0 = p1, p1 = s;
  if (p2 > p3) s = p2, p2 = p3, p3 = s;
  if (p0 > p2) s = p0, p0 = p2, p2 = s;
  if (p1 > p3) s = p1, p1 = p3, p3 = s;
  if (p2 > p3) s = p2, p2 = p3, p3 = s;
  int held = kEmptyChild;
  bool have = false;
#pragma unroll
  for (int i = 3; i >= 0; i--) {
    const int c = __float_as_int(sel4(p0, p1, p2, p3, i)) & 3;
    if ((vm >> c) & 1u) {
      const int cr = sel4(ch.x, ch.y, ch.z, ch.w, c);
      if (have) {
        if (r.sp >= limit) return kOverflow;
        stack[r.sp * stride] = held;
        r.sp++;
      }
      held = cr;
      have = true;
    }
  }
  r.ref = held;
  return kContinue;
}


// Any-hit variant of inner_step: whether the ray is occluded does not depend
// on the order in which hit children are visited (every node whose packed
// interval passes the reference's test is visited until a triangle hits), so
// the order network is skipped: the lowest hit slot continues, the others are
// pushed.
template <bool FASTMM>
__device__ __forceinline__ StepResult inner_step_any(const DevBVH& b, RayState& r, int* stack, int stride, int limit) {
  const QNodeDev* n = b.nodes + r.ref;
  const float4 nx0 = __ldg(&n->bminx), nx1 = __ldg(&n->bmaxx);
  const float4 ny0 = __ldg(&n->bminy), ny1 = __ldg(&n->bmaxy);
  const float4 nz0 = __ldg(&n->bminz), nz1 = __ldg(&n->bmaxz);
  const int4 ch = __ldg(&n->child);
  float tn0, tn1, tn2, tn3, tf0, tf1, tf2, tf3;
  if (FASTMM) {
    fast_slab4(nx0, nx1, ny0, ny1, nz0, nz1, r, tn0, tn1, tn2, tn3, tf0, tf1, tf2, tf3);
  } else {
    slab<false>(nx0.x, nx1.x, ny0.x, ny1.x, nz0.x, nz1.x, r.ox, r.oy, r.oz, r.ix, r.iy, r.iz, tn0, tf0);
    slab<false>(nx0.y, nx1.y, ny0.y, ny1.y, nz0.y, nz1.y, r.ox, r.oy, r.oz, r.ix, r.iy, r.iz, tn1, tf1);
    slab<false>(nx0.z, nx1.z, ny0.z, ny1.z, nz0.z, nz1.z, r.ox, r.oy, r.oz, r.ix, r.iy, r.iz, tn2, tf2);
    slab<false>(nx0.w, nx1.w, ny0.w, ny1.w, nz0.w, nz1.w, r.ox, r.oy, r.oz, r.ix, r.iy, r.iz, tn3, tf3);
  }
  const float p0 = __int_as_float((__float_as_int(tn0) & ~3) | 0);
  const float p1 = __int_as_float((__float_as_int(tn1) & ~3) | 1);
  const float p2 = __int_as_float((__float_as_int(tn2) & ~3) | 2);
  const float p3 = __int_as_float((__float_as_int(tn3) & ~3) | 3);
  const float t = r.t;
  unsigned vm = ((tf0 > 0.0f && p0 <= tf0 && p0 < t && ch.x != kEmptyChild) ? 1u : 0u) |
                ((tf1 > 0.0f && p1 <= tf1 && p1 < t && ch.y != kEmptyChild) ? 2u : 0u) |
                ((tf2 > 0.0f && p2 <= tf2 && p2 < t && ch.z != kEmptyChild) ? 4u : 0u) |
                ((tf3 > 0.0f && p3 <= tf3 && p3 < t && ch.w != kEmptyChild) ? 8u : 0u);
  if (vm == 0) {
    if (r.sp == 0) return kDone;
    r.ref = stack[--r.sp * stride];
    return kContinue;
  }
  // the lowest hit slot continues; the others (never slot 0) are pushed in slot order
  const unsigned rest = vm & (vm - 1);
  if (r.sp + __popc(rest) > limit) return kOverflow;
  if (rest & 2u) stack[r.sp++ * stride] = ch.y;
  if (rest & 4u) stack[r.sp++ * stride] = ch.z;
  if (rest & 8u) stack[r.sp++ * stride] = ch.w;
  r.ref = (vm & 1u) ? ch.x : ((vm & 2u) ? ch.y : ((vm & 4u) ? ch.z : ch.w));
  return kContinue;
}

// Test the leaf r.ref's triangles in primitive order, then pop.
template <bool ANY>
__device__ __forceinline__ StepResult leaf_step(const DevBVH& b, RayState& r, float eps, int* stack, int stride) {
  const uint32_t u = (uint32_t)r.ref;
  const uint32_t first = u & b.first_mask;
  const uint32_t cnt = (u >> b.leaf_shift) & b.count_mask;
  const float4* tp = b.tris + 3 * (size_t)first;
  for (uint32_t k = 0; k < cnt; k++) {
    const float4 a = __ldg(tp + 3 * k), e1 = __ldg(tp + 3 * k + 1), e2 = __ldg(tp + 3 * k + 2);
    if (tri_test(a, e1, e2, r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, eps, r.t)) {
      r.hit = __float_as_int(a.w);
      if (ANY) return kDone;
    }
  }
  if (r.sp == 0) return kDone;
  r.ref = stack[--r.sp * stride];
  return kContinue;
}

// leaf_step that tests at most P triangles per call: the rest of the leaf stays
// in r.ref (first + k, count - k), so a round of the persistent loop is not
// held up by the warp's largest leaf (P = 2 measured best; 1, 3 and 4 close).
// Each ray still tests its triangles in the same order, so results are those
// of leaf_step.
template <bool ANY, int P>
__device__ __forceinline__ StepResult leaf_step_part(const DevBVH& b, RayState& r, float eps, int* stack, int stride) {
  const uint32_t u = (uint32_t)r.ref;
  const uint32_t first = u & b.first_mask;
  const uint32_t cnt = (u >> b.leaf_shift) & b.count_mask;
  const uint32_t m = cnt < (uint32_t)P ? cnt : (uint32_t)P;
  const float4* tp = b.tris + 3 * (size_t)first;
  for (uint32_t k = 0; k < m; k++) {
    const float4 a = __ldg(tp + 3 * k), e1 = __ldg(tp + 3 * k + 1), e2 = __ldg(tp + 3 * k + 2);
    if (tri_test(a, e1, e2, r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, eps, r.t)) {
      r.hit = __float_as_int(a.w);
      if (ANY) return kDone;
    }
  }
  if (cnt > m) {
    r.ref = (int)(u + m - (m << b.leaf_shift));
    return kContinue;
  }
  if (r.sp == 0) return kDone;
  r.ref = stack[--r.sp * stride];
  return kContinue;
}

// Whole traversal of one ray by one thread. ANY = stop at the first hit
// (traverseMBVHShadow: nodes culled against maxDist, triangles accepted below
// it). `stack` is this thread's column of a [entries][stride] shared array.
// Returns false when the stack limit was reached (the ray's result is dropped).
template <bool ANY, bool FASTMM>
__device__ __forceinline__ bool traverse(const DevBVH& b, RayState& r, float eps, int* stack, int stride) {
  const int limit = b.stack_entries;
  while (true) {
    const StepResult s = r.ref >= 0 ? (ANY ? inner_step_any<FASTMM>(b, r, stack, stride, limit)
                                           : (FASTMM ? inner_step_sorted(b, r, stack, stride, limit)
                                                     : inner_step<false>(b, r, stack, stride, limit)))
                                    : leaf_step<ANY>(b, r, eps, stack, stride);
    if (s == kDone) return true;
    if (s == kOverflow) return false;
  }
}

// Persistent traversal with per-warp dynamic ray fetch. Each lane owns a ray
// and performs one step (an inner node or a leaf) per round; lanes whose ray
// finished take the next rays from a device cursor (one atomicAdd per warp),
// so a warp is not held back by its longest ray. A warp refills once at least
// REFILL of its lanes are idle (or all are): refilling costs a cursor atomic
// shared by every warp, a ballot and the new rays' loads and reciprocals, run
// by the whole warp for the lanes that refill, so batching refills pays for
// long incoherent traversals (the wavefront's extend) while short coherent
// queries refill at the first idle lane. Every ray still performs the
// reference's exact sequence of node tests, pushes, pops and triangle tests:
// only the interleaving across lanes changes.
//   IO::load(int i, float4& org, float4& dir, float& t0)
//   IO::store(int i, const RayState& r, bool overflow)
template <bool ANY, bool FASTMM, int REFILL, class IO>
__device__ __forceinline__ void trace_persistent(const DevBVH& b, int n, int* cursor, float eps, IO& io, int* stack,
                                                 int stride) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  const int limit = b.stack_entries;
  int rid = -1;
  bool exhausted = false;
  RayState r;
  r.ref = kEmptyChild;
  while (true) {
    if (!exhausted) {
      const unsigned m = __ballot_sync(FULL, rid < 0);
      if (m == FULL || __popc(m) >= REFILL) {
        const int leader = __ffs(m) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(cursor, __popc(m));
        base = __shfl_sync(FULL, base, leader);
        if (base + __popc(m) >= n) exhausted = true;
        if (rid < 0) {
          const int my = base + __popc(m & below);
          if (my < n) {
            float4 o, d;
            float t0;
            io.load(my, o, d, t0);
            ray_begin(r, o, d, t0);
            rid = my;
          }
        }
      }
    }
    if (__ballot_sync(FULL, rid >= 0) == 0) break;
    if (rid < 0) continue;
    const StepResult s = r.ref >= 0 ? (ANY ? inner_step_any<FASTMM>(b, r, stack, stride, limit)
                                           : (FASTMM ? inner_step_sorted(b, r, stack, stride, limit)
                                                     : inner_step<false>(b, r, stack, stride, limit)))
                                    : leaf_step_part<ANY, 2>(b, r, eps, stack, stride);
    if (s != kContinue) {
      io.store(rid, r, s == kOverflow);
      rid = -1;
    }
  }
}

// trace_persistent with a BVH and epsilon per lane: io.load(i, o, d, t0, b, eps)
// supplies the ray and the tree it is traced against (batches of jobs).
template <bool ANY, bool FASTMM, int REFILL, class IO>
__device__ __forceinline__ void trace_persistent_batch(int n, int* cursor, IO& io, int* stack, int stride) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  int rid = -1;
  bool exhausted = false;
  RayState r;
  r.ref = kEmptyChild;
  DevBVH b;
  float eps = 0.0f;
  while (true) {
    if (!exhausted) {
      const unsigned m = __ballot_sync(FULL, rid < 0);
      if (m == FULL || __popc(m) >= REFILL) {
        const int leader = __ffs(m) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(cursor, __popc(m));
        base = __shfl_sync(FULL, base, leader);
        if (base + __popc(m) >= n) exhausted = true;
        if (rid < 0) {
          const int my = base + __popc(m & below);
          if (my < n) {
            float4 o, d;
            float t0;
            io.load(my, o, d, t0, b, eps);
            ray_begin(r, o, d, t0);
            rid = my;
          }
        }
      }
    }
    if (__ballot_sync(FULL, rid >= 0) == 0) break;
    if (rid < 0) continue;
    const StepResult s =
        r.ref >= 0 ? (ANY ? inner_step_any<FASTMM>(b, r, stack, stride, b.stack_entries)
                          : (FASTMM ? inner_step_sorted(b, r, stack, stride, b.stack_entries)
                                    : inner_step<false>(b, r, stack, stride, b.stack_entries)))
                   : leaf_step_part<ANY, 2>(b, r, eps, stack, stride);
    if (s != kContinue) {
      io.store(rid, r, s == kOverflow);
      rid = -1;
    }
  }
}

}  // namespace ct
