// Ray queries on the 8-wide quantised BVH (WNode8).
//
// Boxes: the builder rounds child bounds outward so that fl(p + 2^e q)
// contains the child; the slab test evaluates each plane as one fused
// multiply-add t = q A + B with per-node constants and widens every interval
// by a bound of its rounding error (SlabSetup), so no box that the ray
// touches in exact arithmetic is rejected. Culling against the best hit keeps
// the margin 1 + 2 gamma(3) of Ize ("Robust BVH ray traversal", JCGT 2013).
//
// Triangles: the watertight test of Woop, Benthin and Wald (JCGT 2013) in FP32:
// shear to ray space, edge functions U, V, W, no epsilon. Each edge function
// carries a first-order bound of its FP32 rounding error (from the magnitudes
// of its operands). A triangle is a certain hit when all three functions
// exceed their bounds with one sign, a certain miss when two exceed them with
// opposite signs, and uncertain otherwise. Uncertain triangles, and certain
// hits whose t lies within the combined t error bound of the best hit, are
// kept as candidates (up to kCand per ray); after traversal the best hit and
// the candidates are re-tested with the same algorithm in FP64 and the
// nearest FP64 hit wins (equal t: lower primitive id). A best hit whose t
// error bound exceeds 9e-6 relative is re-tested the same way, so reported t
// stay within 1e-5 of the exact distance. A ray with more candidates is traced again
// entirely in FP64. The result therefore equals an FP64 watertight closest
// hit over all triangles.
#include <cuda_runtime.h>

#include <algorithm>

#include "ct_internal.h"
#include "trace.cuh"

namespace ct {
namespace {

constexpr int kWStack = 128;  // local-memory stack entries per thread
constexpr float kU = 5.9604645e-08f;          // 2^-24
constexpr float kFarScale = 1.00000036f;      // 1 + 2 * gamma(3), gamma(n) = n u / (1 - n u)
constexpr float kTRel = 9e-6f;                // a best hit whose t bound exceeds this (relative) is re-tested in FP64

struct WRay {
  float ox, oy, oz, dx, dy, dz;
  float ix, iy, iz;   // reciprocal direction (zero components replaced by a huge value)
  int kx, ky, kz;     // watertight axis permutation
  float Sx, Sy, Sz;   // shear constants
  float tmax;
};

__device__ __forceinline__ float comp3(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

__device__ __forceinline__ float safe_rcp(float d) {
  return fabsf(d) > 1e-30f ? __frcp_rn(d) : copysignf(1e30f, d);
}

__device__ __forceinline__ void setup(const float4 o, const float4 d, WRay& r) {
  r.ox = o.x, r.oy = o.y, r.oz = o.z, r.dx = d.x, r.dy = d.y, r.dz = d.z, r.tmax = d.w;
  r.ix = safe_rcp(d.x), r.iy = safe_rcp(d.y), r.iz = safe_rcp(d.z);
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  r.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  r.kx = r.kz == 2 ? 0 : r.kz + 1;
  r.ky = r.kx == 2 ? 0 : r.kx + 1;
  if (comp3(d.x, d.y, d.z, r.kz) < 0.0f) {
    const int t = r.kx;
    r.kx = r.ky;
    r.ky = t;
  }
  const float dz = comp3(d.x, d.y, d.z, r.kz);
  r.Sx = __fdiv_rn(comp3(d.x, d.y, d.z, r.kx), dz);
  r.Sy = __fdiv_rn(comp3(d.x, d.y, d.z, r.ky), dz);
  r.Sz = __frcp_rn(dz);
}

// FP32 watertight test. Returns 0 certain miss, 1 certain hit, 2 uncertain;
// t and terr (bound on |t - t_exact|) are set for 1 and 2 (for an uncertain
// edge-on triangle t = 0, terr = +inf: any distance is possible).
__device__ __forceinline__ int tri32(const WRay& r, const float4& a4, const float4& b4, const float4& c4, float& t,
                                     float& terr) {
  // ray-relative vertices, permuted to (kx, ky, kz)
  const float akx = comp3(a4.x, a4.y, a4.z, r.kx) - comp3(r.ox, r.oy, r.oz, r.kx);
  const float aky = comp3(a4.x, a4.y, a4.z, r.ky) - comp3(r.ox, r.oy, r.oz, r.ky);
  const float akz = comp3(a4.x, a4.y, a4.z, r.kz) - comp3(r.ox, r.oy, r.oz, r.kz);
  const float bkx = comp3(b4.x, b4.y, b4.z, r.kx) - comp3(r.ox, r.oy, r.oz, r.kx);
  const float bky = comp3(b4.x, b4.y, b4.z, r.ky) - comp3(r.ox, r.oy, r.oz, r.ky);
  const float bkz = comp3(b4.x, b4.y, b4.z, r.kz) - comp3(r.ox, r.oy, r.oz, r.kz);
  const float ckx = comp3(c4.x, c4.y, c4.z, r.kx) - comp3(r.ox, r.oy, r.oz, r.kx);
  const float cky = comp3(c4.x, c4.y, c4.z, r.ky) - comp3(r.ox, r.oy, r.oz, r.ky);
  const float ckz = comp3(c4.x, c4.y, c4.z, r.kz) - comp3(r.ox, r.oy, r.oz, r.kz);
  // a difference of two floats is rounded once, relative to its own value:
  // the ray-relative coordinates carry u |x| of error
  const float mAkx = fabsf(akx), mAky = fabsf(aky), mAkz = fabsf(akz);
  const float mBkx = fabsf(bkx), mBky = fabsf(bky), mBkz = fabsf(bkz);
  const float mCkx = fabsf(ckx), mCky = fabsf(cky), mCkz = fabsf(ckz);
  const float Ax = akx - r.Sx * akz, Ay = aky - r.Sy * akz;
  const float Bx = bkx - r.Sx * bkz, By = bky - r.Sy * bkz;
  const float Cx = ckx - r.Sx * ckz, Cy = cky - r.Sy * ckz;
  const float aSx = fabsf(r.Sx), aSy = fabsf(r.Sy);
  const float mAx = mAkx + aSx * mAkz, mAy = mAky + aSy * mAkz;
  const float mBx = mBkx + aSx * mBkz, mBy = mBky + aSy * mBkz;
  const float mCx = mCkx + aSx * mCkz, mCy = mCky + aSy * mCkz;
  const float U = Cx * By - Cy * Bx;
  const float V = Ax * Cy - Ay * Cx;
  const float W = Bx * Ay - By * Ax;
  // 4x the first-order bound: 3u per sheared coordinate, 2u for the products and difference
  const float eU = (12.0f * kU) * (fabsf(Cx) * mBy + fabsf(By) * mCx + fabsf(Cy) * mBx + fabsf(Bx) * mCy) +
                   (8.0f * kU) * (fabsf(Cx * By) + fabsf(Cy * Bx));
  const float eV = (12.0f * kU) * (fabsf(Ax) * mCy + fabsf(Cy) * mAx + fabsf(Ay) * mCx + fabsf(Cx) * mAy) +
                   (8.0f * kU) * (fabsf(Ax * Cy) + fabsf(Ay * Cx));
  const float eW = (12.0f * kU) * (fabsf(Bx) * mAy + fabsf(Ay) * mBx + fabsf(By) * mAx + fabsf(Ax) * mBy) +
                   (8.0f * kU) * (fabsf(Bx * Ay) + fabsf(By * Ax));
  const bool up = U > eU, un = U < -eU, vp = V > eV, vn = V < -eV, wp = W > eW, wn = W < -eW;
  if ((up || vp || wp) && (un || vn || wn)) return 0;
  const bool certain = (up && vp && wp) || (un && vn && wn);
  // distance from the triangle's plane, t = ((a - o) . n) / (d . n) with
  // n = (b - a) x (c - a), and a first-order bound of its rounding (x2)
  const float e1x = b4.x - a4.x, e1y = b4.y - a4.y, e1z = b4.z - a4.z;
  const float e2x = c4.x - a4.x, e2y = c4.y - a4.y, e2z = c4.z - a4.z;
  const float nx = e1y * e2z - e1z * e2y, ny = e1z * e2x - e1x * e2z, nz = e1x * e2y - e1y * e2x;
  const float enx = (6.0f * kU) * (fabsf(e1y * e2z) + fabsf(e1z * e2y));
  const float eny = (6.0f * kU) * (fabsf(e1z * e2x) + fabsf(e1x * e2z));
  const float enz = (6.0f * kU) * (fabsf(e1x * e2y) + fabsf(e1y * e2x));
  const float aox = a4.x - r.ox, aoy = a4.y - r.oy, aoz = a4.z - r.oz;
  const float num = aox * nx + aoy * ny + aoz * nz;
  const float den = r.dx * nx + r.dy * ny + r.dz * nz;
  const float enum_ = fabsf(aox) * enx + fabsf(aoy) * eny + fabsf(aoz) * enz +
                      (4.0f * kU) * (fabsf(aox * nx) + fabsf(aoy * ny) + fabsf(aoz * nz));
  const float eden = fabsf(r.dx) * enx + fabsf(r.dy) * eny + fabsf(r.dz) * enz +
                     (3.0f * kU) * (fabsf(r.dx * nx) + fabsf(r.dy * ny) + fabsf(r.dz * nz));
  if (!(fabsf(den) > 2.0f * eden)) {
    // (nearly) parallel to the plane in FP32: distance unknown
    t = 0.0f;
    terr = __int_as_float(0x7f800000);
    return 2;
  }
  t = __fdiv_rn(num, den);
  terr = fabsf(t) * (2.0f * (enum_ / fmaxf(fabsf(num), 1e-37f) + eden / fabsf(den)) + 4.0f * kU);
  if (!(enum_ < fabsf(num))) terr = fmaxf(terr, 2.0f * enum_ / fabsf(den));  // t near zero
  return certain ? 1 : 2;
}

__device__ __forceinline__ double comp3d(double x, double y, double z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

// The same test in FP64 (no contraction), the arbiter for candidates.
__device__ __forceinline__ bool tri64(double ox, double oy, double oz, int kx, int ky, int kz, double Sx, double Sy,
                                      double Sz, const float4& a4, const float4& b4, const float4& c4, double& t) {
  const double akx = __dsub_rn(comp3d(a4.x, a4.y, a4.z, kx), comp3d(ox, oy, oz, kx));
  const double aky = __dsub_rn(comp3d(a4.x, a4.y, a4.z, ky), comp3d(ox, oy, oz, ky));
  const double akz = __dsub_rn(comp3d(a4.x, a4.y, a4.z, kz), comp3d(ox, oy, oz, kz));
  const double bkx = __dsub_rn(comp3d(b4.x, b4.y, b4.z, kx), comp3d(ox, oy, oz, kx));
  const double bky = __dsub_rn(comp3d(b4.x, b4.y, b4.z, ky), comp3d(ox, oy, oz, ky));
  const double bkz = __dsub_rn(comp3d(b4.x, b4.y, b4.z, kz), comp3d(ox, oy, oz, kz));
  const double ckx = __dsub_rn(comp3d(c4.x, c4.y, c4.z, kx), comp3d(ox, oy, oz, kx));
  const double cky = __dsub_rn(comp3d(c4.x, c4.y, c4.z, ky), comp3d(ox, oy, oz, ky));
  const double ckz = __dsub_rn(comp3d(c4.x, c4.y, c4.z, kz), comp3d(ox, oy, oz, kz));
  const double Ax = __dsub_rn(akx, __dmul_rn(Sx, akz)), Ay = __dsub_rn(aky, __dmul_rn(Sy, akz));
  const double Bx = __dsub_rn(bkx, __dmul_rn(Sx, bkz)), By = __dsub_rn(bky, __dmul_rn(Sy, bkz));
  const double Cx = __dsub_rn(ckx, __dmul_rn(Sx, ckz)), Cy = __dsub_rn(cky, __dmul_rn(Sy, ckz));
  const double U = __dsub_rn(__dmul_rn(Cx, By), __dmul_rn(Cy, Bx));
  const double V = __dsub_rn(__dmul_rn(Ax, Cy), __dmul_rn(Ay, Cx));
  const double W = __dsub_rn(__dmul_rn(Bx, Ay), __dmul_rn(By, Ax));
  if ((U < 0.0 || V < 0.0 || W < 0.0) && (U > 0.0 || V > 0.0 || W > 0.0)) return false;
  const double det = __dadd_rn(__dadd_rn(U, V), W);
  if (det == 0.0) return false;
  const double Az = __dmul_rn(Sz, akz), Bz = __dmul_rn(Sz, bkz), Cz = __dmul_rn(Sz, ckz);
  const double T = __dadd_rn(__dadd_rn(__dmul_rn(U, Az), __dmul_rn(V, Bz)), __dmul_rn(W, Cz));
  t = __ddiv_rn(T, det);
  return t > 0.0;
}

struct Ray64 {
  double ox, oy, oz, Sx, Sy, Sz, tmax;
  int kx, ky, kz;
};
__device__ __forceinline__ Ray64 ray64(const WRay& r) {
  Ray64 q;
  q.ox = r.ox, q.oy = r.oy, q.oz = r.oz;
  q.kx = r.kx, q.ky = r.ky, q.kz = r.kz;
  const double dkz = comp3d(r.dx, r.dy, r.dz, r.kz);
  q.Sx = __ddiv_rn(comp3d(r.dx, r.dy, r.dz, r.kx), dkz);
  q.Sy = __ddiv_rn(comp3d(r.dx, r.dy, r.dz, r.ky), dkz);
  q.Sz = __ddiv_rn(1.0, dkz);
  q.tmax = r.tmax;
  return q;
}
__device__ __forceinline__ bool tri64(const Ray64& q, const float4* tris, uint32_t slot, double& t) {
  const float4* tr = tris + 3 * (size_t)slot;
  return tri64(q.ox, q.oy, q.oz, q.kx, q.ky, q.kz, q.Sx, q.Sy, q.Sz, __ldg(tr), __ldg(tr + 1), __ldg(tr + 2), t) &&
         t < q.tmax;
}

// Slab distances of a node's eight slots, set up once per node and ray.
// Per axis a, with s = 2^(e - 127) the quantisation step and inv = 1/d:
//   A = s * inv (exact: a power of two times a float),  B = (p - o) * inv,
// so a plane q (0..255) lies at t = q * A + B, one fused multiply-add. Only the
// ray's near plane (lo for inv >= 0, hi otherwise) and far plane of each axis
// are evaluated, so no min/max per axis is needed. Every computed t differs
// from the exact distance (L - o) / d of the builder's outward-rounded plane
// L = fl(p + s q) by at most
//   E = 5u (255 |A| + |B| + |p inv|) + 1e-30      (u = 2^-24)
// (the rounding of inv, of p - o, of the product and of the FMA, and the
// half-ulp by which p + s q may lie inside L; the last term covers underflow).
// E is folded into the offsets: near planes use Bn = B - E, far planes
// Bf = B + E (E is raised by the rounding of those two sums), so a slot's
// [max near, min far] interval contains the exact one and no box the ray
// touches is rejected.
struct SlabSetup {
  uint32_t nq[3][2], fq[3][2];  // near / far plane bytes of slots 0-3 and 4-7, per axis
  float A[3], Bn[3], Bf[3];
};

__device__ __forceinline__ void slab_axis(float p, float e_scale, float o, float inv, uint2 lo, uint2 hi,
                                          uint32_t* nq, uint32_t* fq, float& A, float& Bn, float& Bf) {
  A = __fmul_rn(e_scale, inv);
  const float B = __fmul_rn(__fsub_rn(p, o), inv);
  const float u = 5.9604645e-08f;
  float E = (5.0f * u) * (255.0f * fabsf(A) + fabsf(B) + fabsf(__fmul_rn(p, inv))) + 1e-30f;
  E = E + (2.0f * u) * (fabsf(B) + E);  // the rounding of B -/+ E below
  Bn = __fsub_rn(B, E);
  Bf = __fadd_rn(B, E);
  const bool pos = inv >= 0.0f;
  nq[0] = pos ? lo.x : hi.x, nq[1] = pos ? lo.y : hi.y;
  fq[0] = pos ? hi.x : lo.x, fq[1] = pos ? hi.y : lo.y;
}

__device__ __forceinline__ void slab_setup(const WNode8& n, float ox, float oy, float oz, float ix, float iy, float iz,
                                           SlabSetup& S) {
  const uint2* qlo = reinterpret_cast<const uint2*>(&n.qlo[0][0]);
  const uint2* qhi = reinterpret_cast<const uint2*>(&n.qhi[0][0]);
  slab_axis(n.px, __int_as_float((int)n.e[0] << 23), ox, ix, qlo[0], qhi[0], S.nq[0], S.fq[0], S.A[0], S.Bn[0],
            S.Bf[0]);
  slab_axis(n.py, __int_as_float((int)n.e[1] << 23), oy, iy, qlo[1], qhi[1], S.nq[1], S.fq[1], S.A[1], S.Bn[1],
            S.Bf[1]);
  slab_axis(n.pz, __int_as_float((int)n.e[2] << 23), oz, iz, qlo[2], qhi[2], S.nq[2], S.fq[2], S.A[2], S.Bn[2],
            S.Bf[2]);
}

__device__ __forceinline__ float qbyte(const uint32_t* w, int i) { return (float)((w[i >> 2] >> (8 * (i & 3))) & 0xffu); }

// Entry distance of slot i (clamped at 0), or +inf when the slot's box is
// missed or begins beyond tfar.
__device__ __forceinline__ float slot_test(const SlabSetup& S, int i, float tfar) {
  const float nx = __fmaf_rn(qbyte(S.nq[0], i), S.A[0], S.Bn[0]), fx = __fmaf_rn(qbyte(S.fq[0], i), S.A[0], S.Bf[0]);
  const float ny = __fmaf_rn(qbyte(S.nq[1], i), S.A[1], S.Bn[1]), fy = __fmaf_rn(qbyte(S.fq[1], i), S.A[1], S.Bf[1]);
  const float nz = __fmaf_rn(qbyte(S.nq[2], i), S.A[2], S.Bn[2]), fz = __fmaf_rn(qbyte(S.fq[2], i), S.A[2], S.Bf[2]);
  const float tn = fmaxf(fmaxf(nx, ny), fmaxf(nz, 0.0f));
  const float tf = fminf(fminf(fx, fy), fminf(fz, tfar));
  return tn <= tf ? tn : __int_as_float(0x7f800000);
}

__device__ __forceinline__ void load_node(const WNode8* nodes, uint32_t i, WNode8& n) {
  const float4* s = reinterpret_cast<const float4*>(nodes + i);
  float4* d = reinterpret_cast<float4*>(&n);
#pragma unroll
  for (int k = 0; k < 5; k++) d[k] = __ldg(s + k);
}

__device__ __forceinline__ uint32_t meta_at(const WNode8& n, int i) {
  const uint32_t* w = reinterpret_cast<const uint32_t*>(n.meta);
  return ((i < 4 ? w[0] : w[1]) >> (8 * (i & 3))) & 0xffu;
}

// A warp refills its idle lanes from the cursor once this many are idle (or
// all are): fewer cursor atomics and refill passes than refilling at the
// first idle lane. Queries (10M-triangle soup, incoherent rays): 4 ahead of 8
// and 16; frames on the wide tree: 8.
constexpr int kWideRefill = 4;
constexpr int kWideFrameRefill = 8;

// Whole traversal in FP64 triangle tests (boxes as above, culled with the FP64
// best distance rounded up): the fallback for rays with too many candidates.
template <bool ANY>
__device__ bool trace_fp64(const DevWBVH& b, const WRay& r, uint32_t* st_node, float* st_t, uint32_t* err, int& best,
                           double& tb) {
  const Ray64 q = ray64(r);
  best = -1;
  tb = q.tmax;
  int sp = 0;
  st_node[sp] = 0, st_t[sp] = 0.0f, sp++;
  while (sp > 0) {
    sp--;
    const uint32_t ni = st_node[sp];
    const float far = __double2float_ru(tb) * kFarScale;
    if (st_t[sp] > far) continue;
    WNode8 n;
    SlabSetup S;
    load_node(b.nodes, ni, n);
    slab_setup(n, r.ox, r.oy, r.oz, r.ix, r.iy, r.iz, S);
    for (int i = 0; i < 8; i++) {
      const uint32_t m = meta_at(n, i);
      if (!m) continue;
      const float tn = slot_test(S, i, far);
      if (!(tn <= far)) continue;
      if (m & 0x80u) {
        if (sp >= kWStack) {
          atomicOr(err, kErrStackOverflow);
          continue;
        }
        st_node[sp] = n.child_base + (m & 7u), st_t[sp] = tn, sp++;
        continue;
      }
      const uint32_t cnt = m >> 5, off = m & 31u;
      for (uint32_t k = 0; k < cnt; k++) {
        double t;
        const uint32_t slot = n.prim_base + off + k;
        if (!tri64(q, b.tris, slot, t)) continue;
        const int prim = __float_as_int(__ldg(b.tris + 3 * (size_t)slot).w);
        if (ANY) {
          best = prim;
          tb = t;
          return true;
        }
        if (t < tb || (t == tb && prim < best)) tb = t, best = prim;
      }
    }
  }
  return best >= 0;
}

constexpr uint32_t kLeafEntry = 0x80000000u;  // stack entry: bit 31 leaf, bits 29-30 count, 0-28 first triangle

// Settlement records: a ray whose closest hit (or occlusion) FP32 could not
// decide is not settled in the traversal kernel, where the few lanes doing
// FP64 work would hold their warp's other lanes idle (binary64 runs at a small
// fraction of the binary32 rate on this GPU). Instead the traversal appends a
// 32-byte record and k_wide_settle re-tests the records' triangles in FP64,
// one record per thread, so its warps run full.
//   word 0  ray index
//   word 1  the best FP32 hit's triangle slot, or -1
//   word 2  candidate count (<= kRecCand), bit 31: trace the ray entirely in FP64
//   words 3-7  candidate triangle slots
constexpr int kRecCand = 5;
constexpr uint32_t kRecFull = 0x80000000u;

// Persistent traversal: each lane owns a ray and takes one step per round —
// an inner node (eight slab tests; inner children and leaf groups pushed,
// the nearest on top) or one leaf group (up to three triangle tests) — so
// the warp's lanes do similar work each round; a lane whose ray is done takes
// the next ray from the device cursor (one atomicAdd per warp). A ray that
// would overflow the stack or keep more than kRecCand candidates is recorded
// for a traversal entirely in FP64.
//   counters[0]  ray fetch cursor;  counters[1]  records written
template <bool ANY>
// 8 resident blocks of 128 threads per SM (64 registers): measured ahead of 6 (80 registers)
__global__ void __launch_bounds__(128, 8) k_trace_wide(const DevWBVH b, const float4* __restrict__ org,
                                                    const float4* __restrict__ dir, int32_t* __restrict__ hit_out,
                                                    float* __restrict__ t_out, uint8_t* __restrict__ occ_out,
                                                    uint32_t n, int* counters, uint4* recs,
                                                    unsigned long long* stats) {
  uint32_t st_node[kWStack];
  float st_t[kWStack];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  unsigned long long n_rays = 0;
  int rid = -1;
  bool exhausted = false;
  WRay r;
  int best = -1, nc = 0, sp = 0;
  float tb = 0.0f, tberr = 0.0f;
  bool overflow = false, occluded = false;
  uint32_t cur = 0;        // the entry visited next, when have_cur (a node's nearest hit slot)
  bool have_cur = false;
  uint32_t cand[kRecCand];
  float cand_lo[kRecCand];
  while (true) {
    if (!exhausted) {
      const unsigned m = __ballot_sync(FULL, rid < 0);
      if (m == FULL || __popc(m) >= kWideRefill) {  // refill once kWideRefill lanes are idle
        const int leader = __ffs(m) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(counters, __popc(m));
        base = __shfl_sync(FULL, base, leader);
        if ((uint32_t)(base + __popc(m)) >= n) exhausted = true;
        if (rid < 0) {
          const int my = base + __popc(m & below);
          if ((uint32_t)my < n) {
            setup(__ldg(org + my), __ldg(dir + my), r);
            rid = my;
            n_rays++;
            best = -1, nc = 0, tb = r.tmax, tberr = 0.0f, overflow = false, occluded = false;
            sp = 0, cur = 0, have_cur = true;  // the root
          }
        }
      }
    }
    if (__ballot_sync(FULL, rid >= 0) == 0) break;
    bool record = false;
    if (rid >= 0) {
      // ---- one step
      const float far = (tb + tberr) * kFarScale;
      if (!have_cur)
        while (sp > 0 && st_t[sp - 1] > far) sp--;  // culled entries
      bool finished = (!have_cur && sp == 0) || overflow || (ANY && occluded);
      if (!finished) {
        const uint32_t ent = have_cur ? cur : st_node[--sp];
        have_cur = false;
        if (ent & kLeafEntry) {
          const uint32_t cnt = (ent >> 29) & 3u, first = ent & 0x1fffffffu;
          for (uint32_t k = 0; k < cnt; k++) {
            const uint32_t slot = first + k;
            const float4* tr = b.tris + 3 * (size_t)slot;
            float t, terr;
            const int res = tri32(r, __ldg(tr), __ldg(tr + 1), __ldg(tr + 2), t, terr);
            if (res == 0) continue;
            if (res == 1 && t - terr > 0.0f && t + terr < tb - tberr) {
              // certainly in range and certainly nearer than the best so far
              best = (int)slot, tb = t, tberr = terr;
              if (ANY) {
                occluded = true;
                break;
              }
              continue;
            }
            if (!(t - terr < tb + tberr)) continue;  // certainly beyond the best (or the ray's end)
            if (res == 1 && t - terr > 0.0f && t < tb && t + terr < tb + tberr) {
              // a certain hit nearer than the best within their errors: FP64 orders them
              if (best >= 0) {
                if (nc < kRecCand) cand[nc] = (uint32_t)best, cand_lo[nc] = tb - tberr, nc++;
                else overflow = true;
              }
              best = (int)slot, tb = t, tberr = terr;
              continue;
            }
            if (nc < kRecCand) cand[nc] = slot, cand_lo[nc] = t - terr, nc++;
            else overflow = true;
          }
        } else {
          WNode8 nd;
          SlabSetup S;
          load_node(b.nodes, ent, nd);
          slab_setup(nd, r.ox, r.oy, r.oz, r.ix, r.iy, r.iz, S);
          // the nearest hit slot is visited next without a stack round trip; the
          // others are pushed (a slot displaced as nearest is pushed when replaced).
          // Closest hit also keeps the second nearest in a register and pushes it
          // last, so it is the next entry popped (closer hits found sooner cull
          // more; any hit stops at its first hit, where the order only costs)
          float tcur = __int_as_float(0x7f800000), tsec = __int_as_float(0x7f800000);
          uint32_t sec = 0;
          bool have_sec = false;
#pragma unroll
          for (int i = 0; i < 8; i++) {
            const uint32_t m = meta_at(nd, i);
            if (!m) continue;
            const float tn = slot_test(S, i, far);
            if (!(tn <= far)) continue;
            const uint32_t ce = (m & 0x80u) ? nd.child_base + (m & 7u)
                                            : (kLeafEntry | ((m >> 5) << 29) | (nd.prim_base + (m & 31u)));
            uint32_t pe = ce;
            float pt = tn;
            if (tn < tcur) {
              pe = cur, pt = tcur;
              cur = ce, tcur = tn;
              if (!have_cur) {
                have_cur = true;
                continue;
              }
            }
            if (!ANY) {
              if (!have_sec) {
                sec = pe, tsec = pt, have_sec = true;
                continue;
              }
              if (pt < tsec) {
                const uint32_t e2 = sec;
                const float t2 = tsec;
                sec = pe, tsec = pt;
                pe = e2, pt = t2;
              }
            }
            if (sp >= kWStack) {
              overflow = true;  // settled by the full FP64 traversal
              continue;
            }
            st_node[sp] = pe, st_t[sp] = pt, sp++;
          }
          if (!ANY && have_sec) {
            if (sp >= kWStack) overflow = true;
            else st_node[sp] = sec, st_t[sp] = tsec, sp++;
          }
        }
        finished = (!have_cur && sp == 0) || overflow || (ANY && occluded);
      }
      if (finished) {
        if (!overflow) {
          int k2 = 0;
          for (int k = 0; k < nc; k++)
            if (cand_lo[k] < tb + tberr) cand[k2] = cand[k], cand_lo[k2] = cand_lo[k], k2++;
          nc = k2;
        }
        if (ANY && !occluded && best >= 0) occluded = true;
        record = !(ANY && occluded) && (overflow || nc > 0 || (!ANY && best >= 0 && tberr > kTRel * tb));
        if (!record) {
          if (ANY) {
            occ_out[rid] = occluded ? 1 : 0;
          } else {
            hit_out[rid] = best >= 0 ? __float_as_int(__ldg(b.tris + 3 * (size_t)best).w) : -1;
            t_out[rid] = best >= 0 ? tb : r.tmax;
          }
          rid = -1;
        }
      }
    }
    // ---- records of the rays FP32 could not settle (one atomic per warp)
    const unsigned rm = __ballot_sync(FULL, record);
    if (rm) {
      const int leader = __ffs(rm) - 1;
      int base = 0;
      if (lane == leader) base = atomicAdd(counters + 1, __popc(rm));
      base = __shfl_sync(FULL, base, leader);
      if (record) {
        uint4* rec = recs + 2 * (size_t)(base + __popc(rm & below));
        uint32_t c[kRecCand];
#pragma unroll
        for (int k = 0; k < kRecCand; k++) c[k] = k < nc ? cand[k] : 0u;
        rec[0] = make_uint4((uint32_t)rid, (uint32_t)best, (uint32_t)nc | (overflow ? kRecFull : 0u), c[0]);
        rec[1] = make_uint4(c[1], c[2], c[3], c[4]);
        rid = -1;
      }
    }
  }
  if (stats) atomicAdd(stats + 0, n_rays);
}

// FP64 settlement of the records: the best FP32 hit and the candidates are
// re-tested with the watertight test in FP64 and the nearest FP64 hit wins
// (equal t: lower primitive id); a record flagged kRecFull is traced again
// entirely in FP64 (trace_fp64). One record per thread, grid-stride over the
// count the traversal left in counters[1].
template <bool ANY>
__global__ void __launch_bounds__(128) k_wide_settle(const DevWBVH b, const float4* __restrict__ org,
                                                     const float4* __restrict__ dir, int32_t* __restrict__ hit_out,
                                                     float* __restrict__ t_out, uint8_t* __restrict__ occ_out,
                                                     const int* counters, const uint4* __restrict__ recs, uint32_t* err,
                                                     unsigned long long* stats) {
  uint32_t st_node[kWStack];
  float st_t[kWStack];
  const int nrec = counters[1];
  unsigned long long n_retest = 0, n_full = 0, n_tbound = 0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nrec; i += gridDim.x * blockDim.x) {
    const uint4 r0 = recs[2 * (size_t)i], r1 = recs[2 * (size_t)i + 1];
    const int rid = (int)r0.x, best = (int)r0.y;
    const uint32_t nc = r0.z & 0xffu;
    const uint32_t cand[kRecCand] = {r0.w, r1.x, r1.y, r1.z, r1.w};
    WRay r;
    setup(__ldg(org + rid), __ldg(dir + rid), r);
    int out_prim = -1;
    float out_t = r.tmax;
    if (r0.z & kRecFull) {
      n_full++;
      double t64;
      int prim;
      const bool h = trace_fp64<ANY>(b, r, st_node, st_t, err, prim, t64);
      out_prim = h ? prim : -1;
      out_t = h ? (float)t64 : r.tmax;
    } else {
      n_retest++;
      n_tbound += nc == 0;
      const Ray64 q = ray64(r);
      int bp = -1;
      double bt = q.tmax;
      auto consider = [&](uint32_t slot) {
        double t;
        if (!tri64(q, b.tris, slot, t)) return;
        const int prim = __float_as_int(__ldg(b.tris + 3 * (size_t)slot).w);
        if (t < bt || (t == bt && prim < bp)) bt = t, bp = prim;
      };
      if (best >= 0) consider((uint32_t)best);
      for (uint32_t k = 0; k < nc && k < (uint32_t)kRecCand; k++) consider(cand[k]);
      out_prim = bp;
      out_t = bp >= 0 ? (float)bt : r.tmax;
    }
    if (ANY) {
      occ_out[rid] = out_prim >= 0 ? 1 : 0;
    } else {
      hit_out[rid] = out_prim;
      t_out[rid] = out_t;
    }
  }
  if (stats) {
    if (n_retest) atomicAdd(stats + 1, n_retest);
    if (n_full) atomicAdd(stats + 2, n_full);
    if (n_tbound) atomicAdd(stats + 3, n_tbound);
  }
}

// ---------------------------------------------------------------- frames on the wide tree
// The wavefront's closest-hit and shadow stages on the quantised tree, with the
// reference's Moller-Trumbore test and triangle epsilon (src/Core/Triangle.cuh:13-44,
// edges formed as p1 - p0 and p2 - p0 exactly as the quad layout stores them)
// instead of the watertight FP32/FP64 pair: the boxes are conservative, so the
// set of triangles a ray can hit is the reference's; only the visit order (and
// with it the winner of an exact t tie) differs.
struct MRay {
  float ox, oy, oz, dx, dy, dz, ix, iy, iz;
};

// Persistent, one step per round (as k_trace_wide). IO::load(i, o, d, t0, bvh, eps),
// IO::store(i, hit, t, overflow).
template <bool ANY, class IO>
__device__ __forceinline__ void trace_wide_mt(int n, int* cursor, IO& io, uint32_t* st_node, float* st_t) {
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  int rid = -1;
  bool exhausted = false;
  MRay r;
  DevWBVH b;
  float eps = 0.0f, t = 0.0f;
  int hit = -1, sp = 0;
  bool overflow = false;
  while (true) {
    if (!exhausted) {
      const unsigned m = __ballot_sync(FULL, rid < 0);
      if (m == FULL || __popc(m) >= kWideFrameRefill) {  // refill once 8 lanes are idle
        const int leader = __ffs(m) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(cursor, __popc(m));
        base = __shfl_sync(FULL, base, leader);
        if (base + __popc(m) >= n) exhausted = true;
        if (rid < 0) {
          const int my = base + __popc(m & below);
          if (my < n) {
            float4 o, d;
            io.load(my, o, d, t, b, eps);
            r.ox = o.x, r.oy = o.y, r.oz = o.z, r.dx = d.x, r.dy = d.y, r.dz = d.z;
            r.ix = safe_rcp(d.x), r.iy = safe_rcp(d.y), r.iz = safe_rcp(d.z);
            hit = -1, overflow = false;
            st_node[0] = 0, st_t[0] = 0.0f, sp = 1;
            rid = my;
          }
        }
      }
    }
    if (__ballot_sync(FULL, rid >= 0) == 0) break;
    if (rid < 0) continue;
    const float far = t * kFarScale;
    while (sp > 0 && st_t[sp - 1] > far) sp--;
    bool finished = sp == 0;
    if (!finished) {
      const uint32_t ent = st_node[--sp];
      if (ent & kLeafEntry) {
        const uint32_t cnt = (ent >> 29) & 3u, first = ent & 0x1fffffffu;
        for (uint32_t k = 0; k < cnt; k++) {
          const float4* tr = b.tris + 3 * (size_t)(first + k);
          const float4 a = __ldg(tr), p1 = __ldg(tr + 1), p2 = __ldg(tr + 2);
          const float4 e1 = make_float4(__fsub_rn(p1.x, a.x), __fsub_rn(p1.y, a.y), __fsub_rn(p1.z, a.z), 0.0f);
          const float4 e2 = make_float4(__fsub_rn(p2.x, a.x), __fsub_rn(p2.y, a.y), __fsub_rn(p2.z, a.z), 0.0f);
          if (tri_test(a, e1, e2, r.ox, r.oy, r.oz, r.dx, r.dy, r.dz, eps, t)) {
            hit = __float_as_int(a.w);
            if (ANY) break;
          }
        }
        finished = ANY && hit >= 0;
      } else {
        WNode8 nd;
        SlabSetup S;
        load_node(b.nodes, ent, nd);
        slab_setup(nd, r.ox, r.oy, r.oz, r.ix, r.iy, r.iz, S);
        const int sp0 = sp;
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const uint32_t m = meta_at(nd, i);
          if (!m) continue;
          const float tn = slot_test(S, i, far);
          if (!(tn <= far)) continue;
          if (sp >= kWStack) {
            overflow = true;
            continue;
          }
          st_node[sp] = (m & 0x80u) ? nd.child_base + (m & 7u)
                                    : (kLeafEntry | ((m >> 5) << 29) | (nd.prim_base + (m & 31u)));
          st_t[sp] = tn;
          sp++;
        }
        if (!ANY && sp - sp0 > 1) {
          int bi = sp0;
          for (int k = sp0 + 1; k < sp; k++)
            if (st_t[k] < st_t[bi]) bi = k;
          const uint32_t tnode = st_node[bi];
          const float tt = st_t[bi];
          st_node[bi] = st_node[sp - 1], st_t[bi] = st_t[sp - 1];
          st_node[sp - 1] = tnode, st_t[sp - 1] = tt;
        }
      }
      finished = finished || sp == 0 || overflow;
    }
    if (!finished) continue;
    io.store(rid, hit, t, overflow);
    rid = -1;
  }
}

struct WExtendIO {
  const float4* __restrict__ org;
  const float4* __restrict__ dir;
  int2* hit;
  uint32_t* err;
  DevWBVH bvh;
  float eps;
  const int32_t* __restrict__ perm;
  __device__ void load(int i, float4& o, float4& d, float& t0, DevWBVH& b, float& e) {
    if (perm) i = __ldg(perm + i);
    o = __ldg(org + i);
    d = __ldg(dir + i);
    t0 = 1e34f;  // MAX_DISTANCE, src/Core/Ray.cuh:13
    b = bvh;
    e = eps;
  }
  __device__ void store(int i, int h, float t, bool overflow) {
    if (perm) i = __ldg(perm + i);
    if (overflow) {
      atomicOr(err, kErrStackOverflow);
      hit[i] = make_int2(-1, __float_as_int(1e34f));
      return;
    }
    hit[i] = make_int2(h, __float_as_int(t));
  }
};

struct WConnectIO {
  const float4* __restrict__ sorg;
  const float4* __restrict__ sdir;
  const float4* __restrict__ scol;
  float4* accum;
  uint32_t* err;
  DevWBVH bvh;
  float eps;
  __device__ void load(int i, float4& o, float4& d, float& t0, DevWBVH& b, float& e) {
    o = __ldg(sorg + i);
    d = __ldg(sdir + i);
    t0 = d.w;
    b = bvh;
    e = eps;
  }
  __device__ void store(int i, int h, float, bool overflow) {
    if (overflow) {
      atomicOr(err, kErrStackOverflow);
      return;
    }
    if (h >= 0) return;
    const float4 c = __ldg(scol + i);
    const int pix = __float_as_int(__ldg(&sorg[i].w));
    float4 a = accum[pix];
    a.x = __fadd_rn(a.x, c.x);
    a.y = __fadd_rn(a.y, c.y);
    a.z = __fadd_rn(a.z, c.z);
    a.w = __fadd_rn(a.w, 1.0f);
    accum[pix] = a;
  }
};

struct WBatchExtendIO {
  const float4* __restrict__ org;
  const float4* __restrict__ dir;
  int2* hit;
  uint32_t* err;
  const BatchJob* jobs;
  const int32_t* bases;
  int n_jobs;
  const int32_t* __restrict__ perm;
  __device__ void load(int i, float4& o, float4& d, float& t0, DevWBVH& b, float& e) {
    if (perm) i = __ldg(perm + i);
    o = __ldg(org + i);
    d = __ldg(dir + i);
    t0 = 1e34f;
    const BatchJob& J = jobs[batch_job_of(bases, n_jobs, __float_as_int(o.w))];
    b = J.wbvh;
    e = J.f.tri_eps;
  }
  __device__ void store(int i, int h, float t, bool overflow) {
    if (perm) i = __ldg(perm + i);
    if (overflow) {
      atomicOr(err, kErrStackOverflow);
      hit[i] = make_int2(-1, __float_as_int(1e34f));
      return;
    }
    hit[i] = make_int2(h, __float_as_int(t));
  }
};

struct WBatchConnectIO {
  const float4* __restrict__ sorg;
  const float4* __restrict__ sdir;
  const float4* __restrict__ scol;
  uint32_t* err;
  const BatchJob* jobs;
  const int32_t* bases;
  int n_jobs;
  __device__ void load(int i, float4& o, float4& d, float& t0, DevWBVH& b, float& e) {
    o = __ldg(sorg + i);
    d = __ldg(sdir + i);
    t0 = d.w;
    const BatchJob& J = jobs[batch_job_of(bases, n_jobs, __float_as_int(o.w))];
    b = J.wbvh;
    e = J.f.tri_eps;
  }
  __device__ void store(int i, int h, float, bool overflow) {
    if (overflow) {
      atomicOr(err, kErrStackOverflow);
      return;
    }
    if (h >= 0) return;
    const float4 c = __ldg(scol + i);
    const int pix = __float_as_int(__ldg(&sorg[i].w));
    const BatchJob& J = jobs[batch_job_of(bases, n_jobs, pix)];
    float4* acc = J.accum + (pix - J.pix_base);
    float4 a = *acc;
    a.x = __fadd_rn(a.x, c.x);
    a.y = __fadd_rn(a.y, c.y);
    a.z = __fadd_rn(a.z, c.z);
    a.w = __fadd_rn(a.w, 1.0f);
    *acc = a;
  }
};

__global__ void __launch_bounds__(128) k_extend_wide(DevWBVH b, DevQueues q, int qi, float eps) {
  uint32_t st_node[kWStack];
  float st_t[kWStack];
  const int n = q.counts[qi];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    q.counts[qi ^ 1] = 0;
    q.counts[2] = 0;
    q.counts[5] = 0;  // fetch cursor of the connect that follows
    atomicAdd(&q.stats[0], (unsigned long long)n);
  }
  WExtendIO io{q.org_q(qi), q.dir_q(qi), q.hit, q.error, b, eps, q.perm};
  trace_wide_mt<false>(n, q.counts + 4, io, st_node, st_t);
}

__global__ void __launch_bounds__(128) k_connect_wide(DevWBVH b, DevQueues q, float eps) {
  uint32_t st_node[kWStack];
  float st_t[kWStack];
  const int n = q.counts[2];
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&q.stats[1], (unsigned long long)n);
  WConnectIO io{q.sorg, q.sdir, q.scol, q.accum, q.error, b, eps};
  trace_wide_mt<true>(n, q.counts + 5, io, st_node, st_t);
}

__global__ void __launch_bounds__(128) k_batch_extend_wide(DevBatch bt, DevQueues q, int qi) {
  uint32_t st_node[kWStack];
  float st_t[kWStack];
  const int n = q.counts[qi];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    q.counts[qi ^ 1] = 0;
    q.counts[2] = 0;
    q.counts[5] = 0;
    atomicAdd(&q.stats[0], (unsigned long long)n);
  }
  WBatchExtendIO io{q.org_q(qi), q.dir_q(qi), q.hit, q.error, bt.jobs, bt.bases, bt.n_jobs, q.perm};
  trace_wide_mt<false>(n, q.counts + 4, io, st_node, st_t);
}

__global__ void __launch_bounds__(128) k_batch_connect_wide(DevBatch bt, DevQueues q) {
  uint32_t st_node[kWStack];
  float st_t[kWStack];
  const int n = q.counts[2];
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&q.stats[1], (unsigned long long)n);
  WBatchConnectIO io{q.sorg, q.sdir, q.scol, q.error, bt.jobs, bt.bases, bt.n_jobs};
  trace_wide_mt<true>(n, q.counts + 5, io, st_node, st_t);
}

template <typename K>
int mt_grid(K kernel, int capacity) {
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 128, 0);
  const int cap_blocks = (capacity + 127) / 128;
  return std::max(1, std::min(cap_blocks, std::max(1, per) * sm_count()));
}

template <typename K>
int resident_blocks(K kernel) {
  int per = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, kernel, 128, 0);
  return std::max(1, per) * sm_count();
}

template <bool ANY>
cudaError_t launch_wide_query(const DevWBVH& b, const float4* org, const float4* dir, int32_t* hit, float* t,
                              uint8_t* occ, uint32_t n, uint32_t* err, int* counters, uint4* recs,
                              unsigned long long* stats, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(counters, 0, 2 * sizeof(int), s);
  if (e != cudaSuccess) return e;
  static int g_trace = 0, g_settle = 0;
  if (!g_trace) g_trace = resident_blocks(k_trace_wide<ANY>), g_settle = resident_blocks(k_wide_settle<ANY>);
  const int g = std::min<int>(g_trace, (int)((n + 127) / 128));
  k_trace_wide<ANY><<<g, 128, 0, s>>>(b, org, dir, hit, t, occ, n, counters, recs, stats);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  // the record count stays on the device: a grid of resident blocks strides over it
  k_wide_settle<ANY><<<std::min<int>(g_settle, g), 128, 0, s>>>(b, org, dir, hit, t, occ, counters, recs, err, stats);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_trace_wide_closest(const DevWBVH& b, const float4* org, const float4* dir, int32_t* hit, float* t,
                                      uint32_t n, uint32_t* err, int* counters, void* recs,
                                      unsigned long long* stats, cudaStream_t s) {
  return launch_wide_query<false>(b, org, dir, hit, t, nullptr, n, err, counters, (uint4*)recs, stats, s);
}

cudaError_t launch_trace_wide_any(const DevWBVH& b, const float4* org, const float4* dir, uint8_t* occ, uint32_t n,
                                  uint32_t* err, int* counters, void* recs, unsigned long long* stats,
                                  cudaStream_t s) {
  return launch_wide_query<true>(b, org, dir, nullptr, nullptr, occ, n, err, counters, (uint4*)recs, stats, s);
}


cudaError_t launch_extend_wide(const DevWBVH& b, const DevQueues& q, int queue, float eps, cudaStream_t s) {
  k_extend_wide<<<mt_grid(k_extend_wide, q.capacity), 128, 0, s>>>(b, q, queue, eps);
  return cudaGetLastError();
}
cudaError_t launch_connect_wide(const DevWBVH& b, const DevQueues& q, float eps, cudaStream_t s) {
  k_connect_wide<<<mt_grid(k_connect_wide, q.capacity), 128, 0, s>>>(b, q, eps);
  return cudaGetLastError();
}
cudaError_t launch_batch_extend_wide(const DevBatch& b, const DevQueues& q, int queue, cudaStream_t s) {
  k_batch_extend_wide<<<mt_grid(k_batch_extend_wide, q.capacity), 128, 0, s>>>(b, q, queue);
  return cudaGetLastError();
}
cudaError_t launch_batch_connect_wide(const DevBatch& b, const DevQueues& q, cudaStream_t s) {
  k_batch_connect_wide<<<mt_grid(k_batch_connect_wide, q.capacity), 128, 0, s>>>(b, q);
  return cudaGetLastError();
}

}  // namespace ct
