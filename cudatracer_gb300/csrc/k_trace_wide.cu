// Ray queries on the 8-wide quantised BVH (WNode8).
//
// Boxes: child bounds decoded as fma(2^e, q, p), which the builder rounded
// outward, and a slab test whose far distance is scaled by 1 + 2*gamma(3)
// (Ize 2013, "Robust BVH ray traversal"), so no box that the ray touches in
// exact arithmetic is rejected.
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
constexpr int kCand = 8;
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

struct NodeBoxes {
  float px, py, pz, sx, sy, sz;
};

// Slab test of slot i; returns the entry distance or +inf when missed.
__device__ __forceinline__ float slot_box(const WRay& r, const WNode8& n, const NodeBoxes& nb, int i, float tfar) {
  const float lx = __fmaf_rn(nb.sx, (float)n.qlo[0][i], nb.px), hx = __fmaf_rn(nb.sx, (float)n.qhi[0][i], nb.px);
  const float ly = __fmaf_rn(nb.sy, (float)n.qlo[1][i], nb.py), hy = __fmaf_rn(nb.sy, (float)n.qhi[1][i], nb.py);
  const float lz = __fmaf_rn(nb.sz, (float)n.qlo[2][i], nb.pz), hz = __fmaf_rn(nb.sz, (float)n.qhi[2][i], nb.pz);
  const float t0x = (lx - r.ox) * r.ix, t1x = (hx - r.ox) * r.ix;
  const float t0y = (ly - r.oy) * r.iy, t1y = (hy - r.oy) * r.iy;
  const float t0z = (lz - r.oz) * r.iz, t1z = (hz - r.oz) * r.iz;
  const float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), 0.0f));
  const float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tfar)) * kFarScale;
  return tn <= tf ? tn : __int_as_float(0x7f800000);
}

__device__ __forceinline__ void load_node(const WNode8* nodes, uint32_t i, WNode8& n, NodeBoxes& nb) {
  const float4* s = reinterpret_cast<const float4*>(nodes + i);
  float4* d = reinterpret_cast<float4*>(&n);
#pragma unroll
  for (int k = 0; k < 5; k++) d[k] = __ldg(s + k);
  nb.px = n.px, nb.py = n.py, nb.pz = n.pz;
  nb.sx = __int_as_float((int)n.e[0] << 23);
  nb.sy = __int_as_float((int)n.e[1] << 23);
  nb.sz = __int_as_float((int)n.e[2] << 23);
}

__device__ __forceinline__ uint32_t meta_at(const WNode8& n, int i) {
  const uint32_t* w = reinterpret_cast<const uint32_t*>(n.meta);
  return ((i < 4 ? w[0] : w[1]) >> (8 * (i & 3))) & 0xffu;
}

// A warp refills its idle lanes from the cursor once this many are idle (or
// all are): fewer cursor atomics and refill passes than refilling at the
// first idle lane (measured best for queries and frames on the wide tree).
constexpr int kWideRefill = 8;

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
    NodeBoxes nb;
    load_node(b.nodes, ni, n, nb);
    for (int i = 0; i < 8; i++) {
      const uint32_t m = meta_at(n, i);
      if (!m) continue;
      const float tn = slot_box(r, n, nb, i, far);
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

// Persistent traversal: each lane owns a ray and takes one step per round —
// an inner node (eight slab tests; inner children and leaf groups pushed,
// the nearest on top) or one leaf group (up to three triangle tests) — so
// the warp's lanes do similar work each round; a lane whose ray is done takes
// the next ray from the device cursor (one atomicAdd per warp). A ray that
// would overflow the stack is traced again entirely in FP64.
template <bool ANY>
// At least 6 resident blocks per SM: 80 registers with a few spills beat 90
// registers and 5 blocks (290 vs 266 Mrays/s on a 4M-triangle soup).
__global__ void __launch_bounds__(128, 6) k_trace_wide(const DevWBVH b, const float4* __restrict__ org,
                                                    const float4* __restrict__ dir, int32_t* __restrict__ hit_out,
                                                    float* __restrict__ t_out, uint8_t* __restrict__ occ_out,
                                                    uint32_t n, uint32_t* err, int* cursor,
                                                    unsigned long long* stats) {
  uint32_t st_node[kWStack];
  float st_t[kWStack];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31;
  const unsigned below = (1u << lane) - 1u;
  unsigned long long n_rays = 0, n_retest = 0, n_full = 0, n_tbound = 0;
  int rid = -1;
  bool exhausted = false;
  WRay r;
  int best = -1, nc = 0, sp = 0;
  float tb = 0.0f, tberr = 0.0f;
  bool overflow = false, occluded = false;
  uint32_t cand[kCand];
  float cand_lo[kCand];
  while (true) {
    if (!exhausted) {
      const unsigned m = __ballot_sync(FULL, rid < 0);
      if (m == FULL || __popc(m) >= kWideRefill) {  // refill once 8 lanes are idle
        const int leader = __ffs(m) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(cursor, __popc(m));
        base = __shfl_sync(FULL, base, leader);
        if ((uint32_t)(base + __popc(m)) >= n) exhausted = true;
        if (rid < 0) {
          const int my = base + __popc(m & below);
          if ((uint32_t)my < n) {
            setup(__ldg(org + my), __ldg(dir + my), r);
            rid = my;
            n_rays++;
            best = -1, nc = 0, tb = r.tmax, tberr = 0.0f, overflow = false, occluded = false;
            st_node[0] = 0, st_t[0] = 0.0f, sp = 1;
          }
        }
      }
    }
    if (__ballot_sync(FULL, rid >= 0) == 0) break;
    if (rid < 0) continue;
    // ---- one step
    const float far = (tb + tberr) * kFarScale;
    while (sp > 0 && st_t[sp - 1] > far) sp--;  // culled entries
    bool finished = sp == 0 || overflow || (ANY && occluded);
    if (!finished) {
      const uint32_t ent = st_node[--sp];
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
              if (nc < kCand) cand[nc] = (uint32_t)best, cand_lo[nc] = tb - tberr, nc++;
              else overflow = true;
            }
            best = (int)slot, tb = t, tberr = terr;
            continue;
          }
          if (nc < kCand) cand[nc] = slot, cand_lo[nc] = t - terr, nc++;
          else overflow = true;
        }
      } else {
        WNode8 nd;
        NodeBoxes nb;
        load_node(b.nodes, ent, nd, nb);
        const int sp0 = sp;
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const uint32_t m = meta_at(nd, i);
          if (!m) continue;
          const float tn = slot_box(r, nd, nb, i, far);
          if (!(tn <= far)) continue;
          if (sp >= kWStack) {
            overflow = true;  // settled by the full FP64 traversal
            continue;
          }
          st_node[sp] = (m & 0x80u) ? nd.child_base + (m & 7u)
                                    : (kLeafEntry | ((m >> 5) << 29) | (nd.prim_base + (m & 31u)));
          st_t[sp] = tn;
          sp++;
        }
        if (sp - sp0 > 1) {
          int bi = sp0;
          for (int k = sp0 + 1; k < sp; k++)
            if (st_t[k] < st_t[bi]) bi = k;
          const uint32_t tnode = st_node[bi];
          const float tt = st_t[bi];
          st_node[bi] = st_node[sp - 1], st_t[bi] = st_t[sp - 1];
          st_node[sp - 1] = tnode, st_t[sp - 1] = tt;
        }
      }
      finished = sp == 0 || overflow || (ANY && occluded);
    }
    if (!finished) continue;
    // ---- the ray is done: settle what FP32 could not
    if (!overflow) {
      int k2 = 0;
      for (int k = 0; k < nc; k++)
        if (cand_lo[k] < tb + tberr) cand[k2] = cand[k], cand_lo[k2] = cand_lo[k], k2++;
      nc = k2;
    }
    int out_prim = best >= 0 ? __float_as_int(__ldg(b.tris + 3 * (size_t)best).w) : -1;
    float out_t = best >= 0 ? tb : r.tmax;
    if (ANY && !occluded && best >= 0) occluded = true;
    if (!(ANY && occluded) && overflow) {
      n_full++;
      double t64;
      int prim;
      const bool h = trace_fp64<ANY>(b, r, st_node, st_t, err, prim, t64);
      out_prim = h ? prim : -1;
      out_t = h ? (float)t64 : r.tmax;
      occluded = h;
    } else if (!(ANY && occluded) && (nc > 0 || (!ANY && best >= 0 && tberr > kTRel * tb))) {
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
      for (int k = 0; k < nc; k++) consider(cand[k]);
      out_prim = bp;
      out_t = bp >= 0 ? (float)bt : r.tmax;
      occluded = bp >= 0;
    }
    if (ANY) {
      occ_out[rid] = occluded ? 1 : 0;
    } else {
      hit_out[rid] = out_prim;
      t_out[rid] = out_t;
    }
    rid = -1;
  }
  if (stats) {
    atomicAdd(stats + 0, n_rays);
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

__device__ __forceinline__ float mslot_box(const MRay& r, const WNode8& n, const NodeBoxes& nb, int i, float tfar) {
  const float lx = __fmaf_rn(nb.sx, (float)n.qlo[0][i], nb.px), hx = __fmaf_rn(nb.sx, (float)n.qhi[0][i], nb.px);
  const float ly = __fmaf_rn(nb.sy, (float)n.qlo[1][i], nb.py), hy = __fmaf_rn(nb.sy, (float)n.qhi[1][i], nb.py);
  const float lz = __fmaf_rn(nb.sz, (float)n.qlo[2][i], nb.pz), hz = __fmaf_rn(nb.sz, (float)n.qhi[2][i], nb.pz);
  const float t0x = (lx - r.ox) * r.ix, t1x = (hx - r.ox) * r.ix;
  const float t0y = (ly - r.oy) * r.iy, t1y = (hy - r.oy) * r.iy;
  const float t0z = (lz - r.oz) * r.iz, t1z = (hz - r.oz) * r.iz;
  const float tn = fmaxf(fmaxf(fminf(t0x, t1x), fminf(t0y, t1y)), fmaxf(fminf(t0z, t1z), 0.0f));
  const float tf = fminf(fminf(fmaxf(t0x, t1x), fmaxf(t0y, t1y)), fminf(fmaxf(t0z, t1z), tfar)) * kFarScale;
  return tn <= tf ? tn : __int_as_float(0x7f800000);
}

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
      if (m == FULL || __popc(m) >= kWideRefill) {  // refill once 8 lanes are idle
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
        NodeBoxes nb;
        load_node(b.nodes, ent, nd, nb);
        const int sp0 = sp;
#pragma unroll
        for (int i = 0; i < 8; i++) {
          const uint32_t m = meta_at(nd, i);
          if (!m) continue;
          const float tn = mslot_box(r, nd, nb, i, far);
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

int wide_grid() {
  static int g = 0;
  if (!g) {
    int per = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_trace_wide<false>, 128, 0);
    g = std::max(1, per) * sm_count();
  }
  return g;
}

}  // namespace

cudaError_t launch_trace_wide_closest(const DevWBVH& b, const float4* org, const float4* dir, int32_t* hit, float* t,
                                      uint32_t n, uint32_t* err, int* cursor, unsigned long long* stats,
                                      cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(cursor, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  const int g = std::min<int>(wide_grid(), (int)((n + 127) / 128));
  k_trace_wide<false><<<g, 128, 0, s>>>(b, org, dir, hit, t, nullptr, n, err, cursor, stats);
  return cudaGetLastError();
}

cudaError_t launch_trace_wide_any(const DevWBVH& b, const float4* org, const float4* dir, uint8_t* occ, uint32_t n,
                                  uint32_t* err, int* cursor, unsigned long long* stats, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  cudaError_t e = cudaMemsetAsync(cursor, 0, sizeof(int), s);
  if (e != cudaSuccess) return e;
  const int g = std::min<int>(wide_grid(), (int)((n + 127) / 128));
  k_trace_wide<true><<<g, 128, 0, s>>>(b, org, dir, nullptr, nullptr, occ, n, err, cursor, stats);
  return cudaGetLastError();
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
