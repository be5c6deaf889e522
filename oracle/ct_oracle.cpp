/*
 * ct_oracle: CPU restatement of the reference tracer's hot path.
 *
 * TEST INFRASTRUCTURE ONLY. This is the checker the CUDA path is compared
 * against; it is loaded by tests/, by __graft_entry__.smoke() and by bench.py's
 * CPU-baseline leg, never by the product library. It is pinned against the
 * reference's own host code (oracle/_ref, see oracle/ref_build.py) through the
 * golden fixtures in tests/golden/.
 *
 * It restates, in plain scalar C++ with no fused multiply-add
 * (-ffp-contract=off) and glm's operation order (dot = (x*x + y*y) + z*z,
 * cross = (a.y*b.z - b.y*a.z, ...), min(a,b) = b < a ? b : a, max = a < b ? b : a):
 *   triangle::getBounds               src/Core/Triangle.cuh:59-65
 *   BVHNode::SubdivideMT / Partition  src/BVH/BVHNode.cu:70-190 (axis-outer SAH)
 *   MBVHNode::MergeNodes/GetBVHNodeInfo src/BVH/MBVHNode.cu:126-160, 226-277
 *   MBVHNode::intersect               src/BVH/MBVHNode.cuh:69-110
 *   MBVHNode::traverseMBVH(Shadow)    src/BVH/MBVHNode.cuh:126-205
 *   BVHNode::Intersect / traverseBVH  src/BVH/BVHNode.cuh:50-62, 206-254
 *   triangle::intersect               src/Core/Triangle.cuh:13-44
 *   generatePrimaryRays, Ray::generate src/CUDA/Kernel.cu:208-234, src/Core/Ray.cuh:85-95
 *   shade / connect / draw_framebuffer src/CUDA/Kernel.cu:88-206, 247-270
 *   SampleBSDF / EvaluateBSDF         src/Core/BSDF.h:26-63
 *   WangHash / RandomInt / RandomFloat / RandomIntMax  src/Core/Random.cuh:10-34
 *   Tangent2World, DiffuseReflectionCosWeighted       src/Core/Tools.h:110-137, 162-169
 *   convertToLocalSpace               src/Core/Random.cuh:37-42
 *   SceneData::getTextureColor        src/Core/SceneData.cuh:81-97
 *
 * Transcendentals: with exact_math=1 the oracle (and the GPU's matching mode)
 * evaluate sin/cos/atan2/acos with the binary32 functions of
 * cudatracer_gb300/csrc/portable_math.h, fixed sequences of correctly rounded
 * IEEE operations, which makes CPU and GPU agree bit for bit (that header's
 * accuracy against correctly rounded values is tested on its own);
 * exact_math=0 calls the C library's float functions, which differ from
 * CUDA's by an ulp now and then.
 */
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <functional>
#include <memory>
#include <thread>
#include <vector>

#include "../cudatracer_gb300/csrc/portable_math.h"

namespace {

struct V3 {
  float x, y, z;
};
inline V3 v3(float x, float y, float z) { return {x, y, z}; }
inline V3 add(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline V3 sub(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline V3 mul(V3 a, V3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline V3 muls(V3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
inline V3 divs(V3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
inline float dot(V3 a, V3 b) {
  const float x = a.x * b.x, y = a.y * b.y, z = a.z * b.z;
  return (x + y) + z;
}
inline V3 cross(V3 a, V3 b) { return {a.y * b.z - b.y * a.z, a.z * b.x - b.z * a.x, a.x * b.y - b.x * a.y}; }
inline float gmin(float a, float b) { return b < a ? b : a; }
inline float gmax(float a, float b) { return a < b ? b : a; }
inline V3 vmax(V3 a, V3 b) { return {gmax(a.x, b.x), gmax(a.y, b.y), gmax(a.z, b.z)}; }
inline V3 normalize(V3 v) {
  const float inv = 1.0f / std::sqrt(dot(v, v));
  return muls(v, inv);
}
inline float length(V3 v) { return std::sqrt(dot(v, v)); }
inline V3 load3(const float* p, size_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }

inline uint32_t fbits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}
inline float bitsf(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}

constexpr float kMaxDistance = 1e34f;  // MAX_DISTANCE, src/Core/Ray.cuh:13
constexpr float kOneOverPi = 0.318309886183790671537767526745028724f;
constexpr float kTwoPi = 6.28318530717958647692528676655900576f;

/* ---------------- reference-layout node types ---------------- */
struct BNode {  // 32 bytes, BVHNode (src/BVH/BVHNode.cuh:29-40)
  float bmin[3];
  int32_t leftFirst;
  float bmax[3];
  int32_t count;
};
struct QNode {  // 128 bytes, MBVHNode (src/BVH/MBVHNode.cuh:35-63)
  float bminx[4], bmaxx[4], bminy[4], bmaxy[4], bminz[4], bmaxz[4];
  int32_t childs[4], counts[4];
};
static_assert(sizeof(BNode) == 32, "BNode layout");
static_assert(sizeof(QNode) == 128, "QNode layout");

struct Box {
  float mn[3], mx[3];
};
inline Box empty_box() { return {{1e34f, 1e34f, 1e34f}, {-1e34f, -1e34f, -1e34f}}; }
// AABB::Grow via _mm_min_ps/_mm_max_ps (src/BVH/AABB.h:57-60): MINPS(a,b) = a < b ? a : b.
inline void grow(Box& b, const Box& o) {
  for (int k = 0; k < 3; k++) {
    b.mn[k] = b.mn[k] < o.mn[k] ? b.mn[k] : o.mn[k];
    b.mx[k] = b.mx[k] > o.mx[k] ? b.mx[k] : o.mx[k];
  }
}
// AABB::Area (src/BVH/AABB.h:122-129)
inline float area(const Box& b) {
  const float e0 = b.mx[0] - b.mn[0], e1 = b.mx[1] - b.mn[1], e2 = b.mx[2] - b.mn[2];
  const float s = (e0 * e1 + e0 * e2) + e1 * e2;
  return std::fmax(0.0f, s);
}
inline float centroid(const Box& b, int axis) { return (b.mn[axis] + b.mx[axis]) * 0.5f; }

/* ---------------- binary SAH build (reference MT semantics) ---------------- */
struct TNode {
  Box box = empty_box();
  int first = 0, count = 0;
  std::unique_ptr<TNode> left, right;
};

struct Builder {
  const Box* aabbs;
  uint32_t* prims;
  int max_threads;
  std::atomic<int>* active;
};

// BVHNode::CalculateBounds (src/BVH/BVHNode.cu:21-34)
Box calc_bounds(const Builder& B, int first, int count) {
  Box b = empty_box();
  for (int i = 0; i < count; i++) grow(b, B.aabbs[B.prims[first + i]]);
  return b;
}

// BVHNode::Partition, thread-pool variant (src/BVH/BVHNode.cu:121-190): axes
// outer, ten candidate planes inner, strict-less cost comparison.
bool partition(const Builder& B, TNode& n, int& lcount) {
  const int lFirst = n.first;
  const float parentCost = area(n.box) * (float)n.count;
  float lowest = 1e34f, bestCoord = 0.0f;
  int bestAxis = 0;
  float lengths[3];
  for (int k = 0; k < 3; k++) lengths[k] = n.box.mx[k] - n.box.mn[k];
  for (int axis = 0; axis < 3; axis++) {
    for (int i = 1; i < 11; i++) {
      const float binOffset = (float)i / (float)11;
      const float split = n.box.mn[axis] + lengths[axis] * binOffset;
      int lc = 0, rc = 0;
      Box lb = empty_box(), rb = empty_box();
      for (int idx = 0; idx < n.count; idx++) {
        const Box& a = B.aabbs[B.prims[lFirst + idx]];
        if (centroid(a, axis) <= split) {
          grow(lb, a);
          lc++;
        } else {
          grow(rb, a);
          rc++;
        }
      }
      const float cost = area(lb) * (float)lc + area(rb) * (float)rc;
      if (cost < lowest) {
        lowest = cost;
        bestCoord = split;
        bestAxis = axis;
      }
    }
  }
  if (parentCost < lowest) return false;
  int lc = 0;
  for (int idx = 0; idx < n.count; idx++) {
    const Box& a = B.aabbs[B.prims[lFirst + idx]];
    if (centroid(a, bestAxis) <= bestCoord) {
      std::swap(B.prims[lFirst + idx], B.prims[lFirst + lc]);
      lc++;
    }
  }
  lcount = lc;
  return true;
}

// BVHNode::SubdivideMT (src/BVH/BVHNode.cu:70-119): leaf if count < 4 or
// depth >= 64; children get their bounds recomputed before recursing.
void subdivide(const Builder& B, TNode& n, unsigned depth) {
  depth++;
  if (n.count < 4 || depth >= 64) return;
  int lc = 0;
  if (!partition(B, n, lc)) return;
  n.left.reset(new TNode());
  n.right.reset(new TNode());
  n.left->first = n.first;
  n.left->count = lc;
  n.right->first = n.first + lc;
  n.right->count = n.count - lc;
  TNode* L = n.left.get();
  TNode* R = n.right.get();
  auto run_left = [&B, L, depth] {
    if (L->count > 0) {
      L->box = calc_bounds(B, L->first, L->count);
      subdivide(B, *L, depth);
    }
  };
  bool spawned = false;
  std::thread th;
  if (L->count > 20000 && R->count > 20000 && B.active->fetch_add(1) < B.max_threads) {
    th = std::thread(run_left);
    spawned = true;
  }
  if (!spawned) run_left();
  if (R->count > 0) {
    R->box = calc_bounds(B, R->first, R->count);
    subdivide(B, *R, depth);
  }
  if (spawned) th.join();
}

/* Linearise the pointer tree with the pool numbering the reference's
 * single-threaded Subdivide produces: root 0, slot 1 unused, and each split
 * node's two children allocated as a pair at (poolPtr, poolPtr+1) in
 * depth-first order (src/BVH/BVHTree.cpp:33-50). */
void linearise(const TNode& n, int slot, std::vector<BNode>& pool, int& poolPtr) {
  BNode& out = pool[slot];
  for (int k = 0; k < 3; k++) out.bmin[k] = n.box.mn[k], out.bmax[k] = n.box.mx[k];
  if (!n.left) {
    out.leftFirst = n.first;
    out.count = n.count;
    return;
  }
  const int l = poolPtr++, r = poolPtr++;
  out.leftFirst = l;
  out.count = -1;
  linearise(*n.left, l, pool, poolPtr);
  linearise(*n.right, r, pool, poolPtr);
}

/* ---------------- quad collapse ---------------- */
struct Collapser {
  const std::vector<BNode>& pool;
  std::vector<QNode>& tree;
  int finalPtr;
};

void qset(QNode& q, int i, const float mn[3], const float mx[3]) {
  q.bminx[i] = mn[0], q.bminy[i] = mn[1], q.bminz[i] = mn[2];
  q.bmaxx[i] = mx[0], q.bmaxy[i] = mx[1], q.bmaxz[i] = mx[2];
}

// MBVHNode::GetBVHNodeInfo (src/BVH/MBVHNode.cu:226-277)
int node_info(QNode& q, const BNode& node, const std::vector<BNode>& pool) {
  for (int i = 0; i < 4; i++) q.childs[i] = -1, q.counts[i] = -1;
  int num = 0;
  if (node.count > -1) return 0;  // "This node shouldn't be a leaf."
  const BNode& L = pool[node.leftFirst];
  const BNode& R = pool[node.leftFirst + 1];
  if (L.count > -1) {
    const int i = num++;
    qset(q, i, L.bmin, L.bmax);
    q.childs[i] = L.leftFirst;
    q.counts[i] = L.count;
  } else {
    const int a = num++, b = num++;
    q.childs[a] = L.leftFirst;
    q.childs[b] = L.leftFirst + 1;
  }
  if (R.count > -1) {
    const int i = num++;
    qset(q, i, R.bmin, R.bmax);
    q.childs[i] = R.leftFirst;
    q.counts[i] = R.count;
  } else {
    const int a = num++, b = num++;
    qset(q, a, pool[R.leftFirst].bmin, pool[R.leftFirst].bmax);
    qset(q, b, pool[R.leftFirst + 1].bmin, pool[R.leftFirst + 1].bmax);
    q.childs[a] = R.leftFirst;
    q.childs[b] = R.leftFirst + 1;
  }
  return num;
}

// MBVHNode::MergeNodes (src/BVH/MBVHNode.cu:27-61)
void merge(Collapser& C, int qidx, const BNode& node) {
  int num = node_info(C.tree[qidx], node, C.pool);
  for (int i = 0; i < num; i++) {
    QNode& q = C.tree[qidx];
    if (q.counts[i] == -1) {
      const BNode& cur = C.pool[q.childs[i]];
      if (cur.count > -1) {
        q.counts[i] = cur.count;
        q.childs[i] = cur.leftFirst;
        qset(q, i, cur.bmin, cur.bmax);
      } else {
        const int ni = C.finalPtr++;
        q.childs[i] = ni;
        q.counts[i] = -1;
        qset(q, i, cur.bmin, cur.bmax);
        merge(C, ni, cur);
      }
    }
  }
  QNode& q = C.tree[qidx];
  const float big[3] = {1e34f, 1e34f, 1e34f}, nbig[3] = {-1e34f, -1e34f, -1e34f};
  for (int i = num; i < 4; i++) {
    qset(q, i, big, nbig);
    q.counts[i] = 0;
  }
}

/* ---------------- traversal ---------------- */
// triangle::intersect (src/Core/Triangle.cuh:13-44)
inline bool tri_intersect(V3 org, V3 dir, float* rayt, V3 p0, V3 p1, V3 p2, float eps) {
  const V3 e1 = sub(p1, p0), e2 = sub(p2, p0);
  const V3 h = cross(dir, e2);
  const float a = dot(e1, h);
  if (a > -eps && a < eps) return false;
  const float f = 1.f / a;
  const V3 s = sub(org, p0);
  const float u = f * dot(s, h);
  if (u < 0.0f || u > 1.0f) return false;
  const V3 q = cross(s, e1);
  const float v = f * dot(dir, q);
  if (v < 0.0f || u + v > 1.0f) return false;
  const float t = f * dot(e2, q);
  if (t > eps && *rayt > t) {
    *rayt = t;
    return true;
  }
  return false;
}

// Child order after the slab tests: the reference's 5-exchange network, whose
// last pair is (2,3) and which leaves (1,2) unordered (MBVHNode.cuh:98-107), or,
// when g_full_sort is set, a full 4-sort with last pair (1,2) as the fast-math
// GPU frames use. Only the visiting order differs, hence only the work counts
// (and exact-tie choices); every parity test runs with the reference's order.
static std::atomic<int> g_full_sort{0};

// MBVHNode::intersect (src/BVH/MBVHNode.cuh:69-110)
inline void quad_intersect(const QNode& n, V3 o, V3 inv, float t, float tmin[4], bool res[4]) {
  float tmax[4];
  for (int k = 0; k < 4; k++) {
    float t1 = (n.bminx[k] - o.x) * inv.x, t2 = (n.bmaxx[k] - o.x) * inv.x;
    float mn = gmin(t1, t2), mx = gmax(t1, t2);
    t1 = (n.bminy[k] - o.y) * inv.y, t2 = (n.bmaxy[k] - o.y) * inv.y;
    mn = gmax(mn, gmin(t1, t2));
    mx = gmin(mx, gmax(t1, t2));
    t1 = (n.bminz[k] - o.z) * inv.z, t2 = (n.bmaxz[k] - o.z) * inv.z;
    mn = gmax(mn, gmin(t1, t2));
    mx = gmin(mx, gmax(t1, t2));
    tmin[k] = bitsf((fbits(mn) & 0xFFFFFFFCu) | (uint32_t)k);
    tmax[k] = mx;
  }
  for (int k = 0; k < 4; k++) res[k] = tmax[k] > 0.0f && tmin[k] <= tmax[k] && tmin[k] < t;
  auto cs = [&](int a, int b) {
    if (tmin[a] > tmin[b]) std::swap(tmin[a], tmin[b]);
  };
  cs(0, 1);
  cs(2, 3);
  cs(0, 2);
  cs(1, 3);
  if (g_full_sort.load(std::memory_order_relaxed))
    cs(1, 2);
  else
    cs(2, 3);
}

struct Geo {
  const float* verts;
  const uint32_t* idx;
  const uint32_t* prims;
  const QNode* qnodes;
  const BNode* bnodes;
  float eps;
};

// MBVHNode::traverseMBVH (src/BVH/MBVHNode.cuh:126-163). The stack is 128
// deep (the reference's 32 has no overflow check); overflow_out counts rays
// whose stack would have exceeded 32 entries.
// Work counters (node visits, triangle tests) for the algorithmic-bytes model.
struct Work {
  uint64_t rays = 0, nodes = 0, tris = 0;
};

void trace_closest(const Geo& g, V3 org, V3 dir, float* t, int* hit, int* deep, Work* w = nullptr) {
  int stk_first[256], stk_count[256];
  int sp = 0, maxsp = 0;
  if (w) w->rays++;
  stk_first[0] = 0;
  stk_count[0] = -1;
  const V3 inv = v3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
  while (sp >= 0) {
    const int lf = stk_first[sp], cnt = stk_count[sp];
    sp--;
    if (cnt > -1) {
      if (w) w->tris += (uint64_t)cnt;
      for (int i = 0; i < cnt; i++) {
        const uint32_t prim = g.prims[lf + i];
        const uint32_t* ix = g.idx + 3 * (size_t)prim;
        if (tri_intersect(org, dir, t, load3(g.verts, ix[0]), load3(g.verts, ix[1]), load3(g.verts, ix[2]), g.eps))
          *hit = (int)prim;
      }
      continue;
    }
    float tmin[4];
    bool res[4];
    const QNode& n = g.qnodes[lf];
    if (w) w->nodes++;
    quad_intersect(n, org, inv, *t, tmin, res);
    for (int i = 3; i >= 0; i--) {
      const int c = (int)(fbits(tmin[i]) & 3u);
      if (res[c]) {
        sp++;
        if (sp >= 255) return;  // guarded; never reached for depth-64 trees
        stk_first[sp] = n.childs[c];
        stk_count[sp] = n.counts[c];
        if (sp > maxsp) maxsp = sp;
      }
    }
  }
  if (deep) *deep = maxsp >= 32 ? 1 : 0;
}

// MBVHNode::traverseMBVHShadow (src/BVH/MBVHNode.cuh:165-205)
bool trace_any(const Geo& g, V3 org, V3 dir, float maxDist, Work* w = nullptr) {
  int stk_first[256], stk_count[256];
  int sp = 0;
  if (w) w->rays++;
  stk_first[0] = 0;
  stk_count[0] = -1;
  const V3 inv = v3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
  while (sp >= 0) {
    const int lf = stk_first[sp], cnt = stk_count[sp];
    sp--;
    if (cnt > -1) {
      for (int i = 0; i < cnt; i++) {
        if (w) w->tris++;
        const uint32_t prim = g.prims[lf + i];
        const uint32_t* ix = g.idx + 3 * (size_t)prim;
        if (tri_intersect(org, dir, &maxDist, load3(g.verts, ix[0]), load3(g.verts, ix[1]), load3(g.verts, ix[2]),
                          g.eps))
          return true;
      }
      continue;
    }
    float tmin[4];
    bool res[4];
    const QNode& n = g.qnodes[lf];
    if (w) w->nodes++;
    quad_intersect(n, org, inv, maxDist, tmin, res);
    for (int i = 3; i >= 0; i--) {
      const int c = (int)(fbits(tmin[i]) & 3u);
      if (res[c]) {
        sp++;
        if (sp >= 255) return false;
        stk_first[sp] = n.childs[c];
        stk_count[sp] = n.counts[c];
      }
    }
  }
  return false;
}

// BVHNode::Intersect (src/BVH/BVHNode.cuh:50-62)
inline bool bin_intersect(const BNode& n, V3 o, V3 inv, float* tn) {
  const float t1x = (n.bmin[0] - o.x) * inv.x, t1y = (n.bmin[1] - o.y) * inv.y, t1z = (n.bmin[2] - o.z) * inv.z;
  const float t2x = (n.bmax[0] - o.x) * inv.x, t2y = (n.bmax[1] - o.y) * inv.y, t2z = (n.bmax[2] - o.z) * inv.z;
  const float mnx = gmin(t1x, t2x), mny = gmin(t1y, t2y), mnz = gmin(t1z, t2z);
  const float mxx = gmax(t1x, t2x), mxy = gmax(t1y, t2y), mxz = gmax(t1z, t2z);
  const float tmin = gmax(mnx, gmax(mny, mnz));
  const float tmax = gmin(mxx, gmin(mxy, mxz));
  *tn = tmin;
  return tmax >= 0.0f && tmin < tmax;
}

// BVHNode::traverseBVH host (src/BVH/BVHNode.cuh:206-254), stack 64 -> 256 here.
void trace_closest_binary(const Geo& g, V3 org, V3 dir, float* t, int* hit) {
  int stk[256];
  int sp = 0;
  stk[0] = 0;
  const V3 inv = v3(1.0f / dir.x, 1.0f / dir.y, 1.0f / dir.z);
  while (sp >= 0) {
    const BNode& n = g.bnodes[stk[sp]];
    sp--;
    if (n.count > -1) {
      for (int i = 0; i < n.count; i++) {
        const uint32_t prim = g.prims[n.leftFirst + i];
        const uint32_t* ix = g.idx + 3 * (size_t)prim;
        if (tri_intersect(org, dir, t, load3(g.verts, ix[0]), load3(g.verts, ix[1]), load3(g.verts, ix[2]), g.eps))
          *hit = (int)prim;
      }
    } else {
      float tn1, tn2;
      const bool hl = bin_intersect(g.bnodes[n.leftFirst], org, inv, &tn1);
      const bool hr = bin_intersect(g.bnodes[n.leftFirst + 1], org, inv, &tn2);
      if (sp >= 250) return;
      if (hl && hr) {
        if (tn1 < tn2) {
          stk[++sp] = n.leftFirst;
          stk[++sp] = n.leftFirst + 1;
        } else {
          stk[++sp] = n.leftFirst + 1;
          stk[++sp] = n.leftFirst;
        }
      } else if (hl) {
        stk[++sp] = n.leftFirst;
      } else if (hr) {
        stk[++sp] = n.leftFirst + 1;
      }
    }
  }
}

template <typename F>
void parallel_range(int n, int nthreads, F&& f) {
  if (nthreads <= 1 || n < 256) {
    f(0, n);
    return;
  }
  std::vector<std::thread> ts;
  const int chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    const int b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    ts.emplace_back([&f, b, e] { f(b, e); });
  }
  for (auto& th : ts) th.join();
}

/* ---------------- shading (compat restatement of Kernel.cu:88-256) ---------------- */
inline uint32_t wang_hash(uint32_t s) {
  s = (s ^ 61u) ^ (s >> 16);
  s *= 9u;
  s = s ^ (s >> 4);
  s *= 0x27d4eb2du;
  s = s ^ (s >> 15);
  return s;
}
}  // namespace

/* xorshift32 exactly as RandomInt (src/Core/Random.cuh:17-23): all three steps
 * shift LEFT (13, 17, 5). */
static inline uint32_t rnd_int(uint32_t& s) {
  s ^= s << 13;
  s ^= s << 17;
  s ^= s << 5;
  return s;
}
static inline float rnd_float(uint32_t& s) { return (float)rnd_int(s) * 2.3283064365387e-10f; }
static inline int rnd_int_max(uint32_t& s, int maxv) { return (int)(rnd_float(s) * ((float)maxv + 0.99999f)); }

namespace {

struct Material {  // 52 bytes, reference layout (src/Core/Material.cuh:29-41)
  float albedo[3];
  float refractIdx;
  int32_t diffuseTex, normalTex, maskTex, displaceTex;
  int32_t type;
  float roughness;
  float absorption[3];
};
static_assert(sizeof(Material) == 52, "Material layout");

struct SceneView {
  const float* verts;
  const float* normals;
  const float* center_normals;
  const float* uvs;
  const uint32_t* idx;
  const uint32_t* mat_idx;
  const Material* mats;
  const uint32_t* lights;
  uint32_t light_count;
  const float* tex;  // float4 texels
  const uint32_t* tex_dims;
  const uint32_t* tex_offsets;
  int sky_tex;
  int sky_enabled, shadow, indirect;
  float normal_eps, dist_eps, tri_eps;
  const QNode* qnodes;
  const uint32_t* prims;
  int tex_filter;
};

inline float xsin(float x, int exact) { return exact ? ct::pm::sin(x) : sinf(x); }
inline float xcos(float x, int exact) { return exact ? ct::pm::cos(x) : cosf(x); }
inline float xatan2(float y, float x, int exact) { return exact ? ct::pm::atan2(y, x) : atan2f(y, x); }
inline float xacos(float x, int exact) { return exact ? ct::pm::acos(x) : acosf(x); }

// Texel addressing of SceneData::getTextureColor/getTextureNormal
// (src/Core/SceneData.cuh:81-116): grid coordinate u*(width-1); NaN or
// out-of-range coordinates are clamped to the texture (the reference would
// read outside it). tex_filter 1 (bilinear, not in the reference) blends the
// four texels around the grid point, clamped at the last row/column, as
// a + (b - a) * t per axis.
struct T4 {
  float v[4];
};
inline float grid_coord(float x, uint32_t n) {
  const float g = x * (float)(n - 1);
  return g >= 0.0f ? std::fmin(g, (float)(n - 1)) : 0.0f;
}
inline T4 texel(const SceneView& s, int idx, float x, float y) {
  const uint32_t w = s.tex_dims[idx * 2], h = s.tex_dims[idx * 2 + 1];
  const float* base = s.tex + 4 * (size_t)s.tex_offsets[idx];
  const float gx = grid_coord(x, w), gy = grid_coord(y, h);
  const uint32_t ix = (uint32_t)gx, iy = (uint32_t)gy;
  T4 o;
  if (s.tex_filter != 1) {
    std::memcpy(o.v, base + 4 * (size_t)(ix + iy * w), sizeof(o.v));
    return o;
  }
  const uint32_t ix1 = std::min(ix + 1, w - 1), iy1 = std::min(iy + 1, h - 1);
  const float tx = gx - (float)ix, ty = gy - (float)iy;
  const float* c00 = base + 4 * (size_t)(ix + iy * w);
  const float* c10 = base + 4 * (size_t)(ix1 + iy * w);
  const float* c01 = base + 4 * (size_t)(ix + iy1 * w);
  const float* c11 = base + 4 * (size_t)(ix1 + iy1 * w);
  for (int k = 0; k < 4; k++) {
    const float a = c00[k] + (c10[k] - c00[k]) * tx;
    const float b = c01[k] + (c11[k] - c01[k]) * tx;
    o.v[k] = a + (b - a) * ty;
  }
  return o;
}
inline T4 tex_color(const SceneView& s, int idx, float u, float v) {
  float x = std::fmod(u, 1.0f), y = std::fmod(v, 1.0f);
  if (x < 0) x += 1.0f;
  if (y < 0) y += 1.0f;
  return texel(s, idx, x, y);
}
inline V3 tex_normal(const SceneView& s, int idx, float u, float v) {
  float x = u, y = v;
  if (x < 0) x += 1.0f;
  if (y < 0) y += 1.0f;
  const T4 t = texel(s, idx, x, y);
  return normalize(v3(t.v[0], t.v[1], t.v[2]));
}
// sampleToWorld = convertToLocalSpace + localToWorld (src/Core/Random.cuh:37-52)
inline V3 sample_to_world(V3 sm, V3 n) {
  const V3 W = std::fabs(n.x) > 0.99f ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
  const V3 T = normalize(cross(n, W));
  const V3 B = cross(n, T);
  return add(add(muls(T, sm.x), muls(B, sm.y)), muls(n, sm.z));
}

/* SampleBSDF (src/Core/BSDF.h:33-63) with DiffuseReflectionCosWeighted and
 * Tangent2World (src/Core/Tools.h:110-137, 162-169). dir is the incoming ray
 * direction (wi = -dir). type: 0 mirror, 1 diffuse, -1 where the reference
 * leaves it unset (pdf = 0). */
void sample_bsdf(V3 color, float roughness, V3 iN, V3 N, V3 dir, float r3, float r4, int exact, V3& wo, V3& f,
                 float& pdf, int& type) {
  if (roughness < 0.1f) {
    wo = sub(dir, muls(muls(iN, dot(iN, dir)), 2.0f));  // reflect(-wi, iN)
    if (dot(N, wo) <= 0.0f) {
      pdf = 0.0f;
      f = v3(0, 0, 0);
      type = -1;
    } else {
      pdf = 1.0f;
      type = 0;
      f = muls(color, 1.0f / std::fabs(dot(iN, wo)));
    }
    return;
  }
  const float term1 = kTwoPi * r3;
  const float term2 = (float)std::sqrt(1.0 - (double)r4);  // sqrt(1.0 - r1) in double
  const float sn = xsin(term1, exact), cs = xcos(term1, exact);
  const V3 Vl = v3(cs * term2, sn * term2, std::sqrt(r4));
  V3 B, Tt;
  const V3 n = iN;
  if (n.z < 0.) {
    const float a = 1.0f / (1.0f - n.z);
    const float b = (n.x * n.y) * a;
    B = v3(1.0f - (n.x * n.x) * a, -b, n.x);
    Tt = v3(b, (n.y * n.y) * a - 1.0f, -n.y);
  } else {
    const float a = 1.0f / (1.0f + n.z);
    const float b = (-n.x * n.y) * a;
    B = v3(1.0f - (n.x * n.x) * a, b, -n.x);
    Tt = v3(b, 1.0f - (n.y * n.y) * a, -n.y);
  }
  wo = normalize(add(add(muls(Tt, Vl.x), muls(B, Vl.y)), muls(n, Vl.z)));
  if (dot(N, wo) <= 0.0f) {
    pdf = 0.0f;
    f = v3(0, 0, 0);
    type = -1;
  } else {
    type = 1;
    pdf = gmax(0.0f, dot(wo, iN)) * kOneOverPi;
    f = muls(color, kOneOverPi);
  }
}

struct PathState {
  V3 org, dir, T;
  float pdf;
  int specular;  // lastBounceType == SPECULAR
};

inline void accum_add(float* acc, V3 c) {
  acc[0] += c.x;
  acc[1] += c.y;
  acc[2] += c.z;
  acc[3] += 1.0f;
}

/* One path through `depth` extend/shade/connect passes, adding into acc[4]
 * in the order the wavefront kernels do. */
void render_path(const SceneView& s, const Geo& g, int pixel, int px, int py, int W, int H, uint32_t frame, int depth,
                 V3 cam_o, V3 cam_w, V3 hor, V3 ver, int exact, float* acc, Work* wext = nullptr,
                 Work* wshd = nullptr, int32_t* hit_log = nullptr, float* t_log = nullptr) {
  // generatePrimaryRays (Kernel.cu:208-234) with start_position = 0.
  uint32_t seed = ((uint32_t)pixel + frame * 147565741u) * 720898027u;
  const float fx = ((float)px + rnd_float(seed)) - 0.5f;
  const float fy = ((float)py + rnd_float(seed)) - 0.5f;
  const float invw = 1.0f / (float)W, invh = 1.0f / (float)H;
  // Ray::generate (Ray.cuh:85-95)
  const float sx = 2.0f * (fx * invw) - 1.0f;
  const float sy = 1.0f - 2.0f * (fy * invh);
  const V3 p = add(add(cam_w, muls(hor, sx)), muls(ver, sy));
  PathState r{cam_o, normalize(p), v3(1.0f, 1.0f, 1.0f), 1.0f, 1};

  for (int pass = 0; pass < depth; pass++) {
    const int pathLength = pass == 0 ? 0 : pass + 1;  // Kernel.cu:306,330
    float t = kMaxDistance;
    int hit = -1;
    trace_closest(g, r.org, r.dir, &t, &hit, nullptr, wext);
    if (hit_log) hit_log[pass] = hit, t_log[pass] = t;
    // ---- shade (Kernel.cu:88-206) ----
    if (!(t < kMaxDistance)) {
      if (s.sky_enabled) {
        const float u = 1.0f + (xatan2(r.dir.x, -r.dir.z, exact) * kOneOverPi) * 0.5f;
        const float v = 1.0f - xacos(r.dir.y, exact) * kOneOverPi;
        const T4 tc = tex_color(s, s.sky_tex, u, v);
        const V3 c = mul(divs(r.T, r.pdf), v3(tc.v[0], tc.v[1], tc.v[2]));
        accum_add(acc, c);
      }
      return;
    }
    const uint32_t* ti = s.idx + 3 * (size_t)hit;
    V3 N = load3(s.center_normals, hit);
    const V3 p0 = load3(s.verts, ti[0]), p1 = load3(s.verts, ti[1]), p2 = load3(s.verts, ti[2]);
    // triangle::getBaryCoords at the ray ORIGIN (Kernel.cu:107, Triangle.cuh:46-57)
    const V3 o = r.org;
    const float aABC = dot(N, cross(sub(p1, p0), sub(p2, p0)));
    const float aPBC = dot(N, cross(sub(p1, o), sub(p2, o)));
    const float aPCA = dot(N, cross(sub(p2, o), sub(p0, o)));
    const float ba = aPBC / aABC, bb = aPCA / aABC, bc = (1.f - ba) - bb;
    V3 iN = add(add(muls(load3(s.normals, ti[0]), ba), muls(load3(s.normals, ti[1]), bb)),
                muls(load3(s.normals, ti[2]), bc));
    const float* uv0 = s.uvs + 2 * (size_t)ti[0];
    const float* uv1 = s.uvs + 2 * (size_t)ti[1];
    const float* uv2 = s.uvs + 2 * (size_t)ti[2];
    const float tu = (ba * uv0[0] + bb * uv1[0]) + bc * uv2[0];
    const float tv = (ba * uv0[1] + bb * uv1[1]) + bc * uv2[1];
    const Material& mat = s.mats[s.mat_idx[hit]];
    if (mat.normalTex >= 0) iN = sample_to_world(tex_normal(s, mat.normalTex, tu, tv), iN);
    if (mat.type == 0) {  // Light
      if (!s.indirect) return;
      const float DdotNL = -dot(r.dir, iN);
      V3 c;
      if (r.specular) {
        c = mul(r.T, v3(mat.albedo[0], mat.albedo[1], mat.albedo[2]));
      } else {
        const float a = length(sub(p0, p1)), b = length(sub(p1, p2)), cc = length(sub(p2, p0));
        const float sh = ((a + b) + cc) / 2.f;
        const float ar = std::sqrt(((sh * (sh - a)) * (sh - b)) * (sh - cc));
        const float lightPDF = ((t * t) / (DdotNL * ar)) * (float)s.light_count;
        c = muls(mul(r.T, v3(mat.albedo[0], mat.albedo[1], mat.albedo[2])), 1.0f / (r.pdf + lightPDF));
      }
      c = vmax(v3(0, 0, 0), c);
      accum_add(acc, c);
      return;
    }
    r.org = add(r.org, muls(r.dir, t));  // getHitpoint: origin + t * direction
    r.T = vmax(v3(0, 0, 0), divs(r.T, r.pdf));
    const float flip = dot(r.dir, N) > 0 ? -1.0f : 1.0f;
    N = muls(N, flip);
    iN = muls(iN, flip);
    uint32_t sd = wang_hash((uint32_t)pixel * 16789u + frame * 1791u + (uint32_t)pathLength * 720898027u);
    V3 color = v3(mat.albedo[0], mat.albedo[1], mat.albedo[2]);
    if (mat.diffuseTex >= 0) {
      const T4 tc = tex_color(s, mat.diffuseTex, tu, tv);
      color = v3(tc.v[0], tc.v[1], tc.v[2]);
    }
    // convertToLocalSpace (Random.cuh:37-42): T only feeds EvaluateBSDF's unused arg
    // SampleBSDF (BSDF.h:33-63); arguments taken left to right.
    const float r3 = rnd_float(sd), r4 = rnd_float(sd);
    V3 wo, f;
    float pdf;
    // type: 0 specular, 1 diffuse, -1 left unset by the reference (a failed
    // sample). The reference then compares an uninitialised value with
    // DIFFUSE (Kernel.cu:153,156); its own GPU build of Kernel.cu takes it as
    // not diffuse (no NEE), which is what is done here. The path ends at this
    // vertex either way (pdf = 0).
    int type;
    sample_bsdf(color, mat.roughness, iN, N, r.dir, r3, r4, exact, wo, f, pdf, type);
    r.specular = type == 1 ? 0 : 1;
    r.dir = wo;
    if (type == 1 && s.shadow && s.light_count > 0) {
      const int light = std::min(rnd_int_max(sd, (int)s.light_count - 1), (int)s.light_count - 1);
      const uint32_t lprim = s.lights[light];
      const uint32_t* li = s.idx + 3 * (size_t)lprim;
      const V3 l0 = load3(s.verts, li[0]), l1 = load3(s.verts, li[1]), l2 = load3(s.verts, li[2]);
      float q1 = rnd_float(sd), q2 = rnd_float(sd);
      if (q1 + q2 > 1.0f) q1 = 1.0f - q1, q2 = 1.0f - q2;  // getRandomPointOnSurface (Triangle.cuh:67-76)
      const float qa = (1.0f - q1) - q2;
      const V3 lp = add(add(muls(l0, qa), muls(l1, q1)), muls(l2, q2));
      V3 L = sub(lp, r.org);
      const float sq = dot(L, L);
      const float dist = std::sqrt(sq);
      L = divs(L, dist);
      const V3 lN = load3(s.center_normals, lprim);
      const float NdotL = dot(iN, L);
      const float LNdotL = -dot(lN, L);
      if (NdotL > 0 && LNdotL > 0) {
        const float a = length(sub(l0, l1)), b = length(sub(l1, l2)), cc = length(sub(l2, l0));
        const float sh = ((a + b) + cc) / 2.f;
        const float ar = std::sqrt(((sh * (sh - a)) * (sh - b)) * (sh - cc));
        const Material& em = s.mats[s.mat_idx[light]];  // light-list index, as Kernel.cu:178
        const float shadowPDF = std::fabs(dot(L, iN)) * kOneOverPi;  // EvaluateBSDF
        const V3 sb = muls(color, kOneOverPi);
        if (shadowPDF > 0) {
          const float lightPDF = (sq / (LNdotL * ar)) * (float)s.light_count;
          const V3 sc = muls(mul(mul(r.T, v3(em.albedo[0], em.albedo[1], em.albedo[2])), sb),
                             NdotL / (shadowPDF + lightPDF));
          // ---- connect (Kernel.cu:247-256) ----
          const V3 so = add(r.org, muls(L, s.normal_eps));
          const float smax = dist - 2.0f * s.dist_eps;
          if (!trace_any(g, so, L, smax, wshd)) accum_add(acc, sc);
        }
      }
      r.specular = 0;
    }
    if (pdf < 1e-6f || std::isnan(pdf) || std::isnan(r.T.x) || std::isnan(r.T.y) || std::isnan(r.T.z) ||
        (r.T.x <= 0.0f && r.T.y <= 0.0f && r.T.z <= 0.0f))
      return;
    r.T = vmax(v3(0, 0, 0), muls(mul(r.T, f), std::fabs(dot(iN, r.dir))));
    r.org = add(r.org, muls(N, s.normal_eps));
    r.pdf = pdf;
  }
}

}  // namespace

static std::atomic<uint64_t> g_work[6];

extern "C" {

int or_abi_version() { return 1; }

/* Camera constructor: m_PlaneDistance = tanf(radians(fov * 0.5f)) (src/Core/Camera.cpp:16). */
float or_plane_distance(float fov_deg) { return tanf((fov_deg * 0.5f) * 0.01745329251994329576923690768489f); }

void or_triangle_bounds(const float* verts, const uint32_t* idx, int ntri, float* out_min, float* out_max) {
  for (int i = 0; i < ntri; i++) {
    const V3 a = load3(verts, idx[3 * i]), b = load3(verts, idx[3 * i + 1]), c = load3(verts, idx[3 * i + 2]);
    const V3 mn = v3(gmin(a.x, gmin(b.x, c.x)), gmin(a.y, gmin(b.y, c.y)), gmin(a.z, gmin(b.z, c.z)));
    const V3 mx = v3(gmax(a.x, gmax(b.x, c.x)), gmax(a.y, gmax(b.y, c.y)), gmax(a.z, gmax(b.z, c.z)));
    out_min[3 * i] = mn.x - 0.001f, out_min[3 * i + 1] = mn.y - 0.001f, out_min[3 * i + 2] = mn.z - 0.001f;
    out_max[3 * i] = mx.x + 0.01f, out_max[3 * i + 1] = mx.y + 0.01f, out_max[3 * i + 2] = mx.z + 0.01f;
  }
}

struct OrBVH {
  std::vector<BNode> bnodes;
  std::vector<QNode> qnodes;
  std::vector<uint32_t> prims;
};

/* Build the binary SAH tree and its quad collapse; returns an opaque handle. */
void* or_build(const float* verts, const uint32_t* idx, int ntri, int nthreads) {
  auto* out = new OrBVH();
  std::vector<Box> aabbs(ntri);
  std::vector<float> mn(3 * (size_t)ntri), mx(3 * (size_t)ntri);
  or_triangle_bounds(verts, idx, ntri, mn.data(), mx.data());
  for (int i = 0; i < ntri; i++)
    for (int k = 0; k < 3; k++) aabbs[i].mn[k] = mn[3 * i + k], aabbs[i].mx[k] = mx[3 * i + k];
  out->prims.resize(ntri);
  for (int i = 0; i < ntri; i++) out->prims[i] = (uint32_t)i;
  if (ntri == 0) return out;
  std::atomic<int> active{0};
  Builder B{aabbs.data(), out->prims.data(), std::max(0, nthreads - 1), &active};
  TNode root;
  root.first = 0;
  root.count = ntri;
  root.box = calc_bounds(B, 0, ntri);
  subdivide(B, root, 1);
  out->bnodes.assign(2 * (size_t)ntri + 2, BNode{});
  int poolPtr = 2;
  linearise(root, 0, out->bnodes, poolPtr);
  out->bnodes.resize(poolPtr);
  // BVHTree::buildBVH: a split root points at (2,3)
  // Quad collapse (MBVHTree::constructBVH, src/BVH/MBVHTree.cpp:15-30)
  out->qnodes.assign(2 * (size_t)ntri, QNode{});
  Collapser C{out->bnodes, out->qnodes, 1};
  merge(C, 0, out->bnodes[0]);
  out->qnodes.resize(C.finalPtr);
  return out;
}

int or_bvh_count(void* h) { return (int)((OrBVH*)h)->bnodes.size(); }
int or_mbvh_count(void* h) { return (int)((OrBVH*)h)->qnodes.size(); }
void or_export(void* h, void* bnodes, uint32_t* prims, void* qnodes) {
  auto* b = (OrBVH*)h;
  if (bnodes) std::memcpy(bnodes, b->bnodes.data(), b->bnodes.size() * sizeof(BNode));
  if (prims) std::memcpy(prims, b->prims.data(), b->prims.size() * 4);
  if (qnodes) std::memcpy(qnodes, b->qnodes.data(), b->qnodes.size() * sizeof(QNode));
}
void or_free(void* h) { delete (OrBVH*)h; }

/* Closest hit over caller arrays: quad nodes (128-B reference layout) and
 * prim indices. deep_out (optional) flags rays whose stack passed 32. */
void or_trace_closest(const void* qnodes, const uint32_t* prims, const float* verts, const uint32_t* idx, float eps,
                      const float* org, const float* dir, int n, int32_t* hit, float* tout, int32_t* deep_out,
                      int nthreads) {
  Geo g{verts, idx, prims, (const QNode*)qnodes, nullptr, eps};
  parallel_range(n, nthreads, [&](int b, int e) {
    Work w;
    for (int i = b; i < e; i++) {
      float t = kMaxDistance;
      int hi = -1, deep = 0;
      trace_closest(g, load3(org, i), load3(dir, i), &t, &hi, &deep, &w);
      hit[i] = hi;
      tout[i] = t;
      if (deep_out) deep_out[i] = deep;
    }
    g_work[0] += w.rays, g_work[1] += w.nodes, g_work[2] += w.tris;  // counted as extension rays
  });
}

void or_trace_any(const void* qnodes, const uint32_t* prims, const float* verts, const uint32_t* idx, float eps,
                  const float* org, const float* dir, const float* tmax, int n, uint8_t* occluded, int nthreads) {
  Geo g{verts, idx, prims, (const QNode*)qnodes, nullptr, eps};
  parallel_range(n, nthreads, [&](int b, int e) {
    for (int i = b; i < e; i++) occluded[i] = trace_any(g, load3(org, i), load3(dir, i), tmax[i]) ? 1 : 0;
  });
}

void or_trace_closest_binary(const void* bnodes, const uint32_t* prims, const float* verts, const uint32_t* idx,
                             float eps, const float* org, const float* dir, int n, int32_t* hit, float* tout,
                             int nthreads) {
  Geo g{verts, idx, prims, nullptr, (const BNode*)bnodes, eps};
  parallel_range(n, nthreads, [&](int b, int e) {
    for (int i = b; i < e; i++) {
      float t = kMaxDistance;
      int hi = -1;
      trace_closest_binary(g, load3(org, i), load3(dir, i), &t, &hi);
      hit[i] = hi;
      tout[i] = t;
    }
  });
}

/* Scene description for the frame oracle: SceneData contents
 * (src/Core/SceneData.cuh:18-45) as flat arrays. */
struct OrSceneDesc {
  const float* verts;
  const float* normals;
  const float* center_normals;
  const float* uvs;
  const uint32_t* idx;
  const uint32_t* mat_idx;
  const void* materials;  // 52-B reference Material records
  const uint32_t* lights;
  uint32_t light_count;
  const float* tex;
  const uint32_t* tex_dims;
  const uint32_t* tex_offsets;
  int32_t sky_tex;
  int32_t sky_enabled, shadow, indirect;
  float normal_eps, dist_eps, tri_eps;
  const void* qnodes;
  const uint32_t* prims;
  int32_t tex_filter;  // 0 nearest (reference), 1 bilinear
};

/* Camera basis for a frame, as sample() builds it (Kernel.cu:272-290). */
void or_camera_basis(const float* forward, const float* up, float plane_dist, int W, int H, float* hor, float* ver) {
  const V3 w = load3(forward, 0), upv = load3(up, 0);
  const V3 u = normalize(cross(w, upv));
  const V3 v = normalize(cross(u, w));
  V3 h = muls(u, plane_dist), vv = muls(v, plane_dist);
  const float aspect = (float)W / (float)H;
  if (W > H)
    h = muls(h, aspect);
  else
    vv = muls(vv, aspect);
  hor[0] = h.x, hor[1] = h.y, hor[2] = h.z;
  ver[0] = vv.x, ver[1] = vv.y, ver[2] = vv.z;
}

/* One 1-spp frame over pixels [p_begin, p_end) of a W x H image: adds into
 * accum (float4 per pixel, full image size). `frame` is the seed frame index. */
void or_render_frame(const OrSceneDesc* sd, const float* cam_pos, const float* cam_w, const float* hor,
                     const float* ver, int W, int H, uint32_t frame, int depth, int exact_math, float* accum,
                     int p_begin, int p_end, int nthreads) {
  SceneView s{sd->verts, sd->normals, sd->center_normals, sd->uvs, sd->idx, sd->mat_idx, (const Material*)sd->materials,
              sd->lights, sd->light_count, sd->tex, sd->tex_dims, sd->tex_offsets, sd->sky_tex, sd->sky_enabled,
              sd->shadow, sd->indirect, sd->normal_eps, sd->dist_eps, sd->tri_eps, (const QNode*)sd->qnodes,
              sd->prims, sd->tex_filter};
  Geo g{sd->verts, sd->idx, sd->prims, (const QNode*)sd->qnodes, nullptr, sd->tri_eps};
  const V3 co = load3(cam_pos, 0), cw = load3(cam_w, 0), h = load3(hor, 0), v = load3(ver, 0);
  const int n = p_end - p_begin;
  parallel_range(n, nthreads, [&](int b, int e) {
    Work we, ws;
    for (int i = b; i < e; i++) {
      const int pix = p_begin + i;
      render_path(s, g, pix, pix % W, (pix / W) % H, W, H, frame, depth, co, cw, h, v, exact_math,
                  accum + 4 * (size_t)pix, &we, &ws);
    }
    g_work[0] += we.rays, g_work[1] += we.nodes, g_work[2] += we.tris;
    g_work[3] += ws.rays, g_work[4] += ws.nodes, g_work[5] += ws.tris;
  });
}

/* 1-spp frames frames[0..nframes) (seed frame indices, in that order) over the
 * pixels listed in `pixels` of a W x H image, adding into accum (float4 per
 * pixel, full image size). Each pixel accumulates its frames in frame order,
 * exactly as or_render_frame called once per frame would; the threads are
 * started once for all frames and take the listed pixels interleaved, so
 * scattered rows of a frame are rendered in one balanced pass. */
void or_render_pixels(const OrSceneDesc* sd, const float* cam_pos, const float* cam_w, const float* hor,
                      const float* ver, int W, int H, const uint32_t* frames, int nframes, int depth, int exact_math,
                      float* accum, const int32_t* pixels, int npix, int nthreads) {
  SceneView s{sd->verts, sd->normals, sd->center_normals, sd->uvs, sd->idx, sd->mat_idx, (const Material*)sd->materials,
              sd->lights, sd->light_count, sd->tex, sd->tex_dims, sd->tex_offsets, sd->sky_tex, sd->sky_enabled,
              sd->shadow, sd->indirect, sd->normal_eps, sd->dist_eps, sd->tri_eps, (const QNode*)sd->qnodes,
              sd->prims, sd->tex_filter};
  Geo g{sd->verts, sd->idx, sd->prims, (const QNode*)sd->qnodes, nullptr, sd->tri_eps};
  const V3 co = load3(cam_pos, 0), cw = load3(cam_w, 0), h = load3(hor, 0), v = load3(ver, 0);
  const int nt = std::max(1, std::min(nthreads, npix));
  auto work = [&](int t) {
    Work we, ws;
    for (int i = t; i < npix; i += nt) {
      const int pix = pixels[i];
      for (int f = 0; f < nframes; f++)
        render_path(s, g, pix, pix % W, (pix / W) % H, W, H, frames[f], depth, co, cw, h, v, exact_math,
                    accum + 4 * (size_t)pix, &we, &ws);
    }
    g_work[0] += we.rays, g_work[1] += we.nodes, g_work[2] += we.tris;
    g_work[3] += ws.rays, g_work[4] += ws.nodes, g_work[5] += ws.tris;
  };
  if (nt == 1) {
    work(0);
    return;
  }
  std::vector<std::thread> ts;
  for (int t = 0; t < nt; t++) ts.emplace_back(work, t);
  for (auto& th : ts) th.join();
}

/* The closest hit of every extension pass of one pixel's path in one frame:
 * primitive id (-1: miss) and t per pass, -2 and 0 for passes the path does
 * not reach. Comparing the logs of two trees shows at which bounce their
 * answers part, and whether at an equal t (an exact tie, where the winner
 * depends on the order in which the tree presents the two triangles). */
void or_path_hits(const OrSceneDesc* sd, const float* cam_pos, const float* cam_w, const float* hor, const float* ver,
                  int W, int H, uint32_t frame, int depth, int exact_math, int pixel, int32_t* hits, float* ts) {
  SceneView s{sd->verts, sd->normals, sd->center_normals, sd->uvs, sd->idx, sd->mat_idx, (const Material*)sd->materials,
              sd->lights, sd->light_count, sd->tex, sd->tex_dims, sd->tex_offsets, sd->sky_tex, sd->sky_enabled,
              sd->shadow, sd->indirect, sd->normal_eps, sd->dist_eps, sd->tri_eps, (const QNode*)sd->qnodes,
              sd->prims, sd->tex_filter};
  Geo g{sd->verts, sd->idx, sd->prims, (const QNode*)sd->qnodes, nullptr, sd->tri_eps};
  for (int k = 0; k < depth; k++) hits[k] = -2, ts[k] = 0.0f;
  float acc[4] = {0, 0, 0, 0};
  render_path(s, g, pixel, pixel % W, (pixel / W) % H, W, H, frame, depth, load3(cam_pos, 0), load3(cam_w, 0),
              load3(hor, 0), load3(ver, 0), exact_math, acc, nullptr, nullptr, hits, ts);
}

/* Traversal work of the frames rendered since the last reset:
 * [ext rays, ext quad-node visits, ext triangle tests, shadow rays, shadow
 * node visits, shadow triangle tests]. */
void or_work_read(uint64_t* out, int reset) {
  for (int k = 0; k < 6; k++) {
    out[k] = g_work[k].load();
    if (reset) g_work[k] = 0;
  }
}

/* Child order of the quad traversal for the frames that follow: 0 the
 * reference's network (default), 1 a full sort (fast-math GPU frames). */
void or_set_full_sort(int on) { g_full_sort = on ? 1 : 0; }

/* ---- per-function entry points for the known-answer tests ---- */
void or_sample_bsdf(const float* color, float roughness, const float* iN, const float* N, const float* wi, float r3,
                    float r4, int exact, float* f_out, float* wo_out, float* pdf_out, int* type_out) {
  V3 wo, f;
  float pdf;
  int type;
  const V3 w = load3(wi, 0);
  sample_bsdf(load3(color, 0), roughness, load3(iN, 0), load3(N, 0), v3(-w.x, -w.y, -w.z), r3, r4, exact, wo, f, pdf,
              type);
  f_out[0] = f.x, f_out[1] = f.y, f_out[2] = f.z;
  wo_out[0] = wo.x, wo_out[1] = wo.y, wo_out[2] = wo.z;
  *pdf_out = pdf;
  *type_out = type;
}
uint32_t or_wang_hash(uint32_t s) { return wang_hash(s); }
void or_random_stream(uint32_t seed, int n, uint32_t* ints, float* floats) {
  uint32_t a = seed, b = seed;
  for (int i = 0; i < n; i++) {
    ints[i] = rnd_int(a);
    floats[i] = rnd_float(b);
  }
}
int or_tri_intersect(const float* o, const float* d, float* t, const float* p0, const float* p1, const float* p2,
                     float eps) {
  return tri_intersect(load3(o, 0), load3(d, 0), t, load3(p0, 0), load3(p1, 0), load3(p2, 0), eps) ? 1 : 0;
}
void or_quad_intersect(const void* node, const float* o, const float* inv, float t, int32_t* tmini, int32_t* res) {
  float tm[4];
  bool r[4];
  quad_intersect(*(const QNode*)node, load3(o, 0), load3(inv, 0), t, tm, r);
  for (int k = 0; k < 4; k++) tmini[k] = (int32_t)fbits(tm[k]), res[k] = r[k] ? 1 : 0;
}
void or_bary(const float* p, const float* n, const float* a, const float* b, const float* c, float* out) {
  const V3 P = load3(p, 0), N = load3(n, 0), p0 = load3(a, 0), p1 = load3(b, 0), p2 = load3(c, 0);
  const float aABC = dot(N, cross(sub(p1, p0), sub(p2, p0)));
  const float aPBC = dot(N, cross(sub(p1, P), sub(p2, P)));
  const float aPCA = dot(N, cross(sub(p2, P), sub(p0, P)));
  out[0] = aPBC / aABC, out[1] = aPCA / aABC, out[2] = (1.f - out[0]) - out[1];
}
float or_area(const float* a, const float* b, const float* c) {
  const V3 p0 = load3(a, 0), p1 = load3(b, 0), p2 = load3(c, 0);
  const float x = length(sub(p0, p1)), y = length(sub(p1, p2)), z = length(sub(p2, p0));
  const float s = ((x + y) + z) / 2.f;
  return std::sqrt(((s * (s - x)) * (s - y)) * (s - z));
}
void or_random_point(const float* a, const float* b, const float* c, float r1, float r2, float* out) {
  if (r1 + r2 > 1.0f) r1 = 1.0f - r1, r2 = 1.0f - r2;
  const float qa = (1.0f - r1) - r2;
  const V3 q = add(add(muls(load3(a, 0), qa), muls(load3(b, 0), r1)), muls(load3(c, 0), r2));
  out[0] = q.x, out[1] = q.y, out[2] = q.z;
}
void or_tangent2world(const float* v, const float* nn, float* out) {
  const V3 V = load3(v, 0), n = load3(nn, 0);
  V3 B, T;
  if (n.z < 0.) {
    const float a = 1.0f / (1.0f - n.z);
    const float b = (n.x * n.y) * a;
    B = v3(1.0f - (n.x * n.x) * a, -b, n.x);
    T = v3(b, (n.y * n.y) * a - 1.0f, -n.y);
  } else {
    const float a = 1.0f / (1.0f + n.z);
    const float b = (-n.x * n.y) * a;
    B = v3(1.0f - (n.x * n.x) * a, b, -n.x);
    T = v3(b, 1.0f - (n.y * n.y) * a, -n.y);
  }
  const V3 r = add(add(muls(T, V.x), muls(B, V.y)), muls(n, V.z));
  out[0] = r.x, out[1] = r.y, out[2] = r.z;
}
void or_local_space(const float* nn, float* T, float* B) {
  const V3 n = load3(nn, 0);
  const V3 W = std::fabs(n.x) > 0.99f ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
  const V3 t = normalize(cross(n, W)), b = cross(n, t);
  T[0] = t.x, T[1] = t.y, T[2] = t.z, B[0] = b.x, B[1] = b.y, B[2] = b.z;
}
void or_cos_weighted(float r3, float r4, int exact, float* out) {
  const float term1 = kTwoPi * r3;
  const float term2 = (float)std::sqrt(1.0 - (double)r4);
  out[0] = xcos(term1, exact) * term2, out[1] = xsin(term1, exact) * term2, out[2] = std::sqrt(r4);
}

/* The reproducible binary32 functions of portable_math.h over arrays (their
 * accuracy tests): sin, cos, atan2(y, x) and acos. */
void or_pm_eval(const float* x, const float* y, int n, float* s, float* c, float* at2, float* ac) {
  for (int i = 0; i < n; i++) {
    if (s || c) {
      float a, b;
      ct::pm::sincos(x[i], &a, &b);
      if (s) s[i] = a;
      if (c) c[i] = b;
    }
    if (at2) at2[i] = ct::pm::atan2(y[i], x[i]);
    if (ac) ac[i] = ct::pm::acos(x[i]);
  }
}

/* draw_framebuffer (Kernel.cu:258-270): pow(sum.rgb / samples, 1/2.2), alpha 1. */
void or_present(const float* accum, int n, float samples, float* rgba) {
  const float e = 1.0f / 2.2f;
  for (int i = 0; i < n; i++) {
    for (int k = 0; k < 3; k++) rgba[4 * i + k] = std::pow(accum[4 * i + k] / samples, e);
    rgba[4 * i + 3] = 1.0f;
  }
}

}  // extern "C"
