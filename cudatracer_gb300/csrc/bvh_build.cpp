// Host BVH builder: the reference's binned SAH (src/BVH/BVHNode.cu:70-190,
// src/BVH/BVHTree.cpp:22-50) and quad collapse (src/BVH/MBVHNode.cu:27-61,
// 226-277), rebuilt for throughput on many cores.
//
// Same trees, less work: the reference scans all primitives of a node once per
// candidate plane (3 axes x 10 planes). Because the planes of an axis are
// non-decreasing and bounding-box union (min/max) is exact and
// order-independent, one pass that assigns each centroid to the interval
// between consecutive planes, followed by prefix/suffix unions, yields
// bit-identical left/right boxes and counts for all thirty candidates. The
// cost formula, the axis-outer/plane-inner strict-less selection, the leaf
// rules (fewer than 4 primitives, depth 64, parent cost below best) and the
// in-place swap partition are the reference's, so the primitive order and the
// tree topology match it exactly. Large nodes bin in parallel; subtrees are
// built as parallel tasks. Compile with -ffp-contract=off.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <system_error>
#include <thread>

#include "ct_internal.h"

namespace ct {
namespace {

struct Box {
  float mn[3], mx[3];
};
inline Box empty_box() { return {{1e34f, 1e34f, 1e34f}, {-1e34f, -1e34f, -1e34f}}; }
// _mm_min_ps / _mm_max_ps semantics (src/BVH/AABB.h:57-60)
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
inline float gmin(float a, float b) { return b < a ? b : a; }
inline float gmax(float a, float b) { return a < b ? b : a; }

constexpr int kPlanes = 10;  // BINS 11 -> planes i = 1..10 (src/BVH/BVHNode.cu:8)
constexpr int kIntervals = kPlanes + 1;

struct Bins {
  Box box[3][kIntervals];
  int32_t cnt[3][kIntervals];
  void clear() {
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < kIntervals; i++) box[a][i] = empty_box(), cnt[a][i] = 0;
  }
  void merge(const Bins& o) {
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < kIntervals; i++) grow(box[a][i], o.box[a][i]), cnt[a][i] += o.cnt[a][i];
  }
};

struct Node {
  Box box;
  uint32_t first, count;
  int32_t left = -1, right = -1;  // arena indices
};

struct Ctx {
  const Box* aabb;
  const float* cent;  // 3 per primitive: (bmin + bmax) * 0.5f
  uint32_t* prims;
  std::vector<Node>* arena;
  std::atomic<uint32_t>* arena_ptr;
  int nthreads;
  std::atomic<int>* busy;
};

void bin_range(const Ctx& C, const float planes[3][kPlanes], uint32_t b, uint32_t e, Bins& bins) {
  bins.clear();
  for (uint32_t k = b; k < e; k++) {
    const uint32_t p = C.prims[k];
    const float* c = C.cent + 3 * (size_t)p;
    const Box& bb = C.aabb[p];
    for (int a = 0; a < 3; a++) {
      // interval = number of planes the centroid is NOT <= (NaN lands right of all)
      int iv = 0;
      for (int i = 0; i < kPlanes; i++) iv += !(c[a] <= planes[a][i]);
      grow(bins.box[a][iv], bb);
      bins.cnt[a][iv]++;
    }
  }
}

uint32_t alloc_node(const Ctx& C) { return C.arena_ptr->fetch_add(1); }

void build_node(const Ctx& C, uint32_t ni, unsigned depth) {
  Node* n = &(*C.arena)[ni];
  depth++;
  if (n->count < 4 || depth >= 64) return;
  const Box nb = n->box;
  const uint32_t first = n->first, count = n->count;
  float planes[3][kPlanes];
  for (int a = 0; a < 3; a++) {
    const float len = nb.mx[a] - nb.mn[a];
    for (int i = 1; i <= kPlanes; i++) {
      const float off = (float)i / (float)kIntervals;
      planes[a][i - 1] = nb.mn[a] + len * off;
    }
  }
  Bins bins;
  const int want = std::min<int>(C.nthreads, (int)(count / 65536));
  if (want >= 2) {
    std::vector<Bins> part(want);
    std::vector<std::thread> ts;
    const uint32_t chunk = (count + want - 1) / want;
    for (int t = 0; t < want; t++) {
      const uint32_t b = first + t * chunk, e = std::min(first + count, b + chunk);
      try {
        ts.emplace_back([&, t, b, e] { bin_range(C, planes, b, e, part[t]); });
      } catch (const std::system_error&) {
        bin_range(C, planes, b, e, part[t]);
      }
    }
    for (auto& th : ts) th.join();
    bins = part[0];
    for (int t = 1; t < want; t++) bins.merge(part[t]);
  } else {
    bin_range(C, planes, first, first + count, bins);
  }
  // thirty candidates, axis outer, plane inner, strict less (BVHNode.cu:133-163)
  const float parent_cost = area(nb) * (float)count;
  float lowest = 1e34f, best_coord = 0.0f;
  int best_axis = 0, best_plane = -1;
  Box best_l = empty_box(), best_r = empty_box();
  for (int a = 0; a < 3; a++) {
    Box suffix[kIntervals + 1];
    int32_t scnt[kIntervals + 1];
    suffix[kIntervals] = empty_box();
    scnt[kIntervals] = 0;
    for (int i = kIntervals - 1; i >= 0; i--) {
      suffix[i] = suffix[i + 1];
      grow(suffix[i], bins.box[a][i]);
      scnt[i] = scnt[i + 1] + bins.cnt[a][i];
    }
    Box pre = empty_box();
    int32_t pcnt = 0;
    for (int i = 1; i <= kPlanes; i++) {
      grow(pre, bins.box[a][i - 1]);
      pcnt += bins.cnt[a][i - 1];
      const float cost = area(pre) * (float)pcnt + area(suffix[i]) * (float)scnt[i];
      if (cost < lowest) {
        lowest = cost;
        best_coord = planes[a][i - 1];
        best_axis = a;
        best_plane = i;
        best_l = pre;
        best_r = suffix[i];
      }
    }
  }
  if (parent_cost < lowest) return;
  // in-place partition with the reference's swap sequence (BVHNode.cu:167-177)
  uint32_t lc = 0;
  for (uint32_t k = 0; k < count; k++) {
    const uint32_t p = C.prims[first + k];
    if (C.cent[3 * (size_t)p + best_axis] <= best_coord) {
      std::swap(C.prims[first + k], C.prims[first + lc]);
      lc++;
    }
  }
  if (best_plane < 0) {
    // no finite candidate but the parent cost was not below 1e34: the
    // reference still splits at plane coordinate 0 on axis 0; recompute boxes
    best_l = empty_box(), best_r = empty_box();
    for (uint32_t k = 0; k < count; k++) grow(k < lc ? best_l : best_r, C.aabb[C.prims[first + k]]);
  }
  const uint32_t li = alloc_node(C), ri = alloc_node(C);
  n = &(*C.arena)[ni];
  n->left = (int32_t)li;
  n->right = (int32_t)ri;
  Node& L = (*C.arena)[li];
  Node& R = (*C.arena)[ri];
  L = Node{best_l, first, lc, -1, -1};
  R = Node{best_r, first + lc, count - lc, -1, -1};
  // children with no primitives keep CalculateBounds' empty box and stay leaves
  bool spawned = false;
  std::thread th;
  if (lc > 16384 && count - lc > 16384) {
    if (C.busy->fetch_add(1) < C.nthreads - 1) {
      try {
        th = std::thread([&C, li, depth] { build_node(C, li, depth); });
        spawned = true;
      } catch (const std::system_error&) {  // no thread to be had: build it here
        C.busy->fetch_sub(1);
      }
    } else {
      C.busy->fetch_sub(1);
    }
  }
  if (!spawned && lc > 0) build_node(C, li, depth);
  if (count - lc > 0) build_node(C, ri, depth);
  if (spawned) {
    th.join();
    C.busy->fetch_sub(1);
  }
}

// Pool numbering of the reference's single-threaded build: root 0, slot 1
// unused, children allocated pairwise depth-first (BVHTree.cpp:33-50).
void linearise(const std::vector<Node>& arena, uint32_t ni, uint32_t slot, std::vector<BinNode>& pool,
               uint32_t& ptr) {
  // iterative to survive depth-64 trees without deep recursion concerns
  struct Item {
    uint32_t ni, slot;
  };
  std::vector<Item> st;
  st.push_back({ni, slot});
  while (!st.empty()) {
    const Item it = st.back();
    st.pop_back();
    const Node& n = arena[it.ni];
    BinNode& o = pool[it.slot];
    for (int k = 0; k < 3; k++) o.bmin[k] = n.box.mn[k], o.bmax[k] = n.box.mx[k];
    if (n.left < 0) {
      o.leftFirst = (int32_t)n.first;
      o.count = (int32_t)n.count;
      continue;
    }
    const uint32_t l = ptr++, r = ptr++;
    o.leftFirst = (int32_t)l;
    o.count = -1;
    // depth-first: left subtree fully before right -> push right first
    st.push_back({(uint32_t)n.right, r});
    st.push_back({(uint32_t)n.left, l});
  }
}

}  // namespace

void build_binary(const float* verts, const uint32_t* idx, uint32_t ntri, int nthreads, HostBVH& out) {
  const auto t0 = std::chrono::high_resolution_clock::now();
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  std::vector<Box> aabb(ntri);
  std::vector<float> cent(3 * (size_t)ntri);
  out.prims.resize(ntri);
  auto prep = [&](uint32_t b, uint32_t e) {
    for (uint32_t i = b; i < e; i++) {
      const float* p0 = verts + 3 * (size_t)idx[3 * (size_t)i];
      const float* p1 = verts + 3 * (size_t)idx[3 * (size_t)i + 1];
      const float* p2 = verts + 3 * (size_t)idx[3 * (size_t)i + 2];
      Box& b2 = aabb[i];
      for (int k = 0; k < 3; k++) {
        // triangle::getBounds: min - 0.001, max + 0.01 (Triangle.cuh:59-65)
        b2.mn[k] = gmin(p0[k], gmin(p1[k], p2[k])) - 0.001f;
        b2.mx[k] = gmax(p0[k], gmax(p1[k], p2[k])) + 0.01f;
        cent[3 * (size_t)i + k] = (b2.mn[k] + b2.mx[k]) * 0.5f;
      }
      out.prims[i] = i;
    }
  };
  {
    std::vector<std::thread> ts;
    const uint32_t chunk = (ntri + nthreads - 1) / std::max(1, nthreads);
    for (int t = 0; t < nthreads; t++) {
      const uint32_t b = t * chunk, e = std::min(ntri, b + chunk);
      if (b >= e) break;
      try {
        ts.emplace_back(prep, b, e);
      } catch (const std::system_error&) {
        prep(b, e);
      }
    }
    for (auto& th : ts) th.join();
  }
  out.bin.clear();
  if (ntri == 0) return;
  std::vector<Node> arena(2 * (size_t)ntri + 1);
  std::atomic<uint32_t> aptr{1};
  std::atomic<int> busy{0};
  Ctx C{aabb.data(), cent.data(), out.prims.data(), &arena, &aptr, nthreads, &busy};
  // root: CalculateBounds over all primitives (BVHTree.cpp:41)
  Box rb = empty_box();
  for (uint32_t i = 0; i < ntri; i++) grow(rb, aabb[i]);
  arena[0] = Node{rb, 0, ntri, -1, -1};
  build_node(C, 0, 1);
  const uint32_t nodes = aptr.load();
  out.bin.assign(std::max<uint32_t>(2, nodes + 1), BinNode{});
  uint32_t ptr = 2;
  linearise(arena, 0, 0, out.bin, ptr);
  out.bin.resize(std::max<uint32_t>(ptr, 2));
  const auto t1 = std::chrono::high_resolution_clock::now();
  out.build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
}

namespace {
void qset(QuadNode& q, int i, const float mn[3], const float mx[3]) {
  q.bminx[i] = mn[0], q.bminy[i] = mn[1], q.bminz[i] = mn[2];
  q.bmaxx[i] = mx[0], q.bmaxy[i] = mx[1], q.bmaxz[i] = mx[2];
}

// GetBVHNodeInfo (MBVHNode.cu:226-277)
int node_info(QuadNode& q, const BinNode& node, const std::vector<BinNode>& pool) {
  for (int i = 0; i < 4; i++) q.childs[i] = -1, q.counts[i] = -1;
  if (node.count > -1) return 0;
  int num = 0;
  const BinNode& L = pool[node.leftFirst];
  const BinNode& R = pool[node.leftFirst + 1];
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
}  // namespace

void collapse_quad(HostBVH& h) {
  const auto t0 = std::chrono::high_resolution_clock::now();
  h.quad.clear();
  if (h.bin.empty()) return;
  const std::vector<BinNode>& pool = h.bin;
  h.quad.reserve(pool.size() / 2 + 2);
  h.quad.emplace_back();
  const float big[3] = {1e34f, 1e34f, 1e34f}, nbig[3] = {-1e34f, -1e34f, -1e34f};
  if (pool[0].count > -1) {
    // Root leaf: the reference's collapse leaves four empty slots and the
    // scene untraceable (MBVHNode.cu:233-237); keep the leaf as child 0.
    QuadNode& q = h.quad[0];
    qset(q, 0, pool[0].bmin, pool[0].bmax);
    q.childs[0] = pool[0].leftFirst;
    q.counts[0] = pool[0].count;
    for (int i = 1; i < 4; i++) qset(q, i, big, nbig), q.childs[i] = -1, q.counts[i] = 0;
  } else {
    // MergeNodes (MBVHNode.cu:27-61) recursion made iterative; numbering is
    // the recursion's pre-order, exactly as m_FinalPtr++ assigns it.
    struct Frame {
      uint32_t qidx;
      uint32_t bin;
      int num;
      int next;
    };
    std::vector<Frame> st;
    auto open = [&](uint32_t qidx, uint32_t bin) {
      const int num = node_info(h.quad[qidx], pool[bin], pool);
      st.push_back({qidx, bin, num, 0});
    };
    open(0, 0);
    while (!st.empty()) {
      Frame& f = st.back();
      if (f.next >= f.num) {
        QuadNode& q = h.quad[f.qidx];
        for (int i = f.num; i < 4; i++) qset(q, i, big, nbig), q.counts[i] = 0;
        st.pop_back();
        continue;
      }
      const int i = f.next++;
      const uint32_t qidx = f.qidx;
      if (h.quad[qidx].counts[i] != -1) continue;
      const BinNode& cur = pool[h.quad[qidx].childs[i]];
      if (cur.count > -1) {
        QuadNode& q = h.quad[qidx];
        q.counts[i] = cur.count;
        q.childs[i] = cur.leftFirst;
        qset(q, i, cur.bmin, cur.bmax);
      } else {
        const uint32_t ni = (uint32_t)h.quad.size();
        const uint32_t cur_bin = (uint32_t)h.quad[qidx].childs[i];
        h.quad.emplace_back();
        QuadNode& q = h.quad[qidx];
        q.childs[i] = (int32_t)ni;
        q.counts[i] = -1;
        qset(q, i, cur.bmin, cur.bmax);
        open(ni, cur_bin);  // invalidates f
      }
    }
  }
  const auto t1 = std::chrono::high_resolution_clock::now();
  h.collapse_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
}

std::string validate_binary(const std::vector<BinNode>& b, uint32_t prim_count) {
  if (b.empty()) return "binary BVH has no nodes";
  std::vector<uint8_t> seen(b.size(), 0);
  std::vector<uint32_t> st{0};
  size_t visited = 0;
  while (!st.empty()) {
    const uint32_t i = st.back();
    st.pop_back();
    if (i >= b.size()) return "binary BVH child index out of range";
    if (seen[i]) return "binary BVH is not a tree (node reached twice)";
    seen[i] = 1;
    if (++visited > b.size()) return "binary BVH has a cycle";
    const BinNode& n = b[i];
    if (n.count > -1) {
      if ((uint64_t)(uint32_t)n.leftFirst + (uint64_t)n.count > prim_count || n.leftFirst < 0)
        return "binary BVH leaf range exceeds the primitive count";
    } else {
      if (n.leftFirst < 1 || (uint64_t)n.leftFirst + 1 >= b.size()) return "binary BVH child index out of range";
      st.push_back((uint32_t)n.leftFirst);
      st.push_back((uint32_t)n.leftFirst + 1);
    }
  }
  return "";
}

std::string validate_quad(const std::vector<QuadNode>& q, uint32_t prim_count) {
  if (q.empty()) return "quad BVH has no nodes";
  std::vector<uint8_t> seen(q.size(), 0);
  std::vector<uint32_t> st{0};
  while (!st.empty()) {
    const uint32_t i = st.back();
    st.pop_back();
    if (seen[i]) return "quad BVH is not a tree (node reached twice)";
    seen[i] = 1;
    for (int c = 0; c < 4; c++) {
      const int32_t cnt = q[i].counts[c], ch = q[i].childs[c];
      if (cnt == -1) {
        if (ch <= 0 || (uint32_t)ch >= q.size()) return "quad BVH child index out of range";
        st.push_back((uint32_t)ch);
      } else if (cnt > 0) {
        if (ch < 0 || (uint64_t)(uint32_t)ch + (uint64_t)cnt > prim_count)
          return "quad BVH leaf range exceeds the primitive count";
      } else if (cnt < -1) {
        return "quad BVH has a negative leaf count";
      }
    }
  }
  return "";
}

std::string leaf_encoding(uint32_t np, uint32_t max_leaf, uint32_t& shift, uint32_t& first_mask, uint32_t& count_mask) {
  // first in the low `shift` bits, count above, bit 31 flag
  shift = 1;
  while (shift < 31 && (1ull << shift) <= (uint64_t)np) shift++;
  const uint32_t count_bits = 31 - shift;
  if (count_bits == 0 || max_leaf >= (1u << count_bits))
    return "BVH leaf of " + std::to_string(max_leaf) + " primitives cannot be encoded with " + std::to_string(np) +
           " primitives";
  first_mask = (1u << shift) - 1u;
  count_mask = (1u << count_bits) - 1u;
  return "";
}

std::string to_device_layout(const HostBVH& h, const float* verts, const uint32_t* idx, uint32_t ntri,
                             DeviceLayout& out) {
  const uint32_t np = (uint32_t)h.prims.size();
  if (np != ntri) return "primitive index count does not match the scene's triangle count";
  uint32_t max_leaf = 0;
  for (const QuadNode& n : h.quad)
    for (int c = 0; c < 4; c++)
      if (n.counts[c] > 0) max_leaf = std::max<uint32_t>(max_leaf, (uint32_t)n.counts[c]);
  uint32_t shift = 0;
  const std::string enc = leaf_encoding(np, max_leaf, shift, out.first_mask, out.count_mask);
  if (!enc.empty()) return enc;
  out.leaf_shift = shift;
  out.max_leaf = max_leaf;
  const size_t nn = h.quad.size();
  out.nodes.assign(nn * sizeof(QNodeDev), 0);
  // tree depth in inner levels (DFS; imported trees may use any numbering)
  uint32_t depth = 0;
  if (nn) {
    std::vector<std::pair<uint32_t, uint32_t>> st{{0u, 1u}};
    while (!st.empty()) {
      const auto it = st.back();
      st.pop_back();
      depth = std::max(depth, it.second);
      for (int c = 0; c < 4; c++)
        if (h.quad[it.first].counts[c] == -1) st.push_back({(uint32_t)h.quad[it.first].childs[c], it.second + 1});
    }
  }
  for (size_t i = 0; i < nn; i++) {
    const QuadNode& s = h.quad[i];
    QNodeDev d;
    std::memset(&d, 0, sizeof(d));
    d.bminx = make_float4(s.bminx[0], s.bminx[1], s.bminx[2], s.bminx[3]);
    d.bmaxx = make_float4(s.bmaxx[0], s.bmaxx[1], s.bmaxx[2], s.bmaxx[3]);
    d.bminy = make_float4(s.bminy[0], s.bminy[1], s.bminy[2], s.bminy[3]);
    d.bmaxy = make_float4(s.bmaxy[0], s.bmaxy[1], s.bmaxy[2], s.bmaxy[3]);
    d.bminz = make_float4(s.bminz[0], s.bminz[1], s.bminz[2], s.bminz[3]);
    d.bmaxz = make_float4(s.bmaxz[0], s.bmaxz[1], s.bmaxz[2], s.bmaxz[3]);
    int32_t ref[4];
    for (int c = 0; c < 4; c++) {
      const int32_t cnt = s.counts[c], ch = s.childs[c];
      if (cnt == -1) {
        ref[c] = ch;
      } else if (cnt > 0) {
        ref[c] = (int32_t)(0x80000000u | ((uint32_t)cnt << shift) | (uint32_t)ch);
      } else {
        ref[c] = kEmptyChild;
      }
    }
    d.child = make_int4(ref[0], ref[1], ref[2], ref[3]);
    std::memcpy(out.nodes.data() + i * sizeof(QNodeDev), &d, sizeof(d));
  }
  out.depth = depth;
  // every inner level can leave three siblings on the stack
  out.stack_entries = (int32_t)std::min<uint32_t>(3 * depth + 1, 256);
  out.tris.assign(12 * (size_t)np, 0.0f);
  for (uint32_t j = 0; j < np; j++) {
    const uint32_t p = h.prims[j];
    const float* p0 = verts + 3 * (size_t)idx[3 * (size_t)p];
    const float* p1 = verts + 3 * (size_t)idx[3 * (size_t)p + 1];
    const float* p2 = verts + 3 * (size_t)idx[3 * (size_t)p + 2];
    float* o = out.tris.data() + 12 * (size_t)j;
    o[0] = p0[0], o[1] = p0[1], o[2] = p0[2];
    std::memcpy(&o[3], &p, 4);
    o[4] = p1[0] - p0[0], o[5] = p1[1] - p0[1], o[6] = p1[2] - p0[2], o[7] = 0.0f;
    o[8] = p2[0] - p0[0], o[9] = p2[1] - p0[1], o[10] = p2[2] - p0[2], o[11] = 0.0f;
  }
  return "";
}

}  // namespace ct
