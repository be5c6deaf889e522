// Quad BVH built for traversal speed (ct_bvh_build_fast).
//
// The reference's tree (src/BVH/BVHNode.cu:70-190 + src/BVH/MBVHNode.cu:27-61)
// pads every triangle box by -0.001/+0.01 scene units, stops splitting only
// below four primitives or when no plane lowers area x count, and fills a quad
// node with the grandchildren of one binary node, so a node whose binary
// children are leaves keeps empty slots (one per node on average). This
// builder keeps the reference's node and leaf formats and changes the tree:
//
//  * triangle boxes padded per side by 1e-5 x max(|coordinate|, M / 4), M the
//    largest vertex coordinate magnitude, instead of the absolute padding. The
//    fast-math slab plane fma(b, 1/d, -o/d) errs by about 1.2e-7 |o| + 6e-8 |b|
//    in distance, so a ray whose origin lies within about 10 M of the scene's
//    centre of coordinates (every secondary ray, and cameras in that range)
//    never loses a box that holds its hit;
//  * a binary tree over centroid bins (16 per axis, all three axes; ranges of
//    at most 16 primitives sweep every split of the centroid order exactly)
//    split down to one primitive per leaf;
//  * binary-to-quad conversion by dynamic programming over the surface-area
//    cost (the optimal n-wide collapse of Ylitie, Karras and Laine, "Efficient
//    Incoherent Ray Traversal on GPUs Through Compressed Wide BVHs", HPG 2017):
//    C(n, i) is the least cost of subtree n spread over i slots of its parent;
//    a subtree of at most four primitives may become one leaf slot, charged
//    area x 2 x ceil(count / 2) because the traversal tests a leaf's
//    triangles two per round; an inner node is charged its area once;
//  * the slots of a node in descending box area.
//
// The primitive order is the binary tree's leaf order (each subtree covers one
// contiguous range), so every leaf slot is a contiguous range. The result does
// not depend on the thread count: children are always numbered after their
// parent and the collapse walks the tree by structure, not by number. Every
// step is a fixed sequence of IEEE operations and every partition is stable,
// so the device build (bvh_gpu_fast.cu) reproduces the nodes and the primitive
// order byte for byte.
#include <stdint.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <system_error>
#include <thread>
#include <vector>

#include "bvh_build.h"

namespace ct {
namespace {

constexpr int kBins = 16;
constexpr uint32_t kLeafMax = 4;   // largest leaf the collapse may make
constexpr int kDepthLimit = 60;    // binary depth at which a node stays a leaf
constexpr float kPad = 1e-5f;      // relative box padding per side
constexpr uint32_t kSweepMax = 16; // ranges up to this size take the exact SAH sweep

struct FBox {
  float mn[3], mx[3];
};
inline FBox fempty() { return {{1e34f, 1e34f, 1e34f}, {-1e34f, -1e34f, -1e34f}}; }
inline void fgrow(FBox& b, const FBox& o) {
  for (int k = 0; k < 3; k++) b.mn[k] = std::min(b.mn[k], o.mn[k]), b.mx[k] = std::max(b.mx[k], o.mx[k]);
}
// Surface area with the extents scaled by s, a power of two chosen from the
// scene's extent: exact scaling, so the cost comparisons are those of the
// unscaled areas wherever those are finite, and finite for any float scene.
inline float farea(const FBox& b, float s) {
  const float dx = (b.mx[0] - b.mn[0]) * s, dy = (b.mx[1] - b.mn[1]) * s, dz = (b.mx[2] - b.mn[2]) * s;
  if (dx < 0.0f) return 0.0f;
  return 2.0f * (dx * dy + dy * dz + dz * dx);
}

struct FNode {
  FBox box;
  uint32_t first, count;
  int32_t l, r;  // -1: leaf
};

struct FBins {
  FBox box[3][kBins];
  uint32_t cnt[3][kBins];
  void clear() {
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < kBins; i++) box[a][i] = fempty(), cnt[a][i] = 0;
  }
  void merge(const FBins& o) {
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < kBins; i++) fgrow(box[a][i], o.box[a][i]), cnt[a][i] += o.cnt[a][i];
  }
};

struct FCtx {
  const FBox* pb;
  const float* cent;
  uint32_t* prims;
  FNode* nodes;
  std::atomic<uint32_t>* next;
  std::atomic<int>* busy;
  int nthreads;
  float scale;  // area scale (farea)
};

// Bin of a centroid: floor((c - lo) * scale) clamped to [0, kBins - 1], defined
// for every float (NaN bins to 0, +inf to the last bin) so that every machine,
// and the device build, bins alike.
inline int bin_of(float c, float lo, float scale) {
  const float f = (c - lo) * scale;
  if (!(f >= 1.0f)) return 0;
  if (f >= (float)(kBins - 1)) return kBins - 1;
  return (int)f;
}

void bin_range(const FCtx& C, const float lo[3], const float scale[3], uint32_t b, uint32_t e, FBins& out) {
  out.clear();
  for (uint32_t k = b; k < e; k++) {
    const uint32_t p = C.prims[k];
    for (int a = 0; a < 3; a++) {
      if (!(scale[a] > 0.0f)) continue;
      const int i = bin_of(C.cent[3 * (size_t)p + a], lo[a], scale[a]);
      fgrow(out.box[a][i], C.pb[p]);
      out.cnt[a][i]++;
    }
  }
}

struct Cut {
  uint32_t mid;  // primitives in the left child
  FBox lb, rb;   // child boxes
};

// Boxes of the two halves of a range, by a pass over its primitives.
void cut_boxes(const FCtx& C, uint32_t first, uint32_t count, Cut& c) {
  c.lb = fempty(), c.rb = fempty();
  for (uint32_t k = first; k < first + c.mid; k++) fgrow(c.lb, C.pb[C.prims[k]]);
  for (uint32_t k = first + c.mid; k < first + count; k++) fgrow(c.rb, C.pb[C.prims[k]]);
}

// Binned SAH split of [first, first + count): partitions the range; the child
// boxes are the unions of their bins (exact: a bin box is a min/max union).
Cut binned_split(const FCtx& C, uint32_t first, uint32_t count) {
  FBox cb = fempty();
  for (uint32_t k = first; k < first + count; k++) {
    const float* c = C.cent + 3 * (size_t)C.prims[k];
    const FBox t = {{c[0], c[1], c[2]}, {c[0], c[1], c[2]}};
    fgrow(cb, t);
  }
  float lo[3], scale[3];
  for (int a = 0; a < 3; a++) {
    const float ext = cb.mx[a] - cb.mn[a];
    lo[a] = cb.mn[a];
    scale[a] = ext > 0.0f ? (float)kBins / ext : 0.0f;
  }
  FBins bins;
  const int want = std::min<int>(C.nthreads, (int)(count / 65536));
  if (want >= 2) {
    std::vector<FBins> part(want);
    std::vector<std::thread> ts;
    const uint32_t chunk = (count + want - 1) / want;
    for (int t = 0; t < want; t++) {
      const uint32_t b = first + t * chunk, e = std::min(first + count, b + chunk);
      try {
        ts.emplace_back([&, t, b, e] { bin_range(C, lo, scale, b, e, part[t]); });
      } catch (const std::system_error&) {
        bin_range(C, lo, scale, b, e, part[t]);
      }
    }
    for (auto& th : ts) th.join();
    bins = part[0];
    for (int t = 1; t < want; t++) bins.merge(part[t]);
  } else {
    bin_range(C, lo, scale, first, first + count, bins);
  }
  float best = 3e38f;
  int bax = -1, bsp = -1;
  for (int a = 0; a < 3; a++) {
    if (!(scale[a] > 0.0f)) continue;
    float ra[kBins];
    uint32_t rn[kBins];
    FBox r = fempty();
    uint32_t rc = 0;
    for (int i = kBins - 1; i > 0; i--) {
      fgrow(r, bins.box[a][i]);
      rc += bins.cnt[a][i];
      ra[i] = farea(r, C.scale), rn[i] = rc;
    }
    FBox l = fempty();
    uint32_t lc = 0;
    for (int i = 1; i < kBins; i++) {
      fgrow(l, bins.box[a][i - 1]);
      lc += bins.cnt[a][i - 1];
      if (lc == 0 || rn[i] == 0) continue;
      const float cost = farea(l, C.scale) * (float)lc + ra[i] * (float)rn[i];
      if (cost < best) best = cost, bax = a, bsp = i;
    }
  }
  Cut c;
  if (bax >= 0) {
    uint32_t* b = C.prims + first;
    // stable: the order inside each half (and with it the all-in-one-bin
    // halving below and the leaf order) is a function of the input order only
    uint32_t* m = std::stable_partition(b, b + count, [&](uint32_t p) {
      return bin_of(C.cent[3 * (size_t)p + bax], lo[bax], scale[bax]) < bsp;
    });
    c.mid = (uint32_t)(m - b);
    if (c.mid > 0 && c.mid < count) {
      c.lb = fempty(), c.rb = fempty();
      for (int i = 0; i < kBins; i++) fgrow(i < bsp ? c.lb : c.rb, bins.box[bax][i]);
      return c;
    }
  }
  c.mid = count / 2;  // all centroids in one bin: split the range in half
  cut_boxes(C, first, count, c);
  return c;
}

// Exact SAH split of a small range: every split of the centroid order on
// each axis (ties by primitive id). Reorders the range, returns the left count.
Cut sweep_split(const FCtx& C, uint32_t first, uint32_t count) {
  uint32_t ord[3][kSweepMax];
  float best = 3e38f;
  int bax = 0;
  uint32_t bmid = count / 2;
  for (int a = 0; a < 3; a++) {
    uint32_t* o = ord[a];
    for (uint32_t k = 0; k < count; k++) {
      const uint32_t p = C.prims[first + k];
      const float c = C.cent[3 * (size_t)p + a];
      uint32_t j = k;
      for (; j > 0; j--) {
        const uint32_t q = o[j - 1];
        const float cq = C.cent[3 * (size_t)q + a];
        if (cq < c || (cq == c && q < p)) break;
        o[j] = q;
      }
      o[j] = p;
    }
    float ra[kSweepMax];
    FBox r = fempty();
    for (uint32_t i = count - 1; i > 0; i--) {
      fgrow(r, C.pb[o[i]]);
      ra[i] = farea(r, C.scale);
    }
    FBox l = fempty();
    for (uint32_t i = 1; i < count; i++) {
      fgrow(l, C.pb[o[i - 1]]);
      const float cost = farea(l, C.scale) * (float)i + ra[i] * (float)(count - i);
      if (cost < best) best = cost, bax = a, bmid = i;
    }
  }
  memcpy(C.prims + first, ord[bax], count * sizeof(uint32_t));
  Cut c;
  c.mid = bmid;
  cut_boxes(C, first, count, c);
  return c;
}

void build_node(const FCtx& C, uint32_t ni, int depth) {
  FNode& n = C.nodes[ni];
  const uint32_t first = n.first, count = n.count;
  if (count <= 1 || depth >= kDepthLimit) return;
  const Cut cut = count <= kSweepMax ? sweep_split(C, first, count) : binned_split(C, first, count);
  const uint32_t mid = cut.mid;
  const FBox& lb = cut.lb;
  const FBox& rb = cut.rb;
  const uint32_t li = C.next->fetch_add(2), ri = li + 1;
  C.nodes[li] = FNode{lb, first, mid, -1, -1};
  C.nodes[ri] = FNode{rb, first + mid, count - mid, -1, -1};
  n.l = (int32_t)li;
  n.r = (int32_t)ri;
  bool spawned = false;
  std::thread th;
  if (mid > 16384 && count - mid > 16384) {
    if (C.busy->fetch_add(1) < C.nthreads - 1) {
      try {
        th = std::thread([&C, li, depth] { build_node(C, li, depth + 1); });
        spawned = true;
      } catch (const std::system_error&) {  // no thread to be had: build it here
        C.busy->fetch_sub(1);
      }
    } else {
      C.busy->fetch_sub(1);
    }
  }
  if (!spawned) build_node(C, li, depth + 1);
  build_node(C, ri, depth + 1);
  if (spawned) {
    th.join();
    C.busy->fetch_sub(1);
  }
}

// C[n][i], i = 1..4: least cost of subtree n in i slots of its parent
struct Cost {
  float c[5];
  int8_t leaf1;     // with one slot: 1 = a leaf, 0 = an inner quad node
  int8_t split[5];  // with i slots: 0 = as with i - 1, else slots given to the left subtree
};

void solve(const std::vector<FNode>& nodes, uint32_t used, float scale, std::vector<Cost>& d) {
  d.assign(used, Cost{});
  for (uint32_t x = used; x-- > 0;) {  // children are numbered after their parent
    const FNode& n = nodes[x];
    const float A = farea(n.box, scale);
    Cost& e = d[x];
    float leaf = 3e38f;
    if (n.count <= kLeafMax || n.l < 0) leaf = A * (float)(2 * ((n.count + 1) / 2));
    float dist[5] = {3e38f, 3e38f, 3e38f, 3e38f, 3e38f};
    int8_t dk[5] = {0, 0, 0, 0, 0};
    if (n.l >= 0) {
      const Cost& L = d[(uint32_t)n.l];
      const Cost& R = d[(uint32_t)n.r];
      for (int j = 2; j <= 4; j++)
        for (int k = 1; k < j; k++) {
          const float v = L.c[k] + R.c[j - k];
          if (v < dist[j]) dist[j] = v, dk[j] = (int8_t)k;
        }
    }
    const float inner = A + dist[4];
    e.leaf1 = leaf <= inner ? 1 : 0;
    e.c[1] = std::min(leaf, inner);
    e.split[1] = 0;
    for (int i = 2; i <= 4; i++) {
      if (dist[i] < e.c[i - 1]) e.c[i] = dist[i], e.split[i] = dk[i];
      else e.c[i] = e.c[i - 1], e.split[i] = 0;
    }
  }
}

struct Slot {
  uint32_t n;
  bool leaf;
};

void emit(const std::vector<FNode>& nodes, const std::vector<Cost>& d, uint32_t n, int i, std::vector<Slot>& out) {
  while (i > 1 && d[n].split[i] == 0) i--;
  if (i == 1) {
    out.push_back({n, d[n].leaf1 != 0});
    return;
  }
  const int k = d[n].split[i];
  emit(nodes, d, (uint32_t)nodes[n].l, k, out);
  emit(nodes, d, (uint32_t)nodes[n].r, i - k, out);
}

void set_slot(QuadNode& q, int i, const FBox& b) {
  q.bminx[i] = b.mn[0], q.bminy[i] = b.mn[1], q.bminz[i] = b.mn[2];
  q.bmaxx[i] = b.mx[0], q.bmaxy[i] = b.mx[1], q.bmaxz[i] = b.mx[2];
}

// quad nodes in pre-order from node qi (binary inner node bn); iterative
void collapse(const std::vector<FNode>& nodes, const std::vector<Cost>& d, float scale, std::vector<QuadNode>& quad) {
  struct Item {
    uint32_t qi, bn;
  };
  std::vector<Item> st{{0u, 0u}};
  std::vector<Slot> ch;
  const FBox none = fempty();
  while (!st.empty()) {
    const Item it = st.back();
    st.pop_back();
    ch.clear();
    const FNode& n = nodes[it.bn];
    float best = 3e38f;
    int bk = 1;
    for (int k = 1; k < 4; k++) {
      const float v = d[(uint32_t)n.l].c[k] + d[(uint32_t)n.r].c[4 - k];
      if (v < best) best = v, bk = k;
    }
    emit(nodes, d, (uint32_t)n.l, bk, ch);
    emit(nodes, d, (uint32_t)n.r, 4 - bk, ch);
    // largest box first: the any-hit step takes the lowest hit slot next, and a
    // larger child is the likelier occluder (closest-hit frames sort by distance)
    std::stable_sort(ch.begin(), ch.end(), [&](const Slot& a, const Slot& b) {
      return farea(nodes[a.n].box, scale) > farea(nodes[b.n].box, scale);
    });
    Item kids[4];
    int nk = 0;
    for (int i = 0; i < 4; i++) {
      if (i >= (int)ch.size()) {
        set_slot(quad[it.qi], i, none);
        quad[it.qi].childs[i] = -1, quad[it.qi].counts[i] = 0;
        continue;
      }
      const FNode& c = nodes[ch[i].n];
      set_slot(quad[it.qi], i, c.box);
      if (ch[i].leaf) {
        quad[it.qi].childs[i] = (int32_t)c.first, quad[it.qi].counts[i] = (int32_t)c.count;
      } else {
        const uint32_t nq = (uint32_t)quad.size();
        quad.emplace_back();
        quad[it.qi].childs[i] = (int32_t)nq, quad[it.qi].counts[i] = -1;
        kids[nk++] = {nq, ch[i].n};
      }
    }
    // numbering is allocation order; visit the first child next (pre-order walk)
    for (int k = nk; k-- > 0;) st.push_back(kids[k]);
  }
}

}  // namespace

// 2^-e with the largest root extent in [2^(e-1), 2^e): scaled extents below 1
float fast_area_scale(const float mn[3], const float mx[3]) {
  const float ext = std::max(mx[0] - mn[0], std::max(mx[1] - mn[1], mx[2] - mn[2]));
  if (ext > 0.0f && std::isfinite(ext)) {
    int e = 0;
    std::frexp(ext, &e);
    return std::ldexp(1.0f, -e);
  }
  return 1.0f;
}

void build_fast_quad(const float* verts, const uint32_t* idx, uint32_t ntri, int nthreads, HostBVH& out) {
  const auto t0 = std::chrono::high_resolution_clock::now();
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  out.bin.clear();
  out.quad.clear();
  out.prims.assign(ntri, 0);
  if (ntri == 0) return;
  float M = 0.0f;  // largest coordinate magnitude of the triangles' vertices
  for (uint64_t i = 0; i < 3ull * ntri; i++) {
    const float* p = verts + 3 * (size_t)idx[i];
    M = std::max(M, std::max(std::fabs(p[0]), std::max(std::fabs(p[1]), std::fabs(p[2]))));
  }
  const float floor_mag = 0.25f * M;
  std::vector<FBox> pb(ntri);
  std::vector<float> cent(3 * (size_t)ntri);
  auto prep = [&](uint32_t b, uint32_t e) {
    for (uint32_t i = b; i < e; i++) {
      const float* p0 = verts + 3 * (size_t)idx[3 * (size_t)i];
      const float* p1 = verts + 3 * (size_t)idx[3 * (size_t)i + 1];
      const float* p2 = verts + 3 * (size_t)idx[3 * (size_t)i + 2];
      FBox& t = pb[i];
      for (int k = 0; k < 3; k++) {
        float mn = std::min(p0[k], std::min(p1[k], p2[k])), mx = std::max(p0[k], std::max(p1[k], p2[k]));
        const float pad = kPad * std::max(floor_mag, std::max(std::fabs(mn), std::fabs(mx)));
        mn -= pad, mx += pad;
        mn += 0.0f, mx += 0.0f;  // -0 becomes +0: min/max unions then do not depend on the order
        t.mn[k] = mn, t.mx[k] = mx;
        cent[3 * (size_t)i + k] = 0.5f * (mn + mx);
      }
      out.prims[i] = i;
    }
  };
  {
    std::vector<std::thread> ts;
    const uint32_t chunk = (ntri + nthreads - 1) / (uint32_t)nthreads;
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
  std::vector<FNode> nodes(2 * (size_t)ntri);
  FBox root = fempty();
  for (uint32_t i = 0; i < ntri; i++) fgrow(root, pb[i]);
  nodes[0] = FNode{root, 0, ntri, -1, -1};
  std::atomic<uint32_t> next{1};
  std::atomic<int> busy{0};
  const float scale = fast_area_scale(root.mn, root.mx);
  const FCtx C{pb.data(), cent.data(), out.prims.data(), nodes.data(), &next, &busy, nthreads, scale};
  build_node(C, 0, 0);
  const auto t1 = std::chrono::high_resolution_clock::now();
  out.build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  const uint32_t used = next.load();
  out.quad.reserve(used / 3 + 2);
  out.quad.emplace_back();
  if (nodes[0].l < 0) {
    // a single primitive: one leaf slot under the root, three empty slots
    QuadNode& q = out.quad[0];
    const FBox none = fempty();
    set_slot(q, 0, nodes[0].box);
    q.childs[0] = 0, q.counts[0] = (int32_t)nodes[0].count;
    for (int i = 1; i < 4; i++) set_slot(q, i, none), q.childs[i] = -1, q.counts[i] = 0;
  } else {
    std::vector<Cost> d;
    solve(nodes, used, scale, d);
    collapse(nodes, d, scale, out.quad);
  }
  const auto t2 = std::chrono::high_resolution_clock::now();
  out.collapse_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
}

}  // namespace ct
