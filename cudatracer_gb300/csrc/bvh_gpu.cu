// Device BVH builder: the reference's binned SAH (src/BVH/BVHNode.cu:121-190)
// and MergeNodes collapse (src/BVH/MBVHNode.cu:27-61, 226-277) run on the GPU.
//
// The split rule is the host builder's, evaluated with the same IEEE
// operations (no contraction: __fadd_rn/__fmul_rn/__fdiv_rn): ten planes per
// axis at min + len*i/11, a primitive's interval = the number of planes its
// centroid is not <= to, cost = area(left)*nl + area(right)*nr, the first
// lowest cost in axis-outer/plane-inner order, a leaf when the parent's cost
// is lower, when fewer than 4 primitives remain, or at binary depth 62. Bin
// boxes are unions (exact min/max), so every node box, count and primitive
// range equals the host build's: the quad tree comes out bit-identical, with
// the primitives of each leaf in another order (both partitions here are
// stable; the reference's swap partition is not).
//
// Phases:
//   prep      per-primitive padded bounds (triangle::getBounds) and the root box
//   levels    nodes with more than kWarpMax primitives, one level per round:
//             chunks of kChunk primitives bin into shared memory and flush to
//             the node's global bins; one warp per node picks the split; a
//             chunk-ordered scan gives a stable partition through a scratch copy
//   small     one warp builds the whole subtree of each node of <= kWarpMax
//             primitives, bins and partition in shared memory
//   collapse  quad nodes are the inner binary nodes at even depth; subtree
//             quad counts bottom-up (arrival counters), each quad node's
//             pre-order index from its ancestors' left-sibling counts, then
//             every quad node written in place, as MergeNodes numbers them
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "bvh_build.h"
#include "ct_internal.h"

namespace ct {
namespace {

constexpr int kPlanes = 10;
constexpr int kIntervals = kPlanes + 1;
constexpr int kBinFields = 7;  // count, min key x/y/z, max key x/y/z
constexpr int kBinWords = 3 * kIntervals * kBinFields;
constexpr uint32_t kWarpMax = 128;  // nodes up to this size are built by one warp
constexpr uint32_t kChunk = 2048;   // primitives binned by one block
constexpr int32_t kMaxSplitDepth = 61;
constexpr int kSmallStack = 64;
constexpr int kSmallWarps = 8;

enum : uint32_t { kErrDegenerate = 1, kErrArena = 2, kErrStack = 4, kErrPartition = 8 };
enum Counter : int {
  kArenaCount = 0,
  kSmallCount = 1,
  kLargeNext = 2,
  kChunkCursor = 3,
  kError = 4,
  kMaxLeaf = 5,
  kQuadDepth = 6,
  kRootKeys = 8,  // 6 words: min x/y/z, max x/y/z
  kCounterWords = 16
};

struct __align__(16) BNode {
  float mn[3];
  int32_t first;
  float mx[3];
  int32_t count;
  int32_t left;    // -1 for a leaf, else the left child (right = left + 1)
  int32_t parent;  // -1 at the root
  int32_t depth;
  uint32_t qcount;  // quad nodes in the subtree (collapse phase)
};
static_assert(sizeof(BNode) == 48, "BNode");

struct Chunk {
  int32_t slot;
  uint32_t begin, end;
};
struct Split {
  int32_t axis;  // -1: the node stays a leaf
  float coord;
  uint32_t lc;
  uint32_t chunk0;
};

// Carving of the scratch block for n primitives.
struct Layout {
  size_t lo, hi, prims, tmp, arena, arrive, qidx, large0, large1, small, chunks, chunk_left, chunk_loff, split, bins,
      counters, total;
  uint32_t cap, max_large, max_chunks, max_small;
  explicit Layout(uint32_t n) {
    cap = 2 * n + 2;
    max_large = n / (kWarpMax + 1) + 2;
    max_chunks = n / kChunk + max_large + 2;
    max_small = n / 4 + 2;
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o += (bytes + 255) & ~(size_t)255;
      return at;
    };
    lo = take(sizeof(float4) * (size_t)n);
    hi = take(sizeof(float4) * (size_t)n);
    prims = take(4 * (size_t)n);
    tmp = take(4 * (size_t)n);
    arena = take(sizeof(BNode) * (size_t)cap);
    arrive = take(4 * (size_t)cap);
    qidx = take(4 * (size_t)cap);
    large0 = take(4 * (size_t)max_large);
    large1 = take(4 * (size_t)max_large);
    small = take(4 * (size_t)max_small);
    chunks = take(sizeof(Chunk) * (size_t)max_chunks);
    chunk_left = take(4 * (size_t)max_chunks);
    chunk_loff = take(4 * (size_t)max_chunks);
    split = take(sizeof(Split) * (size_t)max_large);
    bins = take(4 * (size_t)kBinWords * max_large);
    counters = take(4 * kCounterWords);
    total = o;
  }
};

template <typename T>
T* at(void* base, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(base) + off);
}

// order-preserving float <-> uint32 keys for atomic min/max
__device__ __forceinline__ uint32_t fkey(float f) {
  const uint32_t u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float unkey(uint32_t k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}
__device__ __forceinline__ uint32_t bin_init(int w) {
  const int f = w % kBinFields;
  return f == 0 ? 0u : (f < 4 ? fkey(1e34f) : fkey(-1e34f));
}

__device__ __forceinline__ float gmin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float gmax(float a, float b) { return a < b ? b : a; }
// AABB::Area (src/BVH/AABB.h:122-129)
__device__ __forceinline__ float area3(const float mn[3], const float mx[3]) {
  const float e0 = __fsub_rn(mx[0], mn[0]), e1 = __fsub_rn(mx[1], mn[1]), e2 = __fsub_rn(mx[2], mn[2]);
  const float s = __fadd_rn(__fadd_rn(__fmul_rn(e0, e1), __fmul_rn(e0, e2)), __fmul_rn(e1, e2));
  return fmaxf(0.0f, s);
}
__device__ __forceinline__ float plane_at(float mn, float mx, int i) {
  const float len = __fsub_rn(mx, mn);
  const float off = __fdiv_rn((float)i, (float)kIntervals);
  return __fadd_rn(mn, __fmul_rn(len, off));
}
__device__ __forceinline__ float centroid(float lo, float hi) { return __fmul_rn(__fadd_rn(lo, hi), 0.5f); }
__device__ __forceinline__ float comp(const float4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// Bin one primitive into 3 x 11 intervals (counts + box keys) with atomics.
__device__ __forceinline__ void bin_prim(uint32_t* bins, const float* planes, const float4& l, const float4& h) {
  const float c[3] = {centroid(l.x, h.x), centroid(l.y, h.y), centroid(l.z, h.z)};
  const uint32_t kl[3] = {fkey(l.x), fkey(l.y), fkey(l.z)};
  const uint32_t kh[3] = {fkey(h.x), fkey(h.y), fkey(h.z)};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    int iv = 0;
#pragma unroll
    for (int j = 0; j < kPlanes; j++) iv += !(c[a] <= planes[a * kPlanes + j]);
    uint32_t* b = bins + (a * kIntervals + iv) * kBinFields;
    atomicAdd(b, 1u);
#pragma unroll
    for (int k = 0; k < 3; k++) {
      atomicMin(b + 1 + k, kl[k]);
      atomicMax(b + 4 + k, kh[k]);
    }
  }
}

struct Cand {
  float cost;
  uint32_t lc, rc;
  float lmn[3], lmx[3], rmn[3], rmx[3];
};

// Lane l < 30 evaluates axis l / 10, plane l % 10 + 1; returns the winning
// lane (first lowest cost below 1e34) or 32 when no candidate qualifies.
__device__ __forceinline__ int choose_split(const uint32_t* bins, int lane, Cand& c) {
  bool valid = false;
  c.cost = 0.0f;
  c.lc = c.rc = 0;
  if (lane < 3 * kPlanes) {
    const int a = lane / kPlanes, i = lane % kPlanes + 1;
    for (int k = 0; k < 3; k++) c.lmn[k] = c.rmn[k] = 1e34f, c.lmx[k] = c.rmx[k] = -1e34f;
    for (int iv = 0; iv < kIntervals; iv++) {
      const uint32_t* e = bins + (a * kIntervals + iv) * kBinFields;
      const uint32_t n = e[0];
      if (iv < i) {
        c.lc += n;
        for (int k = 0; k < 3; k++) c.lmn[k] = gmin(c.lmn[k], unkey(e[1 + k])), c.lmx[k] = gmax(c.lmx[k], unkey(e[4 + k]));
      } else {
        c.rc += n;
        for (int k = 0; k < 3; k++) c.rmn[k] = gmin(c.rmn[k], unkey(e[1 + k])), c.rmx[k] = gmax(c.rmx[k], unkey(e[4 + k]));
      }
    }
    c.cost = __fadd_rn(__fmul_rn(area3(c.lmn, c.lmx), __uint2float_rn(c.lc)),
                       __fmul_rn(area3(c.rmn, c.rmx), __uint2float_rn(c.rc)));
    valid = c.cost < 1e34f;
  }
  float bc = valid ? c.cost : 0.0f;
  int bl = valid ? lane : 32;
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    const float oc = __shfl_xor_sync(0xffffffffu, bc, off);
    const int ol = __shfl_xor_sync(0xffffffffu, bl, off);
    if (ol < 32 && (bl == 32 || oc < bc || (oc == bc && ol < bl))) bc = oc, bl = ol;
  }
  return bl;
}

__device__ __forceinline__ void bcast_cand(Cand& c, int src) {
  c.cost = __shfl_sync(0xffffffffu, c.cost, src);
  c.lc = __shfl_sync(0xffffffffu, c.lc, src);
  c.rc = __shfl_sync(0xffffffffu, c.rc, src);
  for (int k = 0; k < 3; k++) {
    c.lmn[k] = __shfl_sync(0xffffffffu, c.lmn[k], src);
    c.lmx[k] = __shfl_sync(0xffffffffu, c.lmx[k], src);
    c.rmn[k] = __shfl_sync(0xffffffffu, c.rmn[k], src);
    c.rmx[k] = __shfl_sync(0xffffffffu, c.rmx[k], src);
  }
}

__device__ __forceinline__ BNode make_node(const float mn[3], const float mx[3], uint32_t first, uint32_t count,
                                           int32_t parent, int32_t depth) {
  BNode b;
  for (int k = 0; k < 3; k++) b.mn[k] = mn[k], b.mx[k] = mx[k];
  b.first = (int32_t)first;
  b.count = (int32_t)count;
  b.left = -1;
  b.parent = parent;
  b.depth = depth;
  b.qcount = 0;
  return b;
}

// ---------------------------------------------------------------- prep
__global__ void k_init(uint32_t* counters) {
  const int w = threadIdx.x;
  if (w < kCounterWords)
    counters[w] = (w >= kRootKeys && w < kRootKeys + 3) ? fkey(1e34f)
                  : (w >= kRootKeys + 3 && w < kRootKeys + 6) ? fkey(-1e34f)
                                                              : 0u;
}

__global__ void __launch_bounds__(256) k_prep(const float4* __restrict__ v, const uint4* __restrict__ idx, uint32_t n,
                                              float4* __restrict__ lo, float4* __restrict__ hi,
                                              uint32_t* __restrict__ prims, uint32_t* counters) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t kmn[3] = {fkey(1e34f), fkey(1e34f), fkey(1e34f)}, kmx[3] = {fkey(-1e34f), fkey(-1e34f), fkey(-1e34f)};
  if (i < n) {
    const uint4 t = idx[i];
    const float4 a = v[t.x], b = v[t.y], c = v[t.z];
    // triangle::getBounds (src/Core/Triangle.cuh:59-65): min - 0.001, max + 0.01
    const float plo = 0.001f, phi = 0.01f;
    const float mn[3] = {__fsub_rn(gmin(a.x, gmin(b.x, c.x)), plo), __fsub_rn(gmin(a.y, gmin(b.y, c.y)), plo),
                         __fsub_rn(gmin(a.z, gmin(b.z, c.z)), plo)};
    const float mx[3] = {__fadd_rn(gmax(a.x, gmax(b.x, c.x)), phi), __fadd_rn(gmax(a.y, gmax(b.y, c.y)), phi),
                         __fadd_rn(gmax(a.z, gmax(b.z, c.z)), phi)};
    lo[i] = make_float4(mn[0], mn[1], mn[2], 0.0f);
    hi[i] = make_float4(mx[0], mx[1], mx[2], 0.0f);
    prims[i] = i;
    for (int k = 0; k < 3; k++) kmn[k] = fkey(mn[k]), kmx[k] = fkey(mx[k]);
  }
  for (int k = 0; k < 3; k++) {
    kmn[k] = __reduce_min_sync(0xffffffffu, kmn[k]);
    kmx[k] = __reduce_max_sync(0xffffffffu, kmx[k]);
  }
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 3; k++) {
      atomicMin(&counters[kRootKeys + k], kmn[k]);
      atomicMax(&counters[kRootKeys + 3 + k], kmx[k]);
    }
}

__global__ void k_root(BNode* arena, int32_t* large, int32_t* small, uint32_t n, uint32_t* counters) {
  float mn[3], mx[3];
  for (int k = 0; k < 3; k++) mn[k] = unkey(counters[kRootKeys + k]), mx[k] = unkey(counters[kRootKeys + 3 + k]);
  arena[0] = make_node(mn, mx, 0, n, -1, 0);
  counters[kArenaCount] = 1;
  if (n >= 4) {
    if (n > kWarpMax) {
      large[0] = 0;
      counters[kLargeNext] = 1;
    } else {
      small[0] = 0;
      counters[kSmallCount] = 1;
    }
  }
}

// ---------------------------------------------------------------- large nodes, one level
__global__ void k_chunks(const BNode* __restrict__ arena, const int32_t* __restrict__ large, uint32_t nl,
                         Chunk* chunks, Split* split, uint32_t* bins, uint32_t* counters) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nl) return;
  const BNode& nd = arena[large[s]];
  const uint32_t cnt = (uint32_t)nd.count, nc = (cnt + kChunk - 1) / kChunk;
  const uint32_t base = atomicAdd(&counters[kChunkCursor], nc);
  for (uint32_t c = 0; c < nc; c++) {
    const uint32_t b = (uint32_t)nd.first + c * kChunk;
    chunks[base + c] = Chunk{(int32_t)s, b, (uint32_t)nd.first + min(cnt, (c + 1) * kChunk)};
  }
  split[s] = Split{-1, 0.0f, 0u, base};
  uint32_t* b = bins + (size_t)s * kBinWords;
  for (int w = 0; w < kBinWords; w++) b[w] = bin_init(w);
}

__global__ void __launch_bounds__(256) k_bin(const BNode* __restrict__ arena, const int32_t* __restrict__ large,
                                             const Chunk* __restrict__ chunks, const uint32_t* counters,
                                             const float4* __restrict__ lo, const float4* __restrict__ hi,
                                             const uint32_t* __restrict__ prims, uint32_t* gbins) {
  __shared__ float planes[3 * kPlanes];
  __shared__ uint32_t bins[kBinWords];
  if (blockIdx.x >= counters[kChunkCursor]) return;
  const Chunk ch = chunks[blockIdx.x];
  const BNode& nd = arena[large[ch.slot]];
  if (threadIdx.x < 3 * kPlanes) {
    const int a = threadIdx.x / kPlanes, i = threadIdx.x % kPlanes + 1;
    planes[threadIdx.x] = plane_at(nd.mn[a], nd.mx[a], i);
  }
  for (int w = threadIdx.x; w < kBinWords; w += blockDim.x) bins[w] = bin_init(w);
  __syncthreads();
  for (uint32_t k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) {
    const uint32_t p = prims[k];
    bin_prim(bins, planes, lo[p], hi[p]);
  }
  __syncthreads();
  uint32_t* g = gbins + (size_t)ch.slot * kBinWords;
  for (int w = threadIdx.x; w < kBinWords; w += blockDim.x) {
    const uint32_t v = bins[w];
    const int f = w % kBinFields;
    if (f == 0) {
      if (v) atomicAdd(&g[w], v);
    } else if (f < 4) {
      if (v != fkey(1e34f)) atomicMin(&g[w], v);
    } else {
      if (v != fkey(-1e34f)) atomicMax(&g[w], v);
    }
  }
}

// Place a new child: leaf, a node for the next level, or a warp-built subtree root.
__device__ __forceinline__ void classify(int32_t id, uint32_t count, int32_t depth, int32_t* next_large,
                                         int32_t* small, uint32_t* counters) {
  if (count < 4 || depth > kMaxSplitDepth) return;
  if (count > kWarpMax)
    next_large[atomicAdd(&counters[kLargeNext], 1u)] = id;
  else
    small[atomicAdd(&counters[kSmallCount], 1u)] = id;
}

__global__ void __launch_bounds__(256) k_split(BNode* arena, const int32_t* __restrict__ large, uint32_t nl,
                                               const uint32_t* __restrict__ gbins, Split* split, int32_t* next_large,
                                               int32_t* small, uint32_t* counters, uint32_t cap) {
  const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= nl) return;  // whole warp
  const int32_t ni = large[s];
  const BNode nd = arena[ni];
  Cand c;
  const int best = choose_split(gbins + (size_t)s * kBinWords, lane, c);
  const float parent_cost = __fmul_rn(area3(nd.mn, nd.mx), __uint2float_rn((uint32_t)nd.count));
  if (best == 32) {
    // no candidate below 1e34: a leaf unless the parent's cost is not below it either
    if (!(parent_cost < 1e34f) && lane == 0) atomicOr(&counters[kError], kErrDegenerate);
    return;
  }
  bcast_cand(c, best);
  if (parent_cost < c.cost) return;
  if (lane != 0) return;
  const int a = best / kPlanes, i = best % kPlanes + 1;
  const uint32_t cid = atomicAdd(&counters[kArenaCount], 2u);
  if (cid + 2 > cap) {
    atomicOr(&counters[kError], kErrArena);
    return;
  }
  arena[cid] = make_node(c.lmn, c.lmx, (uint32_t)nd.first, c.lc, ni, nd.depth + 1);
  arena[cid + 1] = make_node(c.rmn, c.rmx, (uint32_t)nd.first + c.lc, c.rc, ni, nd.depth + 1);
  arena[ni].left = (int32_t)cid;
  split[s].axis = a;
  split[s].coord = plane_at(nd.mn[a], nd.mx[a], i);
  split[s].lc = c.lc;
  classify((int32_t)cid, c.lc, nd.depth + 1, next_large, small, counters);
  classify((int32_t)cid + 1, c.rc, nd.depth + 1, next_large, small, counters);
}

__device__ __forceinline__ bool goes_left(const float4* lo, const float4* hi, uint32_t p, int axis, float coord) {
  return centroid(comp(lo[p], axis), comp(hi[p], axis)) <= coord;
}

__global__ void __launch_bounds__(256) k_part_count(const Chunk* __restrict__ chunks, const Split* __restrict__ split,
                                                    const uint32_t* counters, const float4* __restrict__ lo,
                                                    const float4* __restrict__ hi, const uint32_t* __restrict__ prims,
                                                    uint32_t* chunk_left) {
  __shared__ uint32_t warp_sum[8];
  if (blockIdx.x >= counters[kChunkCursor]) return;
  const Chunk ch = chunks[blockIdx.x];
  const Split sp = split[ch.slot];
  if (sp.axis < 0) return;
  uint32_t n = 0;
  for (uint32_t k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) n += goes_left(lo, hi, prims[k], sp.axis, sp.coord);
  n = __reduce_add_sync(0xffffffffu, n);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += warp_sum[w];
    chunk_left[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(256) k_part_offsets(const BNode* __restrict__ arena, const int32_t* __restrict__ large,
                                                      uint32_t nl, Split* split,
                                                      const uint32_t* __restrict__ chunk_left, uint32_t* chunk_loff,
                                                      uint32_t* counters) {
  const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= nl) return;
  const Split sp = split[s];
  if (sp.axis < 0) return;
  const uint32_t nc = ((uint32_t)arena[large[s]].count + kChunk - 1) / kChunk;
  uint32_t run = 0;
  for (uint32_t c0 = 0; c0 < nc; c0 += 32) {
    const uint32_t c = c0 + lane;
    const uint32_t v = c < nc ? chunk_left[sp.chunk0 + c] : 0u;
    uint32_t x = v;  // inclusive warp scan
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    if (c < nc) chunk_loff[sp.chunk0 + c] = run + x - v;
    run += __shfl_sync(0xffffffffu, x, 31);
  }
  if (lane == 0 && run != sp.lc) {
    // the flags disagree with the bins: leave the range as it is (the build fails)
    atomicOr(&counters[kError], kErrPartition);
    split[s].axis = -1;
  }
}

__global__ void __launch_bounds__(256) k_part_scatter(const BNode* __restrict__ arena, const int32_t* __restrict__ large,
                                                      const Chunk* __restrict__ chunks, const Split* __restrict__ split,
                                                      const uint32_t* counters, const uint32_t* __restrict__ chunk_loff,
                                                      const float4* __restrict__ lo, const float4* __restrict__ hi,
                                                      const uint32_t* __restrict__ prims, uint32_t* tmp) {
  __shared__ uint32_t wl[8], wr[8];
  if (blockIdx.x >= counters[kChunkCursor]) return;
  const Chunk ch = chunks[blockIdx.x];
  const Split sp = split[ch.slot];
  if (sp.axis < 0) return;
  const uint32_t first = (uint32_t)arena[large[ch.slot]].first;
  const uint32_t loff = chunk_loff[blockIdx.x];
  const uint32_t roff = (ch.begin - first) - loff;
  uint32_t dl = first + loff, dr = first + sp.lc + roff;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  const uint32_t lt = (1u << lane) - 1u;
  for (uint32_t k0 = ch.begin; k0 < ch.end; k0 += blockDim.x) {
    const uint32_t k = k0 + threadIdx.x;
    const bool in = k < ch.end;
    const uint32_t p = in ? prims[k] : 0u;
    const bool left = in && goes_left(lo, hi, p, sp.axis, sp.coord);
    const uint32_t bl = __ballot_sync(0xffffffffu, left), br = __ballot_sync(0xffffffffu, in && !left);
    if (lane == 0) wl[warp] = __popc(bl), wr[warp] = __popc(br);
    __syncthreads();
    uint32_t pl = 0, pr = 0, tl = 0, tr = 0;
    for (int w = 0; w < nw; w++) {
      if (w < warp) pl += wl[w], pr += wr[w];
      tl += wl[w], tr += wr[w];
    }
    if (left) tmp[dl + pl + __popc(bl & lt)] = p;
    else if (in) tmp[dr + pr + __popc(br & lt)] = p;
    dl += tl, dr += tr;
    __syncthreads();
  }
}

__global__ void __launch_bounds__(256) k_part_copy(const Chunk* __restrict__ chunks, const Split* __restrict__ split,
                                                   const uint32_t* counters, const uint32_t* __restrict__ tmp,
                                                   uint32_t* prims) {
  if (blockIdx.x >= counters[kChunkCursor]) return;
  const Chunk ch = chunks[blockIdx.x];
  if (split[ch.slot].axis < 0) return;
  for (uint32_t k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) prims[k] = tmp[k];
}

// ---------------------------------------------------------------- small subtrees, one warp each
__global__ void __launch_bounds__(kSmallWarps * 32) k_small(BNode* arena, const int32_t* __restrict__ small,
                                                            const uint32_t* counters_ro, const float4* __restrict__ lo,
                                                            const float4* __restrict__ hi, uint32_t* prims,
                                                            uint32_t* counters, uint32_t cap) {
  __shared__ uint32_t sbins[kSmallWarps][kBinWords];
  __shared__ float splanes[kSmallWarps][3 * kPlanes];
  __shared__ int32_t sstack[kSmallWarps][kSmallStack];
  __shared__ uint32_t stmp[kSmallWarps][2 * kWarpMax];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t* bins = sbins[warp];
  float* planes = splanes[warp];
  int32_t* stack = sstack[warp];
  uint32_t* tmp = stmp[warp];
  const uint32_t nsmall = counters_ro[kSmallCount];
  for (uint32_t s = blockIdx.x * kSmallWarps + warp; s < nsmall; s += gridDim.x * kSmallWarps) {
    int sp = 0;
    if (lane == 0) stack[0] = small[s];
    sp = 1;
    __syncwarp();
    while (sp > 0) {
      const int32_t ni = stack[--sp];
      __syncwarp();
      const BNode nd = arena[ni];
      const uint32_t first = (uint32_t)nd.first, count = (uint32_t)nd.count;
      if (lane < 3 * kPlanes) planes[lane] = plane_at(nd.mn[lane / kPlanes], nd.mx[lane / kPlanes], lane % kPlanes + 1);
      for (int w = lane; w < kBinWords; w += 32) bins[w] = bin_init(w);
      __syncwarp();
      for (uint32_t k = lane; k < count; k += 32) {
        const uint32_t p = prims[first + k];
        bin_prim(bins, planes, lo[p], hi[p]);
      }
      __syncwarp();
      Cand c;
      const int best = choose_split(bins, lane, c);
      const float parent_cost = __fmul_rn(area3(nd.mn, nd.mx), __uint2float_rn(count));
      if (best == 32) {
        if (!(parent_cost < 1e34f) && lane == 0) atomicOr(&counters[kError], kErrDegenerate);
        continue;
      }
      bcast_cand(c, best);
      if (parent_cost < c.cost) continue;
      const int a = best / kPlanes;
      const float coord = planes[best];
      // stable partition through shared memory
      uint32_t nl = 0, nr = 0;
      for (uint32_t k0 = 0; k0 < count; k0 += 32) {
        const uint32_t k = k0 + lane;
        const bool in = k < count;
        const uint32_t p = in ? prims[first + k] : 0u;
        const bool left = in && goes_left(lo, hi, p, a, coord);
        const uint32_t bl = __ballot_sync(0xffffffffu, left), br = __ballot_sync(0xffffffffu, in && !left);
        if (left) tmp[nl + __popc(bl & lt)] = p;
        else if (in) tmp[kWarpMax + nr + __popc(br & lt)] = p;
        nl += __popc(bl), nr += __popc(br);
      }
      __syncwarp();
      if (nl != c.lc) {
        if (lane == 0) atomicOr(&counters[kError], kErrPartition);
        continue;
      }
      for (uint32_t k = lane; k < count; k += 32) prims[first + k] = k < nl ? tmp[k] : tmp[kWarpMax + k - nl];
      uint32_t cid = 0;
      if (lane == 0) cid = atomicAdd(&counters[kArenaCount], 2u);
      cid = __shfl_sync(0xffffffffu, cid, 0);
      if (cid + 2 > cap) {
        if (lane == 0) atomicOr(&counters[kError], kErrArena);
        continue;
      }
      if (lane == 0) {
        arena[cid] = make_node(c.lmn, c.lmx, first, c.lc, ni, nd.depth + 1);
        arena[cid + 1] = make_node(c.rmn, c.rmx, first + c.lc, c.rc, ni, nd.depth + 1);
        arena[ni].left = (int32_t)cid;
      }
      const bool push_r = c.rc >= 4 && nd.depth + 1 <= kMaxSplitDepth;
      const bool push_l = c.lc >= 4 && nd.depth + 1 <= kMaxSplitDepth;
      if (sp + (int)push_r + (int)push_l > kSmallStack) {
        if (lane == 0) atomicOr(&counters[kError], kErrStack);
        continue;
      }
      if (lane == 0) {
        if (push_r) stack[sp] = (int32_t)cid + 1;
        if (push_l) stack[sp + (int)push_r] = (int32_t)cid;
      }
      sp += (int)push_r + (int)push_l;
      __syncwarp();
    }
  }
}

// ---------------------------------------------------------------- collapse
__device__ __forceinline__ bool is_quad(const BNode& b) { return b.left >= 0 && (b.depth & 1) == 0; }

__global__ void k_qcount(BNode* arena, uint32_t* arrive, const uint32_t* counters_ro, uint32_t* counters) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= counters_ro[kArenaCount]) return;
  if (arena[i].left >= 0) return;
  atomicMax(&counters[kMaxLeaf], (uint32_t)arena[i].count);
  int32_t cur = (int32_t)i;
  while (true) {
    const int32_t p = arena[cur].parent;
    if (p < 0) break;
    __threadfence();
    if (atomicAdd(&arrive[p], 1u) == 0) return;  // the sibling's subtree is not finished yet
    __threadfence();
    const int32_t l = arena[p].left;
    const uint32_t q = __ldcg(&arena[l].qcount) + __ldcg(&arena[l + 1].qcount) + ((arena[p].depth & 1) == 0 ? 1u : 0u);
    __stcg(&arena[p].qcount, q);
    cur = p;
  }
}

__global__ void k_qindex(const BNode* __restrict__ arena, const uint32_t* counters_ro, uint32_t* qidx,
                         uint32_t* counters) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= counters_ro[kArenaCount]) return;
  const BNode b = arena[i];
  if (!is_quad(b)) return;
  // pre-order position: one for each quad ancestor step, plus the quad nodes of
  // every earlier slot (MergeNodes visits slots left to right, depth first)
  uint32_t idx = 0;
  int32_t cur = (int32_t)i;
  while (cur != 0) {
    const int32_t y = arena[cur].parent, p = arena[y].parent;
    const int32_t ly = arena[y].left, lp = arena[p].left;
    idx += 1;
    if (cur == ly + 1) idx += arena[ly].qcount;
    if (y == lp + 1) idx += arena[lp].qcount;
    cur = p;
  }
  qidx[i] = idx;
  atomicMax(&counters[kQuadDepth], (uint32_t)(b.depth / 2 + 1));
}

__device__ __forceinline__ void set_slot(QuadNode& q, int s, const float mn[3], const float mx[3], int32_t child,
                                         int32_t count) {
  q.bminx[s] = mn[0], q.bminy[s] = mn[1], q.bminz[s] = mn[2];
  q.bmaxx[s] = mx[0], q.bmaxy[s] = mx[1], q.bmaxz[s] = mx[2];
  q.childs[s] = child;
  q.counts[s] = count;
}

__global__ void k_qwrite(const BNode* __restrict__ arena, const uint32_t* counters_ro, const uint32_t* __restrict__ qidx,
                         uint32_t nq, QuadNode* quad) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= counters_ro[kArenaCount]) return;
  const BNode b = arena[i];
  const float big[3] = {1e34f, 1e34f, 1e34f}, nbig[3] = {-1e34f, -1e34f, -1e34f};
  QuadNode q;
  int num = 0;
  if (i == 0 && b.left < 0) {
    // a root that is a leaf becomes child 0 of the quad root (the reference
    // would leave the tree empty, src/BVH/MBVHNode.cu:233-237)
    set_slot(q, num++, b.mn, b.mx, b.first, b.count);
  } else {
    if (!is_quad(b)) return;
    auto slot = [&](int32_t s) {
      const BNode& c = arena[s];
      if (c.left < 0) set_slot(q, num++, c.mn, c.mx, c.first, c.count);
      else set_slot(q, num++, c.mn, c.mx, (int32_t)qidx[s], -1);
    };
    for (int side = 0; side < 2; side++) {
      const int32_t ci = b.left + side;
      const BNode& c = arena[ci];
      if (c.left < 0) {
        set_slot(q, num++, c.mn, c.mx, c.first, c.count);
      } else {
        slot(c.left);
        slot(c.left + 1);
      }
    }
  }
  for (int s = num; s < 4; s++) set_slot(q, s, big, nbig, -1, 0);
  const uint32_t at_idx = i == 0 ? 0u : qidx[i];
  if (at_idx < nq) quad[at_idx] = q;
}

__global__ void k_qdev(const QuadNode* __restrict__ quad, uint32_t nq, uint32_t shift, QNodeDev* out) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nq) return;
  const QuadNode& s = quad[i];
  QNodeDev d;
  d.bminx = make_float4(s.bminx[0], s.bminx[1], s.bminx[2], s.bminx[3]);
  d.bmaxx = make_float4(s.bmaxx[0], s.bmaxx[1], s.bmaxx[2], s.bmaxx[3]);
  d.bminy = make_float4(s.bminy[0], s.bminy[1], s.bminy[2], s.bminy[3]);
  d.bmaxy = make_float4(s.bmaxy[0], s.bmaxy[1], s.bmaxy[2], s.bmaxy[3]);
  d.bminz = make_float4(s.bminz[0], s.bminz[1], s.bminz[2], s.bminz[3]);
  d.bmaxz = make_float4(s.bmaxz[0], s.bmaxz[1], s.bmaxz[2], s.bmaxz[3]);
  int32_t ref[4];
  for (int c = 0; c < 4; c++) {
    const int32_t cnt = s.counts[c], ch = s.childs[c];
    ref[c] = cnt == -1 ? ch : (cnt > 0 ? (int32_t)(0x80000000u | ((uint32_t)cnt << shift) | (uint32_t)ch) : kEmptyChild);
  }
  d.child = make_int4(ref[0], ref[1], ref[2], ref[3]);
  d.meta = make_int4(0, 0, 0, 0);
  out[i] = d;
}

__global__ void k_tris(const float4* __restrict__ v, const uint4* __restrict__ idx, const uint32_t* __restrict__ prims,
                       uint32_t n, float4* tris) {
  const uint32_t j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= n) return;
  const uint32_t p = prims[j];
  const uint4 t = idx[p];
  const float4 a = v[t.x], b = v[t.y], c = v[t.z];
  tris[3 * (size_t)j] = make_float4(a.x, a.y, a.z, __uint_as_float(p));
  tris[3 * (size_t)j + 1] = make_float4(__fsub_rn(b.x, a.x), __fsub_rn(b.y, a.y), __fsub_rn(b.z, a.z), 0.0f);
  tris[3 * (size_t)j + 2] = make_float4(__fsub_rn(c.x, a.x), __fsub_rn(c.y, a.y), __fsub_rn(c.z, a.z), 0.0f);
}

unsigned blocks(uint64_t n, unsigned per) { return (unsigned)((n + per - 1) / per); }

#define GB_TRY(call)                      \
  do {                                    \
    cudaError_t e_ = (call);              \
    if (e_ != cudaSuccess) return e_;     \
  } while (0)

}  // namespace

size_t gpu_bvh_scratch_bytes(uint32_t n) { return Layout(n).total; }

cudaError_t gpu_bvh_build(const DevScene& sc, void* scratch, uint32_t* host_counters, cudaStream_t s,
                          GpuBvhResult& r) {
  const uint32_t n = sc.tri_count;
  const Layout L(n);
  uint32_t* counters = at<uint32_t>(scratch, L.counters);
  float4* lo = at<float4>(scratch, L.lo);
  float4* hi = at<float4>(scratch, L.hi);
  uint32_t* prims = at<uint32_t>(scratch, L.prims);
  uint32_t* tmp = at<uint32_t>(scratch, L.tmp);
  BNode* arena = at<BNode>(scratch, L.arena);
  int32_t* large[2] = {at<int32_t>(scratch, L.large0), at<int32_t>(scratch, L.large1)};
  int32_t* small = at<int32_t>(scratch, L.small);
  Chunk* chunks = at<Chunk>(scratch, L.chunks);
  uint32_t* chunk_left = at<uint32_t>(scratch, L.chunk_left);
  uint32_t* chunk_loff = at<uint32_t>(scratch, L.chunk_loff);
  Split* split = at<Split>(scratch, L.split);
  uint32_t* bins = at<uint32_t>(scratch, L.bins);
  uint32_t* arrive = at<uint32_t>(scratch, L.arrive);
  uint32_t* qidx = at<uint32_t>(scratch, L.qidx);

  k_init<<<1, 32, 0, s>>>(counters);
  k_prep<<<blocks(n, 256), 256, 0, s>>>(sc.verts, sc.idx, n, lo, hi, prims, counters);
  k_root<<<1, 1, 0, s>>>(arena, large[0], small, n, counters);
  GB_TRY(cudaGetLastError());
  GB_TRY(cudaMemcpyAsync(host_counters, counters, 4 * kCounterWords, cudaMemcpyDeviceToHost, s));
  GB_TRY(cudaStreamSynchronize(s));
  uint32_t nl = host_counters[kLargeNext];
  int cur = 0;
  r.levels = 0;
  while (nl > 0) {
    if (nl > L.max_large) return cudaErrorInvalidValue;
    GB_TRY(cudaMemsetAsync(counters + kLargeNext, 0, 8, s));  // kLargeNext, kChunkCursor
    k_chunks<<<blocks(nl, 128), 128, 0, s>>>(arena, large[cur], nl, chunks, split, bins, counters);
    const unsigned nchunk = (unsigned)std::min<uint64_t>((uint64_t)n / kChunk + nl + 1, L.max_chunks);
    k_bin<<<nchunk, 256, 0, s>>>(arena, large[cur], chunks, counters, lo, hi, prims, bins);
    k_split<<<blocks((uint64_t)nl * 32, 256), 256, 0, s>>>(arena, large[cur], nl, bins, split, large[cur ^ 1], small,
                                                          counters, L.cap);
    k_part_count<<<nchunk, 256, 0, s>>>(chunks, split, counters, lo, hi, prims, chunk_left);
    k_part_offsets<<<blocks((uint64_t)nl * 32, 256), 256, 0, s>>>(arena, large[cur], nl, split, chunk_left, chunk_loff,
                                                                 counters);
    k_part_scatter<<<nchunk, 256, 0, s>>>(arena, large[cur], chunks, split, counters, chunk_loff, lo, hi, prims, tmp);
    k_part_copy<<<nchunk, 256, 0, s>>>(chunks, split, counters, tmp, prims);
    GB_TRY(cudaGetLastError());
    GB_TRY(cudaMemcpyAsync(host_counters, counters, 4 * kCounterWords, cudaMemcpyDeviceToHost, s));
    GB_TRY(cudaStreamSynchronize(s));
    nl = host_counters[kLargeNext];
    cur ^= 1;
    r.levels++;
    if (host_counters[kError]) break;
  }
  const uint32_t nsmall = host_counters[kSmallCount];
  if (nsmall > 0 && !host_counters[kError]) {
    const int sms = sm_count();
    const unsigned g = (unsigned)std::min<uint64_t>(blocks(nsmall, kSmallWarps), (uint64_t)sms * 8);
    k_small<<<g, kSmallWarps * 32, 0, s>>>(arena, small, counters, lo, hi, prims, counters, L.cap);
    GB_TRY(cudaGetLastError());
  }
  GB_TRY(cudaMemsetAsync(arrive, 0, 4 * (size_t)L.cap, s));
  // arena size bound for the grids below: the count is read on the device
  GB_TRY(cudaMemcpyAsync(host_counters, counters, 4 * kCounterWords, cudaMemcpyDeviceToHost, s));
  GB_TRY(cudaStreamSynchronize(s));
  const uint32_t nb = host_counters[kArenaCount];
  k_qcount<<<blocks(nb, 256), 256, 0, s>>>(arena, arrive, counters, counters);
  k_qindex<<<blocks(nb, 256), 256, 0, s>>>(arena, counters, qidx, counters);
  GB_TRY(cudaGetLastError());
  BNode root;
  GB_TRY(cudaMemcpyAsync(host_counters, counters, 4 * kCounterWords, cudaMemcpyDeviceToHost, s));
  GB_TRY(cudaMemcpyAsync(&root, arena, sizeof(BNode), cudaMemcpyDeviceToHost, s));
  GB_TRY(cudaStreamSynchronize(s));
  r.binary_nodes = host_counters[kArenaCount];
  r.error = host_counters[kError];
  r.max_leaf = host_counters[kMaxLeaf];
  if (root.left < 0) {
    r.quad_nodes = 1;
    r.depth = 1;
  } else {
    r.quad_nodes = root.qcount;
    r.depth = host_counters[kQuadDepth];
  }
  r.small_roots = nsmall;
  return cudaSuccess;
}

cudaError_t launch_quad_to_dev(const QuadNode* quad, uint32_t nq, uint32_t leaf_shift, QNodeDev* nodes, cudaStream_t s) {
  if (nq) k_qdev<<<blocks(nq, 256), 256, 0, s>>>(quad, nq, leaf_shift, nodes);
  return cudaGetLastError();
}

cudaError_t launch_leaf_tris(const DevScene& sc, const uint32_t* prims, uint32_t n, float4* tris, cudaStream_t s) {
  if (n) k_tris<<<blocks(n, 256), 256, 0, s>>>(sc.verts, sc.idx, prims, n, tris);
  return cudaGetLastError();
}

cudaError_t gpu_bvh_emit(const DevScene& sc, void* scratch, const GpuBvhResult& r, uint32_t leaf_shift, void* quad_out,
                         QNodeDev* nodes, float4* tris, uint32_t* prims_out, cudaStream_t s) {
  const uint32_t n = sc.tri_count;
  const Layout L(n);
  const uint32_t* counters = at<uint32_t>(scratch, L.counters);
  const BNode* arena = at<BNode>(scratch, L.arena);
  const uint32_t* qidx = at<uint32_t>(scratch, L.qidx);
  const uint32_t* prims = at<uint32_t>(scratch, L.prims);
  QuadNode* quad = static_cast<QuadNode*>(quad_out);
  k_qwrite<<<blocks(r.binary_nodes, 256), 256, 0, s>>>(arena, counters, qidx, r.quad_nodes, quad);
  k_qdev<<<blocks(r.quad_nodes, 256), 256, 0, s>>>(quad, r.quad_nodes, leaf_shift, nodes);
  k_tris<<<blocks(n, 256), 256, 0, s>>>(sc.verts, sc.idx, prims, n, tris);
  GB_TRY(cudaGetLastError());
  GB_TRY(cudaMemcpyAsync(prims_out, prims, 4 * (size_t)n, cudaMemcpyDeviceToDevice, s));
  return cudaSuccess;
}


// ================================================================ 8-wide quantised collapse
namespace {

enum WCounter : int { kWideCount = 0, kWidePrims = 1, kWideNext = 2, kWideError = 3, kWideCounterWords = 8 };
enum : uint32_t { kWErrSlots = 1, kWErrCapacity = 2, kWErrQuant = 4 };

struct WEntry {
  uint32_t wide, bin;
};

struct WLayout {
  size_t nodes, list0, list1, counters, total;
  uint32_t cap;
  explicit WLayout(uint32_t binary_nodes) {
    cap = binary_nodes / 2 + 2;  // inner binary nodes + the root
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t a = o;
      o += (bytes + 255) & ~(size_t)255;
      return a;
    };
    nodes = take(sizeof(WNode8) * (size_t)cap);
    list0 = take(sizeof(WEntry) * (size_t)cap);
    list1 = take(sizeof(WEntry) * (size_t)cap);
    counters = take(4 * kWideCounterWords);
    total = o;
  }
};

__device__ __forceinline__ uint32_t leaf_slots(int32_t count) { return count <= 0 ? 1u : (uint32_t)(count + 2) / 3u; }
__device__ __forceinline__ float pow2(int biased) { return __int_as_float(biased << 23); }

// Smallest biased exponent whose 255 steps from p reach hi (fma as the traversal evaluates it).
__device__ __forceinline__ int quant_exponent(float p, float hi) {
  const float ext = __fsub_rn(hi, p);
  int e = 1;
  if (ext > 0.0f) {
    int k = 0;
    frexpf(__fdiv_rn(ext, 255.0f), &k);
    e = max(1, min(254, k + 127));
  }
  while (e < 254 && __fmaf_rn(pow2(e), 255.0f, p) < hi) e++;
  return e;
}

// Outward 8-bit bounds of [lo, hi] on the grid p + s*q; false if none fits.
__device__ __forceinline__ bool quantise(float p, float s, float lo, float hi, uint8_t& qlo, uint8_t& qhi) {
  float fl = floorf(__fdiv_rn(__fsub_rn(lo, p), s)), fh = ceilf(__fdiv_rn(__fsub_rn(hi, p), s));
  int ql = (int)fminf(fmaxf(fl, 0.0f), 255.0f), qh = (int)fminf(fmaxf(fh, 0.0f), 255.0f);
  while (ql > 0 && __fmaf_rn(s, (float)ql, p) > lo) ql--;
  while (qh < 255 && __fmaf_rn(s, (float)qh, p) < hi) qh++;
  qlo = (uint8_t)ql, qhi = (uint8_t)qh;
  return __fmaf_rn(s, (float)ql, p) <= lo && __fmaf_rn(s, (float)qh, p) >= hi;
}

__device__ __forceinline__ uint32_t wsplit(const WideCost& c, int i) { return (c.split >> (3 * (i - 2))) & 7u; }

__global__ void __launch_bounds__(128) k_wcollapse(const BNode* __restrict__ arena, const uint32_t* __restrict__ bprims,
                                                   const WideCost* __restrict__ cost, const float4* __restrict__ v,
                                                   const uint4* __restrict__ idx, const WEntry* __restrict__ in,
                                                   uint32_t n_in, WEntry* out, uint32_t* counters, WNode8* wn,
                                                   float4* wtris, uint32_t cap, uint32_t n_prims) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_in) return;
  const WEntry en = in[i];
  const BNode b = arena[en.bin];
  // frontier of binary nodes under this wide node, in left-to-right order;
  // leafy[k]: entry k becomes leaf slots (its primitive range, three per slot)
  int32_t F[8];
  bool leafy[8];
  int nf = 0;
  auto usage = [&](int32_t x, bool lf) {
    const BNode& c = arena[x];
    return lf ? leaf_slots(c.count) : 1u;
  };
  if (b.left < 0) {
    F[nf] = (int32_t)en.bin, leafy[nf++] = true;
  } else {
    // the slots of least cost (the optimal n-wide collapse of Ylitie, Karras and
    // Laine, HPG 2017): k of 8 to the left child, then each side as its table says
    const int32_t L = b.left, R = L + 1;
    float best = 3e38f;
    int bk = 1;
    for (int k = 1; k < 8; k++) {
      const float c = __fadd_rn(cost[L].c[k - 1], cost[R].c[8 - k - 1]);
      if (c < best) best = c, bk = k;
    }
    int32_t stn[16];
    int sti[16];
    int sp = 0;
    stn[sp] = R, sti[sp++] = 8 - bk;
    stn[sp] = L, sti[sp++] = bk;
    while (sp > 0) {
      const int32_t x = stn[--sp];
      int ix = sti[sp];
      const BNode& c = arena[x];
      while (ix > 1 && (c.left < 0 || wsplit(cost[x], ix) == 0)) ix--;
      if (ix == 1) {
        if (nf >= 8) {
          atomicOr(&counters[kWideError], kWErrSlots);
          return;
        }
        F[nf] = x, leafy[nf++] = c.left < 0 || cost[x].leaf1 != 0;
        continue;
      }
      const int k = (int)wsplit(cost[x], ix);
      if (sp + 2 > 16) {
        atomicOr(&counters[kWideError], kWErrSlots);
        return;
      }
      stn[sp] = c.left + 1, sti[sp++] = ix - k;
      stn[sp] = c.left, sti[sp++] = k;
    }
  }
  uint32_t used = 0;
  for (int k = 0; k < nf; k++) used += usage(F[k], leafy[k]);
  if (used > 8) {
    atomicOr(&counters[kWideError], kWErrSlots);
    return;
  }
  uint32_t n_int = 0, n_tri = 0;
  for (int k = 0; k < nf; k++) {
    const BNode& c = arena[F[k]];
    if (!leafy[k]) n_int++;
    else n_tri += (uint32_t)c.count;
  }
  const uint32_t child_base = n_int ? atomicAdd(&counters[kWideCount], n_int) : 0u;
  const uint32_t prim_base = n_tri ? atomicAdd(&counters[kWidePrims], n_tri) : 0u;
  const uint32_t out_base = n_int ? atomicAdd(&counters[kWideNext], n_int) : 0u;
  if (child_base + n_int > cap || prim_base + n_tri > n_prims || out_base + n_int > cap) {
    atomicOr(&counters[kWideError], kWErrCapacity);
    return;
  }
  WNode8 w;
  memset(&w, 0, sizeof(w));
  const float p[3] = {b.mn[0], b.mn[1], b.mn[2]};
  float sc[3];
  for (int a = 0; a < 3; a++) {
    const int e = quant_exponent(p[a], b.mx[a]);
    w.e[a] = (uint8_t)e;
    sc[a] = pow2(e);
  }
  w.px = p[0], w.py = p[1], w.pz = p[2];
  w.child_base = child_base;
  w.prim_base = prim_base;
  bool ok = true;
  int slot = 0;
  uint32_t rank = 0, off = 0;
  for (int k = 0; k < nf; k++) {
    const BNode& c = arena[F[k]];
    if (!leafy[k]) {
      for (int a = 0; a < 3; a++) ok &= quantise(p[a], sc[a], c.mn[a], c.mx[a], w.qlo[a][slot], w.qhi[a][slot]);
      w.meta[slot] = (uint8_t)(0x80u | rank);
      w.imask |= (uint8_t)(1u << slot);
      out[out_base + rank] = WEntry{child_base + rank, (uint32_t)F[k]};
      rank++, slot++;
      continue;
    }
    for (int32_t j = 0; j < c.count; j += 3) {
      const int cnt = min(3, c.count - j);
      float mn[3] = {1e34f, 1e34f, 1e34f}, mx[3] = {-1e34f, -1e34f, -1e34f};
      for (int t = 0; t < cnt; t++) {
        const uint32_t prim = bprims[c.first + j + t];
        const uint4 ti = idx[prim];
        const float4 a = v[ti.x], bb = v[ti.y], cc = v[ti.z];
        mn[0] = fminf(mn[0], fminf(a.x, fminf(bb.x, cc.x))), mx[0] = fmaxf(mx[0], fmaxf(a.x, fmaxf(bb.x, cc.x)));
        mn[1] = fminf(mn[1], fminf(a.y, fminf(bb.y, cc.y))), mx[1] = fmaxf(mx[1], fmaxf(a.y, fmaxf(bb.y, cc.y)));
        mn[2] = fminf(mn[2], fminf(a.z, fminf(bb.z, cc.z))), mx[2] = fmaxf(mx[2], fmaxf(a.z, fmaxf(bb.z, cc.z)));
        float4* o = wtris + 3 * (size_t)(prim_base + off + t);
        o[0] = make_float4(a.x, a.y, a.z, __uint_as_float(prim));
        o[1] = make_float4(bb.x, bb.y, bb.z, 0.0f);
        o[2] = make_float4(cc.x, cc.y, cc.z, 0.0f);
      }
      for (int a = 0; a < 3; a++) ok &= quantise(p[a], sc[a], mn[a], mx[a], w.qlo[a][slot], w.qhi[a][slot]);
      w.meta[slot] = (uint8_t)(((uint32_t)cnt << 5) | off);
      off += (uint32_t)cnt;
      slot++;
    }
  }
  if (!ok) atomicOr(&counters[kWideError], kWErrQuant);
  wn[en.wide] = w;
}

}  // namespace

size_t gpu_wbvh_scratch_bytes(uint32_t binary_nodes) { return WLayout(binary_nodes).total; }

cudaError_t gpu_wbvh_collapse(const DevScene& sc, const void* arena_v, const uint32_t* bprims, const WideCost* cost,
                              void* scratch2, uint32_t binary_nodes, float4* tris, uint32_t* host_counters,
                              cudaStream_t s, uint32_t* wide_nodes, uint32_t* depth, uint32_t* error) {
  const uint32_t n = sc.tri_count;
  const WLayout W(binary_nodes);
  // both binary builders write this 48-byte node layout (BNode here, FNodeD in bvh_gpu_fast.cu)
  const BNode* arena = static_cast<const BNode*>(arena_v);
  WNode8* wn = at<WNode8>(scratch2, W.nodes);
  WEntry* lists[2] = {at<WEntry>(scratch2, W.list0), at<WEntry>(scratch2, W.list1)};
  uint32_t* counters = at<uint32_t>(scratch2, W.counters);
  const uint32_t init[kWideCounterWords] = {1, 0, 0, 0, 0, 0, 0, 0};
  const WEntry root{0, 0};
  GB_TRY(cudaMemcpyAsync(counters, init, sizeof(init), cudaMemcpyHostToDevice, s));
  GB_TRY(cudaMemcpyAsync(lists[0], &root, sizeof(root), cudaMemcpyHostToDevice, s));
  uint32_t n_in = 1, levels = 0;
  int cur = 0;
  while (n_in > 0) {
    GB_TRY(cudaMemsetAsync(counters + kWideNext, 0, 4, s));
    k_wcollapse<<<blocks(n_in, 128), 128, 0, s>>>(arena, bprims, cost, sc.verts, sc.idx, lists[cur], n_in,
                                                  lists[cur ^ 1], counters, wn, tris, W.cap, n);
    GB_TRY(cudaGetLastError());
    GB_TRY(cudaMemcpyAsync(host_counters, counters, 4 * kWideCounterWords, cudaMemcpyDeviceToHost, s));
    GB_TRY(cudaStreamSynchronize(s));
    levels++;
    if (host_counters[kWideError]) break;
    n_in = host_counters[kWideNext];
    cur ^= 1;
  }
  *wide_nodes = host_counters[kWideCount];
  *depth = levels;
  *error = host_counters[kWideError] | (host_counters[kWidePrims] != n ? kWErrCapacity : 0u);
  return cudaSuccess;
}

cudaError_t gpu_wbvh_copy_nodes(void* scratch2, uint32_t binary_nodes, WNode8* out, uint32_t count, cudaStream_t s) {
  const WLayout W(binary_nodes);
  GB_TRY(cudaMemcpyAsync(out, at<WNode8>(scratch2, W.nodes), sizeof(WNode8) * (size_t)count, cudaMemcpyDeviceToDevice, s));
  return cudaSuccess;
}

}  // namespace ct
