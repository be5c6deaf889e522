// Device build of the traversal-speed quad tree (ct_bvh_build_fast_device).
//
// The rules of the host builder (bvh_fast.cpp: triangle boxes padded relative
// to their coordinates, 16 centroid bins per axis, the exact sweep for ranges
// of at most 16 primitives, split to one primitive per leaf, the cost-optimal
// four-wide collapse, slots in descending box area), evaluated with the same
// IEEE operations in the same order (__fadd_rn/__fmul_rn/__fdiv_rn: nothing
// is contracted). Box unions are min/max, which is exact and, with no negative
// zero in any box, independent of the order; every partition is stable, as on
// the host. So the quad nodes and the primitive order equal
// ct_bvh_build_fast's byte for byte.
//
// Phases:
//   prep      the largest coordinate magnitude M, padded boxes and centroids,
//             the root box
//   levels    nodes of more than kWarpMax primitives, one level per round:
//             per chunk of kChunk primitives the centroid bounds, then the bins
//             (shared memory, flushed into the node's global bins); one warp per
//             node evaluates the 45 bin splits; a chunk-ordered scan gives the
//             stable partition through a scratch copy
//   small     one warp builds each subtree of at most kWarpMax primitives
//             (the exact sweep at <= 16 primitives, bins above)
//   cost      the collapse's cost table C(n, 1..4), bottom-up: the second of
//             two sibling subtrees to finish computes the parent
//   collapse  quad nodes level by level from the root, each choosing its slots
//             from the cost table. The host numbers the children of a quad node
//             when it visits that node, visiting in pre-order: so a node's
//             children are numbered from 1 + the number of children of all
//             nodes before it in pre-order (subtree sizes bottom-up, pre-order
//             ranks top-down, an exclusive scan in rank order)
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <vector>

#include "bvh_build.h"
#include "ct_internal.h"

namespace ct {
namespace {

constexpr int kBins = 16;
constexpr int kCands = 3 * (kBins - 1);  // 45 split candidates per node
constexpr int kBinFields = 7;            // count, min key x/y/z, max key x/y/z
constexpr int kBinWords = 3 * kBins * kBinFields;
constexpr uint32_t kLeafMax = 4;
constexpr int32_t kDepthLimit = 60;
constexpr float kPad = 1e-5f;
constexpr uint32_t kSweepMax = 16;
constexpr uint32_t kWarpMax = 128;  // subtrees up to this size: one warp
constexpr uint32_t kChunk = 2048;
constexpr int kSmallWarps = 4;
constexpr int kSmallStack = 64;  // depth limit 60: at most 61 pending nodes
constexpr int kScanBlock = 1024;

enum : uint32_t { kErrRange = 1, kErrArena = 2, kErrStack = 4, kErrPartition = 8, kErrQuad = 16 };
enum Counter : int {
  kArenaCount = 0,
  kSmallCount = 1,
  kLargeNext = 2,
  kChunkCursor = 3,
  kError = 4,
  kMaxLeaf = 5,
  kMag = 6,
  kQNext = 7,
  kRootKeys = 8,  // 6 words: min x/y/z, max x/y/z
  kCounterWords = 16
};

struct __align__(16) FNodeD {
  float mn[3];
  int32_t first;
  float mx[3];
  int32_t count;
  int32_t left;    // -1 for a leaf, else the left child (right = left + 1)
  int32_t parent;  // -1 at the root
  int32_t depth;
  uint32_t pad;
};
static_assert(sizeof(FNodeD) == 48, "FNodeD");

// C(n, i) for i = 1..4 in c[0..3]; meta bit 0: with one slot the subtree is a
// leaf; bits 8(i-1)..: with i slots, the slots given to the left child (0: as
// with i - 1 slots)
struct __align__(16) FCostD {
  float c[4];
  uint32_t meta;
  uint32_t pad[3];
};
static_assert(sizeof(FCostD) == 32, "FCostD");

struct Chunk {
  int32_t slot;
  uint32_t begin, end;
};
struct FSplit {
  int32_t mode;  // -1 not split yet, 0 partition by bin, 1 halves in the current order, -2 no chunks
  int32_t axis;
  float lo, scale;
  int32_t bsp;  // primitives with bin < bsp go left
  uint32_t lc;
  uint32_t chunk0;
  uint32_t pad;
};

// one quad node (index = breadth-first allocation order)
struct QRec {
  int32_t slot[4];  // binary node of each slot, -1 empty
  int32_t kid[4];   // quad record of an inner slot, else -1
  uint32_t leafmask, nk, size, rank;
  uint32_t number, pad[3];
};
static_assert(sizeof(QRec) == 64, "QRec");

struct Layout {
  size_t lo, hi, cent, prims, tmp, arena, cost, arrive, large0, large1, small, chunks, chunk_left, chunk_loff, split,
      bins, cbk, qlist, qrec, scan, sums, counters, total;
  uint32_t cap, qcap, max_large, max_chunks, max_small, max_sums;
  explicit Layout(uint32_t n, int wide = 0) {
    cap = 2 * n + 2;
    qcap = n + 2;
    max_large = n / (kWarpMax + 1) + 2;
    max_chunks = n / kChunk + max_large + 2;
    max_small = n / 2 + 2;
    max_sums = qcap / kScanBlock + 2;
    size_t o = 0;
    auto take = [&](size_t bytes) {
      const size_t at = o;
      o += (bytes + 255) & ~(size_t)255;
      return at;
    };
    lo = take(sizeof(float4) * (size_t)n);
    hi = take(sizeof(float4) * (size_t)n);
    cent = take(sizeof(float4) * (size_t)n);
    prims = take(4 * (size_t)n);
    tmp = take(4 * (size_t)n);
    arena = take(sizeof(FNodeD) * (size_t)cap);
    cost = take((wide ? sizeof(WideCost) : sizeof(FCostD)) * (size_t)cap);
    arrive = take(4 * (size_t)cap);
    large0 = take(4 * (size_t)max_large);
    large1 = take(4 * (size_t)max_large);
    small = take(4 * (size_t)max_small);
    chunks = take(sizeof(Chunk) * (size_t)max_chunks);
    chunk_left = take(4 * (size_t)max_chunks);
    chunk_loff = take(4 * (size_t)max_chunks);
    split = take(sizeof(FSplit) * (size_t)max_large);
    bins = take(4 * (size_t)kBinWords * max_large);
    cbk = take(4 * 6 * (size_t)max_large);
    qlist = take(4 * (size_t)qcap);
    qrec = take(sizeof(QRec) * (size_t)qcap);
    scan = take(4 * (size_t)qcap);
    sums = take(4 * (size_t)max_sums);
    counters = take(4 * kCounterWords);
    total = o;
  }
};

template <typename T>
T* at(void* base, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(base) + off);
}

// order-preserving float <-> uint32 keys for atomic and warp min/max
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
// std::min / std::max as the host evaluates them
__device__ __forceinline__ float gmin(float a, float b) { return b < a ? b : a; }
__device__ __forceinline__ float gmax(float a, float b) { return a < b ? b : a; }
__device__ __forceinline__ float comp(const float4& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }

// farea (bvh_fast.cpp): surface area with extents scaled by s
__device__ __forceinline__ float farea(const float mn[3], const float mx[3], float s) {
  const float dx = __fmul_rn(__fsub_rn(mx[0], mn[0]), s), dy = __fmul_rn(__fsub_rn(mx[1], mn[1]), s),
              dz = __fmul_rn(__fsub_rn(mx[2], mn[2]), s);
  if (dx < 0.0f) return 0.0f;
  return __fmul_rn(2.0f, __fadd_rn(__fadd_rn(__fmul_rn(dx, dy), __fmul_rn(dy, dz)), __fmul_rn(dz, dx)));
}
// bin_of (bvh_fast.cpp)
__device__ __forceinline__ int bin_of(float c, float lo, float scale) {
  const float f = __fmul_rn(__fsub_rn(c, lo), scale);
  if (!(f >= 1.0f)) return 0;
  if (f >= (float)(kBins - 1)) return kBins - 1;
  return (int)f;
}
// per-axis bin origin and scale from a range's centroid bounds (6 keys)
__device__ __forceinline__ void bin_frame(const uint32_t* k, float lo[3], float scale[3]) {
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const float mn = unkey(k[a]), mx = unkey(k[3 + a]);
    const float ext = __fsub_rn(mx, mn);
    lo[a] = mn;
    scale[a] = ext > 0.0f ? __fdiv_rn((float)kBins, ext) : 0.0f;
  }
}

__device__ __forceinline__ void bin_prim(uint32_t* bins, const float lo[3], const float scale[3], const float4& c,
                                         const float4& l, const float4& h) {
  const uint32_t kl[3] = {fkey(l.x), fkey(l.y), fkey(l.z)};
  const uint32_t kh[3] = {fkey(h.x), fkey(h.y), fkey(h.z)};
#pragma unroll
  for (int a = 0; a < 3; a++) {
    if (!(scale[a] > 0.0f)) continue;
    uint32_t* b = bins + (a * kBins + bin_of(comp(c, a), lo[a], scale[a])) * kBinFields;
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
  int32_t j;  // candidate index a * 15 + i - 1; kCands + 32 when none
  uint32_t lc, rc;
  float lmn[3], lmx[3], rmn[3], rmx[3];
};

__device__ __forceinline__ void eval_cand(const uint32_t* bins, const float scale[3], int j, float s, Cand& c) {
  c.j = kCands + 32;
  c.cost = 0.0f;
  const int a = j / (kBins - 1), i = j % (kBins - 1) + 1;
  if (!(scale[a] > 0.0f)) return;
  c.lc = c.rc = 0;
  for (int k = 0; k < 3; k++) c.lmn[k] = c.rmn[k] = 1e34f, c.lmx[k] = c.rmx[k] = -1e34f;
  for (int b = 0; b < kBins; b++) {
    const uint32_t* e = bins + (a * kBins + b) * kBinFields;
    if (b < i) {
      c.lc += e[0];
      for (int k = 0; k < 3; k++) c.lmn[k] = gmin(c.lmn[k], unkey(e[1 + k])), c.lmx[k] = gmax(c.lmx[k], unkey(e[4 + k]));
    } else {
      c.rc += e[0];
      for (int k = 0; k < 3; k++) c.rmn[k] = gmin(c.rmn[k], unkey(e[1 + k])), c.rmx[k] = gmax(c.rmx[k], unkey(e[4 + k]));
    }
  }
  if (c.lc == 0 || c.rc == 0) return;
  const float cost = __fadd_rn(__fmul_rn(farea(c.lmn, c.lmx, s), __uint2float_rn(c.lc)),
                               __fmul_rn(farea(c.rmn, c.rmx, s), __uint2float_rn(c.rc)));
  if (!(cost < 3e38f)) return;  // the host's running best starts at 3e38
  c.cost = cost;
  c.j = j;
}

__device__ __forceinline__ void bcast_cand(Cand& c, int src) {
  c.cost = __shfl_sync(0xffffffffu, c.cost, src);
  c.j = __shfl_sync(0xffffffffu, c.j, src);
  c.lc = __shfl_sync(0xffffffffu, c.lc, src);
  c.rc = __shfl_sync(0xffffffffu, c.rc, src);
  for (int k = 0; k < 3; k++) {
    c.lmn[k] = __shfl_sync(0xffffffffu, c.lmn[k], src);
    c.lmx[k] = __shfl_sync(0xffffffffu, c.lmx[k], src);
    c.rmn[k] = __shfl_sync(0xffffffffu, c.rmn[k], src);
    c.rmx[k] = __shfl_sync(0xffffffffu, c.rmx[k], src);
  }
}

// First lowest cost over the 45 bin splits in axis-major order (the host's
// strict "cost < best" scan); the whole warp returns the winner, j >= kCands
// when no split qualifies.
__device__ __forceinline__ void choose_bin_split(const uint32_t* bins, const float scale[3], float s, int lane,
                                                 Cand& best) {
  eval_cand(bins, scale, lane, s, best);
  if (lane + 32 < kCands) {
    Cand c2;
    eval_cand(bins, scale, lane + 32, s, c2);
    if (c2.j < kCands && (best.j >= kCands || c2.cost < best.cost)) best = c2;
  }
  float bc = best.cost;
  int bj = best.j;
#pragma unroll
  for (int off = 16; off; off >>= 1) {
    const float oc = __shfl_xor_sync(0xffffffffu, bc, off);
    const int oj = __shfl_xor_sync(0xffffffffu, bj, off);
    if (oj < kCands && (bj >= kCands || oc < bc || (oc == bc && oj < bj))) bc = oc, bj = oj;
  }
  if (bj >= kCands) {
    best.j = kCands + 32;
    return;
  }
  bcast_cand(best, bj < 32 ? bj : bj - 32);
}

// Union of the boxes of prims[b, e) by one warp (order-free).
__device__ __forceinline__ void warp_union(const float4* lo, const float4* hi, const uint32_t* prims, uint32_t b,
                                           uint32_t e, int lane, float mn[3], float mx[3]) {
  uint32_t kmn[3] = {fkey(1e34f), fkey(1e34f), fkey(1e34f)}, kmx[3] = {fkey(-1e34f), fkey(-1e34f), fkey(-1e34f)};
  for (uint32_t k = b + lane; k < e; k += 32) {
    const uint32_t p = prims[k];
    const float4 l = lo[p], h = hi[p];
    kmn[0] = min(kmn[0], fkey(l.x)), kmn[1] = min(kmn[1], fkey(l.y)), kmn[2] = min(kmn[2], fkey(l.z));
    kmx[0] = max(kmx[0], fkey(h.x)), kmx[1] = max(kmx[1], fkey(h.y)), kmx[2] = max(kmx[2], fkey(h.z));
  }
  for (int k = 0; k < 3; k++) {
    mn[k] = unkey(__reduce_min_sync(0xffffffffu, kmn[k]));
    mx[k] = unkey(__reduce_max_sync(0xffffffffu, kmx[k]));
  }
}

__device__ __forceinline__ FNodeD make_node(const float mn[3], const float mx[3], uint32_t first, uint32_t count,
                                            int32_t parent, int32_t depth) {
  FNodeD b;
  for (int k = 0; k < 3; k++) b.mn[k] = mn[k], b.mx[k] = mx[k];
  b.first = (int32_t)first;
  b.count = (int32_t)count;
  b.left = -1;
  b.parent = parent;
  b.depth = depth;
  b.pad = 0;
  return b;
}

// A child is split further when it holds more than one primitive above the depth limit.
__device__ __forceinline__ void classify(int32_t id, uint32_t count, int32_t depth, int32_t* next_large,
                                         uint32_t max_large, int32_t* small, uint32_t max_small, uint32_t* counters) {
  if (count <= 1 || depth >= kDepthLimit) return;
  if (count > kWarpMax) {
    const uint32_t s = atomicAdd(&counters[kLargeNext], 1u);
    if (s < max_large) next_large[s] = id;
    else atomicOr(&counters[kError], kErrArena);
  } else {
    const uint32_t s = atomicAdd(&counters[kSmallCount], 1u);
    if (s < max_small) small[s] = id;
    else atomicOr(&counters[kError], kErrArena);
  }
}

// ---------------------------------------------------------------- prep
__global__ void k_finit(uint32_t* counters) {
  const int w = threadIdx.x;
  if (w < kCounterWords)
    counters[w] = (w >= kRootKeys && w < kRootKeys + 3) ? fkey(1e34f)
                  : (w >= kRootKeys + 3 && w < kRootKeys + 6) ? fkey(-1e34f)
                                                              : 0u;
}

__global__ void __launch_bounds__(256) k_fmag(const float4* __restrict__ v, const uint4* __restrict__ idx, uint32_t n,
                                              uint32_t* counters) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  float m = 0.0f;
  if (i < n) {
    const uint4 t = idx[i];
    const float4 p[3] = {v[t.x], v[t.y], v[t.z]};
    for (int k = 0; k < 3; k++) m = gmax(m, gmax(fabsf(p[k].x), gmax(fabsf(p[k].y), fabsf(p[k].z))));
  }
  // non-negative floats order as their bit patterns
  const uint32_t r = __reduce_max_sync(0xffffffffu, __float_as_uint(m));
  if ((threadIdx.x & 31) == 0) atomicMax(&counters[kMag], r);
}

// rel_pad: kPad for the traversal-speed quad tree, 0 (exact bounds) for the wide tree
__global__ void __launch_bounds__(256) k_fprep(const float4* __restrict__ v, const uint4* __restrict__ idx, uint32_t n,
                                               float4* __restrict__ lo, float4* __restrict__ hi,
                                               float4* __restrict__ cent, uint32_t* __restrict__ prims,
                                               uint32_t* counters, float rel_pad) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  uint32_t kmn[3] = {fkey(1e34f), fkey(1e34f), fkey(1e34f)}, kmx[3] = {fkey(-1e34f), fkey(-1e34f), fkey(-1e34f)};
  if (i < n) {
    const float floor_mag = __fmul_rn(0.25f, __uint_as_float(counters[kMag]));
    const uint4 t = idx[i];
    const float4 a = v[t.x], b = v[t.y], c = v[t.z];
    float mn[3], mx[3], ce[3];
    bool ok = true;
    for (int k = 0; k < 3; k++) {
      const float pa = comp(a, k), pb = comp(b, k), pc = comp(c, k);
      float lo_k = gmin(pa, gmin(pb, pc)), hi_k = gmax(pa, gmax(pb, pc));
      const float pad = __fmul_rn(rel_pad, gmax(floor_mag, gmax(fabsf(lo_k), fabsf(hi_k))));
      lo_k = __fadd_rn(__fsub_rn(lo_k, pad), 0.0f);  // -0 becomes +0
      hi_k = __fadd_rn(__fadd_rn(hi_k, pad), 0.0f);
      mn[k] = lo_k, mx[k] = hi_k;
      ce[k] = __fmul_rn(0.5f, __fadd_rn(lo_k, hi_k));
      ok &= isfinite(lo_k) && isfinite(hi_k) && isfinite(ce[k]);
    }
    if (!ok) atomicOr(&counters[kError], kErrRange);
    lo[i] = make_float4(mn[0], mn[1], mn[2], 0.0f);
    hi[i] = make_float4(mx[0], mx[1], mx[2], 0.0f);
    cent[i] = make_float4(ce[0], ce[1], ce[2], 0.0f);
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

__global__ void k_froot(FNodeD* arena, int32_t* large, int32_t* small, uint32_t n, uint32_t* counters) {
  float mn[3], mx[3];
  for (int k = 0; k < 3; k++) mn[k] = unkey(counters[kRootKeys + k]), mx[k] = unkey(counters[kRootKeys + 3 + k]);
  arena[0] = make_node(mn, mx, 0, n, -1, 0);
  counters[kArenaCount] = 1;
  if (n >= 2) {
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
__global__ void k_fchunks(const FNodeD* __restrict__ arena, const int32_t* __restrict__ large, uint32_t nl,
                          uint32_t max_chunks, Chunk* chunks, FSplit* split, uint32_t* bins, uint32_t* cbk,
                          uint32_t* counters) {
  const uint32_t s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nl) return;
  const FNodeD& nd = arena[large[s]];
  const uint32_t cnt = (uint32_t)nd.count, nc = (cnt + kChunk - 1) / kChunk;
  const uint32_t base = atomicAdd(&counters[kChunkCursor], nc);
  if (base + nc > max_chunks) {
    atomicOr(&counters[kError], kErrArena);
    split[s] = FSplit{-2, 0, 0.0f, 0.0f, 0, 0u, 0u, 0u};
    return;
  }
  for (uint32_t c = 0; c < nc; c++) {
    const uint32_t b = (uint32_t)nd.first + c * kChunk;
    chunks[base + c] = Chunk{(int32_t)s, b, (uint32_t)nd.first + min(cnt, (c + 1) * kChunk)};
  }
  split[s] = FSplit{-1, 0, 0.0f, 0.0f, 0, 0u, base, 0u};
  uint32_t* b = bins + (size_t)s * kBinWords;
  for (int w = 0; w < kBinWords; w++) b[w] = bin_init(w);
  uint32_t* k = cbk + 6 * (size_t)s;
  for (int a = 0; a < 3; a++) k[a] = fkey(1e34f), k[3 + a] = fkey(-1e34f);
}

__device__ __forceinline__ uint32_t nchunks_used(const uint32_t* counters, uint32_t max_chunks) {
  return min(counters[kChunkCursor], max_chunks);
}

__global__ void __launch_bounds__(256) k_fcb(const Chunk* __restrict__ chunks, const uint32_t* counters,
                                             uint32_t max_chunks, const float4* __restrict__ cent,
                                             const uint32_t* __restrict__ prims, uint32_t* cbk) {
  __shared__ uint32_t red[6];
  if (blockIdx.x >= nchunks_used(counters, max_chunks)) return;
  const Chunk ch = chunks[blockIdx.x];
  if (threadIdx.x < 6) red[threadIdx.x] = threadIdx.x < 3 ? fkey(1e34f) : fkey(-1e34f);
  __syncthreads();
  uint32_t kmn[3] = {fkey(1e34f), fkey(1e34f), fkey(1e34f)}, kmx[3] = {fkey(-1e34f), fkey(-1e34f), fkey(-1e34f)};
  for (uint32_t k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) {
    const float4 c = cent[prims[k]];
    kmn[0] = min(kmn[0], fkey(c.x)), kmn[1] = min(kmn[1], fkey(c.y)), kmn[2] = min(kmn[2], fkey(c.z));
    kmx[0] = max(kmx[0], fkey(c.x)), kmx[1] = max(kmx[1], fkey(c.y)), kmx[2] = max(kmx[2], fkey(c.z));
  }
  for (int a = 0; a < 3; a++) {
    kmn[a] = __reduce_min_sync(0xffffffffu, kmn[a]);
    kmx[a] = __reduce_max_sync(0xffffffffu, kmx[a]);
  }
  if ((threadIdx.x & 31) == 0)
    for (int a = 0; a < 3; a++) atomicMin(&red[a], kmn[a]), atomicMax(&red[3 + a], kmx[a]);
  __syncthreads();
  if (threadIdx.x < 6) {
    uint32_t* k = cbk + 6 * (size_t)ch.slot;
    if (threadIdx.x < 3) atomicMin(&k[threadIdx.x], red[threadIdx.x]);
    else atomicMax(&k[threadIdx.x], red[threadIdx.x]);
  }
}

__global__ void __launch_bounds__(256) k_fbin(const Chunk* __restrict__ chunks, const uint32_t* counters,
                                              uint32_t max_chunks, const uint32_t* __restrict__ cbk,
                                              const float4* __restrict__ lo, const float4* __restrict__ hi,
                                              const float4* __restrict__ cent, const uint32_t* __restrict__ prims,
                                              uint32_t* gbins) {
  __shared__ uint32_t bins[kBinWords];
  if (blockIdx.x >= nchunks_used(counters, max_chunks)) return;
  const Chunk ch = chunks[blockIdx.x];
  float blo[3], bscale[3];
  bin_frame(cbk + 6 * (size_t)ch.slot, blo, bscale);
  for (int w = threadIdx.x; w < kBinWords; w += blockDim.x) bins[w] = bin_init(w);
  __syncthreads();
  for (uint32_t k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) {
    const uint32_t p = prims[k];
    bin_prim(bins, blo, bscale, cent[p], lo[p], hi[p]);
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

struct LevelArgs {
  FNodeD* arena;
  const int32_t* large;
  uint32_t nl;
  int32_t* next_large;
  uint32_t max_large;
  int32_t* small;
  uint32_t max_small;
  uint32_t* counters;
  uint32_t cap;
  float ascale;
};

// Allocate the two children of node ni and queue them.
__device__ __forceinline__ void add_children(const LevelArgs& A, int32_t ni, const FNodeD& nd, uint32_t mid,
                                             const float lmn[3], const float lmx[3], const float rmn[3],
                                             const float rmx[3]) {
  const uint32_t cid = atomicAdd(&A.counters[kArenaCount], 2u);
  if (cid + 2 > A.cap) {
    atomicOr(&A.counters[kError], kErrArena);
    return;
  }
  const uint32_t count = (uint32_t)nd.count;
  A.arena[cid] = make_node(lmn, lmx, (uint32_t)nd.first, mid, ni, nd.depth + 1);
  A.arena[cid + 1] = make_node(rmn, rmx, (uint32_t)nd.first + mid, count - mid, ni, nd.depth + 1);
  A.arena[ni].left = (int32_t)cid;
  classify((int32_t)cid, mid, nd.depth + 1, A.next_large, A.max_large, A.small, A.max_small, A.counters);
  classify((int32_t)cid + 1, count - mid, nd.depth + 1, A.next_large, A.max_large, A.small, A.max_small, A.counters);
}

__global__ void __launch_bounds__(256) k_fsplit(LevelArgs A, const uint32_t* __restrict__ gbins,
                                                const uint32_t* __restrict__ cbk, FSplit* split,
                                                const float4* __restrict__ lo, const float4* __restrict__ hi,
                                                const uint32_t* __restrict__ prims) {
  const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= A.nl) return;  // whole warp
  if (split[s].mode == -2) return;  // no chunks (the build fails)
  const int32_t ni = A.large[s];
  const FNodeD nd = A.arena[ni];
  float blo[3], bscale[3];
  bin_frame(cbk + 6 * (size_t)s, blo, bscale);
  Cand c;
  choose_bin_split(gbins + (size_t)s * kBinWords, bscale, A.ascale, lane, c);
  const uint32_t count = (uint32_t)nd.count;
  if (c.j < kCands) {
    if (lane == 0) {
      const int a = c.j / (kBins - 1);
      split[s].mode = 0;
      split[s].axis = a;
      split[s].lo = blo[a];
      split[s].scale = bscale[a];
      split[s].bsp = c.j % (kBins - 1) + 1;
      split[s].lc = c.lc;
      add_children(A, ni, nd, c.lc, c.lmn, c.lmx, c.rmn, c.rmx);
    }
    return;
  }
  // every centroid in one bin on every axis: halve the range as it lies
  const uint32_t mid = count / 2;
  float lmn[3], lmx[3], rmn[3], rmx[3];
  warp_union(lo, hi, prims, (uint32_t)nd.first, (uint32_t)nd.first + mid, lane, lmn, lmx);
  warp_union(lo, hi, prims, (uint32_t)nd.first + mid, (uint32_t)nd.first + count, lane, rmn, rmx);
  if (lane == 0) {
    split[s].mode = 1;
    add_children(A, ni, nd, mid, lmn, lmx, rmn, rmx);
  }
}

__device__ __forceinline__ bool goes_left(const float4* cent, uint32_t p, const FSplit& sp) {
  return bin_of(comp(cent[p], sp.axis), sp.lo, sp.scale) < sp.bsp;
}

__global__ void __launch_bounds__(256) k_fpcount(const Chunk* __restrict__ chunks, const FSplit* __restrict__ split,
                                                 const uint32_t* counters, uint32_t max_chunks,
                                                 const float4* __restrict__ cent, const uint32_t* __restrict__ prims,
                                                 uint32_t* chunk_left) {
  __shared__ uint32_t warp_sum[8];
  if (blockIdx.x >= nchunks_used(counters, max_chunks)) return;
  const Chunk ch = chunks[blockIdx.x];
  const FSplit sp = split[ch.slot];
  if (sp.mode != 0) return;
  uint32_t n = 0;
  for (uint32_t k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) n += goes_left(cent, prims[k], sp);
  n = __reduce_add_sync(0xffffffffu, n);
  if ((threadIdx.x & 31) == 0) warp_sum[threadIdx.x >> 5] = n;
  __syncthreads();
  if (threadIdx.x == 0) {
    uint32_t t = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) t += warp_sum[w];
    chunk_left[blockIdx.x] = t;
  }
}

__global__ void __launch_bounds__(256) k_fpoffsets(const FNodeD* __restrict__ arena, const int32_t* __restrict__ large,
                                                   uint32_t nl, FSplit* split, const uint32_t* __restrict__ chunk_left,
                                                   uint32_t* chunk_loff, uint32_t* counters) {
  const uint32_t s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (s >= nl) return;
  const FSplit sp = split[s];
  if (sp.mode != 0) return;
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
    // the bins and the predicate disagree: keep the range (the build fails)
    atomicOr(&counters[kError], kErrPartition);
    split[s].mode = -1;
  }
}

__global__ void __launch_bounds__(256) k_fpscatter(const FNodeD* __restrict__ arena, const int32_t* __restrict__ large,
                                                   const Chunk* __restrict__ chunks, const FSplit* __restrict__ split,
                                                   const uint32_t* counters, uint32_t max_chunks,
                                                   const uint32_t* __restrict__ chunk_loff,
                                                   const float4* __restrict__ cent, const uint32_t* __restrict__ prims,
                                                   uint32_t* tmp) {
  __shared__ uint32_t wl[8], wr[8];
  if (blockIdx.x >= nchunks_used(counters, max_chunks)) return;
  const Chunk ch = chunks[blockIdx.x];
  const FSplit sp = split[ch.slot];
  if (sp.mode != 0) return;
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
    const bool left = in && goes_left(cent, p, sp);
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

__global__ void __launch_bounds__(256) k_fpcopy(const Chunk* __restrict__ chunks, const FSplit* __restrict__ split,
                                                const uint32_t* counters, uint32_t max_chunks,
                                                const uint32_t* __restrict__ tmp, uint32_t* prims) {
  if (blockIdx.x >= nchunks_used(counters, max_chunks)) return;
  const Chunk ch = chunks[blockIdx.x];
  if (split[ch.slot].mode != 0) return;
  for (uint32_t k = ch.begin + threadIdx.x; k < ch.end; k += blockDim.x) prims[k] = tmp[k];
}

// ---------------------------------------------------------------- small subtrees, one warp each
// Exact SAH sweep of a range of 2..16 primitives (sweep_split): every split of
// the centroid order (ties by primitive id) on each axis; reorders the range to
// the winning axis' order. Returns the left count and the child boxes.
__device__ __forceinline__ uint32_t sweep_split(const float4* lo, const float4* hi, const float4* cent, uint32_t* prims,
                                                uint32_t first, uint32_t count, float s, int lane,
                                                uint32_t (*ord)[kSweepMax], float lmn[3], float lmx[3],
                                                float rmn[3], float rmx[3]) {
  const bool in = (uint32_t)lane < count;
  const uint32_t p = in ? prims[first + lane] : 0u;
  const float4 pc = in ? cent[p] : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  float best = 3e38f;
  int bax = 0;
  uint32_t bmid = count / 2;
  for (int a = 0; a < 3; a++) {
    const float c = comp(pc, a);
    uint32_t r = 0;
    for (uint32_t j = 0; j < count; j++) {
      const float cj = __shfl_sync(0xffffffffu, c, j);
      const uint32_t pj = __shfl_sync(0xffffffffu, p, j);
      r += (cj < c || (cj == c && pj < p)) ? 1u : 0u;
    }
    if (in) ord[a][r] = p;
    __syncwarp();
    // lane r holds the box of the r-th primitive in this axis' order
    float bmn[3] = {1e34f, 1e34f, 1e34f}, bmx[3] = {-1e34f, -1e34f, -1e34f};
    if (in) {
      const uint32_t q = ord[a][lane];
      const float4 l = lo[q], h = hi[q];
      bmn[0] = l.x, bmn[1] = l.y, bmn[2] = l.z, bmx[0] = h.x, bmx[1] = h.y, bmx[2] = h.z;
    }
    float pmn[3], pmx[3], smn[3], smx[3];  // inclusive prefix / suffix unions
    for (int k = 0; k < 3; k++) pmn[k] = smn[k] = bmn[k], pmx[k] = smx[k] = bmx[k];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      for (int k = 0; k < 3; k++) {
        const float umn = __shfl_up_sync(0xffffffffu, pmn[k], off), umx = __shfl_up_sync(0xffffffffu, pmx[k], off);
        const float dmn = __shfl_down_sync(0xffffffffu, smn[k], off), dmx = __shfl_down_sync(0xffffffffu, smx[k], off);
        if (lane >= off) pmn[k] = gmin(pmn[k], umn), pmx[k] = gmax(pmx[k], umx);
        if (lane + off < 32) smn[k] = gmin(smn[k], dmn), smx[k] = gmax(smx[k], dmx);
      }
    }
    float lmn_i[3], lmx_i[3];  // union of the first `lane` primitives
    for (int k = 0; k < 3; k++) {
      lmn_i[k] = __shfl_up_sync(0xffffffffu, pmn[k], 1);
      lmx_i[k] = __shfl_up_sync(0xffffffffu, pmx[k], 1);
    }
    const bool cand = lane >= 1 && (uint32_t)lane < count;
    float cost = 0.0f;
    if (cand)
      cost = __fadd_rn(__fmul_rn(farea(lmn_i, lmx_i, s), __uint2float_rn((uint32_t)lane)),
                       __fmul_rn(farea(smn, smx, s), __uint2float_rn(count - (uint32_t)lane)));
    // first lowest cost below the running best, in split order
    float bc = cost;
    int bi = (cand && cost < best) ? lane : 64;
#pragma unroll
    for (int off = 16; off; off >>= 1) {
      const float oc = __shfl_xor_sync(0xffffffffu, bc, off);
      const int oi = __shfl_xor_sync(0xffffffffu, bi, off);
      if (oi < 64 && (bi >= 64 || oc < bc || (oc == bc && oi < bi))) bc = oc, bi = oi;
    }
    if (bi < 64) best = bc, bax = a, bmid = (uint32_t)bi;
  }
  __syncwarp();
  if (in) prims[first + lane] = ord[bax][lane];
  __syncwarp();
  // cut_boxes over the reordered range
  warp_union(lo, hi, prims, first, first + bmid, lane, lmn, lmx);
  warp_union(lo, hi, prims, first + bmid, first + count, lane, rmn, rmx);
  return bmid;
}

__global__ void __launch_bounds__(kSmallWarps * 32) k_fsmall(LevelArgs A, const int32_t* __restrict__ small_ro,
                                                             const float4* __restrict__ lo,
                                                             const float4* __restrict__ hi,
                                                             const float4* __restrict__ cent, uint32_t* prims) {
  __shared__ uint32_t sbins[kSmallWarps][kBinWords];
  __shared__ int32_t sstack[kSmallWarps][kSmallStack];
  __shared__ uint32_t stmp[kSmallWarps][2 * kWarpMax];
  __shared__ uint32_t sord[kSmallWarps][3][kSweepMax];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t lt = (1u << lane) - 1u;
  uint32_t* bins = sbins[warp];
  int32_t* stack = sstack[warp];
  uint32_t* tmp = stmp[warp];
  const uint32_t nsmall = min(A.counters[kSmallCount], A.max_small);
  for (uint32_t sidx = blockIdx.x * kSmallWarps + warp; sidx < nsmall; sidx += gridDim.x * kSmallWarps) {
    if (lane == 0) stack[0] = small_ro[sidx];
    int sp = 1;
    __syncwarp();
    while (sp > 0) {
      const int32_t ni = stack[--sp];
      __syncwarp();
      const FNodeD nd = A.arena[ni];
      const uint32_t first = (uint32_t)nd.first, count = (uint32_t)nd.count;
      float lmn[3], lmx[3], rmn[3], rmx[3];
      uint32_t mid;
      if (count <= kSweepMax) {
        mid = sweep_split(lo, hi, cent, prims, first, count, A.ascale, lane, sord[warp], lmn, lmx, rmn, rmx);
      } else {
        // centroid bounds, bins, the 45 bin splits
        uint32_t kmn[3] = {fkey(1e34f), fkey(1e34f), fkey(1e34f)}, kmx[3] = {fkey(-1e34f), fkey(-1e34f), fkey(-1e34f)};
        for (uint32_t k = lane; k < count; k += 32) {
          const float4 c = cent[prims[first + k]];
          kmn[0] = min(kmn[0], fkey(c.x)), kmn[1] = min(kmn[1], fkey(c.y)), kmn[2] = min(kmn[2], fkey(c.z));
          kmx[0] = max(kmx[0], fkey(c.x)), kmx[1] = max(kmx[1], fkey(c.y)), kmx[2] = max(kmx[2], fkey(c.z));
        }
        uint32_t keys[6];
        for (int a = 0; a < 3; a++) {
          keys[a] = __reduce_min_sync(0xffffffffu, kmn[a]);
          keys[3 + a] = __reduce_max_sync(0xffffffffu, kmx[a]);
        }
        float blo[3], bscale[3];
        bin_frame(keys, blo, bscale);
        for (int w = lane; w < kBinWords; w += 32) bins[w] = bin_init(w);
        __syncwarp();
        for (uint32_t k = lane; k < count; k += 32) {
          const uint32_t p = prims[first + k];
          bin_prim(bins, blo, bscale, cent[p], lo[p], hi[p]);
        }
        __syncwarp();
        Cand c;
        choose_bin_split(bins, bscale, A.ascale, lane, c);
        if (c.j < kCands) {
          FSplit sp_;
          sp_.axis = c.j / (kBins - 1);
          sp_.lo = blo[sp_.axis];
          sp_.scale = bscale[sp_.axis];
          sp_.bsp = c.j % (kBins - 1) + 1;
          uint32_t nl = 0, nr = 0;
          for (uint32_t k0 = 0; k0 < count; k0 += 32) {
            const uint32_t k = k0 + lane;
            const bool in = k < count;
            const uint32_t p = in ? prims[first + k] : 0u;
            const bool left = in && goes_left(cent, p, sp_);
            const uint32_t bl = __ballot_sync(0xffffffffu, left), br = __ballot_sync(0xffffffffu, in && !left);
            if (left) tmp[nl + __popc(bl & lt)] = p;
            else if (in) tmp[kWarpMax + nr + __popc(br & lt)] = p;
            nl += __popc(bl), nr += __popc(br);
          }
          __syncwarp();
          if (nl != c.lc) {
            if (lane == 0) atomicOr(&A.counters[kError], kErrPartition);
            continue;
          }
          for (uint32_t k = lane; k < count; k += 32) prims[first + k] = k < nl ? tmp[k] : tmp[kWarpMax + k - nl];
          mid = nl;
          for (int k = 0; k < 3; k++) lmn[k] = c.lmn[k], lmx[k] = c.lmx[k], rmn[k] = c.rmn[k], rmx[k] = c.rmx[k];
        } else {
          mid = count / 2;
          warp_union(lo, hi, prims, first, first + mid, lane, lmn, lmx);
          warp_union(lo, hi, prims, first + mid, first + count, lane, rmn, rmx);
        }
      }
      __syncwarp();
      uint32_t cid = 0;
      if (lane == 0) cid = atomicAdd(&A.counters[kArenaCount], 2u);
      cid = __shfl_sync(0xffffffffu, cid, 0);
      if (cid + 2 > A.cap) {
        if (lane == 0) atomicOr(&A.counters[kError], kErrArena);
        continue;
      }
      if (lane == 0) {
        A.arena[cid] = make_node(lmn, lmx, first, mid, ni, nd.depth + 1);
        A.arena[cid + 1] = make_node(rmn, rmx, first + mid, count - mid, ni, nd.depth + 1);
        A.arena[ni].left = (int32_t)cid;
      }
      const bool more = nd.depth + 1 < kDepthLimit;
      const bool push_r = more && count - mid > 1, push_l = more && mid > 1;
      if (sp + (int)push_r + (int)push_l > kSmallStack) {
        if (lane == 0) atomicOr(&A.counters[kError], kErrStack);
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

// ---------------------------------------------------------------- cost table
__device__ __forceinline__ void node_cost(const FNodeD& n, const FCostD* cost, float s, FCostD& e) {
  const float A = farea(n.mn, n.mx, s);
  const uint32_t count = (uint32_t)n.count;
  float leaf = 3e38f;
  if (count <= kLeafMax || n.left < 0) leaf = __fmul_rn(A, __uint2float_rn(2u * ((count + 1u) / 2u)));
  float dist[5] = {3e38f, 3e38f, 3e38f, 3e38f, 3e38f};
  uint32_t dk[5] = {0, 0, 0, 0, 0};
  if (n.left >= 0) {
    float L[4], R[4];
    for (int k = 0; k < 4; k++) L[k] = __ldcg(&cost[n.left].c[k]), R[k] = __ldcg(&cost[n.left + 1].c[k]);
    for (int j = 2; j <= 4; j++)
      for (int k = 1; k < j; k++) {
        const float v = __fadd_rn(L[k - 1], R[j - k - 1]);
        if (v < dist[j]) dist[j] = v, dk[j] = (uint32_t)k;
      }
  }
  const float inner = __fadd_rn(A, dist[4]);
  uint32_t meta = leaf <= inner ? 1u : 0u;
  e.c[0] = inner < leaf ? inner : leaf;
  for (int i = 2; i <= 4; i++) {
    if (dist[i] < e.c[i - 2]) {
      e.c[i - 1] = dist[i];
      meta |= dk[i] << (8 * (i - 1));
    } else {
      e.c[i - 1] = e.c[i - 2];
    }
  }
  e.meta = meta;
}

__device__ __forceinline__ void store_cost(FCostD* dst, const FCostD& e) {
  for (int k = 0; k < 4; k++) __stcg(&dst->c[k], e.c[k]);
  __stcg(&dst->meta, e.meta);
}

__global__ void __launch_bounds__(256) k_fcost(const FNodeD* __restrict__ arena, FCostD* cost, uint32_t* arrive,
                                               const uint32_t* counters, uint32_t cap, float s) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= min(counters[kArenaCount], cap)) return;
  if (arena[i].left >= 0) return;
  FCostD e;
  node_cost(arena[i], cost, s, e);
  store_cost(&cost[i], e);
  int32_t cur = (int32_t)i;
  while (true) {
    const int32_t p = arena[cur].parent;
    if (p < 0) break;
    __threadfence();
    if (atomicAdd(&arrive[p], 1u) == 0) return;  // the sibling's subtree is not finished yet
    __threadfence();
    const FNodeD np = arena[p];
    node_cost(np, cost, s, e);
    store_cost(&cost[p], e);
    cur = p;
  }
}

// ---------------------------------------------------------------- 8-wide cost table
// Relative costs of the wide tree's traversal per unit of surface area: a wide
// node (one 80-byte fetch and eight slot tests) and one triangle of a leaf slot.
constexpr float kWideNodeCost = 1.0f;
constexpr float kWideTriCost = 1.0f;

__device__ __forceinline__ void wide_cost(const FNodeD& n, const WideCost* cost, float s, WideCost& e) {
  const float A = farea(n.mn, n.mx, s);
  const uint32_t count = (uint32_t)n.count;
  const float inf = 3e38f;
  e.split = 0;
  e.pad[0] = e.pad[1] = 0;
  if (n.left < 0) {
    // a binary leaf takes ceil(count / 3) slots of three triangles
    const uint32_t need = (count + 2u) / 3u;
    const float leaf = __fmul_rn(A, __fmul_rn(kWideTriCost, __uint2float_rn(count)));
    for (int i = 1; i <= 8; i++) e.c[i - 1] = (uint32_t)i >= need ? leaf : inf;
    e.leaf1 = 1;
    return;
  }
  float L[8], R[8];
  for (int k = 0; k < 8; k++) L[k] = __ldcg(&cost[n.left].c[k]), R[k] = __ldcg(&cost[n.left + 1].c[k]);
  float dist[9];
  uint32_t dk[9];
  for (int j = 0; j <= 8; j++) dist[j] = inf, dk[j] = 0;
  for (int j = 2; j <= 8; j++)
    for (int k = 1; k < j; k++) {
      const float v = __fadd_rn(L[k - 1], R[j - k - 1]);
      if (v < dist[j]) dist[j] = v, dk[j] = (uint32_t)k;
    }
  const float leaf = count <= 3u ? __fmul_rn(A, __fmul_rn(kWideTriCost, __uint2float_rn(count))) : inf;
  const float inner = __fadd_rn(__fmul_rn(A, kWideNodeCost), dist[8]);
  e.leaf1 = (count <= 3u && leaf <= inner) ? 1u : 0u;
  e.c[0] = e.leaf1 ? leaf : inner;
  for (int i = 2; i <= 8; i++) {
    if (dist[i] < e.c[i - 2]) {
      e.c[i - 1] = dist[i];
      e.split |= dk[i] << (3 * (i - 2));
    } else {
      e.c[i - 1] = e.c[i - 2];
    }
  }
}

__device__ __forceinline__ void store_wide_cost(WideCost* dst, const WideCost& e) {
  for (int k = 0; k < 8; k++) __stcg(&dst->c[k], e.c[k]);
  __stcg(&dst->split, e.split);
  __stcg(&dst->leaf1, e.leaf1);
}

__global__ void __launch_bounds__(256) k_fcost8(const FNodeD* __restrict__ arena, WideCost* cost, uint32_t* arrive,
                                                const uint32_t* counters, uint32_t cap, float s) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= min(counters[kArenaCount], cap)) return;
  if (arena[i].left >= 0) return;
  WideCost e;
  wide_cost(arena[i], cost, s, e);
  store_wide_cost(&cost[i], e);
  int32_t cur = (int32_t)i;
  while (true) {
    const int32_t p = arena[cur].parent;
    if (p < 0) break;
    __threadfence();
    if (atomicAdd(&arrive[p], 1u) == 0) return;  // the sibling's subtree is not finished yet
    __threadfence();
    const FNodeD np = arena[p];
    wide_cost(np, cost, s, e);
    store_wide_cost(&cost[p], e);
    cur = p;
  }
}

// ---------------------------------------------------------------- collapse
__device__ __forceinline__ uint32_t split_of(uint32_t meta, int i) { return (meta >> (8 * (i - 1))) & 0xffu; }

__global__ void __launch_bounds__(256) k_fqlevel(const FNodeD* __restrict__ arena, const FCostD* __restrict__ cost,
                                                 uint32_t* qlist, QRec* qrec, uint32_t b, uint32_t e,
                                                 uint32_t next_base, uint32_t qcap, uint32_t* counters, float s) {
  const uint32_t q = b + blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= e) return;
  const int32_t bn = (int32_t)qlist[q];
  const FNodeD n = arena[bn];
  const int32_t L = n.left, R = L + 1;
  if (L < 0) {  // a quad node is an inner binary node (cannot happen for a consistent table)
    atomicOr(&counters[kError], kErrQuad);
    return;
  }
  float best = 3e38f;
  int bk = 1;
  for (int k = 1; k < 4; k++) {
    const float v = __fadd_rn(cost[L].c[k - 1], cost[R].c[4 - k - 1]);
    if (v < best) best = v, bk = k;
  }
  // emit (bvh_fast.cpp): the slots of a subtree given i of them, depth first
  int32_t sl[4];
  bool lf[4];
  int ns = 0;
  int32_t stn[8];
  int sti[8];
  int sp = 0;
  stn[sp] = R, sti[sp++] = 4 - bk;
  stn[sp] = L, sti[sp++] = bk;
  while (sp > 0) {
    const int32_t x = stn[--sp];
    int i = sti[sp];
    const uint32_t meta = cost[x].meta;
    while (i > 1 && split_of(meta, i) == 0) i--;
    if (i == 1) {
      if (ns < 4) sl[ns] = x, lf[ns] = (meta & 1u) != 0, ns++;
      continue;
    }
    const int k = (int)split_of(meta, i);
    const int32_t xl = arena[x].left;
    if (sp + 2 > 8 || xl < 0) {  // cannot happen for a consistent table
      atomicOr(&counters[kError], kErrQuad);
      return;
    }
    stn[sp] = xl + 1, sti[sp++] = i - k;
    stn[sp] = xl, sti[sp++] = k;
  }
  // largest box first, stable
  float ar[4];
  for (int j = 0; j < ns; j++) ar[j] = farea(arena[sl[j]].mn, arena[sl[j]].mx, s);
  for (int j = 1; j < ns; j++) {
    const float a = ar[j];
    const int32_t x = sl[j];
    const bool f = lf[j];
    int k = j;
    while (k > 0 && ar[k - 1] < a) ar[k] = ar[k - 1], sl[k] = sl[k - 1], lf[k] = lf[k - 1], k--;
    ar[k] = a, sl[k] = x, lf[k] = f;
  }
  QRec r;
  r.leafmask = 0;
  r.nk = 0;
  r.size = 0;
  r.rank = 0;
  r.number = 0;
  r.pad[0] = r.pad[1] = r.pad[2] = 0;
  for (int j = 0; j < 4; j++) {
    r.slot[j] = j < ns ? sl[j] : -1;
    r.kid[j] = -1;
    if (j >= ns) continue;
    if (lf[j]) {
      r.leafmask |= 1u << j;
      atomicMax(&counters[kMaxLeaf], (uint32_t)arena[sl[j]].count);
    } else {
      const uint32_t at_ = next_base + atomicAdd(&counters[kQNext], 1u);
      if (at_ >= qcap) {
        atomicOr(&counters[kError], kErrQuad);
        continue;
      }
      qlist[at_] = (uint32_t)sl[j];
      r.kid[j] = (int32_t)at_;
      r.nk++;
    }
  }
  qrec[q] = r;
}

__global__ void k_fqsize(QRec* qrec, uint32_t b, uint32_t e) {
  const uint32_t q = b + blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= e) return;
  uint32_t sz = 1;
  for (int j = 0; j < 4; j++)
    if (qrec[q].kid[j] >= 0) sz += qrec[qrec[q].kid[j]].size;
  qrec[q].size = sz;
}

__global__ void k_fqrank(QRec* qrec, uint32_t b, uint32_t e) {
  const uint32_t q = b + blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= e) return;
  uint32_t r = qrec[q].rank + 1;
  for (int j = 0; j < 4; j++) {
    const int32_t k = qrec[q].kid[j];
    if (k < 0) continue;
    qrec[k].rank = r;
    r += qrec[k].size;
  }
}

__global__ void k_fqscatter(const QRec* __restrict__ qrec, uint32_t nq, uint32_t* scan) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint32_t r = qrec[q].rank;
  if (r < nq) scan[r] = qrec[q].nk;
}

// exclusive scan of scan[0, n): per block, then the block totals, then the offsets
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(uint32_t* scan, uint32_t n, uint32_t* sums) {
  __shared__ uint32_t ws[kScanBlock / 32];
  const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const uint32_t v = i < n ? scan[i] : 0u;
  uint32_t x = v;
#pragma unroll
  for (int off = 1; off < 32; off <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
    if (lane >= off) x += y;
  }
  if (lane == 31) ws[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t w = ws[lane];
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, off);
      if (lane >= off) w += y;
    }
    ws[lane] = w;
  }
  __syncthreads();
  const uint32_t before = warp ? ws[warp - 1] : 0u;
  if (i < n) scan[i] = before + x - v;
  if (threadIdx.x == kScanBlock - 1) sums[blockIdx.x] = before + x;
}

__global__ void __launch_bounds__(32) k_scan_sums(uint32_t* sums, uint32_t nb) {
  const int lane = threadIdx.x;
  uint32_t run = 0;
  for (uint32_t b0 = 0; b0 < nb; b0 += 32) {
    const uint32_t b = b0 + lane;
    const uint32_t v = b < nb ? sums[b] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, off);
      if (lane >= off) x += y;
    }
    if (b < nb) sums[b] = run + x - v;
    run += __shfl_sync(0xffffffffu, x, 31);
  }
}

__global__ void __launch_bounds__(kScanBlock) k_scan_add(uint32_t* scan, uint32_t n, const uint32_t* sums) {
  const uint32_t i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) scan[i] += sums[blockIdx.x];
}

__global__ void k_fqnum(QRec* qrec, uint32_t nq, const uint32_t* __restrict__ scan) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const uint32_t r = qrec[q].rank;
  uint32_t next = 1 + (r < nq ? scan[r] : 0u);
  for (int j = 0; j < 4; j++) {
    const int32_t k = qrec[q].kid[j];
    if (k >= 0) qrec[k].number = next++;
  }
}

__device__ __forceinline__ void put_slot(QuadNode& d, int j, const float mn[3], const float mx[3], int32_t child,
                                         int32_t count) {
  d.bminx[j] = mn[0], d.bminy[j] = mn[1], d.bminz[j] = mn[2];
  d.bmaxx[j] = mx[0], d.bmaxy[j] = mx[1], d.bmaxz[j] = mx[2];
  d.childs[j] = child;
  d.counts[j] = count;
}

__global__ void k_fqwrite(const FNodeD* __restrict__ arena, const QRec* __restrict__ qrec, uint32_t nq,
                          QuadNode* quad, uint32_t* counters) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= nq) return;
  const QRec r = qrec[q];
  const float big[3] = {1e34f, 1e34f, 1e34f}, nbig[3] = {-1e34f, -1e34f, -1e34f};
  QuadNode d;
  for (int j = 0; j < 4; j++) {
    if (r.slot[j] < 0) {
      put_slot(d, j, big, nbig, -1, 0);
      continue;
    }
    const FNodeD& c = arena[r.slot[j]];
    if (r.leafmask & (1u << j)) put_slot(d, j, c.mn, c.mx, c.first, c.count);
    else put_slot(d, j, c.mn, c.mx, r.kid[j] >= 0 ? (int32_t)qrec[r.kid[j]].number : -1, -1);
  }
  if (r.number < nq) quad[r.number] = d;
  else atomicOr(&counters[kError], kErrQuad);
}

// a single primitive: one leaf slot under the root
__global__ void k_fqsingle(const FNodeD* __restrict__ arena, QuadNode* quad, uint32_t* counters) {
  const float big[3] = {1e34f, 1e34f, 1e34f}, nbig[3] = {-1e34f, -1e34f, -1e34f};
  QuadNode d;
  put_slot(d, 0, arena[0].mn, arena[0].mx, 0, arena[0].count);
  for (int j = 1; j < 4; j++) put_slot(d, j, big, nbig, -1, 0);
  quad[0] = d;
  counters[kMaxLeaf] = (uint32_t)arena[0].count;
}

unsigned blocks(uint64_t n, unsigned per) { return (unsigned)((n + per - 1) / per); }

#define FB_TRY(call)                  \
  do {                                \
    cudaError_t e_ = (call);          \
    if (e_ != cudaSuccess) return e_; \
  } while (0)

cudaError_t read_counters(uint32_t* host, const uint32_t* dev, cudaStream_t s) {
  FB_TRY(cudaMemcpyAsync(host, dev, 4 * kCounterWords, cudaMemcpyDeviceToHost, s));
  return cudaStreamSynchronize(s);
}

}  // namespace

size_t gpu_fbvh_scratch_bytes(uint32_t n, int wide) { return Layout(n, wide).total; }

void gpu_fbvh_binary(void* scratch, uint32_t n, int wide, const void** arena, const uint32_t** prims,
                     const WideCost** cost) {
  const Layout Lo(n, wide);
  *arena = at<FNodeD>(scratch, Lo.arena);
  *prims = at<uint32_t>(scratch, Lo.prims);
  *cost = wide ? at<WideCost>(scratch, Lo.cost) : nullptr;
}

cudaError_t gpu_fbvh_build(const DevScene& sc, void* scratch, uint32_t* hc, cudaStream_t s, GpuBvhResult& r, int wide) {
  const uint32_t n = sc.tri_count;
  const Layout Lo(n, wide);
  uint32_t* counters = at<uint32_t>(scratch, Lo.counters);
  float4* lo = at<float4>(scratch, Lo.lo);
  float4* hi = at<float4>(scratch, Lo.hi);
  float4* cent = at<float4>(scratch, Lo.cent);
  uint32_t* prims = at<uint32_t>(scratch, Lo.prims);
  uint32_t* tmp = at<uint32_t>(scratch, Lo.tmp);
  FNodeD* arena = at<FNodeD>(scratch, Lo.arena);
  FCostD* cost = at<FCostD>(scratch, Lo.cost);
  uint32_t* arrive = at<uint32_t>(scratch, Lo.arrive);
  int32_t* large[2] = {at<int32_t>(scratch, Lo.large0), at<int32_t>(scratch, Lo.large1)};
  int32_t* small = at<int32_t>(scratch, Lo.small);
  Chunk* chunks = at<Chunk>(scratch, Lo.chunks);
  uint32_t* chunk_left = at<uint32_t>(scratch, Lo.chunk_left);
  uint32_t* chunk_loff = at<uint32_t>(scratch, Lo.chunk_loff);
  FSplit* split = at<FSplit>(scratch, Lo.split);
  uint32_t* bins = at<uint32_t>(scratch, Lo.bins);
  uint32_t* cbk = at<uint32_t>(scratch, Lo.cbk);
  uint32_t* qlist = at<uint32_t>(scratch, Lo.qlist);
  QRec* qrec = at<QRec>(scratch, Lo.qrec);
  uint32_t* scan = at<uint32_t>(scratch, Lo.scan);
  uint32_t* sums = at<uint32_t>(scratch, Lo.sums);
  r = GpuBvhResult{};

  k_finit<<<1, 32, 0, s>>>(counters);
  k_fmag<<<blocks(n, 256), 256, 0, s>>>(sc.verts, sc.idx, n, counters);
  k_fprep<<<blocks(n, 256), 256, 0, s>>>(sc.verts, sc.idx, n, lo, hi, cent, prims, counters, wide ? 0.0f : kPad);
  k_froot<<<1, 1, 0, s>>>(arena, large[0], small, n, counters);
  FB_TRY(cudaGetLastError());
  FB_TRY(read_counters(hc, counters, s));
  if (hc[kError]) {
    r.error = hc[kError];
    return cudaSuccess;
  }
  float rmn[3], rmx[3];
  for (int k = 0; k < 3; k++) {
    uint32_t a = hc[kRootKeys + k], b = hc[kRootKeys + 3 + k];
    a = (a & 0x80000000u) ? (a & 0x7fffffffu) : ~a;
    b = (b & 0x80000000u) ? (b & 0x7fffffffu) : ~b;
    std::memcpy(&rmn[k], &a, 4);
    std::memcpy(&rmx[k], &b, 4);
  }
  const float ascale = fast_area_scale(rmn, rmx);
  LevelArgs A{arena, nullptr, 0, nullptr, Lo.max_large, small, Lo.max_small, counters, Lo.cap, ascale};
  uint32_t nl = hc[kLargeNext];
  int cur = 0;
  while (nl > 0) {
    if (nl > Lo.max_large) {
      r.error |= kErrArena;
      return cudaSuccess;
    }
    FB_TRY(cudaMemsetAsync(counters + kLargeNext, 0, 8, s));  // kLargeNext, kChunkCursor
    A.large = large[cur];
    A.nl = nl;
    A.next_large = large[cur ^ 1];
    k_fchunks<<<blocks(nl, 128), 128, 0, s>>>(arena, large[cur], nl, Lo.max_chunks, chunks, split, bins, cbk,
                                              counters);
    const unsigned nchunk = (unsigned)std::min<uint64_t>((uint64_t)n / kChunk + nl + 1, Lo.max_chunks);
    k_fcb<<<nchunk, 256, 0, s>>>(chunks, counters, Lo.max_chunks, cent, prims, cbk);
    k_fbin<<<nchunk, 256, 0, s>>>(chunks, counters, Lo.max_chunks, cbk, lo, hi, cent, prims, bins);
    k_fsplit<<<blocks((uint64_t)nl * 32, 256), 256, 0, s>>>(A, bins, cbk, split, lo, hi, prims);
    k_fpcount<<<nchunk, 256, 0, s>>>(chunks, split, counters, Lo.max_chunks, cent, prims, chunk_left);
    k_fpoffsets<<<blocks((uint64_t)nl * 32, 256), 256, 0, s>>>(arena, large[cur], nl, split, chunk_left, chunk_loff,
                                                              counters);
    k_fpscatter<<<nchunk, 256, 0, s>>>(arena, large[cur], chunks, split, counters, Lo.max_chunks, chunk_loff, cent,
                                       prims, tmp);
    k_fpcopy<<<nchunk, 256, 0, s>>>(chunks, split, counters, Lo.max_chunks, tmp, prims);
    FB_TRY(cudaGetLastError());
    FB_TRY(read_counters(hc, counters, s));
    nl = hc[kLargeNext];
    cur ^= 1;
    r.levels++;
    if (hc[kError]) {
      r.error = hc[kError];
      return cudaSuccess;
    }
  }
  const uint32_t nsmall = std::min(hc[kSmallCount], Lo.max_small);
  if (nsmall > 0) {
    const unsigned g = (unsigned)std::min<uint64_t>(blocks(nsmall, kSmallWarps), (uint64_t)sm_count() * 16);
    k_fsmall<<<g, kSmallWarps * 32, 0, s>>>(A, small, lo, hi, cent, prims);
    FB_TRY(cudaGetLastError());
  }
  FB_TRY(read_counters(hc, counters, s));
  if (hc[kError]) {
    r.error = hc[kError];
    return cudaSuccess;
  }
  const uint32_t nb = hc[kArenaCount];
  r.binary_nodes = nb;
  r.small_roots = nsmall;
  if (n == 1) {
    r.quad_nodes = 1;
    r.depth = 1;
    r.max_leaf = 1;
    return cudaSuccess;
  }
  FB_TRY(cudaMemsetAsync(arrive, 0, 4 * (size_t)nb, s));
  if (wide) {
    k_fcost8<<<blocks(nb, 256), 256, 0, s>>>(arena, at<WideCost>(scratch, Lo.cost), arrive, counters, Lo.cap, ascale);
    FB_TRY(cudaGetLastError());
    FB_TRY(read_counters(hc, counters, s));
    r.error = hc[kError];
    return cudaSuccess;
  }
  k_fcost<<<blocks(nb, 256), 256, 0, s>>>(arena, cost, arrive, counters, Lo.cap, ascale);
  // quad levels from the root (binary node 0)
  FB_TRY(cudaMemsetAsync(qlist, 0, 4, s));
  std::vector<uint32_t> off{0u, 1u};
  while (off.back() > off[off.size() - 2]) {
    const uint32_t b = off[off.size() - 2], e = off.back();
    FB_TRY(cudaMemsetAsync(counters + kQNext, 0, 4, s));
    k_fqlevel<<<blocks(e - b, 256), 256, 0, s>>>(arena, cost, qlist, qrec, b, e, e, Lo.qcap, counters, ascale);
    FB_TRY(cudaGetLastError());
    FB_TRY(read_counters(hc, counters, s));
    if (hc[kError]) {
      r.error = hc[kError];
      return cudaSuccess;
    }
    off.push_back(e + hc[kQNext]);
  }
  const uint32_t nq = off.back();
  const size_t nlev = off.size() - 2;  // levels with nodes
  for (size_t l = nlev; l-- > 0;)
    k_fqsize<<<blocks(off[l + 1] - off[l], 256), 256, 0, s>>>(qrec, off[l], off[l + 1]);
  for (size_t l = 0; l < nlev; l++)
    k_fqrank<<<blocks(off[l + 1] - off[l], 256), 256, 0, s>>>(qrec, off[l], off[l + 1]);
  k_fqscatter<<<blocks(nq, 256), 256, 0, s>>>(qrec, nq, scan);
  const uint32_t nsb = blocks(nq, kScanBlock);
  k_scan_blocks<<<nsb, kScanBlock, 0, s>>>(scan, nq, sums);
  k_scan_sums<<<1, 32, 0, s>>>(sums, nsb);
  k_scan_add<<<nsb, kScanBlock, 0, s>>>(scan, nq, sums);
  k_fqnum<<<blocks(nq, 256), 256, 0, s>>>(qrec, nq, scan);
  FB_TRY(cudaGetLastError());
  FB_TRY(read_counters(hc, counters, s));
  r.error = hc[kError];
  r.quad_nodes = nq;
  r.depth = (uint32_t)nlev;
  r.max_leaf = hc[kMaxLeaf];
  return cudaSuccess;
}

cudaError_t gpu_fbvh_emit(const DevScene& sc, void* scratch, const GpuBvhResult& r, uint32_t leaf_shift,
                          void* quad_out, QNodeDev* nodes, float4* tris, uint32_t* prims_out, cudaStream_t s) {
  const uint32_t n = sc.tri_count;
  const Layout Lo(n);
  uint32_t* counters = at<uint32_t>(scratch, Lo.counters);
  const FNodeD* arena = at<FNodeD>(scratch, Lo.arena);
  const QRec* qrec = at<QRec>(scratch, Lo.qrec);
  const uint32_t* prims = at<uint32_t>(scratch, Lo.prims);
  QuadNode* quad = static_cast<QuadNode*>(quad_out);
  if (n == 1) k_fqsingle<<<1, 1, 0, s>>>(arena, quad, counters);
  else k_fqwrite<<<blocks(r.quad_nodes, 256), 256, 0, s>>>(arena, qrec, r.quad_nodes, quad, counters);
  FB_TRY(cudaGetLastError());
  FB_TRY(launch_quad_to_dev(quad, r.quad_nodes, leaf_shift, nodes, s));
  FB_TRY(launch_leaf_tris(sc, prims, n, tris, s));
  return cudaMemcpyAsync(prims_out, prims, 4 * (size_t)n, cudaMemcpyDeviceToDevice, s);
}

uint32_t gpu_fbvh_error(void* scratch, uint32_t n, uint32_t* hc, cudaStream_t s) {
  const Layout Lo(n);  // quad mode (the wide mode reports its errors from gpu_fbvh_build)
  if (read_counters(hc, at<uint32_t>(scratch, Lo.counters), s) != cudaSuccess) return 0xffffffffu;
  return hc[kError];
}

}  // namespace ct
