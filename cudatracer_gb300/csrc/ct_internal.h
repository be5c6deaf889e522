// Internal declarations shared by the host runtime (.cpp) and the kernels (.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <cstddef>

namespace ct {

// ---------------------------------------------------------------------------
// Device data layout (all arrays in HBM, 16-byte vector loads)
// ---------------------------------------------------------------------------

// Quad-BVH node: 128 bytes, 128-byte aligned, read as eight LDG.128. Bounds are
// the reference MBVHNode planes bit for bit (src/BVH/MBVHNode.cuh:35-60) so the
// slab test and its child order reproduce the reference; children are packed
// 32-bit references:
//   >= 0          inner node index
//   kEmptyChild   unused slot (the reference keeps count 0 there)
//   bit 31 set    leaf: first = ref & first_mask, count = (ref >> leaf_shift) & count_mask
struct __align__(128) QNodeDev {
  float4 bminx, bmaxx, bminy, bmaxy, bminz, bmaxz;
  int4 child;
  int4 meta;  // reserved, zero
};
static_assert(sizeof(QNodeDev) == 128, "QNodeDev is 128 bytes");
constexpr int32_t kEmptyChild = -1;

// Triangle in leaf order, 48 bytes: {p0.xyz, prim id}, {p1-p0, 0}, {p2-p0, 0}.
// The edges are the exact float differences the reference forms per test
// (src/Core/Triangle.cuh:15-16), precomputed once.

// 8-wide node with 8-bit child bounds, 80 bytes (five LDG.128). A child box
// is lo = fma(2^(e - 127), qlo, p), hi = fma(2^(e - 127), qhi, p) per axis,
// rounded outward when built, so it contains the child's exact bounds.
//   meta[i] == 0          empty slot
//   meta[i] & 0x80        inner child: node child_base + (meta & 7)
//   otherwise             leaf: (meta >> 5) triangles (1..3) from prim_base + (meta & 31)
struct __align__(16) WNode8 {
  float px, py, pz;
  uint8_t e[3];
  uint8_t imask;
  uint32_t child_base;
  uint32_t prim_base;
  uint8_t meta[8];
  uint8_t qlo[3][8];
  uint8_t qhi[3][8];
};
static_assert(sizeof(WNode8) == 80, "WNode8 is 80 bytes");

// Triangles of the wide tree in leaf order, 48 bytes: {p0, prim id}, {p1, 0}, {p2, 0}
// (raw vertices: the watertight test shears them per ray).
struct DevWBVH {
  const WNode8* nodes;
  const float4* tris;
  uint32_t node_count;
  uint32_t prim_count;
  uint32_t depth;          // levels of wide nodes
  int32_t stack_entries;   // 7 per level + 1
};

struct DevBVH {
  const QNodeDev* nodes;
  const float4* tris;  // 3 float4 per leaf slot
  uint32_t leaf_shift;
  uint32_t first_mask;
  uint32_t count_mask;
  uint32_t prim_count;
  uint32_t node_count;
  int32_t stack_entries;
};

// 64-byte material (reference Material fields, padded to 4 x float4).
struct __align__(16) DevMaterial {
  float4 albedo_ior;      // albedo/emission xyz, refractIdx
  int4 tex;               // diffuse, normal, mask, displace texture ids
  float4 type_rough;      // type (as int bits), roughness, 0, 0
  float4 absorption;      // xyz, 0
};

struct DevScene {
  const float4* verts;     // per vertex, w = 0
  const float4* normals;   // per vertex
  const float2* uvs;       // per vertex
  const uint4* idx;        // per triangle, w = material index
  const float4* cnormals;  // per triangle centre normal
  // per triangle shading record, 8 float4 (one 128-byte line): {p0, material},
  // {p1, 0}, {p2, 0}, {n0, uv0.x}, {n1, uv0.y}, {n2, uv1.x}, {centre normal,
  // uv1.y}, {uv2, 0, 0}: the same values as the per-vertex arrays above, so a
  // hit is shaded from one line instead of an index fetch and ten gathers
  const float4* shade_rec;
  const DevMaterial* mats;
  const uint32_t* lights;
  uint32_t light_count;
  uint32_t tri_count;
  const float4* texels;
  const uint2* tex_dims;
  const uint32_t* tex_offsets;
  int32_t sky_tex;
  uint32_t tex_count;
};

// Per-job wavefront state (SoA queues, 16-byte records).
struct DevQueues {
  float4* org[2];    // origin xyz, w = pixel index (int bits)
  float4* dir[2];    // direction xyz, w = last bounce type (int bits: 0 specular, 1 diffuse)
  float4* thr[2];    // throughput xyz, w = last BSDF pdf
  int2* hit;         // closest hit: x = primitive id, y = t (float bits)
  float4* sorg;      // shadow origin xyz, w = pixel
  float4* sdir;      // shadow direction xyz, w = max distance
  float4* scol;      // shadow contribution xyz, w unused
  float4* accum;     // FP32 RGBA accumulation, one per pixel
  // device counters
  int32_t* counts;   // [0],[1] ray queue sizes, [2] shadow queue size, [4] extend fetch cursor
  unsigned long long* stats;  // [0] extension rays, [1] shadow rays, [2] samples, [3] frames
  uint32_t* error;   // error bits (1 = stack overflow)
  int32_t* perm;     // order in which extend takes the queue's rays (nullptr = queue order); a
                     // stage that sorted the queue passes perm = perm_buf. It never changes a
                     // result, only which rays share a warp
  int32_t* perm_buf; // capacity entries, written by launch_ray_sort
  int32_t capacity;
  // Exact-math frames rendered in a slot (overlapped with other frames): instead
  // of adding to accum, each pixel's contribution of this launch is stored as
  // entry log_entry of log ([entry][pixel], capacity pixels per entry: shade of
  // pass p writes entry 2p, connect entry 2p + 1), w = log_tag (uint bits); the
  // fold replays the entries in order into the job's buffer, so every pixel
  // sees the same additions in the same order as a frame accumulated in place.
  // nullptr: add to accum.
  float4* log;
  uint32_t log_entry;
  uint32_t log_tag;
  // queue selection without dynamic indexing into the (by-value) parameter struct
  __host__ __device__ float4* org_q(int i) const { return i ? org[1] : org[0]; }
  __host__ __device__ float4* dir_q(int i) const { return i ? dir[1] : dir[0]; }
  __host__ __device__ float4* thr_q(int i) const { return i ? thr[1] : thr[0]; }
};

struct FrameConst {
  float3 cam_pos, cam_w, hor, ver;
  int32_t width, height;
  uint32_t frame;
  float normal_eps, dist_eps, tri_eps;
  int32_t shadow, indirect, sky;
  int32_t shading_mode;
  int32_t tex_filter;  // CT_TEX_NEAREST / CT_TEX_BILINEAR
};

enum : uint32_t { kErrStackOverflow = 1u };

// Math modes (CT_MATH_FAST 0, CT_MATH_EXACT 1, CT_MATH_EXACT_SHADE 2): which
// build each stage runs. Only CT_MATH_EXACT traverses with the reference's
// arithmetic and child order (and runs frames strictly in sequence); ray
// generation and shading are the bit-reproducible build in both exact modes.
inline bool math_fast_traversal(int mode) { return mode != 1; }
inline int math_exact_shading(int mode) { return mode != 0 ? 1 : 0; }
inline bool math_mode_valid(int mode) { return mode >= 0 && mode <= 2; }

// ---------------------------------------------------------------------------
// Batches: many render jobs share one queue set and one launch per stage.
// A ray's pixel index (origin.w) is global to the batch; the job owning it is
// found by binary search over the jobs' first pixels.
// ---------------------------------------------------------------------------
struct BatchJob {
  DevScene sc;
  DevBVH bvh;
  DevWBVH wbvh;         // the job's tree when the batch traces wide BVHs
  FrameConst f;         // f.frame advances by 2 per sample, as launchKernels does
  float4* accum;        // the job's own width*height accumulation
  int32_t pix_base;     // first pixel of the job in the batch
  int32_t max_depth;
  int32_t spp_left;     // samples still to take; the job traces while > 0
  int32_t exact;        // unused by the kernels (the batch picks one math mode)
};
struct DevBatch {
  BatchJob* jobs;
  const int32_t* bases;  // n_jobs + 1 ascending first pixels; bases[n_jobs] = total
  int32_t n_jobs;
  int32_t total_pix;
  int32_t max_stack;     // largest traversal stack among the jobs' BVHs
  int32_t wide;          // 1: every job traces its wide BVH (fast-math frames on the quantised tree)
  int32_t frame_step;    // seed frames a job advances per iteration of this table (2, or 4 when
                         // two tables take alternate samples)
};
#ifdef __CUDACC__
__device__ __forceinline__ int batch_job_of(const int32_t* __restrict__ bases, int n, int pix) {
  int lo = 0, hi = n - 1;  // largest j with bases[j] <= pix
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(bases + mid) <= pix) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}
#endif

// ---------------------------------------------------------------------------
// Kernel launchers (defined in the .cu files)
// ---------------------------------------------------------------------------
int sm_count();

// `cursor`: a device int the launch resets; the kernel's warps take ray indices from it
cudaError_t launch_trace_closest(const DevBVH& b, const float4* org, const float4* dir, int32_t* hit, float* t,
                                 uint32_t n, float eps, uint32_t* err, int* cursor, cudaStream_t s);
cudaError_t launch_trace_any(const DevBVH& b, const float4* org, const float4* dir, uint8_t* occ, uint32_t n,
                             float eps, uint32_t* err, int* cursor, cudaStream_t s);

// wavefront stages; the active count lives at counts[queue] on the device and
// extend's fetch cursor at counts[4] (zeroed by raygen and by every shade).
// `fast` selects hardware min/max in the slab test (fast-math frames only).
cudaError_t launch_extend(const DevBVH& b, const DevQueues& q, int queue, float eps, bool fast, cudaStream_t s);
cudaError_t launch_connect(const DevBVH& b, const DevQueues& q, float eps, bool fast, cudaStream_t s);
cudaError_t launch_raygen(const DevQueues& q, const FrameConst& f, int exact, cudaStream_t s);
cudaError_t launch_shade(const DevScene& sc, const DevQueues& q, const FrameConst& f, int queue, int path_length,
                         int exact, cudaStream_t s);
cudaError_t launch_present(const float4* accum, float4* out, int n, float samples, cudaStream_t s);
// Device SAH build (bvh_gpu.cu). gpu_bvh_build runs the binary build and the
// collapse bookkeeping in `scratch` (gpu_bvh_scratch_bytes) and returns the
// sizes; gpu_bvh_emit then writes the reference-layout quad nodes (QuadNode,
// pre-order), the traversal nodes, the leaf-ordered triangles and the
// primitive order into buffers of those sizes. host_counters: 16 words of
// pinned host memory. Both return after their work is queued on `s`; build
// synchronises with `s` once per level to read the level's node count.
struct GpuBvhResult {
  uint32_t binary_nodes = 0, quad_nodes = 0, max_leaf = 0, depth = 0;
  uint32_t error = 0;  // 1 degenerate extent, 2 arena, 4 stack, 8 partition mismatch
  uint32_t levels = 0, small_roots = 0;
};
size_t gpu_bvh_scratch_bytes(uint32_t n);
cudaError_t gpu_bvh_build(const DevScene& sc, void* scratch, uint32_t* host_counters, cudaStream_t s, GpuBvhResult& r);
cudaError_t gpu_bvh_emit(const DevScene& sc, void* scratch, const GpuBvhResult& r, uint32_t leaf_shift, void* quad,
                         QNodeDev* nodes, float4* tris, uint32_t* prims, cudaStream_t s);

struct QuadNode;  // bvh_build.h
// QuadNode -> traversal node conversion, and the leaf-ordered triangle records
// (3 x float4 per primitive: v0 + id, e1, e2), for trees built on the device.
cudaError_t launch_quad_to_dev(const QuadNode* quad, uint32_t nq, uint32_t leaf_shift, QNodeDev* nodes, cudaStream_t s);
cudaError_t launch_leaf_tris(const DevScene& sc, const uint32_t* prims, uint32_t n, float4* tris, cudaStream_t s);

// Cost table of the 8-wide collapse (gpu_fbvh_build with wide = 1): C(n, i),
// i = 1..8, the surface-area cost of binary subtree n spread over i slots of
// its wide parent; split: 3 bits per i = 2..8 (bits 3(i-2)..), the slots given
// to the left child (0: as with i - 1 slots); leaf1: with one slot the subtree
// is one leaf slot.
struct __align__(16) WideCost {
  float c[8];
  uint32_t split;
  uint32_t leaf1;
  uint32_t pad[2];
};
static_assert(sizeof(WideCost) == 48, "WideCost");

// Device build of ct_bvh_build_fast's tree (bvh_gpu_fast.cu), byte-equal to the
// host build: gpu_fbvh_build fills `scratch` (gpu_fbvh_scratch_bytes) and
// returns the sizes (r.error: 1 a padded box is not finite, 2 capacity, 4
// stack, 8 partition mismatch, 16 collapse); gpu_fbvh_emit writes the quad
// nodes, traversal nodes, triangles and primitive order. host_counters: 16
// words of pinned host memory; the build synchronises with `s` once per level.
// wide = 1: the binary tree of the same rules over exact triangle bounds, then
// the 8-wide cost table instead of the quad collapse (for gpu_wbvh_collapse;
// gpu_fbvh_binary gives the arena, primitive order and table).
size_t gpu_fbvh_scratch_bytes(uint32_t n, int wide = 0);
cudaError_t gpu_fbvh_build(const DevScene& sc, void* scratch, uint32_t* host_counters, cudaStream_t s, GpuBvhResult& r,
                           int wide = 0);
void gpu_fbvh_binary(void* scratch, uint32_t n, int wide, const void** arena, const uint32_t** prims,
                     const WideCost** cost);
cudaError_t gpu_fbvh_emit(const DevScene& sc, void* scratch, const GpuBvhResult& r, uint32_t leaf_shift, void* quad,
                          QNodeDev* nodes, float4* tris, uint32_t* prims, cudaStream_t s);
// error word of the last emit (reads the counters back; synchronises with `s`)
uint32_t gpu_fbvh_error(void* scratch, uint32_t n, uint32_t* host_counters, cudaStream_t s);

// Collapse of a binary build into 8-wide quantised nodes. `scratch2` holds gpu_wbvh_scratch_bytes(binary_nodes);
// nodes end up in scratch2 (read back their count in *wide_nodes, then copy
// them out with gpu_wbvh_copy_nodes); triangles go straight to `tris` (n x 48 B).
size_t gpu_wbvh_scratch_bytes(uint32_t binary_nodes);
// arena / prims / cost: the binary tree (48-byte nodes {mn[3], first, mx[3],
// count, left, parent, depth, -}), primitive order and cost table of
// gpu_fbvh_build with wide = 1 (gpu_fbvh_binary); each wide node takes the
// slots of least surface-area cost from the table.
cudaError_t gpu_wbvh_collapse(const DevScene& sc, const void* arena, const uint32_t* prims, const WideCost* cost,
                              void* scratch2, uint32_t binary_nodes, float4* tris, uint32_t* host_counters,
                              cudaStream_t s, uint32_t* wide_nodes, uint32_t* depth, uint32_t* error);
cudaError_t gpu_wbvh_copy_nodes(void* scratch2, uint32_t binary_nodes, WNode8* out, uint32_t count, cudaStream_t s);

// Wide-tree queries: FP32 watertight tests; hits within the FP32 error bound
// of an edge or of another hit's t are settled by FP64 tests in a second
// kernel. counters: 2 device ints the launch zeroes (fetch cursor, record
// count); recs: kWideRecordBytes per ray, 16-byte aligned (settlement
// records). stats (may be null): [0] rays, [1] rays re-tested in FP64, [2]
// rays traced fully in FP64, [3] of [1], rays re-tested only because the best
// hit's t bound was loose.
constexpr size_t kWideRecordBytes = 32;
cudaError_t launch_trace_wide_closest(const DevWBVH& b, const float4* org, const float4* dir, int32_t* hit, float* t,
                                      uint32_t n, uint32_t* err, int* counters, void* recs,
                                      unsigned long long* stats, cudaStream_t s);
cudaError_t launch_trace_wide_any(const DevWBVH& b, const float4* org, const float4* dir, uint8_t* occ, uint32_t n,
                                  uint32_t* err, int* counters, void* recs, unsigned long long* stats,
                                  cudaStream_t s);

// Batch stages (one launch each for every job of the batch). The queue
// capacity is the batch's total pixel count; counts[0] must be zero before
// raygen (launch_batch_advance leaves it so).
cudaError_t launch_batch_raygen(const DevBatch& b, const DevQueues& q, int exact, cudaStream_t s);
// refill: idle lanes (8, 16 or 24 of 32) at which a traversal warp takes new rays
cudaError_t launch_batch_extend(const DevBatch& b, const DevQueues& q, int queue, bool fast, int block, int refill,
                                cudaStream_t s);
cudaError_t launch_batch_shade(const DevBatch& b, const DevQueues& q, int queue, uint32_t path_length, int pass,
                               int exact, int grid_mult, cudaStream_t s);
cudaError_t launch_batch_connect(const DevBatch& b, const DevQueues& q, bool fast, int block, cudaStream_t s);
cudaError_t launch_batch_advance(const DevBatch& b, const DevQueues& q, cudaStream_t s);

// Frame stages on a wide (quantised) BVH: the reference's Moller-Trumbore test
// and epsilon over conservative 8-bit boxes (k_trace_wide.cu).
cudaError_t launch_extend_wide(const DevWBVH& b, const DevQueues& q, int queue, float eps, cudaStream_t s);
cudaError_t launch_connect_wide(const DevWBVH& b, const DevQueues& q, float eps, cudaStream_t s);
cudaError_t launch_batch_extend_wide(const DevBatch& b, const DevQueues& q, int queue, cudaStream_t s);
// Order the rays of queue `queue` within windows of kSortWindow by direction
// class into q.perm_buf (key 1: octant; key 2: cube face x 4x4 cells; 0: nothing).
constexpr int kSortWindow = 2048;
cudaError_t launch_ray_sort(const DevQueues& q, int queue, int key, cudaStream_t s);
cudaError_t launch_batch_connect_wide(const DevBatch& b, const DevQueues& q, cudaStream_t s);

// accum[i] += frame[i]; frame[i] = 0 (folds an overlapped frame's private buffer)
cudaError_t launch_fold(float4* accum, float4* frame, int n, cudaStream_t s);
// accum[i] += each entry k < entries of log[k * stride + i] whose w is `tag`
// (uint bits), in k order: rgb and w + 1 as separate round-to-nearest additions
// (replays an overlapped exact-math frame's contributions, DevQueues::log)
cudaError_t launch_fold_log(float4* accum, const float4* log, int entries, int stride, int n, uint32_t tag,
                            cudaStream_t s);

// allocation-free frame (noalloc.cu): queues in a static device array
uint32_t noalloc_max_pixels();
cudaError_t noalloc_render(int device, const DevScene& sc, const DevBVH& bvh, const FrameConst& f, int max_depth,
                           int exact_math, float4* accum, uint32_t* err, cudaStream_t s);


}  // namespace ct

// Host-side accessors of the runtime objects (api.cpp), for the serving loop.
#include <string>
#include <utility>
#include <vector>

#include "../../include/cudatracer.h"

namespace ct {
const DevScene& rt_scene_dev(const ct_scene* s);
uint32_t rt_scene_tris(const ct_scene* s);
const DevBVH& rt_bvh_dev(const ct_bvh* b);
bool rt_bvh_wide(const ct_bvh* b);
uint32_t rt_bvh_tris(const ct_bvh* b);
int rt_ctx_device(const ct_ctx* c);
uint32_t* rt_ctx_error(const ct_ctx* c);
ct_status rt_fail(ct_ctx* c, ct_status s, const std::string& msg);
// device allocation counted against the context's budget (rt_free gives it back)
ct_status rt_alloc(ct_ctx* c, size_t bytes, void** p);
void rt_free(ct_ctx* c, void* p, size_t bytes);
ct_status rt_alloc_queues(ct_ctx* c, size_t n, DevQueues& q, std::vector<std::pair<void*, size_t>>& owned);
void rt_free_list(ct_ctx* c, std::vector<std::pair<void*, size_t>>& owned);
FrameConst rt_frame_const(const ct_camera* cam, const ct_render_params* p);
const DevWBVH& rt_bvh_wdev(const ct_bvh* b);
// count stream-ordered allocations against the context's budget (false: over budget)
bool rt_account(ct_ctx* c, int64_t delta);
ct_status rt_check_job(ct_ctx* ctx, const ct_batch_job& J);
}  // namespace ct
