// Allocation-free render path: the wavefront queues of one frame live in a
// file-scope __device__ array instead of memory the library allocates.
//
// Who needs it: a host application that owns all device memory itself, or
// whose render thread must never enter the CUDA allocator (cudaMalloc and
// cudaFree can synchronise the device and stall the frame). Such a caller
// creates its scene and BVH once at load time, then renders every frame
// through ct_render_accumulate_noalloc into an accumulation buffer it owns.
//
// Limits and sharing:
//   * at most kNoAllocMaxPixels paths per frame (width * height <= 65,536,
//     e.g. 256 x 256); the array is ~9.5 MiB and every GPU that loads the
//     library holds it until the process exits;
//   * every call uses the same array and it keeps the last call's contents:
//     calls whose work overlaps on the GPU (different streams, threads or
//     contexts on one device) race with each other and must be serialised;
//   * the first call on each device looks up the array's device address
//     with cudaGetSymbolAddress; make that first call before any stream
//     capture begins. The address is kept for the life of the process and
//     belongs to the device's context as it was then: after a cudaDeviceReset
//     of that device it is stale, so the entry point must not be used on a
//     device this process has reset since its first call there.
#include <mutex>

#include "ct_internal.h"

namespace ct {

constexpr uint32_t kNoAllocMaxPixels = 65536;
// nine float4 queues (two ray queues of three, one shadow queue of three),
// the int2 hit buffer, then 16 counters and 8 statistics words
constexpr size_t kQueueBytes = (size_t)kNoAllocMaxPixels * 16;
constexpr size_t kHitBytes = (size_t)kNoAllocMaxPixels * 8;
constexpr size_t kCountsOffset = 9 * kQueueBytes + kHitBytes;
constexpr size_t kStatsOffset = kCountsOffset + 16 * sizeof(int32_t);
constexpr size_t kScratchBytes = kStatsOffset + 8 * sizeof(unsigned long long);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

namespace {
std::mutex g_mu;
void* g_addr[256] = {};  // per device ordinal, looked up once
}  // namespace

uint32_t noalloc_max_pixels() { return kNoAllocMaxPixels; }

// Looks the scratch address up once per device (with that device current).
cudaError_t noalloc_scratch(int device, unsigned char** out) {
  if (device < 0 || device >= 256) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_addr[device]) {
    void* p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_addr[device] = p;
  }
  *out = (unsigned char*)g_addr[device];
  return cudaSuccess;
}

cudaError_t noalloc_render(int device, const DevScene& sc, const DevBVH& bvh, const FrameConst& f, int max_depth,
                           int exact_math, float4* accum, uint32_t* err, cudaStream_t s) {
  unsigned char* base = nullptr;
  cudaError_t e = noalloc_scratch(device, &base);
  if (e != cudaSuccess) return e;
  DevQueues q{};
  float4* qs = (float4*)base;
  const size_t n4 = kNoAllocMaxPixels;
  q.org[0] = qs + 0 * n4;
  q.org[1] = qs + 1 * n4;
  q.dir[0] = qs + 2 * n4;
  q.dir[1] = qs + 3 * n4;
  q.thr[0] = qs + 4 * n4;
  q.thr[1] = qs + 5 * n4;
  q.sorg = qs + 6 * n4;
  q.sdir = qs + 7 * n4;
  q.scol = qs + 8 * n4;
  q.hit = (int2*)(base + 9 * kQueueBytes);
  q.counts = (int32_t*)(base + kCountsOffset);
  q.stats = (unsigned long long*)(base + kStatsOffset);
  q.accum = accum;
  q.error = err;
  q.capacity = f.width * f.height;
  // counters and statistics start at zero on every call (the array keeps the last call's values)
  if ((e = cudaMemsetAsync(base + kCountsOffset, 0, kScratchBytes - kCountsOffset, s)) != cudaSuccess) return e;
  const bool fast = math_fast_traversal(exact_math);
  const int exact_shade = math_exact_shading(exact_math);
  if ((e = launch_raygen(q, f, exact_shade, s)) != cudaSuccess) return e;
  for (int pass = 0; pass < max_depth; pass++) {
    const int cur = pass & 1;
    const int path_length = pass == 0 ? 0 : pass + 1;
    if ((e = launch_extend(bvh, q, cur, f.tri_eps, fast, s)) != cudaSuccess) return e;
    if ((e = launch_shade(sc, q, f, cur, path_length, exact_shade, s)) != cudaSuccess) return e;
    if (f.shadow && (e = launch_connect(bvh, q, f.tri_eps, fast, s)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace ct
