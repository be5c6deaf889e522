// Traversal kernels: public closest/any-hit queries and the wavefront's
// extend (closest hit) and connect (shadow any hit + accumulate) stages.
//
// Launch shape: 128-thread blocks, each thread owns one ray at a time; the
// traversal stack lives in dynamic shared memory laid out [entry][thread] so
// that a warp's pushes and pops hit 32 distinct banks. Queue-driven stages
// read their active count from device memory (no host round trip) and walk
// the queue with a grid-stride loop over a grid sized to fill every SM.
#include "trace.cuh"

namespace ct {

constexpr int kBlock = 128;
constexpr float kMaxDistance = 1e34f;  // MAX_DISTANCE, src/Core/Ray.cuh:13

int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    if (n <= 0) n = 1;
  }
  return n;
}

namespace {

size_t stack_bytes(const DevBVH& b) { return (size_t)b.stack_entries * kBlock * sizeof(int); }

template <typename K>
int resident_grid(K kernel, size_t smem) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, smem);
  if (per_sm <= 0) per_sm = 1;
  return per_sm * sm_count();
}

template <typename K>
cudaError_t prepare(K kernel, size_t smem) {
  if (smem > 48 * 1024) return cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  return cudaSuccess;
}

// ---- public ray queries (ct_trace_closest / ct_trace_any) ----
template <bool ANY>
__global__ void __launch_bounds__(kBlock) k_query(DevBVH b, const float4* __restrict__ org,
                                                   const float4* __restrict__ dir, int32_t* __restrict__ hit_out,
                                                   float* __restrict__ t_out, uint8_t* __restrict__ occ_out,
                                                   uint32_t n, float eps, uint32_t* err) {
  extern __shared__ int s_stack[];
  int* stack = s_stack + threadIdx.x;
  for (uint32_t i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
    const float4 o = __ldg(org + i), d = __ldg(dir + i);
    float t = d.w;
    int hit = -1;
    if (!traverse<ANY>(b, o.x, o.y, o.z, d.x, d.y, d.z, eps, t, hit, stack, kBlock)) {
      atomicOr(err, kErrStackOverflow);
      hit = -1;
      t = d.w;
    }
    if (ANY) {
      occ_out[i] = hit >= 0 ? 1 : 0;
    } else {
      hit_out[i] = hit;
      t_out[i] = t;
    }
  }
}

// ---- wavefront extend: closest hit for every ray of queue `qi` ----
// (the reference's extend, src/CUDA/Kernel.cu:236-245: t reset to MAX_DISTANCE)
__global__ void __launch_bounds__(kBlock) k_extend(DevBVH b, DevQueues q, int qi, float eps) {
  extern __shared__ int s_stack[];
  int* stack = s_stack + threadIdx.x;
  const int n = q.counts[qi];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // the shade stage that follows appends to these (setGlobals, Kernel.cu:75-86)
    q.counts[qi ^ 1] = 0;
    q.counts[2] = 0;
    atomicAdd(&q.stats[0], (unsigned long long)n);
  }
  const float4* __restrict__ org = q.org_q(qi);
  const float4* __restrict__ dir = q.dir_q(qi);
  for (int i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
    const float4 o = __ldg(org + i), d = __ldg(dir + i);
    float t = kMaxDistance;
    int hit = -1;
    if (!traverse<false>(b, o.x, o.y, o.z, d.x, d.y, d.z, eps, t, hit, stack, kBlock)) {
      atomicOr(q.error, kErrStackOverflow);
      hit = -1;
      t = kMaxDistance;
    }
    q.hit[i] = make_int2(hit, __float_as_int(t));
  }
}

// ---- wavefront connect: shadow any hit, add unoccluded contributions ----
// (src/CUDA/Kernel.cu:247-256)
__global__ void __launch_bounds__(kBlock) k_connect(DevBVH b, DevQueues q, float eps) {
  extern __shared__ int s_stack[];
  int* stack = s_stack + threadIdx.x;
  const int n = q.counts[2];
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&q.stats[1], (unsigned long long)n);
  for (int i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
    const float4 o = __ldg(q.sorg + i), d = __ldg(q.sdir + i);
    float t = d.w;
    int hit = -1;
    if (!traverse<true>(b, o.x, o.y, o.z, d.x, d.y, d.z, eps, t, hit, stack, kBlock)) {
      atomicOr(q.error, kErrStackOverflow);
      continue;
    }
    if (hit < 0) {
      const float4 c = __ldg(q.scol + i);
      const int pix = __float_as_int(o.w);
      float4 a = q.accum[pix];  // one shadow ray per pixel per pass: no race
      a.x = __fadd_rn(a.x, c.x);
      a.y = __fadd_rn(a.y, c.y);
      a.z = __fadd_rn(a.z, c.z);
      a.w = __fadd_rn(a.w, 1.0f);
      q.accum[pix] = a;
    }
  }
}

}  // namespace

cudaError_t launch_trace_closest(const DevBVH& b, const float4* org, const float4* dir, int32_t* hit, float* t,
                                 uint32_t n, float eps, uint32_t* err, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const size_t smem = stack_bytes(b);
  cudaError_t e = prepare(k_query<false>, smem);
  if (e != cudaSuccess) return e;
  const uint32_t blocks = (n + kBlock - 1) / kBlock;
  const uint32_t grid = std::min<uint32_t>(blocks, (uint32_t)resident_grid(k_query<false>, smem) * 8u);
  k_query<false><<<grid, kBlock, smem, s>>>(b, org, dir, hit, t, nullptr, n, eps, err);
  return cudaGetLastError();
}

cudaError_t launch_trace_any(const DevBVH& b, const float4* org, const float4* dir, uint8_t* occ, uint32_t n,
                             float eps, uint32_t* err, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const size_t smem = stack_bytes(b);
  cudaError_t e = prepare(k_query<true>, smem);
  if (e != cudaSuccess) return e;
  const uint32_t blocks = (n + kBlock - 1) / kBlock;
  const uint32_t grid = std::min<uint32_t>(blocks, (uint32_t)resident_grid(k_query<true>, smem) * 8u);
  k_query<true><<<grid, kBlock, smem, s>>>(b, org, dir, nullptr, nullptr, occ, n, eps, err);
  return cudaGetLastError();
}

cudaError_t launch_extend(const DevBVH& b, const DevQueues& q, int queue, float eps, cudaStream_t s) {
  const size_t smem = stack_bytes(b);
  cudaError_t e = prepare(k_extend, smem);
  if (e != cudaSuccess) return e;
  const int cap_blocks = (q.capacity + kBlock - 1) / kBlock;
  const int grid = std::max(1, std::min(cap_blocks, resident_grid(k_extend, smem)));
  k_extend<<<grid, kBlock, smem, s>>>(b, q, queue, eps);
  return cudaGetLastError();
}

cudaError_t launch_connect(const DevBVH& b, const DevQueues& q, float eps, cudaStream_t s) {
  const size_t smem = stack_bytes(b);
  cudaError_t e = prepare(k_connect, smem);
  if (e != cudaSuccess) return e;
  const int cap_blocks = (q.capacity + kBlock - 1) / kBlock;
  const int grid = std::max(1, std::min(cap_blocks, resident_grid(k_connect, smem)));
  k_connect<<<grid, kBlock, smem, s>>>(b, q, eps);
  return cudaGetLastError();
}

}  // namespace ct
