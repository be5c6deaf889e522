// Traversal kernels: public closest/any-hit queries and the wavefront's
// extend (closest hit) and connect (shadow any hit + accumulate) stages.
//
// Launch shape: 64-thread blocks (measured ahead of 128 and 256), as many as
// are resident on all SMs. Ray queries and extend use persistent warps that
// pull rays from a device cursor (trace_persistent); connect walks its queue
// with a grid-stride loop, whose warps keep neighbouring shadow rays in step
// (measured ahead of persistent refills and of per-lane continuous loops).
// Queue-driven stages read their active count on the device: no host round
// trip between stages. The traversal stack lives in dynamic shared memory laid
// out [entry][thread], so a warp's pushes and pops hit 32 distinct banks.
#include "trace.cuh"

namespace ct {

constexpr int kBlock = 64;
constexpr int kExtendRefill = 24;  // idle lanes that make an extend warp refill (of 32)
constexpr int kQueryRefill = 8;    // the same for ray queries (shorter, often coherent)
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

// ---- ray sources and result sinks ----
struct QueryIO {
  const float4* __restrict__ org;
  const float4* __restrict__ dir;
  int32_t* hit_out;
  float* t_out;
  uint8_t* occ_out;
  uint32_t* err;
  __device__ void load(int i, float4& o, float4& d, float& t0) {
    o = __ldg(org + i);
    d = __ldg(dir + i);
    t0 = d.w;
  }
  __device__ void store(int i, const RayState& r, bool overflow) {
    int hit = r.hit;
    float t = r.t;
    if (overflow) {
      atomicOr(err, kErrStackOverflow);
      hit = -1;
      t = __ldg(&dir[i].w);
    }
    if (occ_out) {
      occ_out[i] = hit >= 0 ? 1 : 0;
    } else {
      hit_out[i] = hit;
      t_out[i] = t;
    }
  }
};

// extend (src/CUDA/Kernel.cu:236-245): t restarts at MAX_DISTANCE every pass
struct ExtendIO {
  const float4* __restrict__ org;
  const float4* __restrict__ dir;
  int2* hit;
  uint32_t* err;
  const int32_t* __restrict__ perm;
  __device__ void load(int i, float4& o, float4& d, float& t0) {
    if (perm) i = __ldg(perm + i);
    o = __ldg(org + i);
    d = __ldg(dir + i);
    t0 = kMaxDistance;
  }
  __device__ void store(int i, const RayState& r, bool overflow) {
    if (perm) i = __ldg(perm + i);
    if (overflow) {
      atomicOr(err, kErrStackOverflow);
      hit[i] = make_int2(-1, __float_as_int(kMaxDistance));
      return;
    }
    hit[i] = make_int2(r.hit, __float_as_int(r.t));
  }
};

template <bool ANY>
__global__ void __launch_bounds__(kBlock) k_query(DevBVH b, QueryIO io, int n, int* cursor, float eps) {
  extern __shared__ int s_stack[];
  trace_persistent<ANY, false, kQueryRefill>(b, n, cursor, eps, io, s_stack + threadIdx.x, kBlock);
}

template <bool FASTMM>
__global__ void __launch_bounds__(kBlock) k_extend(DevBVH b, DevQueues q, int qi, float eps) {
  extern __shared__ int s_stack[];
  const int n = q.counts[qi];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    // the shade stage that follows appends to these (setGlobals, Kernel.cu:75-86)
    q.counts[qi ^ 1] = 0;
    q.counts[2] = 0;
    atomicAdd(&q.stats[0], (unsigned long long)n);
  }
  ExtendIO io{q.org_q(qi), q.dir_q(qi), q.hit, q.error, q.perm};
  trace_persistent<false, FASTMM, kExtendRefill>(b, n, q.counts + 4, eps, io, s_stack + threadIdx.x, kBlock);
}

// connect (src/CUDA/Kernel.cu:247-256): unoccluded shadow rays add their
// contribution to their pixel (one shadow ray per pixel per pass: no race)
template <bool FASTMM>
__global__ void __launch_bounds__(kBlock) k_connect(DevBVH b, DevQueues q, float eps) {
  extern __shared__ int s_stack[];
  int* stack = s_stack + threadIdx.x;
  const int n = q.counts[2];
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&q.stats[1], (unsigned long long)n);
  for (int i = blockIdx.x * kBlock + threadIdx.x; i < n; i += gridDim.x * kBlock) {
    const float4 o = __ldg(q.sorg + i), d = __ldg(q.sdir + i);
    RayState r;
    ray_begin(r, o, d, d.w);
    if (!traverse<true, FASTMM>(b, r, eps, stack, kBlock)) {
      atomicOr(q.error, kErrStackOverflow);
      continue;
    }
    if (r.hit < 0) {
      const float4 c = __ldg(q.scol + i);
      const int pix = __float_as_int(o.w);
      if (q.log) {  // an exact frame in a slot: this launch's log entry (DevQueues::log)
        q.log[(size_t)q.log_entry * q.capacity + pix] = make_float4(c.x, c.y, c.z, __uint_as_float(q.log_tag));
        continue;
      }
      float4 a = q.accum[pix];
      a.x = __fadd_rn(a.x, c.x);
      a.y = __fadd_rn(a.y, c.y);
      a.z = __fadd_rn(a.z, c.z);
      a.w = __fadd_rn(a.w, 1.0f);
      q.accum[pix] = a;
    }
  }
}

template <bool ANY>
cudaError_t launch_query(const DevBVH& b, const QueryIO& io, uint32_t n, int* cursor, float eps, cudaStream_t s) {
  if (n == 0) return cudaSuccess;
  const size_t smem = stack_bytes(b);
  cudaError_t e = prepare(k_query<ANY>, smem);
  if (e != cudaSuccess) return e;
  if ((e = cudaMemsetAsync(cursor, 0, sizeof(int), s)) != cudaSuccess) return e;
  const uint32_t blocks = (n + kBlock - 1) / kBlock;
  const uint32_t grid = std::min<uint32_t>(blocks, (uint32_t)resident_grid(k_query<ANY>, smem));
  k_query<ANY><<<grid, kBlock, smem, s>>>(b, io, (int)n, cursor, eps);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_trace_closest(const DevBVH& b, const float4* org, const float4* dir, int32_t* hit, float* t,
                                 uint32_t n, float eps, uint32_t* err, int* cursor, cudaStream_t s) {
  return launch_query<false>(b, QueryIO{org, dir, hit, t, nullptr, err}, n, cursor, eps, s);
}

cudaError_t launch_trace_any(const DevBVH& b, const float4* org, const float4* dir, uint8_t* occ, uint32_t n,
                             float eps, uint32_t* err, int* cursor, cudaStream_t s) {
  return launch_query<true>(b, QueryIO{org, dir, nullptr, nullptr, occ, err}, n, cursor, eps, s);
}

cudaError_t launch_extend(const DevBVH& b, const DevQueues& q, int queue, float eps, bool fast, cudaStream_t s) {
  const size_t smem = stack_bytes(b);
  auto kernel = fast ? k_extend<true> : k_extend<false>;
  cudaError_t e = prepare(kernel, smem);
  if (e != cudaSuccess) return e;
  const int cap_blocks = (q.capacity + kBlock - 1) / kBlock;
  const int grid = std::max(1, std::min(cap_blocks, resident_grid(kernel, smem)));
  kernel<<<grid, kBlock, smem, s>>>(b, q, queue, eps);
  return cudaGetLastError();
}

cudaError_t launch_connect(const DevBVH& b, const DevQueues& q, float eps, bool fast, cudaStream_t s) {
  const size_t smem = stack_bytes(b);
  auto kernel = fast ? k_connect<true> : k_connect<false>;
  cudaError_t e = prepare(kernel, smem);
  if (e != cudaSuccess) return e;
  const int cap_blocks = (q.capacity + kBlock - 1) / kBlock;
  const int grid = std::max(1, std::min(cap_blocks, resident_grid(kernel, smem)));
  kernel<<<grid, kBlock, smem, s>>>(b, q, eps);
  return cudaGetLastError();
}


// ------------------------------------------------------------- ray sorting
// Windows of kSortWindow consecutive queue entries are counting-sorted by a
// direction class in shared memory; q.perm_buf[base + rank] = queue index.
// Sorting them by direction puts rays that traverse alike into one warp (the
// queue is roughly in pixel order, so a window's rays already start close
// together). A ray's result does not depend on the order (extend writes each
// hit at its own queue index), so every key gives identical frames.
namespace {

constexpr int kSortThreads = 256;

template <int KEY>
__device__ __forceinline__ int ray_class(float4 d) {
  if (KEY == 1) return (d.x < 0.0f ? 1 : 0) | (d.y < 0.0f ? 2 : 0) | (d.z < 0.0f ? 4 : 0);
  // cube face of the direction and a 4x4 cell grid on that face
  const float ax = fabsf(d.x), ay = fabsf(d.y), az = fabsf(d.z);
  int face;
  float u, v, m;
  if (ax >= ay && ax >= az) {
    face = d.x < 0.0f ? 1 : 0, u = d.y, v = d.z, m = ax;
  } else if (ay >= az) {
    face = d.y < 0.0f ? 3 : 2, u = d.x, v = d.z, m = ay;
  } else {
    face = d.z < 0.0f ? 5 : 4, u = d.x, v = d.y, m = az;
  }
  const float sc = m > 0.0f ? 2.0f / m : 0.0f;  // u / m in [-1, 1] -> [0, 4]
  const int cu = min(3, max(0, (int)(u * sc + 2.0f)));
  const int cv = min(3, max(0, (int)(v * sc + 2.0f)));
  return face * 16 + cv * 4 + cu;
}

template <int KEY>
__global__ void __launch_bounds__(kSortThreads) k_ray_sort(DevQueues q, int qi) {
  constexpr int NB = KEY == 1 ? 8 : 96;
  constexpr int PER = kSortWindow / kSortThreads;
  constexpr int BPL = (NB + 31) / 32;  // bins per lane of the scan
  __shared__ int bins[NB];
  const int n = q.counts[qi];
  const int base = blockIdx.x * kSortWindow;
  if (base >= n) return;
  const int cnt = min(kSortWindow, n - base);
  for (int b = threadIdx.x; b < NB; b += kSortThreads) bins[b] = 0;
  __syncthreads();
  const float4* dir = q.dir_q(qi) + base;
  int key[PER], rank[PER];
#pragma unroll
  for (int k = 0; k < PER; k++) {
    const int i = k * kSortThreads + threadIdx.x;
    key[k] = -1;
    rank[k] = 0;
    if (i < cnt) {
      key[k] = ray_class<KEY>(__ldg(dir + i));
      rank[k] = atomicAdd(&bins[key[k]], 1);
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {  // exclusive scan of the bin counts
    const int lane = threadIdx.x;
    int c[BPL], sum = 0;
#pragma unroll
    for (int j = 0; j < BPL; j++) {
      const int b = lane * BPL + j;
      c[j] = b < NB ? bins[b] : 0;
      sum += c[j];
    }
    int inc = sum;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, inc, off);
      if (lane >= off) inc += y;
    }
    int run = inc - sum;
#pragma unroll
    for (int j = 0; j < BPL; j++) {
      const int b = lane * BPL + j;
      if (b < NB) bins[b] = run;
      run += c[j];
    }
  }
  __syncthreads();
  int32_t* perm = q.perm_buf + base;
#pragma unroll
  for (int k = 0; k < PER; k++)
    if (key[k] >= 0) perm[bins[key[k]] + rank[k]] = base + k * kSortThreads + threadIdx.x;
}

}  // namespace

cudaError_t launch_ray_sort(const DevQueues& q, int queue, int key, cudaStream_t s) {
  if (key == 0 || !q.perm_buf) return cudaSuccess;
  const int grid = std::max(1, (q.capacity + kSortWindow - 1) / kSortWindow);
  if (key == 1)
    k_ray_sort<1><<<grid, kSortThreads, 0, s>>>(q, queue);
  else
    k_ray_sort<2><<<grid, kSortThreads, 0, s>>>(q, queue);
  return cudaGetLastError();
}

// ---------------------------------------------------------------- batches
namespace {

struct BatchExtendIO {
  const float4* __restrict__ org;
  const float4* __restrict__ dir;
  int2* hit;
  uint32_t* err;
  const BatchJob* jobs;
  const int32_t* bases;
  int n_jobs;
  const int32_t* __restrict__ perm;
  __device__ void load(int i, float4& o, float4& d, float& t0, DevBVH& b, float& eps) {
    if (perm) i = __ldg(perm + i);
    o = __ldg(org + i);
    d = __ldg(dir + i);
    t0 = kMaxDistance;
    const BatchJob& J = jobs[batch_job_of(bases, n_jobs, __float_as_int(o.w))];
    b = J.bvh;
    eps = J.f.tri_eps;
  }
  __device__ void store(int i, const RayState& r, bool overflow) {
    if (perm) i = __ldg(perm + i);
    if (overflow) {
      atomicOr(err, kErrStackOverflow);
      hit[i] = make_int2(-1, __float_as_int(kMaxDistance));
      return;
    }
    hit[i] = make_int2(r.hit, __float_as_int(r.t));
  }
};

template <bool FASTMM, int BLOCK, int REFILL>
__global__ void __launch_bounds__(BLOCK) k_batch_extend(DevBatch bt, DevQueues q, int qi) {
  extern __shared__ int s_stack[];
  const int n = q.counts[qi];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    q.counts[qi ^ 1] = 0;
    q.counts[2] = 0;
    atomicAdd(&q.stats[0], (unsigned long long)n);
  }
  BatchExtendIO io{q.org_q(qi), q.dir_q(qi), q.hit, q.error, bt.jobs, bt.bases, bt.n_jobs, q.perm};
  trace_persistent_batch<false, FASTMM, REFILL>(n, q.counts + 4, io, s_stack + threadIdx.x, BLOCK);
}

template <bool FASTMM, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_batch_connect(DevBatch bt, DevQueues q) {
  extern __shared__ int s_stack[];
  int* stack = s_stack + threadIdx.x;
  const int n = q.counts[2];
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&q.stats[1], (unsigned long long)n);
  for (int i = blockIdx.x * BLOCK + threadIdx.x; i < n; i += gridDim.x * BLOCK) {
    const float4 o = __ldg(q.sorg + i), d = __ldg(q.sdir + i);
    const int pix = __float_as_int(o.w);
    const BatchJob& J = bt.jobs[batch_job_of(bt.bases, bt.n_jobs, pix)];
    const DevBVH b = J.bvh;
    RayState r;
    ray_begin(r, o, d, d.w);
    if (!traverse<true, FASTMM>(b, r, J.f.tri_eps, stack, BLOCK)) {
      atomicOr(q.error, kErrStackOverflow);
      continue;
    }
    if (r.hit < 0) {
      const float4 c = __ldg(q.scol + i);
      float4* acc = J.accum + (pix - J.pix_base);
      float4 a = *acc;
      a.x = __fadd_rn(a.x, c.x);
      a.y = __fadd_rn(a.y, c.y);
      a.z = __fadd_rn(a.z, c.z);
      a.w = __fadd_rn(a.w, 1.0f);
      *acc = a;
    }
  }
}

template <bool FASTMM, int BLOCK, int REFILL>
cudaError_t batch_extend(const DevBatch& b, const DevQueues& q, int queue, cudaStream_t s) {
  const size_t smem = (size_t)b.max_stack * BLOCK * sizeof(int);
  auto kernel = k_batch_extend<FASTMM, BLOCK, REFILL>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, BLOCK, smem);
  const int cap_blocks = (q.capacity + BLOCK - 1) / BLOCK;
  const int grid = std::max(1, std::min(cap_blocks, std::max(1, per_sm) * sm_count()));
  kernel<<<grid, BLOCK, smem, s>>>(b, q, queue);
  return cudaGetLastError();
}

template <bool FASTMM, int BLOCK>
cudaError_t batch_connect(const DevBatch& b, const DevQueues& q, cudaStream_t s) {
  const size_t smem = (size_t)b.max_stack * BLOCK * sizeof(int);
  auto kernel = k_batch_connect<FASTMM, BLOCK>;
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, BLOCK, smem);
  const int cap_blocks = (q.capacity + BLOCK - 1) / BLOCK;
  const int grid = std::max(1, std::min(cap_blocks, std::max(1, per_sm) * sm_count()));
  kernel<<<grid, BLOCK, smem, s>>>(b, q);
  return cudaGetLastError();
}

}  // namespace

namespace {
template <int BLOCK, int REFILL>
cudaError_t batch_extend_math(const DevBatch& b, const DevQueues& q, int queue, bool fast, cudaStream_t s) {
  return fast ? batch_extend<true, BLOCK, REFILL>(b, q, queue, s) : batch_extend<false, BLOCK, REFILL>(b, q, queue, s);
}
template <int BLOCK>
cudaError_t batch_extend_refill(const DevBatch& b, const DevQueues& q, int queue, bool fast, int refill,
                                cudaStream_t s) {
  if (refill == 8) return batch_extend_math<BLOCK, 8>(b, q, queue, fast, s);
  if (refill == 16) return batch_extend_math<BLOCK, 16>(b, q, queue, fast, s);
  return batch_extend_math<BLOCK, 24>(b, q, queue, fast, s);
}
}  // namespace

cudaError_t launch_batch_extend(const DevBatch& b, const DevQueues& q, int queue, bool fast, int block, int refill,
                                cudaStream_t s) {
  if (block == 64) return batch_extend_refill<64>(b, q, queue, fast, refill, s);
  if (block == 256) return batch_extend_refill<256>(b, q, queue, fast, refill, s);
  return batch_extend_refill<128>(b, q, queue, fast, refill, s);
}

cudaError_t launch_batch_connect(const DevBatch& b, const DevQueues& q, bool fast, int block, cudaStream_t s) {
  if (block == 64) return fast ? batch_connect<true, 64>(b, q, s) : batch_connect<false, 64>(b, q, s);
  if (block == 256) return fast ? batch_connect<true, 256>(b, q, s) : batch_connect<false, 256>(b, q, s);
  return fast ? batch_connect<true, 128>(b, q, s) : batch_connect<false, 128>(b, q, s);
}

}  // namespace ct
