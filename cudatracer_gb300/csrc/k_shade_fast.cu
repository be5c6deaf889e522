// Fast build of the shading kernels (FMA contraction, CUDA float
// transcendentals), plus the launchers that pick a build and the present pass.
#define CT_SHADE_NS fast
#define CT_EXACT 0
#include "k_shade.cuh"

namespace ct {
namespace exact {
__global__ void __launch_bounds__(128) k_shade(DevScene sc, DevQueues q, FrameConst f, int cur, uint32_t path_length);
__global__ void __launch_bounds__(128) k_raygen(DevQueues q, FrameConst f);
__global__ void __launch_bounds__(128) k_batch_raygen(DevBatch bt, DevQueues q);
__global__ void __launch_bounds__(128) k_batch_shade(DevBatch bt, DevQueues q, int cur, uint32_t path_length, int pass);
__global__ void k_batch_advance(DevBatch bt, DevQueues q);
}  // namespace exact

namespace {
constexpr int kBlock = 128;

template <typename K>
int fill_grid(K kernel, int work) {
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, kBlock, 0);
  if (per_sm <= 0) per_sm = 1;
  const int blocks = (work + kBlock - 1) / kBlock;
  return blocks < per_sm * sm_count() ? (blocks > 0 ? blocks : 1) : per_sm * sm_count();
}

// draw_framebuffer (src/CUDA/Kernel.cu:258-270) into a device buffer.
__global__ void k_present(const float4* __restrict__ accum, float4* __restrict__ out, int n, float samples) {
  const float e = 1.0f / 2.2f;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 a = accum[i];
    out[i] = make_float4(powf(a.x / samples, e), powf(a.y / samples, e), powf(a.z / samples, e), 1.0f);
  }
}
__global__ void k_fold(float4* __restrict__ accum, float4* __restrict__ frame, int n) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 f = frame[i];
    float4 a = accum[i];
    a.x += f.x;
    a.y += f.y;
    a.z += f.z;
    a.w += f.w;
    accum[i] = a;
    frame[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
}
__global__ void k_fold_log(float4* __restrict__ accum, const float4* __restrict__ log, int entries, int stride, int n,
                           uint32_t tag) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    float4 a = accum[i];
    for (int k = 0; k < entries; k++) {
      const float4 e = __ldg(log + (size_t)k * stride + i);
      if (__float_as_uint(e.w) != tag) continue;
      a.x = __fadd_rn(a.x, e.x);
      a.y = __fadd_rn(a.y, e.y);
      a.z = __fadd_rn(a.z, e.z);
      a.w = __fadd_rn(a.w, 1.0f);
    }
    accum[i] = a;
  }
}
}  // namespace

cudaError_t launch_fold_log(float4* accum, const float4* log, int entries, int stride, int n, uint32_t tag,
                            cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int grid = (n + 255) / 256 < 8 * sm_count() ? (n + 255) / 256 : 8 * sm_count();
  k_fold_log<<<grid, 256, 0, s>>>(accum, log, entries, stride, n, tag);
  return cudaGetLastError();
}

cudaError_t launch_fold(float4* accum, float4* frame, int n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int grid = (n + 255) / 256 < 8 * sm_count() ? (n + 255) / 256 : 8 * sm_count();
  k_fold<<<grid, 256, 0, s>>>(accum, frame, n);
  return cudaGetLastError();
}

cudaError_t launch_raygen(const DevQueues& q, const FrameConst& f, int exact_math, cudaStream_t s) {
  const int npix = f.width * f.height;
  if (exact_math) {
    exact::k_raygen<<<fill_grid(exact::k_raygen, npix), kBlock, 0, s>>>(q, f);
  } else {
    fast::k_raygen<<<fill_grid(fast::k_raygen, npix), kBlock, 0, s>>>(q, f);
  }
  return cudaGetLastError();
}

cudaError_t launch_shade(const DevScene& sc, const DevQueues& q, const FrameConst& f, int queue, int path_length,
                         int exact_math, cudaStream_t s) {
  if (exact_math) {
    exact::k_shade<<<fill_grid(exact::k_shade, q.capacity), kBlock, 0, s>>>(sc, q, f, queue, (uint32_t)path_length);
  } else {
    fast::k_shade<<<fill_grid(fast::k_shade, q.capacity), kBlock, 0, s>>>(sc, q, f, queue, (uint32_t)path_length);
  }
  return cudaGetLastError();
}

cudaError_t launch_present(const float4* accum, float4* out, int n, float samples, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const int grid = (n + 255) / 256 < 4096 ? (n + 255) / 256 : 4096;
  k_present<<<grid, 256, 0, s>>>(accum, out, n, samples);
  return cudaGetLastError();
}


cudaError_t launch_batch_raygen(const DevBatch& b, const DevQueues& q, int exact, cudaStream_t s) {
  if (exact)
    exact::k_batch_raygen<<<fill_grid(exact::k_batch_raygen, b.total_pix), kBlock, 0, s>>>(b, q);
  else
    fast::k_batch_raygen<<<fill_grid(fast::k_batch_raygen, b.total_pix), kBlock, 0, s>>>(b, q);
  return cudaGetLastError();
}

cudaError_t launch_batch_shade(const DevBatch& b, const DevQueues& q, int queue, uint32_t path_length, int pass,
                               int exact, int grid_mult, cudaStream_t s) {
  // the live count is on the device: size the grid for the capacity, up to grid_mult waves
  auto k = exact ? exact::k_batch_shade : fast::k_batch_shade;
  int per_sm = 0;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kBlock, 0);
  const int cap_blocks = (q.capacity + kBlock - 1) / kBlock;
  const int grid = std::max(1, std::min(cap_blocks, std::max(1, per_sm) * sm_count() * std::max(1, grid_mult)));
  k<<<grid, kBlock, 0, s>>>(b, q, queue, path_length, pass);
  return cudaGetLastError();
}

cudaError_t launch_batch_advance(const DevBatch& b, const DevQueues& q, cudaStream_t s) {
  fast::k_batch_advance<<<(b.n_jobs + 127) / 128, 128, 0, s>>>(b, q);
  return cudaGetLastError();
}
}  // namespace ct
