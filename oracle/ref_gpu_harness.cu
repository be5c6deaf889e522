// ref_gpu_harness.cu - frames of the REFERENCE tracer's own GPU path.
//
// TEST INFRASTRUCTURE ONLY (oracle). Compiled by oracle/ref_build.py
// (compile_gpu_lib) together with the reference's src/CUDA/Kernel.cu and
// src/Core/Camera.cpp from the patched copy in oracle/_ref/gpu/src, into
// oracle/_ref/libctref_gpu.so; used by tests/golden/make_ref_frame.py to record
// a golden frame and by oracle/ref_gpu_bench.py to time the reference's frame
// loop. Nothing in the product library links it.
//
// It fills the reference's Params and SceneData (src/CUDA/Kernel.cuh:23-72,
// src/Core/SceneData.cuh:18-45) the way Application::allocateTriangles and
// allocateBuffers do (src/Application.cpp:141-193), with a caller-given quad
// BVH (the reference's own MBVHTree nodes and primitive indices), places the
// camera as core::Camera does, and calls the reference's launchKernels
// (src/CUDA/Kernel.cu:355) from the first frame (samples 0). No sky and no
// textures: the reference's texture lookup reads outside its buffer for NaN
// coordinates. The caller must pass a tree whose quad depth keeps the
// traversal stack in bounds: 3 x depth + 1 <= 64 entries in the patched copy
// (32 in the reference as written).
#include <cstdint>
#include <cstring>
#include <vector>

#include "CUDA/Kernel.cuh"
#include "Core/Camera.h"

cudaError launchKernels(cudaArray_const_t array, Params& params, int rayBufferSize);

namespace {
template <typename T>
bool upload(T** dst, const void* src, size_t bytes) {
  if (cudaMalloc((void**)dst, bytes ? bytes : 16) != cudaSuccess) return false;
  if (bytes && src) return cudaMemcpy(*dst, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
  return cudaMemset(*dst, 0, bytes ? bytes : 16) == cudaSuccess;
}
}  // namespace

namespace {
// Params and SceneData filled the way Application::allocateTriangles and
// allocateBuffers do; false when an allocation or copy failed.
bool setup(Params& params, const float* verts, int nv, const float* normals, const float* center_normals,
           const float* uvs, const uint32_t* idx, int nt, const uint32_t* mat_idx, const void* materials, int nmat,
           const uint32_t* lights, int nlights, const void* mbvh_nodes, int n_nodes, const uint32_t* prim_idx,
           int nprims, int W, int H, float normal_eps, float dist_eps, float tri_eps, int shadow, int indirect) {
  SceneData& s = params.gpuScene;
  bool ok = true;
  ok &= upload(&s.vertices, verts, (size_t)nv * sizeof(vec3));
  ok &= upload(&s.normals, normals, (size_t)nv * sizeof(vec3));
  ok &= upload(&s.centerNormals, center_normals, (size_t)nt * sizeof(vec3));
  ok &= upload(&s.texCoords, uvs, (size_t)nv * sizeof(vec2));
  ok &= upload(&s.indices, idx, (size_t)nt * sizeof(uvec3));
  ok &= upload(&s.gpuMatIdxs, mat_idx, (size_t)nt * sizeof(unsigned int));
  ok &= upload(&s.gpuMaterials, materials, (size_t)nmat * sizeof(Material));
  ok &= upload(&s.lightIndices, lights, (size_t)nlights * sizeof(unsigned int));
  ok &= upload(&s.gpuMbvhNodes, mbvh_nodes, (size_t)n_nodes * sizeof(MBVHNode));
  ok &= upload(&s.gpuPrimIndices, prim_idx, (size_t)nprims * sizeof(unsigned int));
  ok &= upload(&s.currentFrame, nullptr, (size_t)W * H * sizeof(vec4));
  ok &= upload(&params.gpuRays, nullptr, (size_t)W * H * sizeof(Ray));
  ok &= upload(&params.gpuNextRays, nullptr, (size_t)W * H * sizeof(Ray));
  ok &= upload(&params.gpuShadowRays, nullptr, (size_t)W * H * sizeof(ShadowRay));
  s.lightCount = (unsigned int)nlights;
  s.skyboxEnabled = false;
  s.skyboxTexture = -1;
  s.shadow = shadow != 0;
  s.indirect = indirect != 0;
  s.normalEpsilon = normal_eps;
  s.distEpsilon = dist_eps;
  s.triangleEpsilon = tri_eps;
  return ok;
}
}  // namespace

// One frame (samples 0) into accum_out (W * H float4).
extern "C" int ctref_gpu_frame(const float* verts, int nv, const float* normals, const float* center_normals,
                               const float* uvs, const uint32_t* idx, int nt, const uint32_t* mat_idx,
                               const void* materials, int nmat, const uint32_t* lights, int nlights,
                               const void* mbvh_nodes, int n_nodes, const uint32_t* prim_idx, int nprims,
                               const float* cam_pos, const float* cam_fwd, const float* cam_up, float fov, int W,
                               int H, float normal_eps, float dist_eps, float tri_eps, int shadow, int indirect,
                               float* accum_out) {
  Params params(W, H);
  if (!setup(params, verts, nv, normals, center_normals, uvs, idx, nt, mat_idx, materials, nmat, lights, nlights,
             mbvh_nodes, n_nodes, prim_idx, nprims, W, H, normal_eps, dist_eps, tri_eps, shadow, indirect))
    return 1;
  core::Camera cam(W, H, fov, ROTATION_SPEED, glm::vec3(cam_pos[0], cam_pos[1], cam_pos[2]));
  cam.m_Forward = glm::vec3(cam_fwd[0], cam_fwd[1], cam_fwd[2]);
  cam.m_Up = glm::vec3(cam_up[0], cam_up[1], cam_up[2]);
  params.camera = &cam;
  params.samples = 0;
  cudaError err = launchKernels(nullptr, params, W * H);
  if (err == cudaSuccess) err = cudaDeviceSynchronize();
  if (err == cudaSuccess)
    err = cudaMemcpy(accum_out, params.gpuScene.currentFrame, (size_t)W * H * sizeof(vec4), cudaMemcpyDeviceToHost);
  params.deallocate();
  return err == cudaSuccess ? 0 : 2;
}

// The reference's own frame loop timed: one untimed frame, then `frames` calls
// of launchKernels (each one 1-spp frame, as Application::run issues them)
// between two CUDA events; *ms_out = the elapsed time, accum_out (may be null)
// = the accumulation after all frames.
extern "C" int ctref_gpu_time(const float* verts, int nv, const float* normals, const float* center_normals,
                              const float* uvs, const uint32_t* idx, int nt, const uint32_t* mat_idx,
                              const void* materials, int nmat, const uint32_t* lights, int nlights,
                              const void* mbvh_nodes, int n_nodes, const uint32_t* prim_idx, int nprims,
                              const float* cam_pos, const float* cam_fwd, const float* cam_up, float fov, int W,
                              int H, float normal_eps, float dist_eps, float tri_eps, int shadow, int indirect,
                              int frames, float* ms_out, float* accum_out) {
  Params params(W, H);
  if (!setup(params, verts, nv, normals, center_normals, uvs, idx, nt, mat_idx, materials, nmat, lights, nlights,
             mbvh_nodes, n_nodes, prim_idx, nprims, W, H, normal_eps, dist_eps, tri_eps, shadow, indirect))
    return 1;
  core::Camera cam(W, H, fov, ROTATION_SPEED, glm::vec3(cam_pos[0], cam_pos[1], cam_pos[2]));
  cam.m_Forward = glm::vec3(cam_fwd[0], cam_fwd[1], cam_fwd[2]);
  cam.m_Up = glm::vec3(cam_up[0], cam_up[1], cam_up[2]);
  params.camera = &cam;
  params.samples = 0;
  cudaError err = launchKernels(nullptr, params, W * H);
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (err == cudaSuccess) err = cudaDeviceSynchronize();
  if (err == cudaSuccess) err = cudaEventCreate(&e0);
  if (err == cudaSuccess) err = cudaEventCreate(&e1);
  if (err == cudaSuccess) err = cudaEventRecord(e0);
  for (int f = 0; f < frames && err == cudaSuccess; f++) err = launchKernels(nullptr, params, W * H);
  if (err == cudaSuccess) err = cudaEventRecord(e1);
  if (err == cudaSuccess) err = cudaEventSynchronize(e1);
  if (err == cudaSuccess) err = cudaEventElapsedTime(ms_out, e0, e1);
  if (err == cudaSuccess && accum_out)
    err = cudaMemcpy(accum_out, params.gpuScene.currentFrame, (size_t)W * H * sizeof(vec4), cudaMemcpyDeviceToHost);
  if (e0) cudaEventDestroy(e0);
  if (e1) cudaEventDestroy(e1);
  params.deallocate();
  return err == cudaSuccess ? 0 : 2;
}
