// C-ABI host runtime: contexts, scenes, BVHs, ray queries and render jobs.
// Compiled with -ffp-contract=off so the camera basis matches the reference's
// host arithmetic (src/CUDA/Kernel.cu:274-290, src/Core/Camera.cpp:11-16).
#include "../../include/cudatracer.h"

#include <cuda_runtime.h>

#include <atomic>
#include <chrono>
#include <cmath>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <new>
#include <vector>

#include "bvh_build.h"
#include "ct_internal.h"

using namespace ct;

struct ct_ctx {
  int device = 0;
  mutable std::mutex mu;
  std::string err;
  uint64_t budget = 0;
  std::atomic<uint64_t> bytes{0};
  uint32_t* d_error = nullptr;  // device error word
  int* d_cursor = nullptr;      // ray-query fetch cursor and record count (inside the same allocation)
  // settlement records of wide-tree queries (kWideRecordBytes per ray), grown on demand
  void* d_recs = nullptr;
  size_t recs_bytes = 0;
};

namespace {

struct Allocs {
  std::vector<std::pair<void*, size_t>> list;
};

ct_status fail(ct_ctx* ctx, ct_status s, const std::string& msg) {
  if (ctx) {
    std::lock_guard<std::mutex> g(ctx->mu);
    ctx->err = msg;
  }
  return s;
}

ct_status cuda_fail(ct_ctx* ctx, cudaError_t e, const char* what) {
  return fail(ctx, e == cudaErrorMemoryAllocation ? CT_ERR_OUT_OF_MEMORY : CT_ERR_CUDA,
              std::string(what) + ": " + cudaGetErrorString(e));
}

#define CT_CUDA(ctx, call)                                  \
  do {                                                      \
    cudaError_t e_ = (call);                                \
    if (e_ != cudaSuccess) return cuda_fail(ctx, e_, #call); \
  } while (0)

ct_status dev_alloc(ct_ctx* ctx, Allocs& a, void** p, size_t bytes) {
  *p = nullptr;
  if (bytes == 0) bytes = 16;
  bytes = (bytes + 255) & ~(size_t)255;
  if (ctx->budget && ctx->bytes.load() + bytes > ctx->budget)
    return fail(ctx, CT_ERR_OUT_OF_MEMORY,
                "device memory budget exceeded: " + std::to_string(ctx->bytes.load() + bytes) + " > " +
                    std::to_string(ctx->budget) + " bytes");
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    cudaGetLastError();
    *p = nullptr;
    return cuda_fail(ctx, e, "cudaMalloc");
  }
  ctx->bytes += bytes;
  a.list.push_back({*p, bytes});
  return CT_OK;
}

void free_all(ct_ctx* ctx, Allocs& a) {
  for (auto& p : a.list) {
    cudaFree(p.first);
    ctx->bytes -= p.second;
  }
  a.list.clear();
}

template <typename T>
ct_status upload(ct_ctx* ctx, Allocs& a, T** dst, const void* src, size_t bytes) {
  void* p = nullptr;
  ct_status s = dev_alloc(ctx, a, &p, bytes);
  if (s != CT_OK) return s;
  if (bytes && src) {
    cudaError_t e = cudaMemcpy(p, src, bytes, cudaMemcpyHostToDevice);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemcpy");
  } else if (bytes) {
    cudaError_t e = cudaMemset(p, 0, bytes);
    if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaMemset");
  }
  // Both calls can return before the device has finished, and they are ordered
  // only on the legacy stream: wait, so that work the caller (or a frame slot)
  // issues on a non-blocking stream never sees the buffer before it is filled.
  cudaError_t e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaStreamSynchronize");
  *dst = (T*)p;
  return CT_OK;
}

bool finite3(const float* p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

float bits_as_float(uint32_t u) {
  float f;
  std::memcpy(&f, &u, sizeof(f));
  return f;
}

}  // namespace

struct ct_scene {
  uint32_t nv = 0, nt = 0;
  std::vector<float> verts;    // 3 per vertex (host copy for BVH builds)
  std::vector<uint32_t> idx;   // 3 per triangle
  std::vector<ct_material> mats;
  DevScene dev{};
  DevMaterial* d_mats = nullptr;
  Allocs allocs;
};

struct ct_bvh {
  HostBVH host;
  DeviceLayout layout;
  DevBVH dev{};
  ct_bvh_info info{};
  uint32_t nt = 0;
  Allocs allocs;
  // device-built trees keep the reference-layout quad nodes and the primitive
  // order on the device only (exported on request)
  bool device_built = false;
  int device = 0;
  void* d_quad = nullptr;
  uint32_t* d_prims = nullptr;
  // 8-wide quantised tree (ct_bvh_build_wide): queries only
  bool wide = false;
  DevWBVH wdev{};
  unsigned long long* d_wstats = nullptr;  // rays, FP64 re-tests, full FP64 traversals
};

// Fast-math frames in flight at once, each in its own queue set and
// accumulation buffer: the last, nearly empty bounces of one frame overlap
// the first passes of the next ones (measured on the 1080p terrain frame with
// the first kernels: 2 slots 600, 4 slots 710, 6 slots 736, 8 slots 744
// Msamples/s; with the current ones, 64-thread blocks: 6 slots 973, 8 slots
// 991, 10 slots 997, 12 slots 995).
constexpr int kFrameSlots = 10;
// Exact-math frames overlap in up to kExactSlots of those slots, each frame
// logging its per-pixel contributions (DevQueues::log: 2 x max_depth entries of
// 16 bytes per pixel) for an in-order replay; the logs of a job may take up to
// kExactLogBytes, beyond which exact frames run one after another (1080p,
// depth 8, 531 MB of log per slot: 2 slots 631, 4 slots 768, 6 slots 800, 8
// slots 805 Msamples/s).
constexpr int kExactSlots = 6;
constexpr size_t kExactLogBytes = (size_t)4 << 30;

struct ct_render {
  int32_t w = 0, h = 0;
  DevQueues q{};
  Allocs allocs;
  // overlapped fast-math frames: private queue sets + accumulation buffers
  struct Slot {
    DevQueues q{};
    cudaStream_t stream = nullptr;
    cudaEvent_t free_ev = nullptr;  // recorded after the slot's buffer was folded
    cudaEvent_t done_ev = nullptr;  // recorded after the slot's frame finished
  } slots[kFrameSlots];
  int next_slot = 0;
  // overlapped exact-math frames: one contribution log per exact slot
  float4* logs[kExactSlots] = {};
  int log_entries = 0;  // entries per pixel the logs hold (2 x max_depth)
  int exact_slots = 0;  // slots with a log
  int next_exact = 0;
  uint32_t log_tag = 0;  // tag of the last exact frame issued into a slot
  Allocs log_allocs;
  // stage profiling: event pairs per stage, recycled through a pool
  bool profile = false;
  std::vector<std::pair<cudaEvent_t, cudaEvent_t>> marks[4];
  std::vector<cudaEvent_t> pool;
  cudaEvent_t take() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
  void recycle() {
    for (auto& m : marks)
      for (auto& p : m) pool.push_back(p.first), pool.push_back(p.second);
    for (auto& m : marks) m.clear();
  }
  ~ct_render() {
    recycle();
    for (cudaEvent_t e : pool) cudaEventDestroy(e);
  }
};

namespace {
// Bracket one stage launch with events when profiling is on.
template <typename F>
cudaError_t staged(ct_render* r, int stage, cudaStream_t st, F&& launch) {
  if (!r->profile) return launch();
  cudaEvent_t a = r->take(), b = r->take();
  cudaEventRecord(a, st);
  cudaError_t e = launch();
  cudaEventRecord(b, st);
  r->marks[stage].push_back({a, b});
  return e;
}
}  // namespace

namespace {

DevMaterial to_dev(const ct_material& m) {
  DevMaterial d;
  d.albedo_ior = make_float4(m.albedo[0], m.albedo[1], m.albedo[2], m.refract_idx);
  d.tex = make_int4(m.diffuse_tex, m.normal_tex, m.mask_tex, m.displace_tex);
  float type_bits;
  std::memcpy(&type_bits, &m.type, 4);
  d.type_rough = make_float4(type_bits, m.roughness, 0.0f, 0.0f);
  d.absorption = make_float4(m.absorption[0], m.absorption[1], m.absorption[2], 0.0f);
  return d;
}

// Frame constants of one job: core::Camera's basis and plane distance
// (Camera constructor, m_PlaneDistance = tanf(radians(fov * 0.5f)),
// src/Core/Camera.cpp:11-16) and sample()'s u = normalize(cross(w, up)),
// v = normalize(cross(u, w)) with the aspect ratio on the longer axis
// (src/CUDA/Kernel.cu:274-290), plus the flags and epsilons of Params. Every
// frame entry point (frames, the allocation-free frame, batches, serving)
// derives its constants here, so they agree bit for bit.
FrameConst frame_const(const ct_camera* cam, const ct_render_params* p) {
  const float dist = tanf((cam->fov_deg * 0.5f) * 0.01745329251994329576923690768489f);
  const float* w = cam->forward;
  const float* up = cam->up;
  float u[3] = {w[1] * up[2] - up[1] * w[2], w[2] * up[0] - up[2] * w[0], w[0] * up[1] - up[0] * w[1]};
  float inv = 1.0f / std::sqrt((u[0] * u[0] + u[1] * u[1]) + u[2] * u[2]);
  u[0] *= inv, u[1] *= inv, u[2] *= inv;
  float v[3] = {u[1] * w[2] - w[1] * u[2], u[2] * w[0] - w[2] * u[0], u[0] * w[1] - w[0] * u[1]};
  inv = 1.0f / std::sqrt((v[0] * v[0] + v[1] * v[1]) + v[2] * v[2]);
  v[0] *= inv, v[1] *= inv, v[2] *= inv;
  float hor[3] = {u[0] * dist, u[1] * dist, u[2] * dist};
  float ver[3] = {v[0] * dist, v[1] * dist, v[2] * dist};
  const float aspect = (float)p->width / (float)p->height;
  if (p->width > p->height)
    hor[0] *= aspect, hor[1] *= aspect, hor[2] *= aspect;
  else
    ver[0] *= aspect, ver[1] *= aspect, ver[2] *= aspect;
  FrameConst f;
  f.cam_pos = make_float3(cam->position[0], cam->position[1], cam->position[2]);
  f.cam_w = make_float3(w[0], w[1], w[2]);
  f.hor = make_float3(hor[0], hor[1], hor[2]);
  f.ver = make_float3(ver[0], ver[1], ver[2]);
  f.width = p->width;
  f.height = p->height;
  f.frame = p->frame_index;
  f.normal_eps = p->normal_eps;
  f.dist_eps = p->dist_eps;
  f.tri_eps = p->tri_eps;
  f.shadow = p->shadow;
  f.indirect = p->indirect;
  f.sky = p->sky;
  f.shading_mode = p->shading_mode;
  f.tex_filter = p->texture_filter;
  return f;
}

ct_status set_device(ct_ctx* ctx) {
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e != cudaSuccess) return cuda_fail(ctx, e, "cudaSetDevice");
  return CT_OK;
}

ct_status finish_bvh(ct_ctx* ctx, const ct_scene* scene, ct_bvh* b) {
  const auto t0 = std::chrono::high_resolution_clock::now();
  std::string err = to_device_layout(b->host, scene->verts.data(), scene->idx.data(), scene->nt, b->layout);
  if (!err.empty()) return fail(ctx, CT_ERR_UNSUPPORTED, err);
  ct_status s;
  QNodeDev* nodes = nullptr;
  float4* tris = nullptr;
  if ((s = upload(ctx, b->allocs, &nodes, b->layout.nodes.data(), b->layout.nodes.size())) != CT_OK) return s;
  if ((s = upload(ctx, b->allocs, &tris, b->layout.tris.data(), b->layout.tris.size() * 4)) != CT_OK) return s;
  b->dev.nodes = nodes;
  b->dev.tris = tris;
  b->dev.leaf_shift = b->layout.leaf_shift;
  b->dev.first_mask = b->layout.first_mask;
  b->dev.count_mask = b->layout.count_mask;
  b->dev.prim_count = (uint32_t)b->host.prims.size();
  b->dev.node_count = (uint32_t)b->host.quad.size();
  b->dev.stack_entries = b->layout.stack_entries;
  b->nt = scene->nt;
  const auto t1 = std::chrono::high_resolution_clock::now();
  ct_bvh_info& i = b->info;
  i.binary_node_count = (uint32_t)b->host.bin.size();
  i.quad_node_count = (uint32_t)b->host.quad.size();
  i.prim_count = (uint32_t)b->host.prims.size();
  i.max_leaf_size = b->layout.max_leaf;
  i.quad_depth = b->layout.depth;
  i.stack_entries = (uint32_t)b->layout.stack_entries;
  i.build_ms = b->host.build_ms;
  i.collapse_ms = b->host.collapse_ms;
  i.upload_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  uint64_t bytes = 0;
  for (auto& p : b->allocs.list) bytes += p.second;
  i.device_bytes = bytes;
  return CT_OK;
}

}  // namespace

extern "C" {

uint32_t ct_abi_version(void) { return CT_ABI_VERSION; }

void ct_render_params_default(ct_render_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->width = 0;
  p->height = 0;
  p->max_depth = 5;  // maxPathLength, src/CUDA/Kernel.cu:320
  p->frame_index = 0;
  p->shading_mode = CT_SHADE_COMPAT;
  p->exact_math = 0;
  p->shadow = 1;
  p->indirect = 1;
  p->sky = 1;
  p->normal_eps = 1e-5f;  // SceneData defaults, src/Core/SceneData.cuh:43-45
  p->dist_eps = 1e-5f;
  p->tri_eps = 1e-3f;
}

ct_status ct_ctx_create(int32_t device, ct_ctx** out) {
  if (!out) return CT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return CT_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) return CT_ERR_INVALID_ARGUMENT;
  if (cudaSetDevice(device) != cudaSuccess) return CT_ERR_NO_DEVICE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return CT_ERR_NO_DEVICE;
  if (prop.major * 10 + prop.minor < 100) return CT_ERR_NO_DEVICE;  // built for sm_103a only
  auto* c = new ct_ctx();
  c->device = device;
  if (cudaMalloc(&c->d_error, 256) != cudaSuccess || cudaMemset(c->d_error, 0, 256) != cudaSuccess ||
      cudaStreamSynchronize(0) != cudaSuccess) {
    delete c;
    return CT_ERR_OUT_OF_MEMORY;
  }
  c->d_cursor = (int*)(c->d_error + 32);  *out = c;
  return CT_OK;
}

ct_status ct_ctx_destroy(ct_ctx* ctx) {
  if (!ctx) return CT_ERR_INVALID_ARGUMENT;
  cudaSetDevice(ctx->device);
  cudaFree(ctx->d_error);
  if (ctx->d_recs) cudaFree(ctx->d_recs);
  delete ctx;
  return CT_OK;
}

const char* ct_last_error(const ct_ctx* ctx) {
  if (!ctx) return "null context";
  std::lock_guard<std::mutex> g(ctx->mu);
  thread_local std::string copy;
  copy = ctx->err;
  return copy.c_str();
}

ct_status ct_ctx_set_memory_budget(ct_ctx* ctx, uint64_t bytes) {
  if (!ctx) return CT_ERR_INVALID_ARGUMENT;
  ctx->budget = bytes;
  return CT_OK;
}

uint64_t ct_ctx_device_bytes(const ct_ctx* ctx) { return ctx ? ctx->bytes.load() : 0; }

ct_status ct_ctx_check(ct_ctx* ctx, void* stream) {
  if (!ctx) return CT_ERR_INVALID_ARGUMENT;
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  CT_CUDA(ctx, cudaStreamSynchronize((cudaStream_t)stream));
  uint32_t err = 0;
  CT_CUDA(ctx, cudaMemcpy(&err, ctx->d_error, 4, cudaMemcpyDeviceToHost));
  if (err) {
    CT_CUDA(ctx, cudaMemset(ctx->d_error, 0, 4));
    CT_CUDA(ctx, cudaStreamSynchronize(0));
    if (err & kErrStackOverflow)
      return fail(ctx, CT_ERR_STACK_OVERFLOW, "a traversal stack limit was reached; affected rays report no hit");
    return fail(ctx, CT_ERR_CUDA, "device error word " + std::to_string(err));
  }
  return CT_OK;
}

ct_status ct_scene_create(ct_ctx* ctx, const ct_scene_desc* d, ct_scene** out) {
  if (!ctx || !d || !out) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (!d->vertices || !d->normals || !d->indices) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "vertices, normals and indices are required");
  if (d->triangle_count == 0 || d->vertex_count == 0) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "empty scene");
  if (!d->materials || d->material_count == 0) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "at least one material is required");
  if (d->triangle_count >= (1u << 30)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "too many triangles");
  const uint32_t nv = d->vertex_count, nt = d->triangle_count;
  for (uint32_t i = 0; i < nv; i++)
    if (!finite3(d->vertices + 3 * (size_t)i)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "non-finite vertex " + std::to_string(i));
  for (uint64_t i = 0; i < 3ull * nt; i++)
    if (d->indices[i] >= nv) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "vertex index out of range in triangle " + std::to_string(i / 3));
  if (d->material_indices)
    for (uint32_t i = 0; i < nt; i++)
      if (d->material_indices[i] >= d->material_count)
        return fail(ctx, CT_ERR_INVALID_ARGUMENT, "material index out of range in triangle " + std::to_string(i));
  if (d->light_count && !d->light_indices) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "light_count without light_indices");
  if (d->light_count > nt) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "more lights than triangles");
  for (uint32_t i = 0; i < d->light_count; i++)
    if (d->light_indices[i] >= nt) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "light index out of range");
  if (d->texture_count && (!d->texture_dims || !d->texture_offsets || !d->texels))
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "texture arrays missing");
  for (uint32_t i = 0; i < d->texture_count; i++) {
    const uint64_t w = d->texture_dims[2 * i], h = d->texture_dims[2 * i + 1];
    if (w == 0 || h == 0 || (uint64_t)d->texture_offsets[i] + w * h > d->texel_count)
      return fail(ctx, CT_ERR_INVALID_ARGUMENT, "texture " + std::to_string(i) + " exceeds the texel array");
  }
  auto tex_ok = [&](int32_t t) { return t < 0 || (uint32_t)t < d->texture_count; };
  if (!tex_ok(d->skybox_texture)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "skybox texture out of range");
  for (uint32_t i = 0; i < d->material_count; i++) {
    const ct_material& m = d->materials[i];
    if (!tex_ok(m.diffuse_tex) || !tex_ok(m.normal_tex)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "material texture out of range");
    if (m.type < 0 || m.type > CT_MAT_FRESNEL_TROWBRIDGE) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown material type");
  }
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  auto* sc = new ct_scene();
  sc->nv = nv;
  sc->nt = nt;
  sc->verts.assign(d->vertices, d->vertices + 3 * (size_t)nv);
  sc->idx.assign(d->indices, d->indices + 3 * (size_t)nt);
  sc->mats.assign(d->materials, d->materials + d->material_count);
  std::vector<float4> v4(nv), n4(nv), cn(nt);
  std::vector<float2> uv(nv, make_float2(0.0f, 0.0f));
  std::vector<uint4> i4(nt);
  for (uint32_t i = 0; i < nv; i++) {
    const float* p = d->vertices + 3 * (size_t)i;
    const float* n = d->normals + 3 * (size_t)i;
    v4[i] = make_float4(p[0], p[1], p[2], 0.0f);
    n4[i] = make_float4(n[0], n[1], n[2], 0.0f);
    if (d->texcoords) uv[i] = make_float2(d->texcoords[2 * (size_t)i], d->texcoords[2 * (size_t)i + 1]);
  }
  for (uint32_t i = 0; i < nt; i++) {
    const uint32_t* t = d->indices + 3 * (size_t)i;
    i4[i] = make_uint4(t[0], t[1], t[2], d->material_indices ? d->material_indices[i] : 0u);
    if (d->center_normals) {
      const float* c = d->center_normals + 3 * (size_t)i;
      cn[i] = make_float4(c[0], c[1], c[2], 0.0f);
    } else {
      // (n0 + n1 + n2) / 3.0f, TriangleList.cpp:140
      const float* a = d->normals + 3 * (size_t)t[0];
      const float* b = d->normals + 3 * (size_t)t[1];
      const float* c = d->normals + 3 * (size_t)t[2];
      cn[i] = make_float4(((a[0] + b[0]) + c[0]) / 3.0f, ((a[1] + b[1]) + c[1]) / 3.0f, ((a[2] + b[2]) + c[2]) / 3.0f,
                          0.0f);
    }
  }
  std::vector<float4> rec((size_t)nt * 8);
  for (uint32_t i = 0; i < nt; i++) {
    const uint4 t = i4[i];
    float4* r = rec.data() + 8 * (size_t)i;
    r[0] = make_float4(v4[t.x].x, v4[t.x].y, v4[t.x].z, bits_as_float(t.w));
    r[1] = make_float4(v4[t.y].x, v4[t.y].y, v4[t.y].z, 0.0f);
    r[2] = make_float4(v4[t.z].x, v4[t.z].y, v4[t.z].z, 0.0f);
    r[3] = make_float4(n4[t.x].x, n4[t.x].y, n4[t.x].z, uv[t.x].x);
    r[4] = make_float4(n4[t.y].x, n4[t.y].y, n4[t.y].z, uv[t.x].y);
    r[5] = make_float4(n4[t.z].x, n4[t.z].y, n4[t.z].z, uv[t.y].x);
    r[6] = make_float4(cn[i].x, cn[i].y, cn[i].z, uv[t.y].y);
    r[7] = make_float4(uv[t.z].x, uv[t.z].y, 0.0f, 0.0f);
  }
  std::vector<DevMaterial> dm(d->material_count);
  for (uint32_t i = 0; i < d->material_count; i++) dm[i] = to_dev(d->materials[i]);
  std::vector<uint2> dims(d->texture_count);
  for (uint32_t i = 0; i < d->texture_count; i++) dims[i] = make_uint2(d->texture_dims[2 * i], d->texture_dims[2 * i + 1]);
  DevScene& ds = sc->dev;
  float4 *dv = nullptr, *dn = nullptr, *dc = nullptr, *dt = nullptr, *drec = nullptr;
  float2* duv = nullptr;
  uint4* di = nullptr;
  uint32_t *dl = nullptr, *doff = nullptr;
  uint2* ddim = nullptr;
  if ((s = upload(ctx, sc->allocs, &dv, v4.data(), v4.size() * sizeof(float4))) != CT_OK ||
      (s = upload(ctx, sc->allocs, &dn, n4.data(), n4.size() * sizeof(float4))) != CT_OK ||
      (s = upload(ctx, sc->allocs, &duv, uv.data(), uv.size() * sizeof(float2))) != CT_OK ||
      (s = upload(ctx, sc->allocs, &di, i4.data(), i4.size() * sizeof(uint4))) != CT_OK ||
      (s = upload(ctx, sc->allocs, &dc, cn.data(), cn.size() * sizeof(float4))) != CT_OK ||
      (s = upload(ctx, sc->allocs, &drec, rec.data(), rec.size() * sizeof(float4))) != CT_OK ||
      (s = upload(ctx, sc->allocs, &sc->d_mats, dm.data(), dm.size() * sizeof(DevMaterial))) != CT_OK ||
      (s = upload(ctx, sc->allocs, &dl, d->light_indices, (size_t)d->light_count * 4)) != CT_OK ||
      (s = upload(ctx, sc->allocs, &dt, d->texels, (size_t)d->texel_count * sizeof(float4))) != CT_OK ||
      (s = upload(ctx, sc->allocs, &ddim, dims.data(), dims.size() * sizeof(uint2))) != CT_OK ||
      (s = upload(ctx, sc->allocs, &doff, d->texture_offsets, (size_t)d->texture_count * 4)) != CT_OK) {
    free_all(ctx, sc->allocs);
    delete sc;
    return s;
  }
  ds.verts = dv;
  ds.normals = dn;
  ds.uvs = duv;
  ds.idx = di;
  ds.cnormals = dc;
  ds.shade_rec = drec;
  ds.mats = sc->d_mats;
  ds.lights = dl;
  ds.light_count = d->light_count;
  ds.tri_count = nt;
  ds.texels = dt;
  ds.tex_dims = ddim;
  ds.tex_offsets = doff;
  ds.sky_tex = d->skybox_texture;
  ds.tex_count = d->texture_count;
  *out = sc;
  return CT_OK;
}

ct_status ct_scene_destroy(ct_ctx* ctx, ct_scene* scene) {
  if (!ctx || !scene) return CT_ERR_INVALID_ARGUMENT;
  set_device(ctx);
  free_all(ctx, scene->allocs);
  delete scene;
  return CT_OK;
}

ct_status ct_scene_set_material(ct_ctx* ctx, ct_scene* scene, uint32_t index, const ct_material* m) {
  if (!ctx || !scene || !m) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  if (index >= scene->mats.size()) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "material index out of range");
  if (m->type < 0 || m->type > CT_MAT_FRESNEL_TROWBRIDGE) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown material type");
  auto tex_ok = [&](int32_t t) { return t < 0 || (uint32_t)t < scene->dev.tex_count; };
  if (!tex_ok(m->diffuse_tex) || !tex_ok(m->normal_tex)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "material texture out of range");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  scene->mats[index] = *m;
  const DevMaterial dm = to_dev(*m);
  CT_CUDA(ctx, cudaMemcpy(scene->d_mats + index, &dm, sizeof(dm), cudaMemcpyHostToDevice));
  CT_CUDA(ctx, cudaStreamSynchronize(0));  // the copy may still be in flight when cudaMemcpy returns
  return CT_OK;
}

ct_status ct_bvh_build(ct_ctx* ctx, const ct_scene* scene, int32_t nthreads, ct_bvh** out) {
  if (!ctx || !scene || !out) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  auto* b = new ct_bvh();
  try {
    build_binary(scene->verts.data(), scene->idx.data(), scene->nt, nthreads, b->host);
    collapse_quad(b->host);
  } catch (const std::bad_alloc&) {
    delete b;
    return fail(ctx, CT_ERR_OUT_OF_MEMORY, "host allocation failed while building the BVH");
  }
  if ((s = finish_bvh(ctx, scene, b)) != CT_OK) {
    free_all(ctx, b->allocs);
    delete b;
    return s;
  }
  *out = b;
  return CT_OK;
}

ct_status ct_bvh_build_fast(ct_ctx* ctx, const ct_scene* scene, int32_t nthreads, ct_bvh** out) {
  if (!ctx || !scene || !out) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  auto* b = new ct_bvh();
  try {
    build_fast_quad(scene->verts.data(), scene->idx.data(), scene->nt, nthreads, b->host);
  } catch (const std::bad_alloc&) {
    delete b;
    return fail(ctx, CT_ERR_OUT_OF_MEMORY, "host allocation failed while building the BVH");
  }
  if ((s = finish_bvh(ctx, scene, b)) != CT_OK) {
    free_all(ctx, b->allocs);
    delete b;
    return s;
  }
  *out = b;
  return CT_OK;
}

}  // extern "C"

namespace {

// Device quad builds: the reference's SAH tree (fast = false, bvh_gpu.cu) or
// ct_bvh_build_fast's tree (fast = true, bvh_gpu_fast.cu).
ct_status build_device_quad(ct_ctx* ctx, const ct_scene* scene, void* stream, ct_bvh** out, bool fast) {
  if (!ctx || !scene || !out) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  const uint32_t n = scene->nt;
  if (n == 0 || n > (1u << 30)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "triangle count out of range for the device builder");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  const auto t0 = std::chrono::high_resolution_clock::now();
  Allocs scratch_allocs;
  void* scratch = nullptr;
  uint32_t* hc = nullptr;
  auto* b = new ct_bvh();
  auto cleanup = [&](ct_status r) {
    if (st) cudaStreamSynchronize(st);
    else cudaDeviceSynchronize();
    free_all(ctx, scratch_allocs);
    if (hc) cudaFreeHost(hc);
    if (r != CT_OK) {
      free_all(ctx, b->allocs);
      delete b;
    }
    return r;
  };
  const size_t scratch_bytes = fast ? gpu_fbvh_scratch_bytes(n) : gpu_bvh_scratch_bytes(n);
  if ((s = dev_alloc(ctx, scratch_allocs, &scratch, scratch_bytes)) != CT_OK) return cleanup(s);
  cudaError_t e = cudaMallocHost((void**)&hc, 64);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "cudaMallocHost"));
  GpuBvhResult r;
  e = fast ? gpu_fbvh_build(scene->dev, scratch, hc, st, r) : gpu_bvh_build(scene->dev, scratch, hc, st, r);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "device BVH build"));
  if ((r.error & 1u) && fast)
    return cleanup(fail(ctx, CT_ERR_UNSUPPORTED,
                        "device BVH build: a padded triangle box is not finite (coordinates near the float "
                        "range); use ct_bvh_build_fast"));
  if (r.error & 1u)
    return cleanup(fail(ctx, CT_ERR_UNSUPPORTED,
                        "device BVH build: scene extent too large for the SAH cost (area x count >= 1e34); "
                        "use ct_bvh_build"));
  if (r.error) return cleanup(fail(ctx, CT_ERR_CUDA, "device BVH build: internal check failed (code " +
                                                         std::to_string(r.error) + ")"));
  const auto t1 = std::chrono::high_resolution_clock::now();
  uint32_t shift = 0, fm = 0, cm = 0;
  const std::string enc = leaf_encoding(n, r.max_leaf, shift, fm, cm);
  if (!enc.empty()) return cleanup(fail(ctx, CT_ERR_UNSUPPORTED, enc));
  void* quad = nullptr;
  void* nodes = nullptr;
  void* tris = nullptr;
  void* prims = nullptr;
  if ((s = dev_alloc(ctx, b->allocs, &quad, (size_t)r.quad_nodes * sizeof(QuadNode))) != CT_OK) return cleanup(s);
  if ((s = dev_alloc(ctx, b->allocs, &nodes, (size_t)r.quad_nodes * sizeof(QNodeDev))) != CT_OK) return cleanup(s);
  if ((s = dev_alloc(ctx, b->allocs, &tris, (size_t)n * 3 * sizeof(float4))) != CT_OK) return cleanup(s);
  if ((s = dev_alloc(ctx, b->allocs, &prims, (size_t)n * 4)) != CT_OK) return cleanup(s);
  e = fast ? gpu_fbvh_emit(scene->dev, scratch, r, shift, quad, (QNodeDev*)nodes, (float4*)tris, (uint32_t*)prims, st)
           : gpu_bvh_emit(scene->dev, scratch, r, shift, quad, (QNodeDev*)nodes, (float4*)tris, (uint32_t*)prims, st);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "device BVH emit"));
  e = st ? cudaStreamSynchronize(st) : cudaDeviceSynchronize();
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "device BVH build"));
  if (fast) {
    const uint32_t werr = gpu_fbvh_error(scratch, n, hc, st);
    if (werr) return cleanup(fail(ctx, CT_ERR_CUDA, "device BVH emit: internal check failed (code " +
                                                        std::to_string(werr) + ")"));
  }
  const auto t2 = std::chrono::high_resolution_clock::now();
  b->device_built = true;
  b->device = ctx->device;
  b->d_quad = quad;
  b->d_prims = (uint32_t*)prims;
  b->dev.nodes = (const QNodeDev*)nodes;
  b->dev.tris = (const float4*)tris;
  b->dev.leaf_shift = shift;
  b->dev.first_mask = fm;
  b->dev.count_mask = cm;
  b->dev.prim_count = n;
  b->dev.node_count = r.quad_nodes;
  b->dev.stack_entries = (int32_t)std::min<uint32_t>(3 * r.depth + 1, 256);
  b->nt = n;
  ct_bvh_info& i = b->info;
  i.binary_node_count = fast ? 0u : r.binary_nodes;  // as ct_bvh_build_fast: a quad tree only
  i.quad_node_count = r.quad_nodes;
  i.prim_count = n;
  i.max_leaf_size = r.max_leaf;
  i.quad_depth = r.depth;
  i.stack_entries = (uint32_t)b->dev.stack_entries;
  i.build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  i.collapse_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
  i.upload_ms = 0.0;
  uint64_t bytes = 0;
  for (auto& p : b->allocs.list) bytes += p.second;
  i.device_bytes = bytes;
  *out = b;
  return cleanup(CT_OK);
}

}  // namespace

extern "C" {

ct_status ct_bvh_build_device(ct_ctx* ctx, const ct_scene* scene, void* stream, ct_bvh** out) {
  return build_device_quad(ctx, scene, stream, out, false);
}

ct_status ct_bvh_build_fast_device(ct_ctx* ctx, const ct_scene* scene, void* stream, ct_bvh** out) {
  return build_device_quad(ctx, scene, stream, out, true);
}

ct_status ct_bvh_build_wide(ct_ctx* ctx, const ct_scene* scene, void* stream, ct_bvh** out) {
  if (!ctx || !scene || !out) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  const uint32_t n = scene->nt;
  // traversal stack entries hold a leaf group's first triangle in 29 bits
  if (n == 0 || n > (1u << 29)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "triangle count out of range for the wide BVH");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  const auto t0 = std::chrono::high_resolution_clock::now();
  Allocs scratch_allocs;
  void* scratch = nullptr;
  void* scratch2 = nullptr;
  uint32_t* hc = nullptr;
  auto* b = new ct_bvh();
  auto cleanup = [&](ct_status r) {
    if (st) cudaStreamSynchronize(st);
    else cudaDeviceSynchronize();
    free_all(ctx, scratch_allocs);
    if (hc) cudaFreeHost(hc);
    if (r != CT_OK) {
      free_all(ctx, b->allocs);
      delete b;
    }
    return r;
  };
  // the binary tree of ct_bvh_build_fast's rules over exact triangle bounds, and
  // the cost table of the 8-wide collapse
  if ((s = dev_alloc(ctx, scratch_allocs, &scratch, gpu_fbvh_scratch_bytes(n, 1))) != CT_OK) return cleanup(s);
  cudaError_t e = cudaMallocHost((void**)&hc, 64);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "cudaMallocHost"));
  GpuBvhResult r;
  e = gpu_fbvh_build(scene->dev, scratch, hc, st, r, 1);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "device BVH build"));
  if (r.error & 1u)
    return cleanup(fail(ctx, CT_ERR_UNSUPPORTED,
                        "wide BVH build: a triangle box is not finite (coordinates near the float range)"));
  if (r.error) return cleanup(fail(ctx, CT_ERR_CUDA, "wide BVH build: internal check failed (code " +
                                                         std::to_string(r.error) + ")"));
  const void* barena = nullptr;
  const uint32_t* bprims = nullptr;
  const WideCost* wcost = nullptr;
  gpu_fbvh_binary(scratch, n, 1, &barena, &bprims, &wcost);
  const auto t1 = std::chrono::high_resolution_clock::now();
  void* tris = nullptr;
  void* stats = nullptr;
  if ((s = dev_alloc(ctx, b->allocs, &tris, (size_t)n * 3 * sizeof(float4))) != CT_OK) return cleanup(s);
  if ((s = upload(ctx, b->allocs, (unsigned long long**)&stats, nullptr, 4 * sizeof(unsigned long long))) != CT_OK)
    return cleanup(s);
  if ((s = dev_alloc(ctx, scratch_allocs, &scratch2, gpu_wbvh_scratch_bytes(r.binary_nodes))) != CT_OK)
    return cleanup(s);
  uint32_t nw = 0, depth = 0, werr = 0;
  e = gpu_wbvh_collapse(scene->dev, barena, bprims, wcost, scratch2, r.binary_nodes, (float4*)tris, hc, st, &nw, &depth,
                        &werr);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "wide BVH collapse"));
  if (werr) return cleanup(fail(ctx, CT_ERR_UNSUPPORTED, "wide BVH collapse failed (code " + std::to_string(werr) +
                                                              "): a leaf needs more than 8 slots or a box did not quantise"));
  void* nodes = nullptr;
  if ((s = dev_alloc(ctx, b->allocs, &nodes, (size_t)nw * sizeof(WNode8))) != CT_OK) return cleanup(s);
  e = gpu_wbvh_copy_nodes(scratch2, r.binary_nodes, (WNode8*)nodes, nw, st);
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "wide BVH copy"));
  e = st ? cudaStreamSynchronize(st) : cudaDeviceSynchronize();
  if (e != cudaSuccess) return cleanup(cuda_fail(ctx, e, "wide BVH build"));
  const auto t2 = std::chrono::high_resolution_clock::now();
  b->wide = true;
  b->device_built = true;
  b->device = ctx->device;
  b->wdev.nodes = (const WNode8*)nodes;
  b->wdev.tris = (const float4*)tris;
  b->wdev.node_count = nw;
  b->wdev.prim_count = n;
  b->wdev.depth = depth;
  b->wdev.stack_entries = (int32_t)(7 * depth + 1);
  b->d_wstats = (unsigned long long*)stats;
  b->nt = n;
  ct_bvh_info& i = b->info;
  i.binary_node_count = r.binary_nodes;
  i.quad_node_count = nw;
  i.prim_count = n;
  i.max_leaf_size = 3;
  i.quad_depth = depth;
  i.stack_entries = (uint32_t)b->wdev.stack_entries;
  i.build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  i.collapse_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
  i.upload_ms = 0.0;
  uint64_t bytes = 0;
  for (auto& p : b->allocs.list) bytes += p.second;
  i.device_bytes = bytes;
  *out = b;
  return cleanup(CT_OK);
}

ct_status ct_bvh_wide_stats(ct_ctx* ctx, const ct_bvh* bvh, uint64_t* rays, uint64_t* fp64_retests,
                            uint64_t* fp64_t_only, uint64_t* fp64_full, int32_t reset) {
  if (!ctx || !bvh || !bvh->wide) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "not a wide BVH");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  unsigned long long h[4] = {0, 0, 0, 0};
  CT_CUDA(ctx, cudaDeviceSynchronize());
  CT_CUDA(ctx, cudaMemcpy(h, bvh->d_wstats, sizeof(h), cudaMemcpyDeviceToHost));
  if (rays) *rays = h[0];
  if (fp64_retests) *fp64_retests = h[1];
  if (fp64_full) *fp64_full = h[2];
  if (fp64_t_only) *fp64_t_only = h[3];
  if (reset) {
    CT_CUDA(ctx, cudaMemset(bvh->d_wstats, 0, sizeof(h)));
    CT_CUDA(ctx, cudaStreamSynchronize(0));
  }
  return CT_OK;
}

ct_status ct_bvh_import_quad(ct_ctx* ctx, const ct_scene* scene, const void* nodes, uint32_t node_count,
                             const uint32_t* prim_indices, uint32_t prim_count, ct_bvh** out) {
  if (!ctx || !scene || !nodes || !prim_indices || !out) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (prim_count != scene->nt) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "prim_count differs from the scene's triangle count");
  for (uint32_t i = 0; i < prim_count; i++)
    if (prim_indices[i] >= scene->nt) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "primitive index out of range");
  auto* b = new ct_bvh();
  b->host.quad.resize(node_count);
  std::memcpy(b->host.quad.data(), nodes, (size_t)node_count * sizeof(QuadNode));
  b->host.prims.assign(prim_indices, prim_indices + prim_count);
  std::string err = validate_quad(b->host.quad, prim_count);
  ct_status s = err.empty() ? set_device(ctx) : fail(ctx, CT_ERR_INVALID_ARGUMENT, err);
  if (s == CT_OK) s = finish_bvh(ctx, scene, b);
  if (s != CT_OK) {
    free_all(ctx, b->allocs);
    delete b;
    return s;
  }
  *out = b;
  return CT_OK;
}

ct_status ct_bvh_import_binary(ct_ctx* ctx, const ct_scene* scene, const void* nodes, uint32_t node_count,
                               const uint32_t* prim_indices, uint32_t prim_count, ct_bvh** out) {
  if (!ctx || !scene || !nodes || !prim_indices || !out) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (prim_count != scene->nt) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "prim_count differs from the scene's triangle count");
  for (uint32_t i = 0; i < prim_count; i++)
    if (prim_indices[i] >= scene->nt) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "primitive index out of range");
  auto* b = new ct_bvh();
  b->host.bin.resize(node_count);
  std::memcpy(b->host.bin.data(), nodes, (size_t)node_count * sizeof(BinNode));
  b->host.prims.assign(prim_indices, prim_indices + prim_count);
  std::string err = validate_binary(b->host.bin, prim_count);
  ct_status s = err.empty() ? set_device(ctx) : fail(ctx, CT_ERR_INVALID_ARGUMENT, err);
  if (s == CT_OK) {
    collapse_quad(b->host);
    s = finish_bvh(ctx, scene, b);
  }
  if (s != CT_OK) {
    free_all(ctx, b->allocs);
    delete b;
    return s;
  }
  *out = b;
  return CT_OK;
}

ct_status ct_bvh_info_get(const ct_bvh* bvh, ct_bvh_info* info) {
  if (!bvh || !info) return CT_ERR_INVALID_ARGUMENT;
  *info = bvh->info;
  return CT_OK;
}

ct_status ct_bvh_export(const ct_bvh* bvh, ct_bvh_layout layout, void* nodes, uint32_t* prim_indices) {
  if (!bvh) return CT_ERR_INVALID_ARGUMENT;
  if (bvh->wide) {
    if (layout != CT_BVH_WIDE8_Q8) return nodes ? CT_ERR_UNSUPPORTED : CT_OK;
    if (cudaSetDevice(bvh->device) != cudaSuccess) return CT_ERR_CUDA;
    if (nodes && cudaMemcpy(nodes, bvh->wdev.nodes, (size_t)bvh->wdev.node_count * sizeof(WNode8),
                            cudaMemcpyDeviceToHost) != cudaSuccess)
      return CT_ERR_CUDA;
    if (prim_indices) {
      std::vector<float4> tri((size_t)bvh->nt * 3);
      if (cudaMemcpy(tri.data(), bvh->wdev.tris, tri.size() * sizeof(float4), cudaMemcpyDeviceToHost) != cudaSuccess)
        return CT_ERR_CUDA;
      for (uint32_t i = 0; i < bvh->nt; i++) std::memcpy(&prim_indices[i], &tri[3 * (size_t)i].w, 4);
    }
    return CT_OK;
  }
  if (layout == CT_BVH_WIDE8_Q8) return nodes ? CT_ERR_UNSUPPORTED : CT_OK;
  if (bvh->device_built) {
    if (layout == CT_BVH_BINARY) return nodes ? CT_ERR_UNSUPPORTED : CT_OK;
    if (layout != CT_BVH_QUAD) return CT_ERR_INVALID_ARGUMENT;
    if (cudaSetDevice(bvh->device) != cudaSuccess) return CT_ERR_CUDA;
    if (nodes && cudaMemcpy(nodes, bvh->d_quad, (size_t)bvh->info.quad_node_count * sizeof(QuadNode),
                            cudaMemcpyDeviceToHost) != cudaSuccess)
      return CT_ERR_CUDA;
    if (prim_indices &&
        cudaMemcpy(prim_indices, bvh->d_prims, (size_t)bvh->nt * 4, cudaMemcpyDeviceToHost) != cudaSuccess)
      return CT_ERR_CUDA;
    return CT_OK;
  }
  if (layout == CT_BVH_BINARY) {
    if (bvh->host.bin.empty() && nodes) return CT_ERR_UNSUPPORTED;
    if (nodes) std::memcpy(nodes, bvh->host.bin.data(), bvh->host.bin.size() * sizeof(BinNode));
  } else if (layout == CT_BVH_QUAD) {
    if (nodes) std::memcpy(nodes, bvh->host.quad.data(), bvh->host.quad.size() * sizeof(QuadNode));
  } else {
    return CT_ERR_INVALID_ARGUMENT;
  }
  if (prim_indices) std::memcpy(prim_indices, bvh->host.prims.data(), bvh->host.prims.size() * 4);
  return CT_OK;
}

ct_status ct_bvh_destroy(ct_ctx* ctx, ct_bvh* bvh) {
  if (!ctx || !bvh) return CT_ERR_INVALID_ARGUMENT;
  set_device(ctx);
  free_all(ctx, bvh->allocs);
  delete bvh;
  return CT_OK;
}

struct ct_host_bvh {
  HostBVH host;
};

ct_status ct_host_bvh_build(const float* vertices, uint32_t vertex_count, const uint32_t* indices,
                            uint32_t triangle_count, int32_t nthreads, ct_host_bvh** out) {
  if (!vertices || !indices || !out || triangle_count == 0 || vertex_count == 0) return CT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  for (uint32_t i = 0; i < vertex_count; i++)
    if (!finite3(vertices + 3 * (size_t)i)) return CT_ERR_INVALID_ARGUMENT;
  for (uint64_t i = 0; i < 3ull * triangle_count; i++)
    if (indices[i] >= vertex_count) return CT_ERR_INVALID_ARGUMENT;
  auto* h = new ct_host_bvh();
  try {
    build_binary(vertices, indices, triangle_count, nthreads, h->host);
    collapse_quad(h->host);
  } catch (const std::bad_alloc&) {
    delete h;
    return CT_ERR_OUT_OF_MEMORY;
  }
  *out = h;
  return CT_OK;
}

ct_status ct_host_bvh_build_fast(const float* vertices, uint32_t vertex_count, const uint32_t* indices,
                                 uint32_t triangle_count, int32_t nthreads, ct_host_bvh** out) {
  if (!vertices || !indices || !out || triangle_count == 0 || vertex_count == 0) return CT_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  for (uint32_t i = 0; i < vertex_count; i++)
    if (!finite3(vertices + 3 * (size_t)i)) return CT_ERR_INVALID_ARGUMENT;
  for (uint64_t i = 0; i < 3ull * triangle_count; i++)
    if (indices[i] >= vertex_count) return CT_ERR_INVALID_ARGUMENT;
  auto* h = new ct_host_bvh();
  try {
    build_fast_quad(vertices, indices, triangle_count, nthreads, h->host);
  } catch (const std::bad_alloc&) {
    delete h;
    return CT_ERR_OUT_OF_MEMORY;
  }
  *out = h;
  return CT_OK;
}

ct_status ct_host_bvh_counts(const ct_host_bvh* h, uint32_t* binary_nodes, uint32_t* quad_nodes, uint32_t* prims,
                             double* build_ms, double* collapse_ms) {
  if (!h) return CT_ERR_INVALID_ARGUMENT;
  if (binary_nodes) *binary_nodes = (uint32_t)h->host.bin.size();
  if (quad_nodes) *quad_nodes = (uint32_t)h->host.quad.size();
  if (prims) *prims = (uint32_t)h->host.prims.size();
  if (build_ms) *build_ms = h->host.build_ms;
  if (collapse_ms) *collapse_ms = h->host.collapse_ms;
  return CT_OK;
}

ct_status ct_host_bvh_export(const ct_host_bvh* h, ct_bvh_layout layout, void* nodes, uint32_t* prim_indices) {
  if (!h) return CT_ERR_INVALID_ARGUMENT;
  if (layout == CT_BVH_BINARY) {
    if (h->host.bin.empty() && nodes) return CT_ERR_UNSUPPORTED;
    if (nodes) std::memcpy(nodes, h->host.bin.data(), h->host.bin.size() * sizeof(BinNode));
  } else if (layout == CT_BVH_QUAD) {
    if (nodes) std::memcpy(nodes, h->host.quad.data(), h->host.quad.size() * sizeof(QuadNode));
  } else {
    return CT_ERR_INVALID_ARGUMENT;
  }
  if (prim_indices) std::memcpy(prim_indices, h->host.prims.data(), h->host.prims.size() * 4);
  return CT_OK;
}

ct_status ct_host_bvh_destroy(ct_host_bvh* h) {
  if (!h) return CT_ERR_INVALID_ARGUMENT;
  delete h;
  return CT_OK;
}

static ct_status check_rays(ct_ctx* ctx, const ct_bvh* bvh, const float* org, const float* dir, uint32_t n) {
  if (!ctx || !bvh) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  if (n && (!org || !dir)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null ray buffer");
  if (((uintptr_t)org | (uintptr_t)dir) & 15) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "ray buffers must be 16-byte aligned");
  return set_device(ctx);
}

// Settlement records for a wide-tree query of n rays: the context keeps one
// buffer and grows it (after the device has finished with the old one) when a
// query needs more; the bytes count against the context's budget.
static ct_status ensure_wide_records(ct_ctx* ctx, uint32_t n) {
  const size_t need = ((size_t)std::max<uint32_t>(n, 1) * kWideRecordBytes + 255) & ~(size_t)255;
  if (ctx->recs_bytes >= need) return CT_OK;
  if (ctx->budget && ctx->bytes.load() - ctx->recs_bytes + need > ctx->budget)
    return fail(ctx, CT_ERR_OUT_OF_MEMORY, "device memory budget exceeded by the wide-query records of " +
                                               std::to_string(n) + " rays");
  if (ctx->d_recs) {
    CT_CUDA(ctx, cudaDeviceSynchronize());
    cudaFree(ctx->d_recs);
    ctx->bytes -= ctx->recs_bytes;
    ctx->d_recs = nullptr, ctx->recs_bytes = 0;
  }
  cudaError_t e = cudaMalloc(&ctx->d_recs, need);
  if (e != cudaSuccess) {
    cudaGetLastError();
    ctx->d_recs = nullptr;
    return cuda_fail(ctx, e, "cudaMalloc (wide-query records)");
  }
  ctx->recs_bytes = need;
  ctx->bytes += need;
  return CT_OK;
}

ct_status ct_trace_closest(ct_ctx* ctx, const ct_bvh* bvh, const float* org, const float* dir, int32_t* hit, float* t,
                           uint32_t n, float tri_eps, void* stream) {
  ct_status s = check_rays(ctx, bvh, org, dir, n);
  if (s != CT_OK) return s;
  if (n && (!hit || !t)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null output buffer");
  if (bvh->wide) {
    if ((s = ensure_wide_records(ctx, n)) != CT_OK) return s;
    CT_CUDA(ctx, launch_trace_wide_closest(bvh->wdev, (const float4*)org, (const float4*)dir, hit, t, n, ctx->d_error,
                                           ctx->d_cursor, ctx->d_recs, bvh->d_wstats, (cudaStream_t)stream));
    return CT_OK;
  }
  CT_CUDA(ctx, launch_trace_closest(bvh->dev, (const float4*)org, (const float4*)dir, hit, t, n, tri_eps, ctx->d_error,
                                    ctx->d_cursor, (cudaStream_t)stream));
  return CT_OK;
}

ct_status ct_trace_any(ct_ctx* ctx, const ct_bvh* bvh, const float* org, const float* dir, uint8_t* occluded,
                       uint32_t n, float tri_eps, void* stream) {
  ct_status s = check_rays(ctx, bvh, org, dir, n);
  if (s != CT_OK) return s;
  if (n && !occluded) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null output buffer");
  if (bvh->wide) {
    if ((s = ensure_wide_records(ctx, n)) != CT_OK) return s;
    CT_CUDA(ctx, launch_trace_wide_any(bvh->wdev, (const float4*)org, (const float4*)dir, occluded, n, ctx->d_error,
                                       ctx->d_cursor, ctx->d_recs, bvh->d_wstats, (cudaStream_t)stream));
    return CT_OK;
  }
  CT_CUDA(ctx, launch_trace_any(bvh->dev, (const float4*)org, (const float4*)dir, occluded, n, tri_eps, ctx->d_error,
                                ctx->d_cursor, (cudaStream_t)stream));
  return CT_OK;
}

// One queue set: a single zero-filled allocation carved into 256-byte aligned
// buffers (one cudaMalloc, one fill and one wait per set, so the ten frame
// slots of a small job cost a few calls, not a hundred).
static ct_status alloc_queues(ct_ctx* ctx, Allocs& a, size_t n, DevQueues& q) {
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t f4 = al(n * sizeof(float4)), hb = al(n * sizeof(int2)), pb = al(n * sizeof(int32_t));
  const size_t cb = al(16 * sizeof(int32_t)), sb = al(8 * sizeof(unsigned long long));
  char* base = nullptr;
  const ct_status s = upload(ctx, a, &base, nullptr, 10 * f4 + hb + pb + cb + sb);
  if (s != CT_OK) return s;
  char* p = base;
  auto take = [&p](size_t bytes) {
    char* r = p;
    p += bytes;
    return r;
  };
  q.capacity = (int32_t)n;
  q.org[0] = (float4*)take(f4), q.org[1] = (float4*)take(f4);
  q.dir[0] = (float4*)take(f4), q.dir[1] = (float4*)take(f4);
  q.thr[0] = (float4*)take(f4), q.thr[1] = (float4*)take(f4);
  q.sorg = (float4*)take(f4), q.sdir = (float4*)take(f4), q.scol = (float4*)take(f4);
  q.accum = (float4*)take(f4);
  q.hit = (int2*)take(hb);
  q.perm_buf = (int32_t*)take(pb);
  q.counts = (int32_t*)take(cb);
  q.stats = (unsigned long long*)take(sb);
  q.error = ctx->d_error;
  q.perm = nullptr;  // queue order unless a stage sorted the queue
  return CT_OK;
}

ct_status ct_render_create(ct_ctx* ctx, int32_t width, int32_t height, ct_render** out) {
  if (!ctx || !out) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  if (width <= 0 || height <= 0 || (int64_t)width * height > (1ll << 28))
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "bad render size");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  auto* r = new ct_render();
  r->w = width;
  r->h = height;
  if ((s = alloc_queues(ctx, r->allocs, (size_t)width * height, r->q)) != CT_OK) {
    free_all(ctx, r->allocs);
    delete r;
    return s;
  }
  *out = r;
  return CT_OK;
}

ct_status ct_render_destroy(ct_ctx* ctx, ct_render* r) {
  if (!ctx || !r) return CT_ERR_INVALID_ARGUMENT;
  set_device(ctx);
  for (auto& sl : r->slots) {
    if (sl.stream) {
      cudaStreamSynchronize(sl.stream);
      cudaStreamDestroy(sl.stream);
      cudaEventDestroy(sl.free_ev);
      cudaEventDestroy(sl.done_ev);
    }
  }
  free_all(ctx, r->log_allocs);
  free_all(ctx, r->allocs);
  delete r;
  return CT_OK;
}

// Frame slots for overlapped fast-math frames, created on first use.
static ct_status ensure_slots(ct_ctx* ctx, ct_render* r) {
  if (r->slots[0].stream) return CT_OK;
  const size_t n = (size_t)r->w * r->h;
  for (auto& sl : r->slots) {
    ct_status s = alloc_queues(ctx, r->allocs, n, sl.q);
    if (s != CT_OK) return s;
    CT_CUDA(ctx, cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking));
    CT_CUDA(ctx, cudaEventCreateWithFlags(&sl.free_ev, cudaEventDisableTiming));
    CT_CUDA(ctx, cudaEventCreateWithFlags(&sl.done_ev, cudaEventDisableTiming));
  }
  return CT_OK;
}

// Contribution logs for overlapped exact frames of up to max_depth passes;
// false (exact frames then run in sequence) when they would exceed
// kExactLogBytes. Growing them waits for the slots that use the old ones.
static ct_status ensure_logs(ct_ctx* ctx, ct_render* r, int max_depth, bool* ok) {
  const int entries = 2 * max_depth;
  const size_t n = (size_t)r->w * r->h;
  const size_t per_slot = (size_t)entries * n * sizeof(float4);
  const int slots = (int)std::min<size_t>(kExactSlots, kExactLogBytes / std::max<size_t>(per_slot, 1));
  *ok = slots >= 2;
  if (!*ok || (r->log_entries >= entries && r->exact_slots > 0)) return CT_OK;
  for (int k = 0; k < kExactSlots; k++)
    if (r->slots[k].stream) CT_CUDA(ctx, cudaStreamSynchronize(r->slots[k].stream));
  CT_CUDA(ctx, cudaDeviceSynchronize());  // folds on callers' streams may still read the old logs
  free_all(ctx, r->log_allocs);
  for (auto& l : r->logs) l = nullptr;
  r->log_entries = 0, r->exact_slots = 0, r->next_exact = 0;
  // within the context's budget and what the device has left; else in sequence
  if (ctx->budget && ctx->bytes.load() + (size_t)slots * per_slot > ctx->budget) {
    *ok = false;
    return CT_OK;
  }
  for (int k = 0; k < slots; k++) {
    if (cudaMalloc((void**)&r->logs[k], per_slot) != cudaSuccess) {
      cudaGetLastError();
      r->logs[k] = nullptr;
      free_all(ctx, r->log_allocs);
      for (auto& l : r->logs) l = nullptr;
      *ok = false;
      return CT_OK;
    }
    ctx->bytes += per_slot;
    r->log_allocs.list.push_back({r->logs[k], per_slot});
    CT_CUDA(ctx, cudaMemset(r->logs[k], 0, per_slot));  // tag 0 is never issued
  }
  r->log_entries = entries, r->exact_slots = slots;
  return CT_OK;
}

// Issue one frame's stages on stream st into queues q.
static ct_status emit_frame(ct_ctx* ctx, ct_render* r, const DevQueues& q, const ct_scene* scene, const ct_bvh* bvh,
                            const FrameConst& f, const ct_render_params* p, cudaStream_t st) {
  const bool fast = math_fast_traversal(p->exact_math);
  const int exact_shade = math_exact_shading(p->exact_math);
  CT_CUDA(ctx, staged(r, 0, st, [&] { return launch_raygen(q, f, exact_shade, st); }));
  for (int pass = 0; pass < p->max_depth; pass++) {
    const int cur = pass & 1;
    const int path_length = pass == 0 ? 0 : pass + 1;  // Kernel.cu:306, 330
    DevQueues qx = q;  // extend's view: sorted order for bounce rays when asked
    if (pass > 0 && p->ray_sort != CT_SORT_NONE && q.perm_buf) {
      CT_CUDA(ctx, staged(r, 1, st, [&] { return launch_ray_sort(q, cur, p->ray_sort, st); }));
      qx.perm = q.perm_buf;
    }
    if (bvh->wide)
      CT_CUDA(ctx, staged(r, 1, st, [&] { return launch_extend_wide(bvh->wdev, qx, cur, p->tri_eps, st); }));
    else
      CT_CUDA(ctx, staged(r, 1, st, [&] { return launch_extend(bvh->dev, qx, cur, p->tri_eps, fast, st); }));
    DevQueues qs = q, qc = q;  // log entries of this pass (used when q.log is set)
    qs.log_entry = 2u * (uint32_t)pass;
    qc.log_entry = 2u * (uint32_t)pass + 1u;
    CT_CUDA(ctx, staged(r, 2, st, [&] { return launch_shade(scene->dev, qs, f, cur, path_length, exact_shade, st); }));
    if (p->shadow) {
      if (bvh->wide)
        CT_CUDA(ctx, staged(r, 3, st, [&] { return launch_connect_wide(bvh->wdev, qc, p->tri_eps, st); }));
      else
        CT_CUDA(ctx, staged(r, 3, st, [&] { return launch_connect(bvh->dev, qc, p->tri_eps, fast, st); }));
    }
  }
  return CT_OK;
}

ct_status ct_render_reset(ct_ctx* ctx, ct_render* r, void* stream) {
  if (!ctx || !r) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  CT_CUDA(ctx, cudaMemsetAsync(r->q.accum, 0, (size_t)r->w * r->h * sizeof(float4), (cudaStream_t)stream));
  return CT_OK;
}

ct_status ct_render_accumulate(ct_ctx* ctx, const ct_scene* scene, const ct_bvh* bvh, const ct_camera* cam,
                               const ct_render_params* p, ct_render* r, void* stream) {
  if (!ctx || !scene || !bvh || !cam || !p || !r) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  if (p->width != r->w || p->height != r->h) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "params size differs from the render job's");
  if (p->max_depth < 1 || p->max_depth > 64) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "max_depth must be in [1, 64]");
  if (bvh->nt != scene->nt) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "BVH was built for another scene");
  if (p->shading_mode != CT_SHADE_COMPAT && p->shading_mode != CT_SHADE_FULL)
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown shading mode");
  if (!math_mode_valid(p->exact_math)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown math mode");
  if (p->texture_filter != CT_TEX_NEAREST && p->texture_filter != CT_TEX_BILINEAR)
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown texture filter");
  if (p->ray_sort < CT_SORT_NONE || p->ray_sort > CT_SORT_FACE_CELLS)
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown ray-sort key");
  if (!finite3(cam->position) || !finite3(cam->forward) || !finite3(cam->up) || !std::isfinite(cam->fov_deg))
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "non-finite camera");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  const FrameConst f = frame_const(cam, p);
  // profiling times kernels alone: frames in sequence
  if (r->profile) return emit_frame(ctx, r, r->q, scene, bvh, f, p, st);
  if (p->exact_math == CT_MATH_EXACT) {
    // Exact frames overlap too, but keep the sequential accumulation bit for
    // bit: a frame in a slot logs each pixel's contributions (shade, connect;
    // pass by pass) instead of adding them, and the log is replayed into the
    // job's buffer on the caller's stream in frame order, with the same
    // additions in the same order as a frame accumulated in place. Compat
    // shading on quad trees only; FULL shading and wide trees run in sequence.
    bool ok = p->shading_mode == CT_SHADE_COMPAT && !bvh->wide;
    if (ok && (s = ensure_slots(ctx, r)) != CT_OK) return s;
    if (ok && (s = ensure_logs(ctx, r, p->max_depth, &ok)) != CT_OK) return s;
    if (!ok) return emit_frame(ctx, r, r->q, scene, bvh, f, p, st);
    const int k = r->next_exact;
    r->next_exact = (k + 1) % r->exact_slots;
    ct_render::Slot& sl = r->slots[k];
    if (++r->log_tag == 0) r->log_tag = 1;
    DevQueues ql = sl.q;
    ql.log = r->logs[k];
    ql.log_tag = r->log_tag;
    CT_CUDA(ctx, cudaStreamWaitEvent(sl.stream, sl.free_ev, 0));
    if ((s = emit_frame(ctx, r, ql, scene, bvh, f, p, sl.stream)) != CT_OK) return s;
    CT_CUDA(ctx, cudaEventRecord(sl.done_ev, sl.stream));
    CT_CUDA(ctx, cudaStreamWaitEvent(st, sl.done_ev, 0));
    CT_CUDA(ctx, launch_fold_log(r->q.accum, r->logs[k], 2 * p->max_depth, r->w * r->h, r->w * r->h, r->log_tag, st));
    CT_CUDA(ctx, cudaEventRecord(sl.free_ev, st));
    return CT_OK;
  }
  // Fast-math frames overlap: the frame renders into one of kFrameSlots
  // private slots (queues + accumulation) on the slot's own stream, so its
  // first passes can run while earlier frames' last bounces are still
  // draining; the slot is then added to the job's buffer on the caller's
  // stream, in frame order.
  if ((s = ensure_slots(ctx, r)) != CT_OK) return s;
  ct_render::Slot& sl = r->slots[r->next_slot];
  r->next_slot = (r->next_slot + 1) % kFrameSlots;
  CT_CUDA(ctx, cudaStreamWaitEvent(sl.stream, sl.free_ev, 0));
  if ((s = emit_frame(ctx, r, sl.q, scene, bvh, f, p, sl.stream)) != CT_OK) return s;
  CT_CUDA(ctx, cudaEventRecord(sl.done_ev, sl.stream));
  CT_CUDA(ctx, cudaStreamWaitEvent(st, sl.done_ev, 0));
  CT_CUDA(ctx, launch_fold(r->q.accum, sl.q.accum, r->w * r->h, st));
  CT_CUDA(ctx, cudaEventRecord(sl.free_ev, st));
  return CT_OK;
}

ct_status ct_render_accumulate_noalloc(ct_ctx* ctx, const ct_scene* scene, const ct_bvh* bvh, const ct_camera* cam,
                                       const ct_render_params* p, float* accum_device, void* stream) {
  if (!ctx || !scene || !bvh || !cam || !p || !accum_device) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  if (((uintptr_t)accum_device) & 15) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "accumulation buffer must be 16-byte aligned");
  if (p->width <= 0 || p->height <= 0) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "bad frame size");
  if ((int64_t)p->width * p->height > (int64_t)noalloc_max_pixels())
    return fail(ctx, CT_ERR_INVALID_ARGUMENT,
                "frame of " + std::to_string((int64_t)p->width * p->height) + " pixels exceeds the allocation-free limit of " +
                    std::to_string(noalloc_max_pixels()) + " (CT_NOALLOC_MAX_PIXELS)");
  if (p->max_depth < 1 || p->max_depth > 64) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "max_depth must be in [1, 64]");
  if (bvh->nt != scene->nt) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "BVH was built for another scene");
  if (bvh->wide) return fail(ctx, CT_ERR_UNSUPPORTED, "frames trace quad BVHs; the wide BVH serves ray queries");
  if (p->shading_mode != CT_SHADE_COMPAT && p->shading_mode != CT_SHADE_FULL)
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown shading mode");
  if (!math_mode_valid(p->exact_math)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown math mode");
  if (p->texture_filter != CT_TEX_NEAREST && p->texture_filter != CT_TEX_BILINEAR)
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown texture filter");
  if (!finite3(cam->position) || !finite3(cam->forward) || !finite3(cam->up) || !std::isfinite(cam->fov_deg))
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "non-finite camera");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  const FrameConst f = frame_const(cam, p);
  CT_CUDA(ctx, noalloc_render(ctx->device, scene->dev, bvh->dev, f, p->max_depth, p->exact_math,
                              (float4*)accum_device, ctx->d_error, (cudaStream_t)stream));
  return CT_OK;
}

ct_status ct_render_accum(const ct_render* r, float** accum_device) {
  if (!r || !accum_device) return CT_ERR_INVALID_ARGUMENT;
  *accum_device = (float*)r->q.accum;
  return CT_OK;
}

ct_status ct_present(ct_ctx* ctx, const ct_render* r, float samples, float* rgba_device, void* stream) {
  if (!ctx || !r || !rgba_device) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  if (((uintptr_t)rgba_device) & 15) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "output must be 16-byte aligned");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  CT_CUDA(ctx, launch_present(r->q.accum, (float4*)rgba_device, r->w * r->h, samples, (cudaStream_t)stream));
  return CT_OK;
}

ct_status ct_render_stats(ct_ctx* ctx, ct_render* r, ct_frame_stats* stats, int32_t reset, void* stream) {
  if (!ctx || !r || !stats) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  unsigned long long tot[4] = {0, 0, 0, 0};
  CT_CUDA(ctx, cudaStreamSynchronize((cudaStream_t)stream));
  const DevQueues* qs[kFrameSlots + 1];
  qs[0] = &r->q;
  for (int k = 0; k < kFrameSlots; k++) qs[k + 1] = &r->slots[k].q;
  for (const DevQueues* q : qs) {
    if (!q->stats) continue;
    unsigned long long h[4] = {0, 0, 0, 0};
    CT_CUDA(ctx, cudaMemcpy(h, q->stats, sizeof(h), cudaMemcpyDeviceToHost));
    for (int k = 0; k < 4; k++) tot[k] += h[k];
    if (reset) CT_CUDA(ctx, cudaMemset(q->stats, 0, sizeof(h)));
  }
  if (reset) CT_CUDA(ctx, cudaStreamSynchronize(0));
  stats->extension_rays = tot[0];
  stats->shadow_rays = tot[1];
  stats->samples = tot[2];
  stats->frames = (uint32_t)tot[3];
  return CT_OK;
}

ct_status ct_render_profile(ct_ctx* ctx, ct_render* r, int32_t enable) {
  if (!ctx || !r) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  r->profile = enable != 0;
  return CT_OK;
}

ct_status ct_render_profile_read(ct_ctx* ctx, ct_render* r, ct_stage_times* out, int32_t reset) {
  if (!ctx || !r || !out) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  for (int k = 0; k < 4; k++) {
    double ms = 0.0;
    for (auto& p : r->marks[k]) {
      CT_CUDA(ctx, cudaEventSynchronize(p.second));
      float e = 0.0f;
      CT_CUDA(ctx, cudaEventElapsedTime(&e, p.first, p.second));
      ms += e;
    }
    out->ms[k] = ms;
    out->launches[k] = (uint32_t)r->marks[k].size();
  }
  if (reset) r->recycle();
  return CT_OK;
}

}  // extern "C"

// ============================================================ batches
// Lanes of a fast-math batch (measured on the 256-job workload: 2 lanes 1,317,
// 3 lanes 1,375, 4 lanes 1,394 Msamples/s). Fixed, because a job's summation
// grouping depends on it: each lane holds a queue set for every pixel of the
// batch (172 bytes per pixel).
constexpr int kBatchLanes = 4;

struct ct_batch {
  int32_t n = 0;
  int32_t exact = 0;
  int32_t max_depth = 1;
  uint32_t max_spp = 0;
  // Fast-math batches run L = kBatchLanes lanes: lane l takes samples l, l + L,
  // l + 2L, ... of every job, with its own job table, queue set, accumulation
  // and stream, so one lane's last bounces overlap the other lanes' passes;
  // the lanes' accumulations are added to lane 0's, in lane order, when the
  // run ends. Exact-math batches run one lane (bit-identical to
  // ct_render_accumulate). Lane 0 is q/dev/jobs0; lanes >= 1 are in the arrays.
  int lanes = 1;
  DevQueues q{};
  DevBatch dev{};
  Allocs allocs;
  std::vector<BatchJob> jobs0;  // job table at the first sample (lane 0)
  DevQueues lq[kBatchLanes] = {};
  DevBatch ldev[kBatchLanes] = {};
  std::vector<BatchJob> ljobs0[kBatchLanes];
  std::vector<int32_t> bases;
  ct_batch_tuning tune{128, 128, 1, 1, CT_SORT_NONE, 24};
  cudaStream_t cap = nullptr;  // capture stream
  cudaGraphExec_t exec[kBatchLanes] = {};
  ct_batch_tuning exec_tune{0, 0, 0, 0, 0, 0};
  cudaStream_t side[kBatchLanes] = {};  // lane streams
  cudaEvent_t fork_ev = nullptr, join_ev[kBatchLanes] = {};
  const DevQueues& lane_q(int l) const { return l ? lq[l] : q; }
  const DevBatch& lane_dev(int l) const { return l ? ldev[l] : dev; }
  ~ct_batch() {
    for (auto& x : exec)
      if (x) cudaGraphExecDestroy(x);
    if (cap) cudaStreamDestroy(cap);
    for (auto& x : side)
      if (x) cudaStreamDestroy(x);
    if (fork_ev) cudaEventDestroy(fork_ev);
    for (auto& x : join_ev)
      if (x) cudaEventDestroy(x);
  }
};

namespace {


// One iteration: every job that still takes samples traces one more.
cudaError_t batch_iteration(ct_batch* b, int lane, const ct_batch_tuning& t, cudaStream_t st) {
  const DevBatch& dev = b->lane_dev(lane);
  const DevQueues& q = b->lane_q(lane);
  cudaError_t e = launch_batch_raygen(dev, q, math_exact_shading(b->exact), st);
  for (int pass = 0; pass < b->max_depth && e == cudaSuccess; pass++) {
    const int cur = pass & 1;
    const uint32_t path_length = pass == 0 ? 0u : (uint32_t)pass + 1u;  // Kernel.cu:306, 330
    DevQueues qx = q;
    if (pass > 0 && t.sort_key != CT_SORT_NONE) {
      e = launch_ray_sort(q, cur, t.sort_key, st);
      qx.perm = q.perm_buf;
    }
    if (e == cudaSuccess)
      e = dev.wide ? launch_batch_extend_wide(dev, qx, cur, st)
                   : launch_batch_extend(dev, qx, cur, math_fast_traversal(b->exact), t.extend_block, t.refill, st);
    if (e == cudaSuccess) e = launch_batch_shade(dev, q, cur, path_length, pass, math_exact_shading(b->exact), t.shade_waves, st);
    if (e == cudaSuccess)
      e = dev.wide ? launch_batch_connect_wide(dev, q, st)
                   : launch_batch_connect(dev, q, math_fast_traversal(b->exact), t.connect_block, st);
  }
  if (e == cudaSuccess) e = launch_batch_advance(dev, q, st);
  return e;
}

cudaError_t batch_graph(ct_batch* b) {
  if (b->exec[0] && std::memcmp(&b->exec_tune, &b->tune, sizeof(b->tune)) == 0) return cudaSuccess;
  for (auto& x : b->exec)
    if (x) cudaGraphExecDestroy(x), x = nullptr;
  cudaError_t e = cudaSuccess;
  if (!b->cap) e = cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking);
  for (int lane = 0; lane < b->lanes && e == cudaSuccess; lane++) {
    e = cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeRelaxed);
    if (e != cudaSuccess) return e;
    const cudaError_t le = batch_iteration(b, lane, b->tune, b->cap);
    cudaGraph_t g = nullptr;
    e = cudaStreamEndCapture(b->cap, &g);
    if (le != cudaSuccess) e = le;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&b->exec[lane], g, 0);
    if (g) cudaGraphDestroy(g);
  }
  if (e == cudaSuccess) b->exec_tune = b->tune;
  return e;
}

// Reset the job table to the first sample and the queues' counters.
cudaError_t batch_reset(ct_batch* b, cudaStream_t st, bool zero_accum) {
  cudaError_t e = cudaMemcpyAsync(b->dev.jobs, b->jobs0.data(), b->jobs0.size() * sizeof(BatchJob),
                                  cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(b->q.counts, 0, 16 * sizeof(int32_t), st);
  if (e == cudaSuccess && zero_accum)
    e = cudaMemsetAsync(b->q.accum, 0, (size_t)b->dev.total_pix * sizeof(float4), st);
  for (int l = 1; l < b->lanes; l++) {
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(b->ldev[l].jobs, b->ljobs0[l].data(), b->ljobs0[l].size() * sizeof(BatchJob),
                          cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b->lq[l].counts, 0, 16 * sizeof(int32_t), st);
    if (e == cudaSuccess && zero_accum)
      e = cudaMemsetAsync(b->lq[l].accum, 0, (size_t)b->dev.total_pix * sizeof(float4), st);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);  // the job tables are pageable host memory
  return e;
}

// `iters` iterations on `st`: one lane in order, or the lanes in turn on their
// own streams (forked from and joined back into `st`).
cudaError_t batch_iterations(ct_batch* b, uint32_t iters, cudaStream_t st) {
  cudaError_t e = cudaSuccess;
  if (b->tune.use_graph) e = batch_graph(b);
  if (e != cudaSuccess) return e;
  if (b->lanes == 1) {
    for (uint32_t k = 0; k < iters && e == cudaSuccess; k++)
      e = b->tune.use_graph ? cudaGraphLaunch(b->exec[0], st) : batch_iteration(b, 0, b->tune, st);
    return e;
  }
  e = cudaEventRecord(b->fork_ev, st);
  for (int l = 0; l < b->lanes && e == cudaSuccess; l++) e = cudaStreamWaitEvent(b->side[l], b->fork_ev, 0);
  for (uint32_t k = 0; k < iters && e == cudaSuccess; k++) {
    const int l = (int)(k % (uint32_t)b->lanes);
    e = b->tune.use_graph ? cudaGraphLaunch(b->exec[l], b->side[l]) : batch_iteration(b, l, b->tune, b->side[l]);
  }
  for (int l = 0; l < b->lanes && e == cudaSuccess; l++) {
    e = cudaEventRecord(b->join_ev[l], b->side[l]);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, b->join_ev[l], 0);
  }
  return e;
}

bool tuning_ok(const ct_batch_tuning& t) {
  auto blk = [](int32_t v) { return v == 64 || v == 128 || v == 256; };
  return blk(t.extend_block) && blk(t.connect_block) && t.shade_waves >= 1 && t.shade_waves <= 8 &&
         (t.use_graph == 0 || t.use_graph == 1) && t.sort_key >= CT_SORT_NONE && t.sort_key <= CT_SORT_FACE_CELLS &&
         (t.refill == 8 || t.refill == 16 || t.refill == 24);
}

}  // namespace

extern "C" {

ct_status ct_batch_create(ct_ctx* ctx, const ct_batch_job* jobs, uint32_t n, int32_t exact_math, ct_batch** out) {
  if (!ctx || !jobs || !out || n == 0) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument or empty batch");
  *out = nullptr;
  if (!math_mode_valid(exact_math)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown math mode");
  int64_t total = 0;
  int32_t max_stack = 1, max_depth = 1;
  uint32_t max_spp = 0;
  for (uint32_t j = 0; j < n; j++) {
    const ct_batch_job& J = jobs[j];
    const ct_render_params* p = &J.params;
    const std::string at = "job " + std::to_string(j) + ": ";
    if (!J.scene || !J.bvh) return fail(ctx, CT_ERR_INVALID_ARGUMENT, at + "null scene or BVH");
    if (J.bvh->nt != J.scene->nt) return fail(ctx, CT_ERR_INVALID_ARGUMENT, at + "BVH was built for another scene");
    if (J.bvh->wide != jobs[0].bvh->wide)
      return fail(ctx, CT_ERR_UNSUPPORTED, at + "a batch traces either quad or wide BVHs, not both");
    if (p->width <= 0 || p->height <= 0 || (int64_t)p->width * p->height > (1 << 26))
      return fail(ctx, CT_ERR_INVALID_ARGUMENT, at + "bad frame size");
    if (p->max_depth < 1 || p->max_depth > 64) return fail(ctx, CT_ERR_INVALID_ARGUMENT, at + "max_depth must be in [1, 64]");
    if (p->shading_mode != CT_SHADE_COMPAT && p->shading_mode != CT_SHADE_FULL)
      return fail(ctx, CT_ERR_INVALID_ARGUMENT, at + "unknown shading mode");
    if (p->texture_filter != CT_TEX_NEAREST && p->texture_filter != CT_TEX_BILINEAR)
      return fail(ctx, CT_ERR_INVALID_ARGUMENT, at + "unknown texture filter");
    if (p->ray_sort < CT_SORT_NONE || p->ray_sort > CT_SORT_FACE_CELLS)
      return fail(ctx, CT_ERR_INVALID_ARGUMENT, at + "unknown ray-sort key");
    if (J.spp == 0) return fail(ctx, CT_ERR_INVALID_ARGUMENT, at + "spp must be at least 1");
    if (!finite3(J.camera.position) || !finite3(J.camera.forward) || !finite3(J.camera.up) ||
        !std::isfinite(J.camera.fov_deg))
      return fail(ctx, CT_ERR_INVALID_ARGUMENT, at + "non-finite camera");
    total += (int64_t)p->width * p->height;
    max_stack = std::max(max_stack, J.bvh->dev.stack_entries);
    max_depth = std::max(max_depth, p->max_depth);
    max_spp = std::max(max_spp, J.spp);
  }
  if (total > (int64_t)INT32_MAX / 2) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "batch has too many pixels");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  auto* b = new ct_batch();
  b->n = (int32_t)n;
  b->exact = exact_math;
  b->max_depth = max_depth;
  b->max_spp = max_spp;
  b->lanes = exact_math == CT_MATH_EXACT ? 1 : kBatchLanes;
  b->jobs0.resize(n);
  b->bases.resize(n + 1);
  int32_t base = 0;
  for (uint32_t j = 0; j < n; j++) {
    const ct_batch_job& J = jobs[j];
    BatchJob& d = b->jobs0[j];
    std::memset(&d, 0, sizeof(d));
    d.sc = J.scene->dev;
    d.bvh = J.bvh->dev;
    d.wbvh = J.bvh->wdev;
    d.f = frame_const(&J.camera, &J.params);
    d.pix_base = base;
    d.max_depth = J.params.max_depth;
    d.spp_left = (int32_t)((J.spp + b->lanes - 1) / b->lanes);  // lane 0: samples 0, L, 2L, ...
    d.exact = b->exact;
    b->bases[j] = base;
    base += J.params.width * J.params.height;
  }
  b->bases[n] = base;
  BatchJob* djobs = nullptr;
  int32_t* dbases = nullptr;
  if ((s = alloc_queues(ctx, b->allocs, (size_t)base, b->q)) != CT_OK ||
      (s = upload(ctx, b->allocs, &djobs, b->jobs0.data(), n * sizeof(BatchJob))) != CT_OK ||
      (s = upload(ctx, b->allocs, &dbases, b->bases.data(), (n + 1) * sizeof(int32_t))) != CT_OK) {
    free_all(ctx, b->allocs);
    delete b;
    return s;
  }
  for (uint32_t j = 0; j < n; j++) b->jobs0[j].accum = b->q.accum + b->bases[j];
  cudaError_t e = cudaMemcpy(djobs, b->jobs0.data(), n * sizeof(BatchJob), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaStreamSynchronize(0);
  if (e != cudaSuccess) {
    free_all(ctx, b->allocs);
    delete b;
    return cuda_fail(ctx, e, "batch job table");
  }
  b->dev.jobs = djobs;
  b->dev.bases = dbases;
  b->dev.n_jobs = (int32_t)n;
  b->dev.total_pix = base;
  b->dev.max_stack = max_stack;
  b->dev.wide = jobs[0].bvh->wide ? 1 : 0;
  b->dev.frame_step = 2 * b->lanes;
  if (b->lanes > 1) {
    // lane l >= 1: samples l, l + L, ... (frames + 2l, + 2l + 2L, ...) into its own queues and accumulation
    for (int l = 1; l < b->lanes && s == CT_OK; l++) {
      BatchJob* dj = nullptr;
      b->ljobs0[l] = b->jobs0;
      for (uint32_t j = 0; j < n; j++) {
        BatchJob& d = b->ljobs0[l][j];
        d.spp_left = (int32_t)(jobs[j].spp > (uint32_t)l ? (jobs[j].spp - l + b->lanes - 1) / b->lanes : 0);
        d.f.frame += 2u * (uint32_t)l;
      }
      if ((s = alloc_queues(ctx, b->allocs, (size_t)base, b->lq[l])) == CT_OK) {
        for (uint32_t j = 0; j < n; j++) b->ljobs0[l][j].accum = b->lq[l].accum + b->bases[j];
        s = upload(ctx, b->allocs, &dj, b->ljobs0[l].data(), n * sizeof(BatchJob));
      }
      b->ldev[l] = b->dev;
      b->ldev[l].jobs = dj;
    }
    cudaError_t ce = cudaSuccess;
    for (int l = 0; l < b->lanes && s == CT_OK && ce == cudaSuccess; l++) {
      ce = cudaStreamCreateWithFlags(&b->side[l], cudaStreamNonBlocking);
      if (ce == cudaSuccess) ce = cudaEventCreateWithFlags(&b->join_ev[l], cudaEventDisableTiming);
    }
    if (s == CT_OK && ce == cudaSuccess) ce = cudaEventCreateWithFlags(&b->fork_ev, cudaEventDisableTiming);
    if (s != CT_OK || ce != cudaSuccess) {
      free_all(ctx, b->allocs);
      delete b;
      return s != CT_OK ? s : cuda_fail(ctx, ce, "batch lanes");
    }
  }
  *out = b;
  return CT_OK;
}

ct_status ct_batch_destroy(ct_ctx* ctx, ct_batch* b) {
  if (!ctx || !b) return CT_ERR_INVALID_ARGUMENT;
  set_device(ctx);
  cudaDeviceSynchronize();
  free_all(ctx, b->allocs);
  delete b;
  return CT_OK;
}

ct_status ct_batch_run(ct_ctx* ctx, ct_batch* b, void* stream) {
  if (!ctx || !b) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  CT_CUDA(ctx, batch_reset(b, st, true));
  CT_CUDA(ctx, batch_iterations(b, b->max_spp, st));
  for (int l = 1; l < b->lanes; l++) CT_CUDA(ctx, launch_fold(b->q.accum, b->lq[l].accum, b->dev.total_pix, st));
  return CT_OK;
}

ct_status ct_batch_accum(const ct_batch* b, uint32_t job, float** accum_device, uint32_t* pixels) {
  if (!b || job >= (uint32_t)b->n) return CT_ERR_INVALID_ARGUMENT;
  if (accum_device) *accum_device = (float*)(b->q.accum + b->bases[job]);
  if (pixels) *pixels = (uint32_t)(b->bases[job + 1] - b->bases[job]);
  return CT_OK;
}

ct_status ct_batch_set_tuning(ct_ctx* ctx, ct_batch* b, const ct_batch_tuning* t) {
  if (!b || !t) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  if (!tuning_ok(*t)) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "tuning out of range");
  b->tune = *t;
  return CT_OK;
}

ct_status ct_batch_get_tuning(const ct_batch* b, ct_batch_tuning* t) {
  if (!b || !t) return CT_ERR_INVALID_ARGUMENT;
  *t = b->tune;
  return CT_OK;
}

ct_status ct_batch_autotune(ct_ctx* ctx, ct_batch* b, void* stream, ct_batch_tuning* chosen, double* ms_per_iteration) {
  if (!ctx || !b) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  CT_CUDA(ctx, cudaEventCreate(&e0));
  CT_CUDA(ctx, cudaEventCreate(&e1));
  // time `iters` iterations of the first samples of every job under tuning t
  const uint32_t iters = std::max<uint32_t>(1, std::min<uint32_t>(2, b->max_spp));
  auto measure = [&](const ct_batch_tuning& t, float& ms) -> cudaError_t {
    b->tune = t;
    cudaError_t e = batch_reset(b, st, false);
    if (e == cudaSuccess) e = batch_iterations(b, 1, st);  // warm-up (and graph instantiation)
    if (e == cudaSuccess) e = batch_reset(b, st, false);
    if (e == cudaSuccess) e = cudaEventRecord(e0, st);
    if (e == cudaSuccess) e = batch_iterations(b, iters, st);
    if (e == cudaSuccess) e = cudaEventRecord(e1, st);
    if (e == cudaSuccess) e = cudaEventSynchronize(e1);
    if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
    ms /= (float)iters;
    return e;
  };
  ct_batch_tuning best = b->tune;
  float best_ms = 1e30f;
  cudaError_t err = cudaSuccess;
  auto trial = [&](const ct_batch_tuning& t) {
    if (err != cudaSuccess) return;
    float ms = 0.0f;
    err = measure(t, ms);
    if (err == cudaSuccess && ms < best_ms) best_ms = ms, best = t;
  };
  // coordinate search: traversal block sizes, then the refill (lane
  // compaction) threshold, the ray-sort key, shade waves and graph replay
  for (int eb : {64, 128, 256})
    for (int cb : {128, 256}) trial(ct_batch_tuning{eb, cb, 1, 1, CT_SORT_NONE, 24});
  for (int rf : {8, 16}) trial(ct_batch_tuning{best.extend_block, best.connect_block, 1, 1, CT_SORT_NONE, rf});
  for (int key : {CT_SORT_OCTANT, CT_SORT_FACE_CELLS})
    trial(ct_batch_tuning{best.extend_block, best.connect_block, 1, 1, key, best.refill});
  trial(ct_batch_tuning{best.extend_block, best.connect_block, 2, 1, best.sort_key, best.refill});
  trial(ct_batch_tuning{best.extend_block, best.connect_block, best.shade_waves, 0, best.sort_key, best.refill});
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (err != cudaSuccess) return cuda_fail(ctx, err, "batch autotune");
  b->tune = best;
  if (chosen) *chosen = best;
  if (ms_per_iteration) *ms_per_iteration = best_ms;
  return CT_OK;
}

ct_status ct_batch_stats(ct_ctx* ctx, ct_batch* b, ct_frame_stats* out, int32_t reset, void* stream) {
  if (!ctx || !b || !out) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null argument");
  ct_status s = set_device(ctx);
  if (s != CT_OK) return s;
  cudaStream_t st = (cudaStream_t)stream;
  unsigned long long h[8] = {0};
  for (int l = 0; l < b->lanes; l++) {
    unsigned long long hl[8] = {0};
    const DevQueues& q = b->lane_q(l);
    CT_CUDA(ctx, cudaMemcpyAsync(hl, q.stats, sizeof(hl), cudaMemcpyDeviceToHost, st));
    CT_CUDA(ctx, cudaStreamSynchronize(st));
    for (int k = 0; k < 8; k++) h[k] += hl[k];
    if (reset) CT_CUDA(ctx, cudaMemsetAsync(q.stats, 0, sizeof(hl), st));
  }
  CT_CUDA(ctx, cudaStreamSynchronize(st));
  out->extension_rays = h[0];
  out->shadow_rays = h[1];
  out->samples = h[2];
  out->frames = (uint32_t)h[3];
  return CT_OK;
}

}  // extern "C"

// ============================================================ accessors for the serving loop (server.cpp)
namespace ct {
const DevScene& rt_scene_dev(const ct_scene* s) { return s->dev; }
uint32_t rt_scene_tris(const ct_scene* s) { return s->nt; }
const DevBVH& rt_bvh_dev(const ct_bvh* b) { return b->dev; }
bool rt_bvh_wide(const ct_bvh* b) { return b->wide; }
uint32_t rt_bvh_tris(const ct_bvh* b) { return b->nt; }
int rt_ctx_device(const ct_ctx* c) { return c->device; }
uint32_t* rt_ctx_error(const ct_ctx* c) { return c->d_error; }
ct_status rt_fail(ct_ctx* c, ct_status s, const std::string& msg) { return fail(c, s, msg); }
ct_status rt_alloc(ct_ctx* c, size_t bytes, void** p) {
  Allocs a;
  const ct_status s = dev_alloc(c, a, p, bytes);
  return s;
}
void rt_free(ct_ctx* c, void* p, size_t bytes) {
  if (!p) return;
  bytes = (bytes == 0 ? 16 : bytes);
  bytes = (bytes + 255) & ~(size_t)255;
  cudaFree(p);
  c->bytes -= bytes;
}
ct_status rt_alloc_queues(ct_ctx* c, size_t n, DevQueues& q, std::vector<std::pair<void*, size_t>>& owned) {
  Allocs a;
  const ct_status s = alloc_queues(c, a, n, q);
  owned = a.list;
  if (s != CT_OK) {
    free_all(c, a);
    owned.clear();
  }
  return s;
}
void rt_free_list(ct_ctx* c, std::vector<std::pair<void*, size_t>>& owned) {
  Allocs a;
  a.list = owned;
  free_all(c, a);
  owned.clear();
}
FrameConst rt_frame_const(const ct_camera* cam, const ct_render_params* p) { return frame_const(cam, p); }
const DevWBVH& rt_bvh_wdev(const ct_bvh* b) { return b->wdev; }
bool rt_account(ct_ctx* c, int64_t delta) {
  if (delta > 0 && c->budget && c->bytes.load() + (uint64_t)delta > c->budget) return false;
  c->bytes += (uint64_t)delta;
  return true;
}
ct_status rt_check_job(ct_ctx* ctx, const ct_batch_job& J) {
  const ct_render_params* p = &J.params;
  if (!J.scene || !J.bvh) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "null scene or BVH");
  if (J.bvh->nt != J.scene->nt) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "BVH was built for another scene");
  if (J.bvh->wide) return fail(ctx, CT_ERR_UNSUPPORTED, "the serving loop renders on quad BVHs");
  if (p->width <= 0 || p->height <= 0 || (int64_t)p->width * p->height > (1 << 26))
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "bad frame size");
  if (p->max_depth < 1 || p->max_depth > 64) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "max_depth must be in [1, 64]");
  if (p->shading_mode != CT_SHADE_COMPAT && p->shading_mode != CT_SHADE_FULL)
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown shading mode");
  if (p->texture_filter != CT_TEX_NEAREST && p->texture_filter != CT_TEX_BILINEAR)
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown texture filter");
  if (p->ray_sort < CT_SORT_NONE || p->ray_sort > CT_SORT_FACE_CELLS)
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "unknown ray-sort key");
  if (J.spp == 0) return fail(ctx, CT_ERR_INVALID_ARGUMENT, "spp must be at least 1");
  if (!finite3(J.camera.position) || !finite3(J.camera.forward) || !finite3(J.camera.up) ||
      !std::isfinite(J.camera.fov_deg))
    return fail(ctx, CT_ERR_INVALID_ARGUMENT, "non-finite camera");
  return CT_OK;
}
}  // namespace ct
