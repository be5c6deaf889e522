/*
 * C-ABI harness around the REFERENCE tracer's own host code (meirbon/CudaTracer),
 * compiled from a build-time patched copy of its sources by oracle/ref_build.py.
 *
 * TEST INFRASTRUCTURE ONLY. This library (oracle/_ref/libctref.so) is the
 * checker's pin: it generates the golden fixtures under tests/golden/ and is
 * the "reference" CPU baseline timed by bench.py. The product never links it.
 *
 * Everything that computes here is the reference's code:
 *   - SAH binary build      BVHTree::constructBVH         src/BVH/BVHTree.cpp:13-50
 *                           BVHNode::SubdivideMT/Partition src/BVH/BVHNode.cu:70-190
 *   - quad collapse         MBVHTree::constructBVH        src/BVH/MBVHTree.cpp:15-30
 *   - host closest hit      MBVHNode::traverseMBVH (host)  src/BVH/MBVHNode.cuh:207-244
 *   - host binary closest   BVHNode::traverseBVH (host)    src/BVH/BVHNode.cuh:206-254
 *   - camera rays           Camera::generateRay            src/Core/Camera.cpp:19-37
 *   - per-triangle bounds   triangle::getBounds            src/Core/Triangle.cuh:59-65
 *   - shading helpers       Random.cuh, Tools.h, BSDF.h, Microfacet.cuh, Triangle.cuh
 * The only code written here is marshalling between flat arrays and the
 * reference's containers, plus a std::thread split of rays for timing.
 */
#include <atomic>
#include <chrono>
#include <cstdint>
#include <cstring>
#include <iostream>
#include <sstream>
#include <thread>
#include <vector>

#include "BVH/BVHTree.h"
#include "BVH/MBVHTree.h"
#include "BVH/MBVHNode.cuh"
#include "Core/BSDF.h"
#include "Core/Camera.h"
#include "Core/Material.cuh"
#include "Core/Microfacet.cuh"
#include "Core/Random.cuh"
#include "Core/Tools.h"
#include "Core/Triangle.cuh"
#include "Core/TriangleList.h"

// TriangleList's constructor/destructor live in Core/TriangleList.cpp, which
// needs assimp and FreeImage (Windows binaries only). The BVH path reads only
// the public vectors, so empty definitions suffice.
TriangleList::TriangleList() : m_Pool(nullptr) {}
TriangleList::~TriangleList() {}

namespace {

struct RefScene {
  TriangleList list;
  ctpl::ThreadPool* pool = nullptr;
  BVHTree* bvh = nullptr;
  MBVHTree* mbvh = nullptr;
  double build_ms = 0.0;
  double mbvh_ms = 0.0;
};

template <typename F>
void parallel_for_rays(int n, int nthreads, F&& f) {
  if (nthreads <= 1 || n < 1024) {
    f(0, n);
    return;
  }
  std::vector<std::thread> ts;
  const int chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    const int b = t * chunk, e = std::min(n, b + chunk);
    if (b >= e) break;
    ts.emplace_back([&f, b, e] { f(b, e); });
  }
  for (auto& t : ts) t.join();
}

}  // namespace

extern "C" {

int ctref_sizeof_bvhnode() { return (int)sizeof(BVHNode); }
int ctref_sizeof_mbvhnode() { return (int)sizeof(MBVHNode); }
int ctref_hardware_threads() { return (int)std::thread::hardware_concurrency(); }

/* Build the reference binary SAH BVH and its quad collapse over ntri triangles.
 * nthreads > 0 uses the reference ctpl pool + SubdivideMT (the Application path,
 * src/Application.cpp:132); nthreads == 0 uses the single-threaded Subdivide. */
void* ctref_build(const float* verts, int nverts, const uint32_t* idx, int ntri, int nthreads) {
  auto* s = new RefScene();
  s->list.m_Vertices.resize(nverts);
  for (int i = 0; i < nverts; i++) s->list.m_Vertices[i] = glm::vec3(verts[3 * i], verts[3 * i + 1], verts[3 * i + 2]);
  s->list.m_Indices.resize(ntri);
  s->list.m_AABBs.resize(ntri);
  for (int i = 0; i < ntri; i++) {
    s->list.m_Indices[i] = glm::uvec3(idx[3 * i], idx[3 * i + 1], idx[3 * i + 2]);
    const auto& v = s->list.m_Vertices;
    s->list.m_AABBs[i] = triangle::getBounds(v[idx[3 * i]], v[idx[3 * i + 1]], v[idx[3 * i + 2]]);
  }
  if (nthreads > 0) s->pool = new ctpl::ThreadPool(nthreads);
  std::streambuf* old = std::cout.rdbuf();
  std::ostringstream sink;
  std::cout.rdbuf(sink.rdbuf());  // the reference prints build times; keep stdout clean
  auto t0 = std::chrono::high_resolution_clock::now();
  s->bvh = new BVHTree(&s->list, s->pool);
  s->bvh->constructBVH();
  auto t1 = std::chrono::high_resolution_clock::now();
  s->mbvh = new MBVHTree(s->bvh);
  s->mbvh->constructBVH();
  auto t2 = std::chrono::high_resolution_clock::now();
  std::cout.rdbuf(old);
  s->build_ms = std::chrono::duration<double, std::milli>(t1 - t0).count();
  s->mbvh_ms = std::chrono::duration<double, std::milli>(t2 - t1).count();
  return s;
}

double ctref_build_ms(void* h) { return ((RefScene*)h)->build_ms; }
double ctref_mbvh_ms(void* h) { return ((RefScene*)h)->mbvh_ms; }
int ctref_bvh_count(void* h) { return (int)((RefScene*)h)->bvh->m_BVHPool.size(); }
int ctref_mbvh_count(void* h) { return (int)((RefScene*)h)->mbvh->m_FinalPtr; }
int ctref_prim_count(void* h) { return (int)((RefScene*)h)->bvh->m_PrimitiveIndices.size(); }

/* Raw node copies: BVHNode is 32 bytes {min.xyz, leftFirst, max.xyz, count};
 * MBVHNode is 128 bytes {bminx4,bmaxx4,bminy4,bmaxy4,bminz4,bmaxz4,childs,counts}. */
void ctref_export(void* h, void* bvh_out, uint32_t* prim_out, void* mbvh_out) {
  auto* s = (RefScene*)h;
  if (bvh_out) std::memcpy(bvh_out, s->bvh->m_BVHPool.data(), s->bvh->m_BVHPool.size() * sizeof(BVHNode));
  if (prim_out)
    std::memcpy(prim_out, s->bvh->m_PrimitiveIndices.data(), s->bvh->m_PrimitiveIndices.size() * sizeof(uint32_t));
  if (mbvh_out) std::memcpy(mbvh_out, s->mbvh->m_Tree.data(), s->mbvh->m_FinalPtr * sizeof(MBVHNode));
}

/* Host closest hit, reference quad traversal (MBVHNode.cuh:207). t starts at
 * MAX_DISTANCE and hit at -1, as Ray's constructor sets them (Ray.cuh:51-58). */
void ctref_trace_mbvh(void* h, const float* org, const float* dir, int n, int32_t* hit, float* tout, int nthreads) {
  auto* s = (RefScene*)h;
  const MBVHNode* nodes = s->mbvh->m_Tree.data();
  const unsigned int* prims = s->mbvh->m_PrimitiveIndices.data();
  parallel_for_rays(n, nthreads, [&](int b, int e) {
    for (int i = b; i < e; i++) {
      glm::vec3 o(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
      glm::vec3 d(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
      float t = MAX_DISTANCE;
      int hi = -1;
      MBVHNode::traverseMBVH(o, d, &t, &hi, nodes, prims, s->list);
      hit[i] = hi;
      tout[i] = t;
    }
  });
}

/* Host closest hit, reference binary traversal (BVHNode.cuh:206). */
void ctref_trace_bvh(void* h, const float* org, const float* dir, int n, int32_t* hit, float* tout, int nthreads) {
  auto* s = (RefScene*)h;
  const unsigned int* prims = s->bvh->m_PrimitiveIndices.data();
  parallel_for_rays(n, nthreads, [&](int b, int e) {
    for (int i = b; i < e; i++) {
      glm::vec3 o(org[3 * i], org[3 * i + 1], org[3 * i + 2]);
      glm::vec3 d(dir[3 * i], dir[3 * i + 1], dir[3 * i + 2]);
      float t = MAX_DISTANCE;
      int hi = -1;
      BVHNode::traverseBVH(o, d, &t, &hi, s->bvh->m_BVHPool, prims, s->list);
      hit[i] = hi;
      tout[i] = t;
    }
  });
}

void ctref_free(void* h) {
  auto* s = (RefScene*)h;
  delete s->mbvh;
  delete s->bvh;
  delete s->pool;
  delete s;
}

/* Primary rays exactly as Camera::generateRay(float(x), float(y)) makes them for
 * a camera at pos looking down -z (the constructor's forward, Camera.cpp:11). */
void ctref_camera_rays(const float* pos, float fov_deg, int w, int h, float* org_out, float* dir_out) {
  core::Camera cam(w, h, fov_deg, ROTATION_SPEED, glm::vec3(pos[0], pos[1], pos[2]));
  for (int y = 0; y < h; y++)
    for (int x = 0; x < w; x++) {
      const Ray r = cam.generateRay(float(x), float(y));
      const size_t i = (size_t)y * w + x;
      for (int k = 0; k < 3; k++) {
        org_out[3 * i + k] = r.origin[k];
        dir_out[3 * i + k] = r.direction[k];
      }
    }
}

float ctref_camera_plane_distance(float fov_deg) {
  core::Camera cam(4, 4, fov_deg, ROTATION_SPEED, glm::vec3(0.0f));
  return cam.getPlaneDistance();
}

/* ---- known-answer helpers over the reference's __host__ __device__ math ---- */

uint32_t ctref_wang_hash(uint32_t s) { return WangHash(s); }

void ctref_random_stream(uint32_t seed, int n, uint32_t* ints, float* floats) {
  uint32_t s = seed, s2 = seed;
  for (int i = 0; i < n; i++) {
    if (ints) ints[i] = RandomInt(s);
    if (floats) floats[i] = RandomFloat(s2);
  }
}

int ctref_random_int_max(uint32_t* seed, int maxv) { return RandomIntMax(*seed, maxv); }

int ctref_triangle_intersect(const float* o, const float* d, float* t, const float* p0, const float* p1,
                             const float* p2, float eps) {
  return triangle::intersect(glm::vec3(o[0], o[1], o[2]), glm::vec3(d[0], d[1], d[2]), t,
                             glm::vec3(p0[0], p0[1], p0[2]), glm::vec3(p1[0], p1[1], p1[2]),
                             glm::vec3(p2[0], p2[1], p2[2]), eps)
             ? 1
             : 0;
}

void ctref_triangle_bounds(const float* p0, const float* p1, const float* p2, float* mn, float* mx) {
  const AABB b = triangle::getBounds(glm::vec3(p0[0], p0[1], p0[2]), glm::vec3(p1[0], p1[1], p1[2]),
                                     glm::vec3(p2[0], p2[1], p2[2]));
  for (int k = 0; k < 3; k++) mn[k] = b.bmin[k], mx[k] = b.bmax[k];
}

void ctref_bary(const float* p, const float* n, const float* p0, const float* p1, const float* p2, float* out) {
  const glm::vec3 b = triangle::getBaryCoords(glm::vec3(p[0], p[1], p[2]), glm::vec3(n[0], n[1], n[2]),
                                              glm::vec3(p0[0], p0[1], p0[2]), glm::vec3(p1[0], p1[1], p1[2]),
                                              glm::vec3(p2[0], p2[1], p2[2]));
  out[0] = b.x, out[1] = b.y, out[2] = b.z;
}

float ctref_area(const float* p0, const float* p1, const float* p2) {
  return triangle::getArea(glm::vec3(p0[0], p0[1], p0[2]), glm::vec3(p1[0], p1[1], p1[2]),
                           glm::vec3(p2[0], p2[1], p2[2]));
}

void ctref_random_point(const float* p0, const float* p1, const float* p2, float r1, float r2, float* out) {
  const glm::vec3 q = triangle::getRandomPointOnSurface(glm::vec3(p0[0], p0[1], p0[2]), glm::vec3(p1[0], p1[1], p1[2]),
                                                        glm::vec3(p2[0], p2[1], p2[2]), r1, r2);
  out[0] = q.x, out[1] = q.y, out[2] = q.z;
}

/* The quad-node slab test (MBVHNode.cuh:69-110): packed tmin bits after the
 * sort network, and the per-child hit mask. */
void ctref_mbvh_intersect(const void* node, const float* org, const float* invdir, float t, int32_t* tmini_out,
                          int32_t* result_out) {
  const MBVHNode* n = (const MBVHNode*)node;
  const MBVHHit hit = n->intersect(glm::vec3(org[0], org[1], org[2]), glm::vec3(invdir[0], invdir[1], invdir[2]), &t);
  for (int k = 0; k < 4; k++) {
    tmini_out[k] = hit.tmini[k];
    result_out[k] = hit.result[k] ? 1 : 0;
  }
}

void ctref_local_space(const float* n, float* T, float* B) {
  glm::vec3 t, b;
  convertToLocalSpace(glm::vec3(n[0], n[1], n[2]), &t, &b);
  for (int k = 0; k < 3; k++) T[k] = t[k], B[k] = b[k];
}

void ctref_tangent2world(const float* v, const float* n, float* out) {
  const glm::vec3 r = Tangent2World(glm::vec3(v[0], v[1], v[2]), glm::vec3(n[0], n[1], n[2]));
  out[0] = r.x, out[1] = r.y, out[2] = r.z;
}

void ctref_cos_weighted(float r0, float r1, float* out) {
  const glm::vec3 r = DiffuseReflectionCosWeighted(r0, r1);
  out[0] = r.x, out[1] = r.y, out[2] = r.z;
}

float ctref_fresnel_exact(const float* wo, const float* n, float eta) {
  return FresnelDielectricExact(glm::vec3(wo[0], wo[1], wo[2]), glm::vec3(n[0], n[1], n[2]), eta);
}

/* SampleBSDF (BSDF.h:33): returns the BSDF value; writes wo, pdf and type.
 * type is -1 when the reference leaves it unset (the pdf = 0 exits). */
void ctref_sample_bsdf(const float* color, float roughness, float eta, const float* iN, const float* N, const float* T,
                       const float* B, const float* wi, float r3, float r4, float* f_out, float* wo_out,
                       float* pdf_out, int* type_out) {
  ShadingData d;
  d.color = glm::vec3(color[0], color[1], color[2]);
  d.roughness = roughness;
  d.eta = eta;
  glm::vec3 wo(0.0f);
  float pdf = -1.0f;
  BSDFType type = (BSDFType)-1;
  const glm::vec3 f = SampleBSDF(d, glm::vec3(iN[0], iN[1], iN[2]), glm::vec3(N[0], N[1], N[2]),
                                 glm::vec3(T[0], T[1], T[2]), glm::vec3(B[0], B[1], B[2]),
                                 glm::vec3(wi[0], wi[1], wi[2]), r3, r4, wo, pdf, type);
  for (int k = 0; k < 3; k++) f_out[k] = f[k], wo_out[k] = wo[k];
  *pdf_out = pdf;
  *type_out = (int)type;
}

float ctref_roughness_to_alpha(float r) { return microfacet::RoughnessToAlpha(r); }

/* Microfacet dispatch via Material::sample / Material::evaluate
 * (Material.cuh:175-215) for material type `type`. */
void ctref_mf_sample(int type, float ax, float ay, int visibility, const float* wi, float r1, float r2, float* out) {
  Material m = Material::lambertian(glm::vec3(1.0f));
  m.type = (MaterialType)type;
  const microfacet::Microfacet mf(ax, ay, visibility != 0);
  const glm::vec3 r = m.sample(mf, glm::vec3(wi[0], wi[1], wi[2]), r1, r2);
  out[0] = r.x, out[1] = r.y, out[2] = r.z;
}

float ctref_mf_pdf(int type, float ax, float ay, int visibility, const float* wo, const float* wm, const float* wi) {
  Material m = Material::lambertian(glm::vec3(1.0f));
  m.type = (MaterialType)type;
  const microfacet::Microfacet mf(ax, ay, visibility != 0);
  return m.evaluate(mf, glm::vec3(wo[0], wo[1], wo[2]), glm::vec3(wm[0], wm[1], wm[2]),
                    glm::vec3(wi[0], wi[1], wi[2]));
}

int ctref_sizeof_material() { return (int)sizeof(Material); }

}  // extern "C"
