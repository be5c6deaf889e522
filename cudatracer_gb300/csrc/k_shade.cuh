// Ray generation, shading and presentation kernels of the wavefront loop.
//
// This file is compiled twice: k_shade_exact.cu (-fmad=false, sin/cos/atan2/
// acos from portable_math.h: reproducible bit for bit by the CPU oracle) and
// k_shade_fast.cu (FMA contraction and CUDA's float transcendentals).
// CT_SHADE_NS names the namespace, CT_EXACT selects the math.
//
// Compat shading restates the reference's `shade` kernel
// (src/CUDA/Kernel.cu:88-206) with its BSDF (src/Core/BSDF.h:26-63): every
// non-emitter is shaded by roughness (mirror below 0.1, cosine-weighted
// Lambert otherwise) and next-event estimation samples one light triangle
// with the balance heuristic. Surviving paths and shadow rays are appended to
// their queues with one atomic per warp (ballot + popcount prefix) instead of
// the reference's per-thread atomicAdd.
#pragma once

#include "bsdf_full.cuh"
#include "ct_internal.h"
#include "portable_math.h"
#include "vmath.cuh"

#ifndef CT_MODE_FULL
#define CT_MODE_FULL 1     // CT_SHADE_FULL in include/cudatracer.h
#define CT_TEX_BILINEAR_ 1  // CT_TEX_BILINEAR in include/cudatracer.h
#endif

#ifndef CT_SHADE_NS
#error "define CT_SHADE_NS"
#endif

namespace ct {
namespace CT_SHADE_NS {

constexpr float kMaxDistance = 1e34f;
constexpr float kOneOverPi = 0.318309886183790671537767526745028724f;
constexpr float kTwoPi = 6.28318530717958647692528676655900576f;
constexpr int kBlock = 128;

#if CT_EXACT
// reproducible binary32 functions (portable_math.h): the oracle evaluates the
// same operations on the host, so exact frames agree bit for bit
__device__ __forceinline__ float xsin(float x) { return pm::sin(x); }
__device__ __forceinline__ float xcos(float x) { return pm::cos(x); }
__device__ __forceinline__ float xatan2(float y, float x) { return pm::atan2(y, x); }
__device__ __forceinline__ float xacos(float x) { return pm::acos(x); }
#else
__device__ __forceinline__ float xsin(float x) { return sinf(x); }
__device__ __forceinline__ float xcos(float x) { return cosf(x); }
__device__ __forceinline__ float xatan2(float y, float x) { return atan2f(y, x); }
__device__ __forceinline__ float xacos(float x) { return acosf(x); }
#endif

// ---- RNG: src/Core/Random.cuh:10-34 ----
__device__ __forceinline__ uint32_t wang_hash(uint32_t s) {
  s = (s ^ 61u) ^ (s >> 16);
  s *= 9u;
  s = s ^ (s >> 4);
  s *= 0x27d4eb2du;
  s = s ^ (s >> 15);
  return s;
}
__device__ __forceinline__ uint32_t rnd_int(uint32_t& s) {
  s ^= s << 13;
  s ^= s << 17;
  s ^= s << 5;
  return s;
}
__device__ __forceinline__ float rnd_float(uint32_t& s) { return (float)rnd_int(s) * 2.3283064365387e-10f; }
__device__ __forceinline__ int rnd_int_max(uint32_t& s, int maxv) {
  return (int)(rnd_float(s) * ((float)maxv + 0.99999f));
}

// Texel grid of SceneData::getTextureColor (src/Core/SceneData.cuh:81-97):
// coordinate u*(width-1). For finite uv the nearest texel is the reference's
// index; NaN or out-of-range values are clamped to the texture instead of
// reading past it. CT_TEX_BILINEAR blends the four texels around the same
// grid point, clamped at the last row and column: a + (b - a) * t per axis.
__device__ __forceinline__ float grid_coord(float x, uint32_t n) {
  const float g = x * (float)(n - 1);
  return g >= 0.0f ? fminf(g, (float)(n - 1)) : 0.0f;
}
__device__ __forceinline__ float4 lerp4(const float4& a, const float4& b, float t) {
  return make_float4(a.x + (b.x - a.x) * t, a.y + (b.y - a.y) * t, a.z + (b.z - a.z) * t, a.w + (b.w - a.w) * t);
}
__device__ __forceinline__ float4 texel_at(const DevScene& sc, int tex, float x, float y, int filter) {
  const uint2 dim = __ldg(sc.tex_dims + tex);
  const float4* t = sc.texels + __ldg(sc.tex_offsets + tex);
  const float gx = grid_coord(x, dim.x), gy = grid_coord(y, dim.y);
  const uint32_t ix = (uint32_t)gx, iy = (uint32_t)gy;
  if (filter != CT_TEX_BILINEAR_) return __ldg(t + (ix + iy * dim.x));
  const uint32_t ix1 = min(ix + 1, dim.x - 1), iy1 = min(iy + 1, dim.y - 1);
  const float tx = gx - (float)ix, ty = gy - (float)iy;
  const float4 c00 = __ldg(t + (ix + iy * dim.x)), c10 = __ldg(t + (ix1 + iy * dim.x));
  const float4 c01 = __ldg(t + (ix + iy1 * dim.x)), c11 = __ldg(t + (ix1 + iy1 * dim.x));
  return lerp4(lerp4(c00, c10, tx), lerp4(c01, c11, tx), ty);
}
__device__ __forceinline__ float4 tex_color(const DevScene& sc, int tex, float u, float v, int filter) {
  float x = fmodf(u, 1.0f), y = fmodf(v, 1.0f);
  if (x < 0) x += 1.0f;
  if (y < 0) y += 1.0f;
  return texel_at(sc, tex, x, y, filter);
}
// SceneData::getTextureNormal (src/Core/SceneData.cuh:99-116): no wrap, only +1 for negatives
__device__ __forceinline__ V3 tex_normal(const DevScene& sc, int tex, float u, float v, int filter) {
  float x = u, y = v;
  if (x < 0) x += 1.0f;
  if (y < 0) y += 1.0f;
  return normalize(v3(texel_at(sc, tex, x, y, filter)));
}
// convertToLocalSpace (src/Core/Random.cuh:37-42) + localToWorld
__device__ __forceinline__ V3 sample_to_world(V3 s, V3 n) {
  const V3 W = fabsf(n.x) > 0.99f ? v3(0.0f, 1.0f, 0.0f) : v3(1.0f, 0.0f, 0.0f);
  const V3 T = normalize(cross(n, W));
  const V3 B = cross(n, T);
  return (T * s.x + B * s.y) + n * s.z;
}

__device__ __forceinline__ void accum_add(float4* accum, int pix, V3 c) {
  float4 a = accum[pix];
  a.x += c.x;
  a.y += c.y;
  a.z += c.z;
  a.w += 1.0f;
  accum[pix] = a;
}

// A compat-shading contribution: added to the job's buffer, or, for an exact
// frame in a slot, stored in this launch's log entry (DevQueues::log).
__device__ __forceinline__ void add_contribution(const DevQueues& q, float4* acc, int pix, int pix_base, V3 c) {
  if (q.log) {
    q.log[(size_t)q.log_entry * q.capacity + pix] = make_float4(c.x, c.y, c.z, __uint_as_float(q.log_tag));
    return;
  }
  accum_add(acc ? acc : q.accum, acc ? pix - pix_base : pix, c);
}

// Heron's formula, triangle::getArea (src/Core/Triangle.cuh:89-95)
__device__ __forceinline__ float tri_area(V3 p0, V3 p1, V3 p2) {
  const float a = length(p0 - p1), b = length(p1 - p2), c = length(p2 - p0);
  const float s = ((a + b) + c) / 2.f;
  return sqrtf(((s * (s - a)) * (s - b)) * (s - c));
}

struct Emit {
  bool cont, shadow;
  float4 no, nd, nt;  // continuation ray
  float4 so, sd, sc;  // shadow ray
};

// One ray of the compat shade stage.
// pix_base: first pixel of the job in a batch (0 for a single job); seeds use
// the job's own pixel index so a job renders the same alone and in a batch.
// acc: where the job's pixels accumulate (q.accum when null); indexed by pix - pix_base.
// A hit triangle's shading inputs from its 128-byte record (DevScene::shade_rec):
// eight independent 16-byte loads of one line.
struct TriRec {
  V3 p0, p1, p2, n0, n1, n2, cn;
  float2 uv0, uv1, uv2;
  uint32_t mat;
};
__device__ __forceinline__ TriRec load_tri(const DevScene& sc, int prim) {
  const float4* r = sc.shade_rec + 8 * (size_t)prim;
  const float4 a = __ldg(r), b = __ldg(r + 1), c = __ldg(r + 2), d = __ldg(r + 3);
  const float4 e = __ldg(r + 4), g = __ldg(r + 5), k = __ldg(r + 6), m = __ldg(r + 7);
  TriRec t;
  t.p0 = v3(a), t.p1 = v3(b), t.p2 = v3(c);
  t.n0 = v3(d), t.n1 = v3(e), t.n2 = v3(g), t.cn = v3(k);
  t.uv0 = make_float2(d.w, e.w), t.uv1 = make_float2(g.w, k.w), t.uv2 = make_float2(m.x, m.y);
  t.mat = __float_as_uint(a.w);
  return t;
}

__device__ __forceinline__ void shade_compat(const DevScene& sc, const DevQueues& q, const FrameConst& f, int cur,
                                             int i, uint32_t path_length, Emit& e, int pix_base = 0,
                                             float4* acc = nullptr) {
  const float4 o4 = q.org_q(cur)[i], d4 = q.dir_q(cur)[i], t4 = q.thr_q(cur)[i];
  const int2 h = q.hit[i];
  const int pix = __float_as_int(o4.w);
  V3 org = v3(o4), dir = v3(d4), T = v3(t4);
  const float last_pdf = t4.w;
  const bool last_specular = __float_as_int(d4.w) == 0;
  const float t = __int_as_float(h.y);
  if (!(t < kMaxDistance)) {
    if (f.sky && sc.sky_tex >= 0) {
      const float u = 1.0f + (xatan2(dir.x, -dir.z) * kOneOverPi) * 0.5f;
      const float v = 1.0f - xacos(dir.y) * kOneOverPi;
      const float4 tc = tex_color(sc, sc.sky_tex, u, v, f.tex_filter);
      add_contribution(q, acc, pix, pix_base, (T / last_pdf) * v3(tc));
    }
    return;
  }
  const int prim = h.x;
  const TriRec tri = load_tri(sc, prim);
  V3 N = tri.cn;
  const V3 p0 = tri.p0, p1 = tri.p1, p2 = tri.p2;
  // triangle::getBaryCoords at the ray ORIGIN, before it moves (Kernel.cu:107)
  const float aABC = dot(N, cross(p1 - p0, p2 - p0));
  const float aPBC = dot(N, cross(p1 - org, p2 - org));
  const float aPCA = dot(N, cross(p2 - org, p0 - org));
  const float ba = aPBC / aABC, bb = aPCA / aABC, bc = (1.f - ba) - bb;
  V3 iN = (tri.n0 * ba + tri.n1 * bb) + tri.n2 * bc;
  const float2 uv0 = tri.uv0, uv1 = tri.uv1, uv2 = tri.uv2;
  const float tu = (uv0.x * ba + uv1.x * bb) + uv2.x * bc;
  const float tv = (uv0.y * ba + uv1.y * bb) + uv2.y * bc;
  const DevMaterial* mp = sc.mats + tri.mat;
  const float4 alb = __ldg(&mp->albedo_ior);
  const int4 mtex = __ldg(&mp->tex);
  const float4 tr = __ldg(&mp->type_rough);
  const int mtype = __float_as_int(tr.x);
  if (mtex.y >= 0) iN = sample_to_world(tex_normal(sc, mtex.y, tu, tv, f.tex_filter), iN);
  if (mtype == 0) {  // emitter (Kernel.cu:114-136)
    if (!f.indirect) return;
    const float DdotNL = -dot(dir, iN);
    V3 c;
    if (last_specular) {
      c = T * v3(alb);
    } else {
      const float lightPDF = ((t * t) / (DdotNL * tri_area(p0, p1, p2))) * (float)sc.light_count;
      c = (T * v3(alb)) * (1.0f / (last_pdf + lightPDF));
    }
    add_contribution(q, acc, pix, pix_base, vmax0(c));
    return;
  }
  org = org + dir * t;  // getHitpoint
  T = vmax0(T / last_pdf);
  const float flip = dot(dir, N) > 0 ? -1.0f : 1.0f;
  N = N * flip;
  iN = iN * flip;
  uint32_t seed = wang_hash((uint32_t)(pix - pix_base) * 16789u + f.frame * 1791u + path_length * 720898027u);
  V3 color = v3(alb);
  if (mtex.x >= 0) color = v3(tex_color(sc, mtex.x, tu, tv, f.tex_filter));
  // SampleBSDF (BSDF.h:33-63); its two random numbers are drawn left to right
  const float r3 = rnd_float(seed), r4 = rnd_float(seed);
  V3 wo, fval;
  float pdf;
  // diffuse: the reference's reflectedType == DIFFUSE. A failed sample (pdf = 0) leaves the
  // type unset; the reference's GPU build then runs no NEE, and the path ends here either way.
  bool diffuse;
  if (tr.y < 0.1f) {
    wo = dir - (iN * dot(iN, dir)) * 2.0f;  // reflect(-wi, iN)
    diffuse = false;
    if (dot(N, wo) <= 0.0f) {
      pdf = 0.0f;
      fval = v3(0, 0, 0);
    } else {
      pdf = 1.0f;
      fval = color * (1.0f / fabsf(dot(iN, wo)));
    }
  } else {
    // DiffuseReflectionCosWeighted (Tools.h:162-169): sqrt(1.0 - r1) in double
    const float term1 = kTwoPi * r3;
    const float term2 = (float)sqrt(1.0 - (double)r4);
    const float sn = xsin(term1), cs = xcos(term1);
    const V3 vl = v3(cs * term2, sn * term2, sqrtf(r4));
    // Tangent2World (Tools.h:110-137)
    V3 B, Tt;
    const V3 n = iN;
    if (n.z < 0.) {
      const float a = 1.0f / (1.0f - n.z);
      const float b = (n.x * n.y) * a;
      B = v3(1.0f - (n.x * n.x) * a, -b, n.x);
      Tt = v3(b, (n.y * n.y) * a - 1.0f, -n.y);
    } else {
      const float a = 1.0f / (1.0f + n.z);
      const float b = (-n.x * n.y) * a;
      B = v3(1.0f - (n.x * n.x) * a, b, -n.x);
      Tt = v3(b, 1.0f - (n.y * n.y) * a, -n.y);
    }
    wo = normalize((Tt * vl.x + B * vl.y) + n * vl.z);
    diffuse = dot(N, wo) > 0.0f;
    if (!diffuse) {
      pdf = 0.0f;
      fval = v3(0, 0, 0);
    } else {
      pdf = gmax(0.0f, dot(wo, iN)) * kOneOverPi;
      fval = color * kOneOverPi;
    }
  }
  bool specular_next = !diffuse;
  dir = wo;
  if (diffuse && f.shadow && sc.light_count > 0) {
    // RandomIntMax; clamped because float rounding can reach light_count above 2^24 lights
    const int light = min(rnd_int_max(seed, (int)sc.light_count - 1), (int)sc.light_count - 1);
    const uint32_t lprim = __ldg(sc.lights + light);
    const uint4 li = __ldg(sc.idx + lprim);
    const V3 l0 = v3(__ldg(sc.verts + li.x)), l1 = v3(__ldg(sc.verts + li.y)), l2 = v3(__ldg(sc.verts + li.z));
    float q1 = rnd_float(seed), q2 = rnd_float(seed);
    if (q1 + q2 > 1.0f) q1 = 1.0f - q1, q2 = 1.0f - q2;  // getRandomPointOnSurface
    const float qa = (1.0f - q1) - q2;
    const V3 lp = (l0 * qa + l1 * q1) + l2 * q2;
    V3 L = lp - org;
    const float sq = dot(L, L);
    const float dist = sqrtf(sq);
    L = L / dist;
    const V3 lN = v3(__ldg(sc.cnormals + lprim));
    const float NdotL = dot(iN, L);
    const float LNdotL = -dot(lN, L);
    if (NdotL > 0 && LNdotL > 0) {
      const float area = tri_area(l0, l1, l2);
      // emission of material m_MaterialIdxs[light]: the light-LIST index (Kernel.cu:178)
      const uint32_t em_mat = __ldg(&sc.idx[light].w);
      const V3 em = v3(__ldg(&sc.mats[em_mat].albedo_ior));
      const float shadowPDF = fabsf(dot(L, iN)) * kOneOverPi;  // EvaluateBSDF (BSDF.h:26-31)
      const V3 sb = color * kOneOverPi;
      if (shadowPDF > 0) {
        const float lightPDF = (sq / (LNdotL * area)) * (float)sc.light_count;
        const V3 scol = ((T * em) * sb) * (NdotL / (shadowPDF + lightPDF));
        e.shadow = true;
        e.so = f4(org + L * f.normal_eps, __int_as_float(pix));
        e.sd = f4(L, dist - 2.0f * f.dist_eps);
        e.sc = f4(scol, 0.0f);
      }
    }
    specular_next = false;
  }
  if (pdf < 1e-6f || isnan(pdf) || isnan(T.x) || isnan(T.y) || isnan(T.z) ||
      (T.x <= 0.0f && T.y <= 0.0f && T.z <= 0.0f))
    return;
  T = vmax0((T * fval) * fabsf(dot(iN, dir)));
  org = org + N * f.normal_eps;
  e.cont = true;
  e.no = f4(org, __int_as_float(pix));
  e.nd = f4(dir, __int_as_float(specular_next ? 0 : 1));
  e.nt = f4(T, pdf);
}

// ---------------------------------------------------------------------------
// CT_SHADE_FULL: every material type of the reference's Material record
// (bsdf_full.cuh), next-event estimation for the non-delta reflective lobes,
// power-heuristic MIS between light sampling and BSDF sampling. Unlike compat
// mode the geometry is taken at the hit point: barycentrics of the hit, a
// normalised interpolated normal, the face normal for ray offsets, and the
// emitter's own material for NEE.
//   ray flags (dir.w bits): 2 = the previous vertex sampled a light, so an
//   emitter hit is weighted against the light-sampling density
//   throughput.w: solid-angle density of the sampled direction
// ---------------------------------------------------------------------------
constexpr int kFlagMis = 2;
constexpr float kShadowRel = 1e-4f;  // shadow rays end at dist * (1 - kShadowRel) - 2 * dist_eps

// orthonormal basis around n (Duff et al. 2017)
__device__ __forceinline__ void onb(V3 n, V3& t, V3& b) {
  const float sign = copysignf(1.0f, n.z);
  const float a = -1.0f / (sign + n.z);
  const float bb = n.x * n.y * a;
  t = v3(1.0f + sign * n.x * n.x * a, sign * bb, -sign * n.x);
  b = v3(bb, sign + n.y * n.y * a, -n.y);
}

__device__ __forceinline__ void shade_full(const DevScene& sc, const DevQueues& q, const FrameConst& f, int cur, int i,
                                           uint32_t path_length, Emit& e, int pix_base = 0,
                                           float4* acc = nullptr) {
  const float4 o4 = q.org_q(cur)[i], d4 = q.dir_q(cur)[i], t4 = q.thr_q(cur)[i];
  const int2 h = q.hit[i];
  const int pix = __float_as_int(o4.w);
  const V3 dir = v3(d4);
  V3 T = v3(t4);
  const float last_pdf = t4.w;
  const int flags = __float_as_int(d4.w);
  const float t = __int_as_float(h.y);
  if (!(t < kMaxDistance)) {
    if (f.sky && sc.sky_tex >= 0) {
      const float u = 1.0f + (xatan2(dir.x, -dir.z) * kOneOverPi) * 0.5f;
      const float v = 1.0f - xacos(fminf(fmaxf(dir.y, -1.0f), 1.0f)) * kOneOverPi;
      accum_add(acc ? acc : q.accum, acc ? pix - pix_base : pix, T * v3(tex_color(sc, sc.sky_tex, u, v, f.tex_filter)));
    }
    return;
  }
  const int prim = h.x;
  const TriRec tri = load_tri(sc, prim);
  const V3 p0 = tri.p0, p1 = tri.p1, p2 = tri.p2;
  const V3 p = v3(o4) + dir * t;
  V3 Ngf = cross(p1 - p0, p2 - p0);
  const float area2 = sqrtf(dot(Ngf, Ngf));
  Ngf = Ngf * (1.0f / area2);
  // barycentrics of the hit point
  const float b1 = dot(Ngf, cross(p2 - p, p0 - p)) / area2, b2 = dot(Ngf, cross(p0 - p, p1 - p)) / area2;
  const float b0 = 1.0f - b1 - b2;
  V3 Ns = tri.n0 * b0 + tri.n1 * b1 + tri.n2 * b2;
  const float nl = dot(Ns, Ns);
  Ns = nl > 0.0f ? Ns * (1.0f / sqrtf(nl)) : Ngf;
  const float2 uv0 = tri.uv0, uv1 = tri.uv1, uv2 = tri.uv2;
  const float tu = uv0.x * b0 + uv1.x * b1 + uv2.x * b2, tv = uv0.y * b0 + uv1.y * b1 + uv2.y * b2;
  const DevMaterial* mp = sc.mats + tri.mat;
  const float4 alb = __ldg(&mp->albedo_ior);
  const int4 mtex = __ldg(&mp->tex);
  const float4 tr = __ldg(&mp->type_rough);
  const int mtype = __float_as_int(tr.x);
  if (mtex.y >= 0) Ns = normalize(sample_to_world(tex_normal(sc, mtex.y, tu, tv, f.tex_filter), Ns));
  if (mtype == full::kLight) {
    if (!f.indirect) return;
    // emitters radiate on the side their centre normal faces (as the reference's NEE assumes)
    const V3 cn = normalize(tri.cn);
    const float cos_l = -dot(cn, dir);
    if (cos_l <= 0.0f) return;
    float w = 1.0f;
    if ((flags & kFlagMis) && sc.light_count > 0) {
      const float light_pdf = (t * t) / (cos_l * 0.5f * area2 * (float)sc.light_count);
      w = (last_pdf * last_pdf) / (last_pdf * last_pdf + light_pdf * light_pdf);
    }
    accum_add(acc ? acc : q.accum, acc ? pix - pix_base : pix, vmax0(T * v3(alb) * w));
    return;
  }
  const bool dielectric = full::is_dielectric(mtype);
  const bool front = dot(dir, Ngf) < 0.0f;
  const V3 Ng = front ? Ngf : -Ngf;  // faces the incoming ray
  // shading frame: towards the incoming ray for reflectors, outward for dielectrics
  V3 N = dielectric ? (dot(Ns, Ngf) < 0.0f ? -Ns : Ns) : (dot(Ns, Ng) < 0.0f ? -Ns : Ns);
  V3 Tt, Bt;
  onb(N, Tt, Bt);
  const V3 wo = -dir;
  const V3 wo_l = v3(dot(wo, Tt), dot(wo, Bt), dot(wo, N));
  V3 color = v3(alb);
  if (mtex.x >= 0) color = v3(tex_color(sc, mtex.x, tu, tv, f.tex_filter));
  uint32_t seed = wang_hash((uint32_t)(pix - pix_base) * 16789u + f.frame * 1791u + path_length * 720898027u);
  const float u1 = rnd_float(seed), u2 = rnd_float(seed), u3 = rnd_float(seed);
  const float rough = tr.y;
  const float alpha = full::roughness_to_alpha(rough);
  bool nee = false;
  if (full::has_nee(mtype) && f.shadow && sc.light_count > 0 && wo_l.z > 0.0f) {
    nee = true;
    const int light = min(rnd_int_max(seed, (int)sc.light_count - 1), (int)sc.light_count - 1);
    const uint32_t lprim = __ldg(sc.lights + light);
    const uint4 li = __ldg(sc.idx + lprim);
    const V3 l0 = v3(__ldg(sc.verts + li.x)), l1 = v3(__ldg(sc.verts + li.y)), l2 = v3(__ldg(sc.verts + li.z));
    float q1 = rnd_float(seed), q2 = rnd_float(seed);
    if (q1 + q2 > 1.0f) q1 = 1.0f - q1, q2 = 1.0f - q2;
    const V3 lp = l0 * (1.0f - q1 - q2) + l1 * q1 + l2 * q2;
    V3 L = lp - p;
    const float sq = dot(L, L);
    const float dist = sqrtf(sq);
    L = L * (1.0f / dist);
    const V3 lcn = normalize(v3(__ldg(sc.cnormals + lprim)));
    const float cos_l = -dot(lcn, L);
    const V3 lc = cross(l1 - l0, l2 - l0);
    const float larea = 0.5f * sqrtf(dot(lc, lc));
    if (cos_l > 0.0f && dot(Ng, L) > 0.0f && larea > 0.0f) {
      const V3 wi_l = v3(dot(L, Tt), dot(L, Bt), dot(L, N));
      float pb;
      const V3 fv = full::eval(mtype, color, alpha, wo_l, wi_l, pb);
      if (pb > 0.0f) {
        const float light_pdf = sq / (cos_l * larea * (float)sc.light_count);
        const float w = (light_pdf * light_pdf) / (light_pdf * light_pdf + pb * pb);
        const V3 le = v3(__ldg(&sc.mats[__ldg(&sc.idx[lprim].w)].albedo_ior));
        const V3 contrib = T * fv * le * (wi_l.z * w / light_pdf);
        if (contrib.x > 0.0f || contrib.y > 0.0f || contrib.z > 0.0f) {
          e.shadow = true;
          e.so = f4(p + Ng * f.normal_eps, __int_as_float(pix));
          // stop short of the light by a relative margin as well: at distances of tens of
          // units the light's own FP32 hit distance can fall inside an absolute 2 * dist_eps
          e.sd = f4(L, dist * (1.0f - kShadowRel) - 2.0f * f.dist_eps);
          e.sc = f4(contrib, 0.0f);
        }
      }
    }
  }
  const full::Sample s = full::sample(mtype, color, rough, alb.w, wo_l, u1, u2, u3);
  if (!s.valid) return;
  const V3 wi = Tt * s.wi.x + Bt * s.wi.y + N * s.wi.z;
  T = T * s.weight;
  if (isnan(T.x) || isnan(T.y) || isnan(T.z) || (T.x <= 0.0f && T.y <= 0.0f && T.z <= 0.0f)) return;
  const float side = dot(wi, Ngf) > 0.0f ? 1.0f : -1.0f;
  e.cont = true;
  e.no = f4(p + Ngf * (side * f.normal_eps), __int_as_float(pix));
  e.nd = f4(wi, __int_as_float((nee && !s.delta) ? kFlagMis : 0));
  e.nt = f4(T, s.pdf);
}

// Warp-aggregated append: one atomicAdd per warp, lanes take popc-prefix slots.
__device__ __forceinline__ int warp_append(bool want, int* counter) {
  const unsigned m = __ballot_sync(0xffffffffu, want);
  if (m == 0) return -1;
  const int lane = threadIdx.x & 31;
  int base = 0;
  if (lane == __ffs(m) - 1) base = atomicAdd(counter, __popc(m));
  base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
  return want ? base + __popc(m & ((1u << lane) - 1u)) : -1;
}

__global__ void __launch_bounds__(kBlock) k_shade(DevScene sc, DevQueues q, FrameConst f, int cur,
                                                   uint32_t path_length) {
  const int n = q.counts[cur];
  const int nxt = cur ^ 1;
  if (blockIdx.x == 0 && threadIdx.x == 0) q.counts[4] = 0;  // fetch cursor of the next extend
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * kBlock;
  for (int base = blockIdx.x * kBlock + (threadIdx.x & ~31); base < n; base += stride) {
    const int i = base + lane;
    Emit e;
    e.cont = false;
    e.shadow = false;
    if (i < n) {
      if (f.shading_mode == CT_MODE_FULL)
        shade_full(sc, q, f, cur, i, path_length, e);
      else
        shade_compat(sc, q, f, cur, i, path_length, e);
    }
    const int si = warp_append(e.shadow, &q.counts[2]);
    if (si >= 0) {
      q.sorg[si] = e.so;
      q.sdir[si] = e.sd;
      q.scol[si] = e.sc;
    }
    const int ci = warp_append(e.cont, &q.counts[nxt]);
    if (ci >= 0) {
      q.org_q(nxt)[ci] = e.no;
      q.dir_q(nxt)[ci] = e.nd;
      q.thr_q(nxt)[ci] = e.nt;
    }
  }
}

// generatePrimaryRays + Ray::generate (Kernel.cu:208-234, Ray.cuh:85-95) with
// start_position = 0: buffer index == pixel.
// Pixel of primary-queue slot j: 8x4 tiles in row-major tile order over the
// largest region whose sides are multiples of 8 and 4, then the right strip and
// the bottom strip row by row. A bijection on [0, w*h): each warp's 32 rays
// cover one compact tile, so they traverse alike; ray results are per pixel,
// so the order changes no result.
__device__ __forceinline__ int tile_pixel(int j, int w, int h) {
  const int w8 = w & ~7, h4 = h & ~3;
  const int main = w8 * h4;
  if (j < main) {
    const int t = j >> 5, k = j & 31, tiles_x = w8 >> 3;
    const int x = ((t % tiles_x) << 3) + (k & 7), y = ((t / tiles_x) << 2) + (k >> 3);
    return y * w + x;
  }
  j -= main;
  const int rw = w - w8, right = rw * h4;
  if (j < right) return (j / rw) * w + w8 + j % rw;
  j -= right;
  return (h4 + j / w) * w + j % w;
}

__global__ void __launch_bounds__(kBlock) k_raygen(DevQueues q, FrameConst f) {
  const int npix = f.width * f.height;
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    q.counts[0] = npix;
    q.counts[4] = 0;  // fetch cursor of the first extend
    atomicAdd(&q.stats[2], (unsigned long long)npix);
    atomicAdd(&q.stats[3], 1ull);
  }
  const float invw = 1.0f / (float)f.width, invh = 1.0f / (float)f.height;
  const V3 w = v3(f.cam_w.x, f.cam_w.y, f.cam_w.z), hor = v3(f.hor.x, f.hor.y, f.hor.z),
           ver = v3(f.ver.x, f.ver.y, f.ver.z);
  for (int j = blockIdx.x * kBlock + threadIdx.x; j < npix; j += gridDim.x * kBlock) {
    const int i = tile_pixel(j, f.width, f.height);
    uint32_t seed = ((uint32_t)i + f.frame * 147565741u) * 720898027u;
    const int x = i % f.width, y = (i / f.width) % f.height;
    const float px = ((float)x + rnd_float(seed)) - 0.5f;
    const float py = ((float)y + rnd_float(seed)) - 0.5f;
    const float sx = 2.0f * (px * invw) - 1.0f;
    const float sy = 1.0f - 2.0f * (py * invh);
    const V3 p = (w + hor * sx) + ver * sy;
    q.org_q(0)[j] = make_float4(f.cam_pos.x, f.cam_pos.y, f.cam_pos.z, __int_as_float(i));
    q.dir_q(0)[j] = f4(normalize(p), __int_as_float(0));  // lastBounceType = SPECULAR
    q.thr_q(0)[j] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);  // throughput 1, lastBsdfPDF 1
  }
}

// ---- batches: one launch per stage for every job (see DevBatch)

// Primary rays of the jobs that still take samples, appended to queue 0.
__global__ void __launch_bounds__(kBlock) k_batch_raygen(DevBatch bt, DevQueues q) {
  if (blockIdx.x == 0 && threadIdx.x == 0) q.counts[4] = 0;
  for (int base = blockIdx.x * kBlock + (threadIdx.x & ~31); base < bt.total_pix; base += gridDim.x * kBlock) {
    const int g = base + (threadIdx.x & 31);
    bool want = false;
    float4 o, d;
    if (g < bt.total_pix) {
      const BatchJob& J = bt.jobs[batch_job_of(bt.bases, bt.n_jobs, g)];
      if (J.spp_left > 0) {
        const FrameConst& f = J.f;
        const int i = tile_pixel(g - J.pix_base, f.width, f.height);  // the job's pixels in 8x4 tiles
        uint32_t seed = ((uint32_t)i + f.frame * 147565741u) * 720898027u;
        const int x = i % f.width, y = (i / f.width) % f.height;
        const float invw = 1.0f / (float)f.width, invh = 1.0f / (float)f.height;
        const float px = ((float)x + rnd_float(seed)) - 0.5f;
        const float py = ((float)y + rnd_float(seed)) - 0.5f;
        const float sx = 2.0f * (px * invw) - 1.0f;
        const float sy = 1.0f - 2.0f * (py * invh);
        const V3 w = v3(f.cam_w.x, f.cam_w.y, f.cam_w.z), hor = v3(f.hor.x, f.hor.y, f.hor.z),
                 ver = v3(f.ver.x, f.ver.y, f.ver.z);
        const V3 p = (w + hor * sx) + ver * sy;
        o = make_float4(f.cam_pos.x, f.cam_pos.y, f.cam_pos.z, __int_as_float(J.pix_base + i));
        d = f4(normalize(p), __int_as_float(0));
        want = true;
      }
    }
    const int k = warp_append(want, &q.counts[0]);
    if (k >= 0) {
      q.org_q(0)[k] = o;
      q.dir_q(0)[k] = d;
      q.thr_q(0)[k] = make_float4(1.0f, 1.0f, 1.0f, 1.0f);
    }
  }
}

// Shade every ray of the batch with its job's scene and frame constants; a
// job's paths stop after its own max_depth passes.
__global__ void __launch_bounds__(kBlock) k_batch_shade(DevBatch bt, DevQueues q, int cur, uint32_t path_length,
                                                        int pass) {
  const int n = q.counts[cur];
  const int nxt = cur ^ 1;
  if (blockIdx.x == 0 && threadIdx.x == 0) q.counts[4] = 0;
  const int lane = threadIdx.x & 31;
  const int stride = gridDim.x * kBlock;
  for (int base = blockIdx.x * kBlock + (threadIdx.x & ~31); base < n; base += stride) {
    const int i = base + lane;
    Emit e;
    e.cont = false;
    e.shadow = false;
    if (i < n) {
      const int pix = __float_as_int(q.org_q(cur)[i].w);
      const BatchJob& J = bt.jobs[batch_job_of(bt.bases, bt.n_jobs, pix)];
      if (J.f.shading_mode == CT_MODE_FULL)
        shade_full(J.sc, q, J.f, cur, i, path_length, e, J.pix_base, J.accum);
      else
        shade_compat(J.sc, q, J.f, cur, i, path_length, e, J.pix_base, J.accum);
      if (pass + 1 >= J.max_depth) e.cont = false;
    }
    const int si = warp_append(e.shadow, &q.counts[2]);
    if (si >= 0) {
      q.sorg[si] = e.so;
      q.sdir[si] = e.sd;
      q.scol[si] = e.sc;
    }
    const int ci = warp_append(e.cont, &q.counts[nxt]);
    if (ci >= 0) {
      q.org_q(nxt)[ci] = e.no;
      q.dir_q(nxt)[ci] = e.nd;
      q.thr_q(nxt)[ci] = e.nt;
    }
  }
}

// End of a batch iteration: each job that took a sample advances its frame
// seed by 2 (launchKernels' samples += 2) and counts the sample; queue 0 is
// emptied for the next raygen.
__global__ void k_batch_advance(DevBatch bt, DevQueues q) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j == 0) {
    q.counts[0] = 0;
    q.counts[4] = 0;
    atomicAdd(&q.stats[3], 1ull);
  }
  if (j >= bt.n_jobs) return;
  BatchJob& J = bt.jobs[j];
  if (J.spp_left > 0) {
    atomicAdd(&q.stats[2], (unsigned long long)(J.f.width * J.f.height));
    J.spp_left -= 1;
    J.f.frame += bt.frame_step;
  }
}

}  // namespace CT_SHADE_NS
}  // namespace ct
