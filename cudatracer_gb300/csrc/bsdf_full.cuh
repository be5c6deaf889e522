// Full-material BSDFs for CT_SHADE_FULL.
//
// The reference defines the material parameters and the microfacet sampling
// routines (src/Core/Material.cuh:29-215, src/Core/Microfacet.cuh:15-565,
// src/Core/Tools.h:96) but its kernel never calls them. This file gives them a
// complete scattering model:
//   Lambertian     cosine-weighted diffuse, f = albedo / pi
//   Specular       perfect mirror tinted by albedo
//   Fresnel        smooth dielectric: reflect with the exact dielectric
//                  Fresnel term, otherwise refract (index refract_idx)
//   Beckmann, GGX, Trowbridge
//                  rough reflector, f = albedo D G2 / (4 |cos_o| |cos_i|) with
//                  separable Smith G2 = G1(wo) G1(wi); alpha from
//                  RoughnessToAlpha (pbrt's fit); Beckmann and GGX sample the
//                  visible normals of wo (Heitz & d'Eon 2014), Trowbridge
//                  samples the full distribution (as the reference's
//                  sample_trowbridge_reitz does)
//   Fresnel*       rough dielectric (Walter et al. 2007) over the same
//                  distributions
// All lobes are evaluated in a local frame whose z axis is the shading normal.
// Sampling returns the throughput weight f |cos| / pdf directly.
#pragma once

#include "vmath.cuh"

namespace ct {
namespace full {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.318309886183790671537767526745028724f;

enum MatType : int {
  kLight = 0, kSpecular = 1, kFresnel = 2, kLambert = 3, kBeckmann = 4, kGGX = 5, kTrowbridge = 6,
  kFresnelBeckmann = 7, kFresnelGGX = 8, kFresnelTrowbridge = 9
};

__device__ __forceinline__ int distribution_of(int type) {
  // 0 Beckmann, 1 GGX (visible normals), 2 Trowbridge-Reitz (full distribution)
  return (type == kBeckmann || type == kFresnelBeckmann) ? 0 : ((type == kGGX || type == kFresnelGGX) ? 1 : 2);
}

// pbrt's roughness -> alpha fit (the reference's RoughnessToAlpha)
__device__ __forceinline__ float roughness_to_alpha(float r) {
  r = fmaxf(r, 1e-3f);
  const float x = logf(r);
  return fminf(1.0f, 1.62142f + 0.819955f * x + 0.1734f * x * x + 0.0171201f * x * x * x +
                         0.000640711f * x * x * x * x);
}

__device__ __forceinline__ float tan2_theta(V3 w) {
  const float c2 = w.z * w.z;
  return fmaxf(0.0f, 1.0f - c2) / c2;
}

// Normal distribution (isotropic alpha)
__device__ __forceinline__ float D(int dist, V3 m, float a) {
  if (m.z <= 0.0f) return 0.0f;
  const float c2 = m.z * m.z, t2 = tan2_theta(m);
  if (isinf(t2)) return 0.0f;
  const float a2 = a * a;
  if (dist == 0) return expf(-t2 / a2) / (kPi * a2 * c2 * c2);
  const float e = 1.0f + t2 / a2;
  return 1.0f / (kPi * a2 * c2 * c2 * e * e);
}

// Smith Lambda
__device__ __forceinline__ float lambda(int dist, V3 w, float a) {
  const float t2 = tan2_theta(w);
  if (isinf(t2)) return 0.0f;
  const float tanv = sqrtf(t2);
  if (tanv == 0.0f) return 0.0f;
  if (dist == 0) {
    const float aa = 1.0f / (a * tanv);
    if (aa >= 1.6f) return 0.0f;
    return (1.0f - 1.259f * aa + 0.396f * aa * aa) / (3.535f * aa + 2.181f * aa * aa);
  }
  return (-1.0f + sqrtf(1.0f + a * a * t2)) * 0.5f;
}
__device__ __forceinline__ float G1(int dist, V3 w, float a) { return 1.0f / (1.0f + lambda(dist, w, a)); }

// Error function (Abramowitz & Stegun 7.1.26) and its inverse (Giles 2010)
__device__ __forceinline__ float erf_as(float x) {
  const float s = x < 0.0f ? -1.0f : 1.0f;
  x = fabsf(x);
  const float t = 1.0f / (1.0f + 0.3275911f * x);
  const float y =
      1.0f - (((((1.061405429f * t - 1.453152027f) * t) + 1.421413741f) * t - 0.284496736f) * t + 0.254829592f) * t *
                 expf(-x * x);
  return s * y;
}
__device__ __forceinline__ float erfinv_giles(float x) {
  x = fminf(fmaxf(x, -0.99999f), 0.99999f);
  float w = -logf((1.0f - x) * (1.0f + x)), p;
  if (w < 5.0f) {
    w -= 2.5f;
    p = 2.81022636e-08f;
    p = 3.43273939e-07f + p * w;
    p = -3.5233877e-06f + p * w;
    p = -4.39150654e-06f + p * w;
    p = 0.00021858087f + p * w;
    p = -0.00125372503f + p * w;
    p = -0.00417768164f + p * w;
    p = 0.246640727f + p * w;
    p = 1.50140941f + p * w;
  } else {
    w = sqrtf(w) - 3.0f;
    p = -0.000200214257f;
    p = 0.000100950558f + p * w;
    p = 0.00134934322f + p * w;
    p = -0.00367342844f + p * w;
    p = 0.00573950773f + p * w;
    p = -0.0076224613f + p * w;
    p = 0.00943887047f + p * w;
    p = 1.00167406f + p * w;
    p = 2.83297682f + p * w;
  }
  return p * x;
}

// Slopes of the visible normals for alpha = 1 (pbrt-v3 sample11 routines).
__device__ __forceinline__ void beckmann_sample11(float cos_i, float u1, float u2, float& sx, float& sy) {
  if (cos_i > 0.9999f) {
    const float r = sqrtf(-logf(1.0f - u1)), ph = 2.0f * kPi * u2;
    sx = r * cosf(ph);
    sy = r * sinf(ph);
    return;
  }
  const float sin_i = sqrtf(fmaxf(0.0f, 1.0f - cos_i * cos_i));
  const float tan_i = sin_i / cos_i, cot_i = 1.0f / tan_i;
  float a = -1.0f, c = erf_as(cot_i);
  const float sample_x = fmaxf(u1, 1e-6f);
  const float theta_i = acosf(cos_i);
  const float fit = 1.0f + theta_i * (-0.876f + theta_i * (0.4265f - 0.0594f * theta_i));
  float b = c - (1.0f + c) * powf(1.0f - sample_x, fit);
  const float sqrt_pi_inv = 0.564189583547756f;
  const float norm = 1.0f / (1.0f + c + sqrt_pi_inv * tan_i * expf(-cot_i * cot_i));
  for (int it = 1; it < 10; it++) {
    if (!(b >= a && b <= c)) b = 0.5f * (a + c);
    const float inv = erfinv_giles(b);
    const float value = norm * (1.0f + b + sqrt_pi_inv * tan_i * expf(-inv * inv)) - sample_x;
    const float deriv = norm * (1.0f - inv * tan_i);
    if (fabsf(value) < 1e-5f) break;
    if (value > 0.0f) c = b; else a = b;
    b -= value / deriv;
  }
  sx = erfinv_giles(b);
  sy = erfinv_giles(2.0f * fmaxf(u2, 1e-6f) - 1.0f);
}

__device__ __forceinline__ void ggx_sample11(float cos_i, float u1, float u2, float& sx, float& sy) {
  if (cos_i > 0.9999f) {
    const float r = sqrtf(u1 / (1.0f - u1)), ph = 2.0f * kPi * u2;
    sx = r * cosf(ph);
    sy = r * sinf(ph);
    return;
  }
  const float sin_i = sqrtf(fmaxf(0.0f, 1.0f - cos_i * cos_i));
  const float tan_i = sin_i / cos_i;
  const float a = 1.0f / tan_i;
  const float g1 = 2.0f / (1.0f + sqrtf(1.0f + 1.0f / (a * a)));
  const float A = 2.0f * u1 / g1 - 1.0f;
  const float tmp = fminf(1.0f / (A * A - 1.0f), 1e10f);
  const float B = tan_i;
  const float Dd = sqrtf(fmaxf(B * B * tmp * tmp - (A * A - B * B) * tmp, 0.0f));
  const float x1 = B * tmp - Dd, x2 = B * tmp + Dd;
  sx = (A < 0.0f || x2 > 1.0f / tan_i) ? x1 : x2;
  float S;
  if (u2 > 0.5f) {
    S = 1.0f;
    u2 = 2.0f * (u2 - 0.5f);
  } else {
    S = -1.0f;
    u2 = 2.0f * (0.5f - u2);
  }
  const float z = (u2 * (u2 * (u2 * 0.27385f - 0.73369f) + 0.46341f)) /
                  (u2 * (u2 * (u2 * 0.093073f + 0.309420f) - 1.0f) + 0.597999f);
  sy = S * z * sqrtf(1.0f + sx * sx);
}

// Sample a microfacet normal around +z for direction wo (wo.z > 0).
__device__ __forceinline__ V3 sample_m(int dist, V3 wo, float a, float u1, float u2) {
  if (dist == 2) {  // full distribution (Trowbridge-Reitz)
    const float t2 = a * a * u1 / (1.0f - u1);
    const float ct = 1.0f / sqrtf(1.0f + t2), st = sqrtf(fmaxf(0.0f, 1.0f - ct * ct)), ph = 2.0f * kPi * u2;
    return v3(st * cosf(ph), st * sinf(ph), ct);
  }
  // stretch, sample slopes, rotate, unstretch (visible normals)
  const V3 ws = normalize(v3(a * wo.x, a * wo.y, wo.z));
  float sx, sy;
  if (dist == 0) beckmann_sample11(ws.z, u1, u2, sx, sy); else ggx_sample11(ws.z, u1, u2, sx, sy);
  const float sin_t = sqrtf(fmaxf(0.0f, 1.0f - ws.z * ws.z));
  const float cp = sin_t == 0.0f ? 1.0f : fminf(fmaxf(ws.x / sin_t, -1.0f), 1.0f);
  const float sp = sin_t == 0.0f ? 0.0f : fminf(fmaxf(ws.y / sin_t, -1.0f), 1.0f);
  const float tx = cp * sx - sp * sy;
  sy = sp * sx + cp * sy;
  sx = tx;
  return normalize(v3(-a * sx, -a * sy, 1.0f));
}

// Density of sample_m's normal m (per solid angle of m).
__device__ __forceinline__ float pdf_m(int dist, V3 wo, V3 m, float a) {
  const float d = D(dist, m, a);
  if (dist == 2) return d * fabsf(m.z);
  return G1(dist, wo, a) * fmaxf(0.0f, dot(wo, m)) * d / fabsf(wo.z);
}

// Exact dielectric Fresnel reflectance for cos_i on the incident side, eta = n_t / n_i.
__device__ __forceinline__ float fresnel_dielectric(float cos_i, float eta) {
  cos_i = fminf(fmaxf(cos_i, 0.0f), 1.0f);
  const float sin2_t = (1.0f - cos_i * cos_i) / (eta * eta);
  if (sin2_t >= 1.0f) return 1.0f;
  const float cos_t = sqrtf(1.0f - sin2_t);
  const float rs = (cos_i - eta * cos_t) / (cos_i + eta * cos_t);
  const float rp = (eta * cos_i - cos_t) / (eta * cos_i + cos_t);
  return 0.5f * (rs * rs + rp * rp);
}

__device__ __forceinline__ V3 reflect_about(V3 wo, V3 m) { return m * (2.0f * dot(wo, m)) - wo; }

// Refract wo (pointing away from the surface, on m's side) through m; eta = n_t / n_i.
__device__ __forceinline__ bool refract_about(V3 wo, V3 m, float eta, V3& wi) {
  const float c = dot(wo, m);
  const float s2 = fmaxf(0.0f, 1.0f - c * c) / (eta * eta);
  if (s2 >= 1.0f) return false;
  const float ct = sqrtf(1.0f - s2);
  wi = (-wo) * (1.0f / eta) + m * (c / eta - ct);
  return true;
}

struct Sample {
  V3 wi;        // local frame
  V3 weight;    // f |cos| / pdf
  float pdf;    // solid-angle density of wi (0 for delta lobes is reported as 1)
  bool delta;   // specular lobe: no NEE, no MIS
  bool valid;
};

__device__ __forceinline__ bool is_dielectric(int type) {
  return type == kFresnel || type == kFresnelBeckmann || type == kFresnelGGX || type == kFresnelTrowbridge;
}
__device__ __forceinline__ bool has_nee(int type) {
  return type == kLambert || type == kBeckmann || type == kGGX || type == kTrowbridge;
}

// Evaluate f and the sampling density for the non-delta reflective lobes (NEE).
__device__ __forceinline__ V3 eval(int type, V3 color, float a, V3 wo, V3 wi, float& pdf) {
  pdf = 0.0f;
  if (wo.z <= 0.0f || wi.z <= 0.0f) return v3(0, 0, 0);
  if (type == kLambert) {
    pdf = wi.z * kInvPi;
    return color * kInvPi;
  }
  const int dist = distribution_of(type);
  V3 m = wo + wi;
  const float l2 = dot(m, m);
  if (l2 == 0.0f) return v3(0, 0, 0);
  m = m * (1.0f / sqrtf(l2));
  const float dm = D(dist, m, a);
  const float g2 = G1(dist, wo, a) * G1(dist, wi, a);
  pdf = pdf_m(dist, wo, m, a) / (4.0f * dot(wo, m));
  return color * (dm * g2 / (4.0f * wo.z * wi.z));
}

// Sample a lobe. wo.z may be negative only for dielectrics (inside the surface).
// eta is the material index (outside medium: vacuum).
__device__ __forceinline__ Sample sample(int type, V3 color, float roughness, float eta, V3 wo, float u1, float u2,
                                         float u3) {
  Sample s;
  s.valid = false;
  s.delta = false;
  s.pdf = 0.0f;
  s.weight = v3(0, 0, 0);
  if (type == kLambert) {
    if (wo.z <= 0.0f) return s;
    const float r = sqrtf(u1), ph = 2.0f * kPi * u2;
    s.wi = v3(r * cosf(ph), r * sinf(ph), sqrtf(fmaxf(0.0f, 1.0f - u1)));
    s.pdf = s.wi.z * kInvPi;
    s.weight = color;
    s.valid = s.wi.z > 0.0f;
    return s;
  }
  if (type == kSpecular) {
    if (wo.z <= 0.0f) return s;
    s.wi = v3(-wo.x, -wo.y, wo.z);
    s.pdf = 1.0f;
    s.delta = true;
    s.weight = color;
    s.valid = true;
    return s;
  }
  const float a = roughness_to_alpha(roughness);
  if (!is_dielectric(type)) {
    if (wo.z <= 0.0f) return s;
    const int dist = distribution_of(type);
    const V3 m = sample_m(dist, wo, a, u1, u2);
    s.wi = reflect_about(wo, m);
    if (s.wi.z <= 0.0f || dot(wo, m) <= 0.0f) return s;
    float pdf;
    const V3 f = eval(type, color, a, wo, s.wi, pdf);
    if (pdf <= 0.0f) return s;
    s.pdf = pdf;
    s.weight = f * (s.wi.z / pdf);
    s.valid = true;
    return s;
  }
  // dielectrics: work on the side wo is on
  const bool entering = wo.z > 0.0f;
  const float etai = entering ? 1.0f : eta, etat = entering ? eta : 1.0f;
  const float rel = etat / etai;
  const V3 wo_s = entering ? wo : -wo;  // wo flipped to +z
  V3 m = v3(0.0f, 0.0f, 1.0f);
  bool smooth = type == kFresnel || roughness < 1e-3f;
  int dist = distribution_of(type);
  if (!smooth) m = sample_m(dist, wo_s, a, u1, u2);
  const float c = dot(wo_s, m);
  if (c <= 0.0f) return s;
  const float F = fresnel_dielectric(c, rel);
  V3 wi_s;
  bool reflect = u3 < F;
  if (!reflect && !refract_about(wo_s, m, rel, wi_s)) reflect = true;
  if (reflect) wi_s = reflect_about(wo_s, m);
  if (reflect ? wi_s.z <= 0.0f : wi_s.z >= 0.0f) return s;
  V3 w = color;
  if (!smooth) {
    // visible-normal sampling: f |cos| / pdf = G1(wi); full-distribution sampling adds |wo.m| / (|wo.z| m.z)
    const float g = G1(dist, wi_s.z < 0.0f ? -wi_s : wi_s, a);
    const float extra = dist == 2 ? G1(dist, wo_s, a) * c / (fabsf(wo_s.z) * m.z) : 1.0f;
    w = w * (g * extra);
  }
  if (!reflect) w = w * (1.0f / (rel * rel));  // radiance scaling across the interface
  s.wi = entering ? wi_s : -wi_s;
  s.pdf = 1.0f;
  s.delta = true;
  s.weight = w;
  s.valid = true;
  return s;
}

}  // namespace full
}  // namespace ct
