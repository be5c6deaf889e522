/*
 * ct_fp64: double-precision Monte Carlo oracle for the full-material shading
 * mode (CT_SHADE_FULL).
 *
 * TEST INFRASTRUCTURE ONLY (loaded by tests/ through oracle/oracle.py). It
 * restates, in double precision and with its own random numbers (splitmix64),
 * the estimator the GPU's full mode computes: pinhole rays jittered inside the
 * pixel, closest hit with the reference's Moller-Trumbore test
 * (src/Core/Triangle.cuh:13-44, absolute determinant epsilon), the material
 * model documented in cudatracer_gb300/csrc/bsdf_full.cuh (Lambert, mirror,
 * smooth/rough dielectric, Beckmann/GGX/Trowbridge-Reitz reflectors with the
 * reference's sampling schemes, src/Core/Microfacet.cuh), one-light NEE with
 * the power heuristic, sky lookups (src/Core/SceneData.cuh:81-97). Converged
 * images from the GPU must agree with it within 3 standard errors.
 *
 * It also holds the FP64 closest-hit / any-hit oracle of the precision
 * extension (fp64_trace): the watertight ray/triangle test of Woop, Benthin
 * and Wald (JCGT 2013) evaluated in double, over the padded quad BVH, nearest
 * t first and the lower primitive id on equal t.
 */
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <thread>
#include <vector>

namespace {

struct D3 {
  double x, y, z;
};
inline D3 d3(double x, double y, double z) { return {x, y, z}; }
inline D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
inline D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
inline D3 operator-(D3 a) { return {-a.x, -a.y, -a.z}; }
inline D3 operator*(D3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
inline D3 mulv(D3 a, D3 b) { return {a.x * b.x, a.y * b.y, a.z * b.z}; }
inline double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline D3 cross(D3 a, D3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
inline D3 normalize(D3 v) { return v * (1.0 / std::sqrt(dot(v, v))); }
inline D3 ld3(const float* p, size_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }
constexpr double kPi = 3.14159265358979323846;

struct Rng {
  uint64_t s;
  double next() {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  }
};

struct Material {  // 52-byte reference record
  float albedo[3];
  float refractIdx;
  int32_t diffuseTex, normalTex, maskTex, displaceTex;
  int32_t type;
  float roughness;
  float absorption[3];
};

struct QNode {
  float bminx[4], bmaxx[4], bminy[4], bmaxy[4], bminz[4], bmaxz[4];
  int32_t childs[4], counts[4];
};

}  // namespace

extern "C" struct Fp64Scene {
  const float* verts;
  const float* normals;
  const float* center_normals;
  const float* uvs;
  const uint32_t* idx;
  const uint32_t* mat_idx;
  const void* materials;
  const uint32_t* lights;
  uint32_t light_count;
  const float* tex;
  const uint32_t* tex_dims;
  const uint32_t* tex_offsets;
  int32_t sky_tex;
  int32_t sky, shadow, indirect;
  float normal_eps, dist_eps, tri_eps;
  const void* qnodes;
  const uint32_t* prims;
  int32_t tex_filter;  // 0 nearest, 1 bilinear
};

namespace {

struct Scene {
  const Fp64Scene* s;
  const Material* m;
  const QNode* q;
};

bool tri_hit(const Scene& S, uint32_t prim, D3 o, D3 d, double eps, double& t) {
  const uint32_t* ix = S.s->idx + 3 * (size_t)prim;
  const D3 p0 = ld3(S.s->verts, ix[0]), p1 = ld3(S.s->verts, ix[1]), p2 = ld3(S.s->verts, ix[2]);
  const D3 e1 = p1 - p0, e2 = p2 - p0, h = cross(d, e2);
  const double a = dot(e1, h);
  if (a > -eps && a < eps) return false;
  const double f = 1.0 / a;
  const D3 sv = o - p0;
  const double u = f * dot(sv, h);
  if (u < 0.0 || u > 1.0) return false;
  const D3 qv = cross(sv, e1);
  const double v = f * dot(d, qv);
  if (v < 0.0 || u + v > 1.0) return false;
  const double tt = f * dot(e2, qv);
  if (tt > eps && tt < t) {
    t = tt;
    return true;
  }
  return false;
}

// closest (any=false) or any hit below tmax; boxes are tested in double
bool trace(const Scene& S, D3 o, D3 d, double& t, int& hit, bool any) {
  int stk[512];
  int sp = 0;
  stk[sp++] = 0;
  const D3 inv = d3(1.0 / d.x, 1.0 / d.y, 1.0 / d.z);
  const double eps = S.s->tri_eps;
  while (sp > 0) {
    const int ni = stk[--sp];
    const QNode& n = S.q[ni];
    for (int c = 0; c < 4; c++) {
      if (n.counts[c] == 0) continue;
      double t0 = 0.0, t1 = t;
      const double lo[3] = {n.bminx[c], n.bminy[c], n.bminz[c]}, hi[3] = {n.bmaxx[c], n.bmaxy[c], n.bmaxz[c]};
      const double oo[3] = {o.x, o.y, o.z}, ii[3] = {inv.x, inv.y, inv.z};
      bool ok = true;
      for (int a = 0; a < 3 && ok; a++) {
        double ta = (lo[a] - oo[a]) * ii[a], tb = (hi[a] - oo[a]) * ii[a];
        if (std::isnan(ta) || std::isnan(tb)) continue;  // origin on the plane of a parallel ray: inside
        if (ta > tb) std::swap(ta, tb);
        t0 = std::max(t0, ta);
        t1 = std::min(t1, tb);
        ok = t0 <= t1;
      }
      if (!ok) continue;
      if (n.counts[c] == -1) {
        if (sp < 511) stk[sp++] = n.childs[c];
      } else {
        for (int k = 0; k < n.counts[c]; k++) {
          const uint32_t prim = S.s->prims[n.childs[c] + k];
          if (tri_hit(S, prim, o, d, eps, t)) {
            hit = (int)prim;
            if (any) return true;
          }
        }
      }
    }
  }
  return hit >= 0;
}

D3 texel(const Fp64Scene* s, int idx, double u, double v, bool wrap) {
  double x = wrap ? std::fmod(u, 1.0) : u, y = wrap ? std::fmod(v, 1.0) : v;
  if (x < 0) x += 1.0;
  if (y < 0) y += 1.0;
  const uint32_t w = s->tex_dims[2 * idx], h = s->tex_dims[2 * idx + 1];
  double fx = x * (double)(w - 1), fy = y * (double)(h - 1);
  fx = fx >= 0 ? std::min(fx, (double)(w - 1)) : 0.0;
  fy = fy >= 0 ? std::min(fy, (double)(h - 1)) : 0.0;
  const uint32_t ixx = (uint32_t)fx, iyy = (uint32_t)fy;
  const float* base = s->tex + 4 * (size_t)s->tex_offsets[idx];
  auto at = [&](uint32_t i, uint32_t j) {
    const float* t = base + 4 * (size_t)(i + j * w);
    return d3(t[0], t[1], t[2]);
  };
  if (s->tex_filter != 1) return at(ixx, iyy);
  const uint32_t ix1 = std::min(ixx + 1, w - 1), iy1 = std::min(iyy + 1, h - 1);
  const double tx = fx - ixx, ty = fy - iyy;
  const D3 a = at(ixx, iyy) * (1.0 - tx) + at(ix1, iyy) * tx;
  const D3 b = at(ixx, iy1) * (1.0 - tx) + at(ix1, iy1) * tx;
  return a * (1.0 - ty) + b * ty;
}

// ---- material model (double restatement of bsdf_full.cuh) ----
int dist_of(int type) { return (type == 4 || type == 7) ? 0 : ((type == 5 || type == 8) ? 1 : 2); }
bool is_diel(int type) { return type == 2 || type >= 7; }
bool has_nee(int type) { return type == 3 || type == 4 || type == 5 || type == 6; }
double r2a(double r) {
  r = std::max(r, 1e-3);
  const double x = std::log(r);
  return std::min(1.0, 1.62142 + 0.819955 * x + 0.1734 * x * x + 0.0171201 * x * x * x + 0.000640711 * x * x * x * x);
}
double tan2(D3 w) { return std::max(0.0, 1.0 - w.z * w.z) / (w.z * w.z); }
double Dm(int dist, D3 m, double a) {
  if (m.z <= 0) return 0;
  const double c2 = m.z * m.z, t2 = tan2(m), a2 = a * a;
  if (std::isinf(t2)) return 0;
  if (dist == 0) return std::exp(-t2 / a2) / (kPi * a2 * c2 * c2);
  const double e = 1 + t2 / a2;
  return 1 / (kPi * a2 * c2 * c2 * e * e);
}
double lam(int dist, D3 w, double a) {
  const double t2 = tan2(w);
  if (std::isinf(t2)) return 0;
  const double tv = std::sqrt(t2);
  if (tv == 0) return 0;
  if (dist == 0) {
    const double aa = 1 / (a * tv);
    if (aa >= 1.6) return 0;
    return (1 - 1.259 * aa + 0.396 * aa * aa) / (3.535 * aa + 2.181 * aa * aa);
  }
  return (-1 + std::sqrt(1 + a * a * t2)) * 0.5;
}
double G1(int dist, D3 w, double a) { return 1 / (1 + lam(dist, w, a)); }
double erf_as(double x) {
  const double s = x < 0 ? -1 : 1;
  x = std::fabs(x);
  const double t = 1 / (1 + 0.3275911 * x);
  return s * (1 - (((((1.061405429 * t - 1.453152027) * t) + 1.421413741) * t - 0.284496736) * t + 0.254829592) *
                      t * std::exp(-x * x));
}
double erfinv(double x) {
  x = std::min(std::max(x, -0.99999), 0.99999);
  double w = -std::log((1 - x) * (1 + x)), p;
  if (w < 5) {
    w -= 2.5;
    p = 2.81022636e-08;
    p = 3.43273939e-07 + p * w;
    p = -3.5233877e-06 + p * w;
    p = -4.39150654e-06 + p * w;
    p = 0.00021858087 + p * w;
    p = -0.00125372503 + p * w;
    p = -0.00417768164 + p * w;
    p = 0.246640727 + p * w;
    p = 1.50140941 + p * w;
  } else {
    w = std::sqrt(w) - 3;
    p = -0.000200214257;
    p = 0.000100950558 + p * w;
    p = 0.00134934322 + p * w;
    p = -0.00367342844 + p * w;
    p = 0.00573950773 + p * w;
    p = -0.0076224613 + p * w;
    p = 0.00943887047 + p * w;
    p = 1.00167406 + p * w;
    p = 2.83297682 + p * w;
  }
  return p * x;
}
void beck11(double ci, double u1, double u2, double& sx, double& sy) {
  if (ci > 0.9999) {
    const double r = std::sqrt(-std::log(1 - u1)), ph = 2 * kPi * u2;
    sx = r * std::cos(ph);
    sy = r * std::sin(ph);
    return;
  }
  const double si = std::sqrt(std::max(0.0, 1 - ci * ci)), ti = si / ci, ct = 1 / ti;
  double a = -1, c = erf_as(ct);
  const double sample_x = std::max(u1, 1e-6);
  const double th = std::acos(ci);
  const double fit = 1 + th * (-0.876 + th * (0.4265 - 0.0594 * th));
  double b = c - (1 + c) * std::pow(1 - sample_x, fit);
  const double spi = 1 / std::sqrt(kPi);
  const double norm = 1 / (1 + c + spi * ti * std::exp(-ct * ct));
  for (int it = 1; it < 10; it++) {
    if (!(b >= a && b <= c)) b = 0.5 * (a + c);
    const double inv = erfinv(b);
    const double value = norm * (1 + b + spi * ti * std::exp(-inv * inv)) - sample_x;
    const double der = norm * (1 - inv * ti);
    if (std::fabs(value) < 1e-5) break;
    if (value > 0) c = b; else a = b;
    b -= value / der;
  }
  sx = erfinv(b);
  sy = erfinv(2 * std::max(u2, 1e-6) - 1);
}
void ggx11(double ci, double u1, double u2, double& sx, double& sy) {
  if (ci > 0.9999) {
    const double r = std::sqrt(u1 / (1 - u1)), ph = 2 * kPi * u2;
    sx = r * std::cos(ph);
    sy = r * std::sin(ph);
    return;
  }
  const double si = std::sqrt(std::max(0.0, 1 - ci * ci)), ti = si / ci, a = 1 / ti;
  const double g1 = 2 / (1 + std::sqrt(1 + 1 / (a * a)));
  const double A = 2 * u1 / g1 - 1, tmp = std::min(1 / (A * A - 1), 1e10), B = ti;
  const double Dd = std::sqrt(std::max(B * B * tmp * tmp - (A * A - B * B) * tmp, 0.0));
  const double x1 = B * tmp - Dd, x2 = B * tmp + Dd;
  sx = (A < 0 || x2 > 1 / ti) ? x1 : x2;
  double S;
  if (u2 > 0.5) S = 1, u2 = 2 * (u2 - 0.5); else S = -1, u2 = 2 * (0.5 - u2);
  const double z = (u2 * (u2 * (u2 * 0.27385 - 0.73369) + 0.46341)) / (u2 * (u2 * (u2 * 0.093073 + 0.309420) - 1.0) + 0.597999);
  sy = S * z * std::sqrt(1 + sx * sx);
}
D3 sample_m(int dist, D3 wo, double a, double u1, double u2) {
  if (dist == 2) {
    const double t2 = a * a * u1 / (1 - u1), ct = 1 / std::sqrt(1 + t2), st = std::sqrt(std::max(0.0, 1 - ct * ct));
    const double ph = 2 * kPi * u2;
    return d3(st * std::cos(ph), st * std::sin(ph), ct);
  }
  const D3 ws = normalize(d3(a * wo.x, a * wo.y, wo.z));
  double sx, sy;
  if (dist == 0) beck11(ws.z, u1, u2, sx, sy); else ggx11(ws.z, u1, u2, sx, sy);
  const double st = std::sqrt(std::max(0.0, 1 - ws.z * ws.z));
  const double cp = st == 0 ? 1 : std::min(std::max(ws.x / st, -1.0), 1.0);
  const double sp = st == 0 ? 0 : std::min(std::max(ws.y / st, -1.0), 1.0);
  const double tx = cp * sx - sp * sy;
  sy = sp * sx + cp * sy;
  sx = tx;
  return normalize(d3(-a * sx, -a * sy, 1));
}
double pdf_m(int dist, D3 wo, D3 m, double a) {
  const double d = Dm(dist, m, a);
  if (dist == 2) return d * std::fabs(m.z);
  return G1(dist, wo, a) * std::max(0.0, dot(wo, m)) * d / std::fabs(wo.z);
}
double fresnel(double ci, double eta) {
  ci = std::min(std::max(ci, 0.0), 1.0);
  const double s2 = (1 - ci * ci) / (eta * eta);
  if (s2 >= 1) return 1;
  const double ct = std::sqrt(1 - s2);
  const double rs = (ci - eta * ct) / (ci + eta * ct), rp = (eta * ci - ct) / (eta * ci + ct);
  return 0.5 * (rs * rs + rp * rp);
}
D3 eval(int type, D3 col, double a, D3 wo, D3 wi, double& pdf) {
  pdf = 0;
  if (wo.z <= 0 || wi.z <= 0) return d3(0, 0, 0);
  if (type == 3) {
    pdf = wi.z / kPi;
    return col * (1 / kPi);
  }
  const int dist = dist_of(type);
  D3 m = wo + wi;
  const double l2 = dot(m, m);
  if (l2 == 0) return d3(0, 0, 0);
  m = m * (1 / std::sqrt(l2));
  pdf = pdf_m(dist, wo, m, a) / (4 * dot(wo, m));
  return col * (Dm(dist, m, a) * G1(dist, wo, a) * G1(dist, wi, a) / (4 * wo.z * wi.z));
}
struct Smp {
  D3 wi, w;
  double pdf;
  bool delta, valid;
};
Smp sample(int type, D3 col, double rough, double eta, D3 wo, double u1, double u2, double u3) {
  Smp s{d3(0, 0, 0), d3(0, 0, 0), 0, false, false};
  if (type == 3) {
    if (wo.z <= 0) return s;
    const double r = std::sqrt(u1), ph = 2 * kPi * u2;
    s.wi = d3(r * std::cos(ph), r * std::sin(ph), std::sqrt(std::max(0.0, 1 - u1)));
    s.pdf = s.wi.z / kPi;
    s.w = col;
    s.valid = s.wi.z > 0;
    return s;
  }
  if (type == 1) {
    if (wo.z <= 0) return s;
    s.wi = d3(-wo.x, -wo.y, wo.z);
    s.pdf = 1;
    s.delta = true;
    s.w = col;
    s.valid = true;
    return s;
  }
  const double a = r2a(rough);
  if (!is_diel(type)) {
    if (wo.z <= 0) return s;
    const int dist = dist_of(type);
    const D3 m = sample_m(dist, wo, a, u1, u2);
    s.wi = m * (2 * dot(wo, m)) - wo;
    if (s.wi.z <= 0 || dot(wo, m) <= 0) return s;
    double pdf;
    const D3 f = eval(type, col, a, wo, s.wi, pdf);
    if (pdf <= 0) return s;
    s.pdf = pdf;
    s.w = f * (s.wi.z / pdf);
    s.valid = true;
    return s;
  }
  const bool entering = wo.z > 0;
  const double rel = entering ? eta : 1.0 / eta;
  const D3 wo_s = entering ? wo : -wo;
  D3 m = d3(0, 0, 1);
  const bool smooth = type == 2 || rough < 1e-3;
  const int dist = dist_of(type);
  if (!smooth) m = sample_m(dist, wo_s, a, u1, u2);
  const double c = dot(wo_s, m);
  if (c <= 0) return s;
  const double F = fresnel(c, rel);
  D3 wi_s;
  bool refl = u3 < F;
  if (!refl) {
    const double s2 = std::max(0.0, 1 - c * c) / (rel * rel);
    if (s2 >= 1) refl = true;
    else wi_s = (-wo_s) * (1 / rel) + m * (c / rel - std::sqrt(1 - s2));
  }
  if (refl) wi_s = m * (2 * c) - wo_s;
  if (refl ? wi_s.z <= 0 : wi_s.z >= 0) return s;
  D3 w = col;
  if (!smooth) {
    const double g = G1(dist, wi_s.z < 0 ? -wi_s : wi_s, a);
    const double extra = dist == 2 ? G1(dist, wo_s, a) * c / (std::fabs(wo_s.z) * m.z) : 1.0;
    w = w * (g * extra);
  }
  if (!refl) w = w * (1 / (rel * rel));
  s.wi = entering ? wi_s : -wi_s;
  s.pdf = 1;
  s.delta = true;
  s.w = w;
  s.valid = true;
  return s;
}

void onb(D3 n, D3& t, D3& b) {
  const double sign = std::copysign(1.0, n.z), a = -1 / (sign + n.z), bb = n.x * n.y * a;
  t = d3(1 + sign * n.x * n.x * a, sign * bb, -sign * n.x);
  b = d3(bb, sign + n.y * n.y * a, -n.y);
}

D3 radiance(const Scene& S, D3 o, D3 d, int depth, Rng& rng) {
  const Fp64Scene* s = S.s;
  D3 L = d3(0, 0, 0), T = d3(1, 1, 1);
  double last_pdf = 1;
  bool mis = false;
  for (int pass = 0; pass < depth; pass++) {
    double t = 1e34;
    int hit = -1;
    trace(S, o, d, t, hit, false);
    if (hit < 0) {
      if (s->sky && s->sky_tex >= 0) {
        const double u = 1 + std::atan2(d.x, -d.z) / (2 * kPi), v = 1 - std::acos(std::max(-1.0, std::min(1.0, d.y))) / kPi;
        L = L + mulv(T, texel(s, s->sky_tex, u, v, true));
      }
      break;
    }
    const uint32_t* ix = s->idx + 3 * (size_t)hit;
    const D3 p0 = ld3(s->verts, ix[0]), p1 = ld3(s->verts, ix[1]), p2 = ld3(s->verts, ix[2]);
    const D3 p = o + d * t;
    D3 Ngf = cross(p1 - p0, p2 - p0);
    const double area2 = std::sqrt(dot(Ngf, Ngf));
    Ngf = Ngf * (1 / area2);
    const double b1 = dot(Ngf, cross(p2 - p, p0 - p)) / area2, b2 = dot(Ngf, cross(p0 - p, p1 - p)) / area2;
    const double b0 = 1 - b1 - b2;
    D3 Ns = ld3(s->normals, ix[0]) * b0 + ld3(s->normals, ix[1]) * b1 + ld3(s->normals, ix[2]) * b2;
    Ns = dot(Ns, Ns) > 0 ? normalize(Ns) : Ngf;
    const Material& mat = S.m[s->mat_idx[hit]];
    const float* uv0 = s->uvs + 2 * (size_t)ix[0];
    const float* uv1 = s->uvs + 2 * (size_t)ix[1];
    const float* uv2 = s->uvs + 2 * (size_t)ix[2];
    const double tu = uv0[0] * b0 + uv1[0] * b1 + uv2[0] * b2, tv = uv0[1] * b0 + uv1[1] * b1 + uv2[1] * b2;
    if (mat.normalTex >= 0) {
      // tangent-space normal map: the texel (normalised) expressed in a frame around Ns
      const D3 sm = normalize(texel(s, mat.normalTex, tu, tv, false));
      const D3 W = std::fabs(Ns.x) > 0.99 ? d3(0, 1, 0) : d3(1, 0, 0);
      const D3 Tn = normalize(cross(Ns, W)), Bn = cross(Ns, Tn);
      Ns = normalize(Tn * sm.x + Bn * sm.y + Ns * sm.z);
    }
    const D3 alb = d3(mat.albedo[0], mat.albedo[1], mat.albedo[2]);
    if (mat.type == 0) {
      if (!s->indirect) break;
      const D3 cn = normalize(ld3(s->center_normals, hit));
      const double cl = -dot(cn, d);
      if (cl <= 0) break;
      double w = 1;
      if (mis && s->light_count > 0) {
        const double lp = t * t / (cl * 0.5 * area2 * s->light_count);
        w = last_pdf * last_pdf / (last_pdf * last_pdf + lp * lp);
      }
      L = L + mulv(T, alb) * w;
      break;
    }
    const bool diel = is_diel(mat.type);
    const bool front = dot(d, Ngf) < 0;
    const D3 Ng = front ? Ngf : -Ngf;
    const D3 N = diel ? (dot(Ns, Ngf) < 0 ? -Ns : Ns) : (dot(Ns, Ng) < 0 ? -Ns : Ns);
    D3 Tt, Bt;
    onb(N, Tt, Bt);
    const D3 wo = -d, wo_l = d3(dot(wo, Tt), dot(wo, Bt), dot(wo, N));
    D3 col = alb;
    if (mat.diffuseTex >= 0) col = texel(s, mat.diffuseTex, tu, tv, true);
    const double a = r2a(mat.roughness);
    const double u1 = rng.next(), u2 = rng.next(), u3 = rng.next();
    bool nee = false;
    if (has_nee(mat.type) && s->shadow && s->light_count > 0 && wo_l.z > 0) {
      nee = true;
      const int li = std::min((int)(rng.next() * s->light_count), (int)s->light_count - 1);
      const uint32_t lprim = s->lights[li];
      const uint32_t* lx = s->idx + 3 * (size_t)lprim;
      const D3 l0 = ld3(s->verts, lx[0]), l1 = ld3(s->verts, lx[1]), l2 = ld3(s->verts, lx[2]);
      double q1 = rng.next(), q2 = rng.next();
      if (q1 + q2 > 1) q1 = 1 - q1, q2 = 1 - q2;
      const D3 lp = l0 * (1 - q1 - q2) + l1 * q1 + l2 * q2;
      D3 Ld = lp - p;
      const double sq = dot(Ld, Ld), dist = std::sqrt(sq);
      Ld = Ld * (1 / dist);
      const double cl = -dot(normalize(ld3(s->center_normals, lprim)), Ld);
      const D3 lc = cross(l1 - l0, l2 - l0);
      const double larea = 0.5 * std::sqrt(dot(lc, lc));
      if (cl > 0 && dot(Ng, Ld) > 0 && larea > 0) {
        const D3 wi_l = d3(dot(Ld, Tt), dot(Ld, Bt), dot(Ld, N));
        double pb;
        const D3 fv = eval(mat.type, col, a, wo_l, wi_l, pb);
        if (pb > 0) {
          const double lpdf = sq / (cl * larea * s->light_count);
          const double w = lpdf * lpdf / (lpdf * lpdf + pb * pb);
          const Material& lm = S.m[s->mat_idx[lprim]];
          const D3 le = d3(lm.albedo[0], lm.albedo[1], lm.albedo[2]);
          double tt = dist * (1.0 - 1e-4) - 2.0 * s->dist_eps;  // the full mode's shadow-ray end
          int h2 = -1;
          const D3 so = p + Ng * s->normal_eps;
          if (!trace(S, so, Ld, tt, h2, true)) L = L + mulv(mulv(T, fv), le) * (wi_l.z * w / lpdf);
        }
      }
    }
    const Smp sm = sample(mat.type, col, mat.roughness, mat.refractIdx, wo_l, u1, u2, u3);
    if (!sm.valid) break;
    const D3 wi = Tt * sm.wi.x + Bt * sm.wi.y + N * sm.wi.z;
    T = mulv(T, sm.w);
    if (!(T.x > 0 || T.y > 0 || T.z > 0)) break;
    const double side = dot(wi, Ngf) > 0 ? 1 : -1;
    o = p + Ngf * (side * s->normal_eps);
    d = wi;
    last_pdf = sm.pdf;
    mis = nee && !sm.delta;
  }
  return L;
}

}  // namespace

extern "C" {

/* Microfacet pieces for the known-answer tests: the sampled normal for
 * material `type` (4-9) at isotropic alpha and the Smith G1 of `wo`. */
void fp64_microfacet(int type, double a, const float* wi, double u1, double u2, const float* wo, double* m_out,
                     double* g1_out) {
  const D3 w = d3(wi[0], wi[1], wi[2]);
  const D3 m = sample_m(dist_of(type), w, a, u1, u2);
  m_out[0] = m.x, m_out[1] = m.y, m_out[2] = m.z;
  *g1_out = G1(dist_of(type), d3(wo[0], wo[1], wo[2]), a);
}

double fp64_roughness_to_alpha(double r) { return r2a(r); }

/* spp samples per pixel of a W x H image for a camera (pos, w, hor, ver as
 * sample() builds them); writes per-pixel sums and sums of squares (rgb). */
void fp64_render(const Fp64Scene* desc, const float* pos, const float* cw, const float* hor, const float* ver, int W,
                 int H, int spp, int depth, uint64_t seed, double* sum, double* sumsq, int nthreads) {
  Scene S{desc, (const Material*)desc->materials, (const QNode*)desc->qnodes};
  const D3 co = ld3(pos, 0), w = ld3(cw, 0), h = ld3(hor, 0), v = ld3(ver, 0);
  const int n = W * H;
  auto work = [&](int b, int e) {
    for (int pix = b; pix < e; pix++) {
      const int x = pix % W, y = pix / W;
      Rng rng{seed * 0x100000001B3ull + (uint64_t)pix * 0x9E3779B97F4A7C15ull};
      for (int k = 0; k < spp; k++) {
        const double px = x + rng.next() - 0.5, py = y + rng.next() - 0.5;
        const double sx = 2 * (px / W) - 1, sy = 1 - 2 * (py / H);
        const D3 d = normalize(w + h * sx + v * sy);
        const D3 L = radiance(S, co, d, depth, rng);
        const double c[3] = {L.x, L.y, L.z};
        for (int ch = 0; ch < 3; ch++) {
          sum[3 * (size_t)pix + ch] += c[ch];
          sumsq[3 * (size_t)pix + ch] += c[ch] * c[ch];
        }
      }
    }
  };
  nthreads = std::max(1, nthreads);
  std::vector<std::thread> ts;
  const int chunk = (n + nthreads - 1) / nthreads;
  for (int t = 0; t < nthreads; t++) {
    const int b = t * chunk, e = std::min(n, b + chunk);
    if (b < e) ts.emplace_back(work, b, e);
  }
  for (auto& t : ts) t.join();
}

}  // extern "C"

namespace {
inline double c3(double x, double y, double z, int k) { return k == 0 ? x : (k == 1 ? y : z); }
inline float c3f(float x, float y, float z, int k) { return k == 0 ? x : (k == 1 ? y : z); }

struct WtRay {
  double ox, oy, oz, Sx, Sy, Sz, tmax;
  int kx, ky, kz;
};

// Axis choice and shear exactly as the GPU's ray setup (float comparisons).
WtRay wt_ray(const float* o, const float* d) {
  WtRay r;
  r.ox = o[0], r.oy = o[1], r.oz = o[2], r.tmax = d[3];
  const float ax = std::fabs(d[0]), ay = std::fabs(d[1]), az = std::fabs(d[2]);
  r.kz = (ax > ay) ? (ax > az ? 0 : 2) : (ay > az ? 1 : 2);
  r.kx = r.kz == 2 ? 0 : r.kz + 1;
  r.ky = r.kx == 2 ? 0 : r.kx + 1;
  if (c3f(d[0], d[1], d[2], r.kz) < 0.0f) std::swap(r.kx, r.ky);
  const double dkz = c3f(d[0], d[1], d[2], r.kz);
  r.Sx = (double)c3f(d[0], d[1], d[2], r.kx) / dkz;
  r.Sy = (double)c3f(d[0], d[1], d[2], r.ky) / dkz;
  r.Sz = 1.0 / dkz;
  return r;
}

// Watertight test in double: the operation order of the GPU's FP64 arbiter.
bool wt_hit(const WtRay& r, const float* a, const float* b, const float* c, double& t) {
  const double akx = c3(a[0], a[1], a[2], r.kx) - c3(r.ox, r.oy, r.oz, r.kx);
  const double aky = c3(a[0], a[1], a[2], r.ky) - c3(r.ox, r.oy, r.oz, r.ky);
  const double akz = c3(a[0], a[1], a[2], r.kz) - c3(r.ox, r.oy, r.oz, r.kz);
  const double bkx = c3(b[0], b[1], b[2], r.kx) - c3(r.ox, r.oy, r.oz, r.kx);
  const double bky = c3(b[0], b[1], b[2], r.ky) - c3(r.ox, r.oy, r.oz, r.ky);
  const double bkz = c3(b[0], b[1], b[2], r.kz) - c3(r.ox, r.oy, r.oz, r.kz);
  const double ckx = c3(c[0], c[1], c[2], r.kx) - c3(r.ox, r.oy, r.oz, r.kx);
  const double cky = c3(c[0], c[1], c[2], r.ky) - c3(r.ox, r.oy, r.oz, r.ky);
  const double ckz = c3(c[0], c[1], c[2], r.kz) - c3(r.ox, r.oy, r.oz, r.kz);
  const double Ax = akx - r.Sx * akz, Ay = aky - r.Sy * akz;
  const double Bx = bkx - r.Sx * bkz, By = bky - r.Sy * bkz;
  const double Cx = ckx - r.Sx * ckz, Cy = cky - r.Sy * ckz;
  const double U = Cx * By - Cy * Bx;
  const double V = Ax * Cy - Ay * Cx;
  const double W = Bx * Ay - By * Ax;
  if ((U < 0.0 || V < 0.0 || W < 0.0) && (U > 0.0 || V > 0.0 || W > 0.0)) return false;
  const double det = (U + V) + W;
  if (det == 0.0) return false;
  const double Az = r.Sz * akz, Bz = r.Sz * bkz, Cz = r.Sz * ckz;
  const double T = ((U * Az) + (V * Bz)) + (W * Cz);
  t = T / det;
  return t > 0.0 && t < r.tmax;
}
}  // namespace

extern "C" {
/* FP64 watertight closest hit (any_hit = 0) or occlusion (any_hit = 1) for n
 * rays (org/dir float4, dir.w = tmax) over a quad BVH in the reference layout
 * (padded boxes, so double slab tests lose nothing). hit: primitive or -1;
 * t: its double distance (tmax on a miss). */
void fp64_trace(const float* verts, const uint32_t* idx, const void* qnodes, const uint32_t* prims, const float* org,
                const float* dir, uint32_t n, int any_hit, int32_t* hit, double* t_out, int nthreads) {
  const QNode* Q = (const QNode*)qnodes;
  auto work = [&](uint32_t b, uint32_t e) {
    std::vector<int> stk(4096);
    for (uint32_t i = b; i < e; i++) {
      const float* o = org + 4 * (size_t)i;
      const float* d = dir + 4 * (size_t)i;
      const WtRay r = wt_ray(o, d);
      const double inv[3] = {1.0 / (double)d[0], 1.0 / (double)d[1], 1.0 / (double)d[2]};
      const double oo[3] = {o[0], o[1], o[2]};
      int best = -1;
      double tb = r.tmax;
      int sp = 0;
      stk[sp++] = 0;
      bool done = false;
      while (sp > 0 && !done) {
        const QNode& nd = Q[stk[--sp]];
        for (int c = 0; c < 4 && !done; c++) {
          if (nd.counts[c] == 0) continue;
          double t0 = 0.0, t1 = tb;
          const double lo[3] = {nd.bminx[c], nd.bminy[c], nd.bminz[c]}, hi[3] = {nd.bmaxx[c], nd.bmaxy[c], nd.bmaxz[c]};
          bool ok = true;
          for (int a = 0; a < 3 && ok; a++) {
            double ta = (lo[a] - oo[a]) * inv[a], tb2 = (hi[a] - oo[a]) * inv[a];
            if (std::isnan(ta) || std::isnan(tb2)) continue;
            if (ta > tb2) std::swap(ta, tb2);
            t0 = std::max(t0, ta);
            t1 = std::min(t1, tb2);
            ok = t0 <= t1;
          }
          if (!ok) continue;
          if (nd.counts[c] == -1) {
            if (sp < (int)stk.size()) stk[sp++] = nd.childs[c];
            continue;
          }
          for (int k = 0; k < nd.counts[c]; k++) {
            const uint32_t prim = prims[nd.childs[c] + k];
            const uint32_t* ix = idx + 3 * (size_t)prim;
            double tt;
            if (!wt_hit(r, verts + 3 * (size_t)ix[0], verts + 3 * (size_t)ix[1], verts + 3 * (size_t)ix[2], tt)) continue;
            if (tt < tb || (tt == tb && (int)prim < best)) tb = tt, best = (int)prim;
            if (any_hit) {
              done = true;
              break;
            }
          }
        }
      }
      hit[i] = best;
      t_out[i] = best >= 0 ? tb : r.tmax;
    }
  };
  nthreads = std::max(1, nthreads);
  std::vector<std::thread> ts;
  const uint32_t chunk = (n + nthreads - 1) / nthreads;
  for (int k = 0; k < nthreads; k++) {
    const uint32_t b = k * chunk, e = std::min(n, b + chunk);
    if (b < e) ts.emplace_back(work, b, e);
  }
  for (auto& th : ts) th.join();
}
}  // extern "C"
