// Model and texture ingest for the host side: the import half of
// TriangleList::loadModel (src/Core/TriangleList.cpp:63-146) and
// processMesh (src/Core/TriangleList.cpp:203-348), and the 8-bit image path of
// core::Surface (src/Utils/Surface.cpp:33-98). The reference links assimp and
// FreeImage for these; this file reads Wavefront OBJ/MTL and TGA itself.
//
// What the reference asks assimp for, and what the OBJ reader does instead:
//   one mesh per material   faces are grouped by material in order of first
//                           use; vertices are never shared between groups
//   FlipWindingOrder        each polygon's corner list is reversed
//   Triangulate             the reversed polygon becomes a fan from its first
//                           corner (for triangles and quads this is the split
//                           assimp makes for convex faces; longer convex
//                           polygons cover the same surface with other triangles)
//   JoinIdenticalVertices   one vertex per distinct (position, texcoord, normal)
//                           within a group, numbered by first use
//   GenSmoothNormals        corners without a normal get the normalised sum of
//                           the unit normals of the group's faces that share the
//                           position (the file's counter-clockwise winding, so
//                           outward on closed models); no angle limit
//   PTV_NORMALIZE           optional: centre the model's bounds and scale the
//                           largest half-extent to 1
//   materials               an MTL entry starts from the OBJ defaults (diffuse
//                           0.6 grey, black specular and emission, shininess 0,
//                           index of refraction 1, transmission white) and
//                           every colour counts as present, as the importer
//                           reports them; processMesh's choice is then made
// Not reproduced: ImproveCacheLocality (a triangle reorder), FixInfacingNormals.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <sstream>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/cudatracer.h"

struct ct_mesh {
  std::vector<float> v, n, t;  // 3, 3, 2 floats per vertex
  std::vector<uint32_t> idx;   // 3 per triangle
  std::vector<uint32_t> mat;   // per triangle, into materials
  std::vector<ct_material> materials;
  std::vector<std::string> diffuse_maps, normal_maps;  // per material, path or ""
};

namespace {

thread_local std::string g_mesh_error;

ct_status fail(ct_status s, const std::string& msg) {
  g_mesh_error = msg;
  return s;
}

struct MtlDesc {
  float kd[3] = {0.6f, 0.6f, 0.6f}, ks[3] = {0, 0, 0}, ke[3] = {0, 0, 0}, tf[3] = {1, 1, 1};
  float ns = 0.0f, ni = 1.0f;
  std::string map_kd, map_norm;
};

bool nonzero(const float c[3]) { return c[0] > 0.0001f && c[1] > 0.0001f && c[2] > 0.0001f; }

ct_material blank_material() {
  ct_material m;
  std::memset(&m, 0, sizeof(m));
  m.refract_idx = 1.0f;
  m.diffuse_tex = m.normal_tex = m.mask_tex = m.displace_tex = -1;
  m.type = CT_MAT_LAMBERTIAN;
  return m;
}

// processMesh's material choice (src/Core/TriangleList.cpp:276-346), before
// textures are numbered. `textured` is whether a diffuse map was given.
ct_material choose(const MtlDesc& d) {
  ct_material m = blank_material();
  auto set = [&](const float c[3]) { m.albedo[0] = c[0], m.albedo[1] = c[1], m.albedo[2] = c[2]; };
  if (!d.map_kd.empty()) {
    const float white[3] = {1, 1, 1};
    set(white);
    if (d.ns >= 2.0f) m.roughness = d.ns, m.type = CT_MAT_GGX;
    return m;
  }
  if (nonzero(d.ke)) {
    m.type = CT_MAT_LIGHT;
    for (int k = 0; k < 3; k++) m.albedo[k] = std::fmax(d.ke[k], 0.01f);  // Material::light
    return m;
  }
  if (nonzero(d.kd)) {
    float c[3] = {d.kd[0], d.kd[1], d.kd[2]};
    const float sd = d.ks[0] * d.ks[0] + d.ks[1] * d.ks[1] + d.ks[2] * d.ks[2];
    const float dd = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
    if (sd > dd) c[0] = d.ks[0], c[1] = d.ks[1], c[2] = d.ks[2];
    set(c);
    if (d.ns >= 1.0f) m.roughness = d.ns, m.type = CT_MAT_GGX;
    return m;
  }
  if (nonzero(d.ks)) {
    set(d.ks);
    m.type = CT_MAT_SPECULAR;  // Material::specular(colour, 1.0f)
    m.roughness = 0.0001f;
    return m;
  }
  if (nonzero(d.tf)) {
    set(d.tf);
    m.type = CT_MAT_FRESNEL;
    m.refract_idx = d.ni;
    m.absorption[0] = d.tf[0], m.absorption[1] = d.tf[1], m.absorption[2] = d.tf[2];
    if (d.ns >= 1.0f) m.roughness = d.ns, m.type = CT_MAT_FRESNEL_GGX;
    return m;
  }
  return m;  // every colour black: a black Lambertian
}

std::string dir_of(const std::string& p) {
  const size_t k = p.find_last_of('/');
  return k == std::string::npos ? std::string(".") : p.substr(0, k);
}

std::string rest_of(std::istringstream& ss) {
  std::string rest;
  std::getline(ss, rest);
  const size_t b = rest.find_first_not_of(" \t");
  if (b == std::string::npos) return "";
  const size_t e = rest.find_last_not_of(" \t\r");
  rest = rest.substr(b, e - b + 1);
  // texture options ("-bm 1 file.tga"): the file name is the last word
  if (rest[0] == '-') {
    const size_t s = rest.find_last_of(" \t");
    if (s != std::string::npos) rest = rest.substr(s + 1);
  }
  return rest;
}

std::string lower(std::string s) {
  for (char& c : s) c = (char)std::tolower((unsigned char)c);
  return s;
}

void parse_mtl(const std::string& path, std::map<std::string, MtlDesc>& out) {
  std::ifstream f(path);
  if (!f) return;  // a missing library leaves its materials at the defaults
  std::string line, cur;
  while (std::getline(f, line)) {
    std::istringstream ss(line);
    std::string k;
    if (!(ss >> k) || k[0] == '#') continue;
    if (k == "newmtl") {
      ss >> cur;
      out[cur] = MtlDesc();
      continue;
    }
    if (cur.empty()) continue;
    MtlDesc& d = out[cur];
    auto rd3 = [&](float* c) {
      ss >> c[0];
      if (!(ss >> c[1] >> c[2])) c[1] = c[2] = c[0];
    };
    const std::string kl = lower(k);
    if (k == "Kd") rd3(d.kd);
    else if (k == "Ks") rd3(d.ks);
    else if (k == "Ke") rd3(d.ke);
    else if (k == "Tf") rd3(d.tf);
    else if (k == "Ns") ss >> d.ns;
    else if (k == "Ni") ss >> d.ni;
    else if (kl == "map_kd") d.map_kd = rest_of(ss);
    else if (kl == "norm" || kl == "map_kn") d.map_norm = rest_of(ss);
  }
}

struct Corner {
  int v, t, n;
};

// "v", "v/t", "v//n", "v/t/n": 1-based, negative values count back from the end
bool parse_corner(const std::string& tok, int nv, int nt, int nn, Corner& c) {
  int vals[3] = {0, 0, 0};
  bool present[3] = {false, false, false};
  size_t pos = 0;
  for (int part = 0; part < 3; part++) {
    const size_t slash = tok.find('/', pos);
    const std::string s = tok.substr(pos, slash == std::string::npos ? std::string::npos : slash - pos);
    if (!s.empty()) {
      char* end = nullptr;
      vals[part] = (int)std::strtol(s.c_str(), &end, 10);
      if (*end != 0 || vals[part] == 0) return false;
      present[part] = true;
    }
    if (slash == std::string::npos) break;
    pos = slash + 1;
  }
  auto fix = [](int x, int count) { return x > 0 ? x - 1 : count + x; };
  if (!present[0]) return false;
  c.v = fix(vals[0], nv);
  c.t = present[1] ? fix(vals[1], nt) : -1;
  c.n = present[2] ? fix(vals[2], nn) : -1;
  return c.v >= 0 && c.v < nv && (!present[1] || (c.t >= 0 && c.t < nt)) && (!present[2] || (c.n >= 0 && c.n < nn));
}

struct Face {
  uint32_t material;
  uint32_t first, count;  // into the corner list
};

}  // namespace

extern "C" {

const char* ct_mesh_last_error(void) { return g_mesh_error.c_str(); }

ct_status ct_mesh_load_obj(const char* path, int32_t normalize, ct_mesh** out) {
  if (!path || !out) return fail(CT_ERR_INVALID_ARGUMENT, "null argument");
  *out = nullptr;
  std::ifstream f(path);
  if (!f) return fail(CT_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
  const std::string base = dir_of(path);
  std::vector<float> P, T, N;
  std::map<std::string, MtlDesc> library;
  std::vector<std::string> mat_names;  // in order of first use by a face
  std::map<std::string, uint32_t> mat_ids;
  std::vector<Corner> corners;
  std::vector<Face> faces;
  std::string cur = "";  // faces before any usemtl take the importer's default material
  std::string line;
  size_t line_no = 0;
  while (std::getline(f, line)) {
    line_no++;
    std::istringstream ss(line);
    std::string k;
    if (!(ss >> k) || k[0] == '#') continue;
    if (k == "v" || k == "vn") {
      float x = 0, y = 0, z = 0;
      if (!(ss >> x >> y >> z)) return fail(CT_ERR_INVALID_ARGUMENT, "bad vector at line " + std::to_string(line_no));
      (k == "v" ? P : N).insert((k == "v" ? P : N).end(), {x, y, z});
    } else if (k == "vt") {
      float u = 0, v = 0;
      if (!(ss >> u)) return fail(CT_ERR_INVALID_ARGUMENT, "bad texcoord at line " + std::to_string(line_no));
      ss >> v;
      T.insert(T.end(), {u, v});
    } else if (k == "mtllib") {
      std::string name;
      while (ss >> name) parse_mtl(base + "/" + name, library);
    } else if (k == "usemtl") {
      ss >> cur;
    } else if (k == "f") {
      Face fc;
      fc.first = (uint32_t)corners.size();
      std::string tok;
      while (ss >> tok) {
        Corner c;
        if (!parse_corner(tok, (int)P.size() / 3, (int)T.size() / 2, (int)N.size() / 3, c))
          return fail(CT_ERR_INVALID_ARGUMENT, "bad face corner '" + tok + "' at line " + std::to_string(line_no));
        corners.push_back(c);
      }
      fc.count = (uint32_t)corners.size() - fc.first;
      if (fc.count < 3) return fail(CT_ERR_INVALID_ARGUMENT, "face with fewer than 3 corners at line " + std::to_string(line_no));
      auto it = mat_ids.find(cur);
      if (it == mat_ids.end()) {
        it = mat_ids.emplace(cur, (uint32_t)mat_names.size()).first;
        mat_names.push_back(cur);
      }
      fc.material = it->second;
      faces.push_back(fc);
    }
  }
  if (faces.empty()) return fail(CT_ERR_INVALID_ARGUMENT, std::string("no faces in ") + path);

  auto* m = new ct_mesh();
  for (uint32_t g = 0; g < (uint32_t)mat_names.size(); g++) {
    std::map<std::tuple<int, int, int>, uint32_t> joined;
    const uint32_t v0 = (uint32_t)(m->v.size() / 3);
    const size_t t0 = m->idx.size();
    std::vector<int> vpos;  // position index of each of this group's vertices
    std::vector<char> vhas_n;
    auto vertex = [&](const Corner& c) -> uint32_t {
      const auto key = std::make_tuple(c.v, c.t, c.n);
      auto it = joined.find(key);
      if (it != joined.end()) return it->second;
      const uint32_t id = (uint32_t)(m->v.size() / 3);
      joined.emplace(key, id);
      vpos.push_back(c.v);
      vhas_n.push_back(c.n >= 0);
      m->v.insert(m->v.end(), {P[3 * c.v], P[3 * c.v + 1], P[3 * c.v + 2]});
      if (c.n >= 0) m->n.insert(m->n.end(), {N[3 * c.n], N[3 * c.n + 1], N[3 * c.n + 2]});
      else m->n.insert(m->n.end(), {0.0f, 0.0f, 0.0f});
      // processMesh gives untextured vertices (0.5, 0.5)
      if (c.t >= 0) m->t.insert(m->t.end(), {T[2 * c.t], T[2 * c.t + 1]});
      else m->t.insert(m->t.end(), {0.5f, 0.5f});
      return id;
    };
    for (const Face& fc : faces) {
      if (fc.material != g) continue;
      std::vector<uint32_t> q(fc.count);
      for (uint32_t i = 0; i < fc.count; i++) q[i] = vertex(corners[fc.first + fc.count - 1 - i]);  // reversed
      for (uint32_t i = 1; i + 1 < fc.count; i++) {
        m->idx.insert(m->idx.end(), {q[0], q[i], q[i + 1]});
        m->mat.push_back(g);
      }
    }
    // generated normals for this group's vertices that have none
    bool missing = false;
    for (char h : vhas_n) missing |= !h;
    if (missing) {
      std::map<int, std::vector<double>> sum;  // position index -> summed unit face normals
      for (size_t t = t0; t < m->idx.size(); t += 3) {
        // the stored triangle is reversed; its file-order normal is cross(c - a, b - a)
        const int a = vpos[m->idx[t] - v0], b = vpos[m->idx[t + 1] - v0], c = vpos[m->idx[t + 2] - v0];
        const double e1[3] = {P[3 * c] - (double)P[3 * a], P[3 * c + 1] - (double)P[3 * a + 1], P[3 * c + 2] - (double)P[3 * a + 2]};
        const double e2[3] = {P[3 * b] - (double)P[3 * a], P[3 * b + 1] - (double)P[3 * a + 1], P[3 * b + 2] - (double)P[3 * a + 2]};
        double cr[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        const double l = std::sqrt(cr[0] * cr[0] + cr[1] * cr[1] + cr[2] * cr[2]);
        if (!(l > 0)) continue;  // degenerate faces add nothing
        for (int p : {a, b, c}) {
          auto& s = sum[p];
          if (s.empty()) s.assign(3, 0.0);
          for (int k = 0; k < 3; k++) s[k] += cr[k] / l;
        }
      }
      for (size_t i = 0; i < vpos.size(); i++) {
        if (vhas_n[i]) continue;
        auto it = sum.find(vpos[i]);
        float* dst = &m->n[3 * (v0 + i)];
        if (it == sum.end()) continue;
        const auto& s = it->second;
        const double l = std::sqrt(s[0] * s[0] + s[1] * s[1] + s[2] * s[2]);
        if (l > 0)
          for (int k = 0; k < 3; k++) dst[k] = (float)(s[k] / l);
      }
    }
  }
  // processMesh normalises every normal it reads (glm::normalize: v * inversesqrt(dot(v, v)))
  for (size_t i = 0; i < m->n.size(); i += 3) {
    float* q = &m->n[i];
    const float d = q[0] * q[0] + q[1] * q[1] + q[2] * q[2];
    if (d > 0) {
      const float s = 1.0f / std::sqrt(d);
      q[0] *= s, q[1] *= s, q[2] *= s;
    }
  }
  if (normalize) {
    float lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (size_t i = 0; i < m->v.size(); i += 3)
      for (int k = 0; k < 3; k++) lo[k] = std::fmin(lo[k], m->v[i + k]), hi[k] = std::fmax(hi[k], m->v[i + k]);
    float half = 0.0f, ctr[3];
    for (int k = 0; k < 3; k++) ctr[k] = lo[k] + 0.5f * (hi[k] - lo[k]), half = std::fmax(half, 0.5f * (hi[k] - lo[k]));
    const float s = half > 0 ? 1.0f / half : 1.0f;
    for (size_t i = 0; i < m->v.size(); i += 3)
      for (int k = 0; k < 3; k++) m->v[i + k] = (m->v[i + k] - ctr[k]) * s;
  }
  for (const std::string& name : mat_names) {
    auto it = library.find(name);
    const MtlDesc d = it == library.end() ? MtlDesc() : it->second;
    m->materials.push_back(choose(d));
    m->diffuse_maps.push_back(d.map_kd.empty() ? "" : base + "/" + d.map_kd);
    m->normal_maps.push_back(d.map_norm.empty() ? "" : base + "/" + d.map_norm);
  }
  *out = m;
  return CT_OK;
}

ct_status ct_mesh_info(const ct_mesh* m, uint32_t* vertex_count, uint32_t* triangle_count, uint32_t* material_count) {
  if (!m) return fail(CT_ERR_INVALID_ARGUMENT, "null mesh");
  if (vertex_count) *vertex_count = (uint32_t)(m->v.size() / 3);
  if (triangle_count) *triangle_count = (uint32_t)(m->idx.size() / 3);
  if (material_count) *material_count = (uint32_t)m->materials.size();
  return CT_OK;
}

ct_status ct_mesh_arrays(const ct_mesh* m, float* vertices, float* normals, float* texcoords, uint32_t* indices,
                         uint32_t* material_idxs) {
  if (!m) return fail(CT_ERR_INVALID_ARGUMENT, "null mesh");
  if (vertices) std::memcpy(vertices, m->v.data(), m->v.size() * sizeof(float));
  if (normals) std::memcpy(normals, m->n.data(), m->n.size() * sizeof(float));
  if (texcoords) std::memcpy(texcoords, m->t.data(), m->t.size() * sizeof(float));
  if (indices) std::memcpy(indices, m->idx.data(), m->idx.size() * sizeof(uint32_t));
  if (material_idxs) std::memcpy(material_idxs, m->mat.data(), m->mat.size() * sizeof(uint32_t));
  return CT_OK;
}

ct_status ct_mesh_material(const ct_mesh* m, uint32_t i, ct_material* out, char* diffuse_map, char* normal_map,
                           uint32_t path_capacity) {
  if (!m || !out || i >= m->materials.size()) return fail(CT_ERR_INVALID_ARGUMENT, "bad material index");
  *out = m->materials[i];
  const std::string* paths[2] = {&m->diffuse_maps[i], &m->normal_maps[i]};
  char* dst[2] = {diffuse_map, normal_map};
  for (int k = 0; k < 2; k++) {
    if (!dst[k]) continue;
    if (paths[k]->size() + 1 > path_capacity) return fail(CT_ERR_INVALID_ARGUMENT, "path buffer too small");
    std::memcpy(dst[k], paths[k]->c_str(), paths[k]->size() + 1);
  }
  return CT_OK;
}

ct_status ct_mesh_destroy(ct_mesh* m) {
  if (!m) return fail(CT_ERR_INVALID_ARGUMENT, "null mesh");
  delete m;
  return CT_OK;
}

// Truevision TGA, image types 1/2/3 (colour-mapped, true-colour, grey) and
// their run-length forms 9/10/11, 8/16/24/32 bits per pixel. Texels come out
// as the reference's Surface stores 8-bit images: channel / 255, alpha 1,
// row 0 at the bottom of the picture.
ct_status ct_image_load(const char* path, uint32_t* width, uint32_t* height, float* rgba) {
  if (!path || !width || !height) return fail(CT_ERR_INVALID_ARGUMENT, "null argument");
  std::ifstream f(path, std::ios::binary);
  if (!f) return fail(CT_ERR_INVALID_ARGUMENT, std::string("cannot open ") + path);
  std::vector<unsigned char> b((std::istreambuf_iterator<char>(f)), std::istreambuf_iterator<char>());
  if (b.size() < 18) return fail(CT_ERR_INVALID_ARGUMENT, "truncated TGA header");
  const unsigned id_len = b[0], cmap_type = b[1], type = b[2];
  const unsigned cmap_first = b[3] | (b[4] << 8), cmap_len = b[5] | (b[6] << 8), cmap_bits = b[7];
  const unsigned w = b[12] | (b[13] << 8), h = b[14] | (b[15] << 8), bpp = b[16], desc = b[17];
  const unsigned base_type = type & 7;
  const bool rle = (type & 8) != 0;
  if (!(base_type >= 1 && base_type <= 3) || (base_type == 1 && cmap_type != 1) || w == 0 || h == 0)
    return fail(CT_ERR_UNSUPPORTED, std::string("unsupported TGA image type in ") + path);
  const unsigned px_bytes = (bpp + 7) / 8;
  if (!(bpp == 8 || bpp == 15 || bpp == 16 || bpp == 24 || bpp == 32) || (base_type == 1 && bpp != 8 && bpp != 16))
    return fail(CT_ERR_UNSUPPORTED, std::string("unsupported TGA pixel depth in ") + path);
  *width = w;
  *height = h;
  if (!rgba) return CT_OK;
  size_t pos = 18 + id_len;
  const unsigned cmap_entry = (cmap_bits + 7) / 8;
  const size_t cmap_pos = pos;
  if (cmap_type == 1) pos += (size_t)cmap_len * cmap_entry;
  if (pos > b.size()) return fail(CT_ERR_INVALID_ARGUMENT, "truncated TGA colour map");
  auto decode = [&](const unsigned char* p, unsigned bits, float* o) -> bool {
    unsigned r, g, bl;
    if (bits == 8) {
      r = g = bl = p[0];
    } else if (bits == 15 || bits == 16) {
      const unsigned v = p[0] | (p[1] << 8);
      r = ((v >> 10) & 31) * 255 / 31, g = ((v >> 5) & 31) * 255 / 31, bl = (v & 31) * 255 / 31;
    } else {
      bl = p[0], g = p[1], r = p[2];
    }
    o[0] = (float)r / 255.0f, o[1] = (float)g / 255.0f, o[2] = (float)bl / 255.0f, o[3] = 1.0f;
    return true;
  };
  auto pixel = [&](const unsigned char* p, float* o) -> bool {
    if (base_type == 1) {
      const unsigned i = px_bytes == 1 ? p[0] : (p[0] | (p[1] << 8));
      if (i < cmap_first || i - cmap_first >= cmap_len) return false;
      return decode(&b[cmap_pos + (size_t)(i - cmap_first) * cmap_entry], cmap_bits, o);
    }
    return decode(p, base_type == 3 ? 8 : bpp, o);
  };
  const size_t npx = (size_t)w * h;
  std::vector<float> img(npx * 4);  // file order
  size_t i = 0;
  while (i < npx) {
    if (!rle) {
      if (pos + px_bytes > b.size()) return fail(CT_ERR_INVALID_ARGUMENT, "truncated TGA pixel data");
      if (!pixel(&b[pos], &img[4 * i])) return fail(CT_ERR_INVALID_ARGUMENT, "TGA colour index out of range");
      pos += px_bytes, i++;
      continue;
    }
    if (pos >= b.size()) return fail(CT_ERR_INVALID_ARGUMENT, "truncated TGA packet");
    const unsigned hdr = b[pos++], run = (hdr & 127) + 1;
    if (i + run > npx) return fail(CT_ERR_INVALID_ARGUMENT, "TGA packet runs past the image");
    if (hdr & 128) {
      if (pos + px_bytes > b.size()) return fail(CT_ERR_INVALID_ARGUMENT, "truncated TGA packet");
      float o[4];
      if (!pixel(&b[pos], o)) return fail(CT_ERR_INVALID_ARGUMENT, "TGA colour index out of range");
      pos += px_bytes;
      for (unsigned k = 0; k < run; k++, i++) std::memcpy(&img[4 * i], o, sizeof(o));
    } else {
      if (pos + (size_t)run * px_bytes > b.size()) return fail(CT_ERR_INVALID_ARGUMENT, "truncated TGA packet");
      for (unsigned k = 0; k < run; k++, i++, pos += px_bytes)
        if (!pixel(&b[pos], &img[4 * i])) return fail(CT_ERR_INVALID_ARGUMENT, "TGA colour index out of range");
    }
  }
  // bit 5 of the descriptor: rows stored top first; bit 4: columns right to left
  const bool top_first = (desc & 0x20) != 0, right_first = (desc & 0x10) != 0;
  for (unsigned y = 0; y < h; y++) {
    const unsigned sy = top_first ? h - 1 - y : y;
    for (unsigned x = 0; x < w; x++) {
      const unsigned sx = right_first ? w - 1 - x : x;
      std::memcpy(&rgba[4 * ((size_t)y * w + x)], &img[4 * ((size_t)sy * w + sx)], 4 * sizeof(float));
    }
  }
  return CT_OK;
}

}  // extern "C"
