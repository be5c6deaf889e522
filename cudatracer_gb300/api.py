"""Host-side mirror of the reference tracer's interface over the C ABI.

Names follow the reference's classes so code written against it reads the same:

  reference (meirbon/CudaTracer)                    here
  ------------------------------------------------  ------------------------------
  Material + factories  src/Core/Material.cuh:29-97 Material.light/lambertian/...
  TriangleList          src/Core/TriangleList.h     TriangleList (add_triangle,
                                                    add_material, add_mesh)
  BVHTree / MBVHTree    src/BVH/BVHTree.h, MBVHTree.h  BVH (build / import / export)
  core::Camera          src/Core/Camera.h           Camera
  Params / launchKernels src/CUDA/Kernel.cuh:23-74  Params, launch_kernels
  MBVHNode::traverseMBVH src/BVH/MBVHNode.cuh:126-244  trace_closest / trace_any

Everything that computes runs in libcudatracer.so; this module only marshals.
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import check, ptr

MAT_LIGHT, MAT_SPECULAR, MAT_FRESNEL, MAT_LAMBERTIAN = 0, 1, 2, 3
MAT_BECKMANN, MAT_GGX, MAT_TROWBRIDGE = 4, 5, 6
MAT_FRESNEL_BECKMANN, MAT_FRESNEL_GGX, MAT_FRESNEL_TROWBRIDGE = 7, 8, 9
MAX_DISTANCE = 1e34  # src/Core/Ray.cuh:13


@dataclass
class Material:
    """The reference Material record (52 bytes). `albedo` is the emission of lights."""

    albedo: tuple = (1.0, 1.0, 1.0)
    refract_idx: float = 1.0
    diffuse_tex: int = -1
    normal_tex: int = -1
    mask_tex: int = -1
    displace_tex: int = -1
    type: int = MAT_LAMBERTIAN
    roughness: float = 0.0
    absorption: tuple = (0.0, 0.0, 0.0)

    # factories: src/Core/Material.cuh:50-97
    @staticmethod
    def light(emission) -> "Material":
        e = tuple(max(float(c), 0.01) for c in emission)  # glm::max(emission, vec3(0.01f))
        return Material(albedo=e, type=MAT_LIGHT, roughness=0.0)

    @staticmethod
    def lambertian(albedo, diffuse_tex=-1, normal_tex=-1, mask_tex=-1, displace_tex=-1, refract_idx=1.0):
        return Material(tuple(map(float, albedo)), float(refract_idx), diffuse_tex, normal_tex, mask_tex,
                        displace_tex, MAT_LAMBERTIAN, 0.0)

    @staticmethod
    def specular(albedo, refract_idx) -> "Material":
        return Material(tuple(map(float, albedo)), float(refract_idx), type=MAT_SPECULAR, roughness=0.0001)

    @staticmethod
    def fresnel(albedo, refract_idx, absorption=(0.0, 0.0, 0.0), roughness=0.0, diffuse_tex=-1, normal_tex=-1):
        return Material(tuple(map(float, albedo)), float(refract_idx), diffuse_tex, normal_tex, -1, -1, MAT_FRESNEL,
                        float(roughness), tuple(map(float, absorption)))

    def to_ct(self) -> _lib.ct_material:
        m = _lib.ct_material()
        m.albedo[:] = [float(c) for c in self.albedo]
        m.refract_idx = self.refract_idx
        m.diffuse_tex, m.normal_tex = self.diffuse_tex, self.normal_tex
        m.mask_tex, m.displace_tex = self.mask_tex, self.displace_tex
        m.type = self.type
        m.roughness = self.roughness
        m.absorption[:] = [float(c) for c in self.absorption]
        return m

    @staticmethod
    def from_ct(m: _lib.ct_material) -> "Material":
        return Material(tuple(float(c) for c in m.albedo), float(m.refract_idx), int(m.diffuse_tex),
                        int(m.normal_tex), int(m.mask_tex), int(m.displace_tex), int(m.type), float(m.roughness),
                        tuple(float(c) for c in m.absorption))


def _mesh_check(status: int) -> None:
    if status != _lib.CT_OK:
        raw = _lib.load().ct_mesh_last_error()
        raise _lib.CTError(status, raw.decode(errors="replace") if raw else "")


def load_obj(path: str, normalize: bool = True) -> dict:
    """Import a Wavefront OBJ (+ MTL) through libcudatracer (ct_mesh_load_obj):
    what assimp hands processMesh in TriangleList::loadModel
    (src/Core/TriangleList.cpp:63-91, 203-348). Returns float32/uint32 arrays
    `vertices` (V,3), `normals` (V,3), `texcoords` (V,2), `indices` (T,3),
    `material_idxs` (T,) into `materials`, and per material the `diffuse_maps`
    and `normal_maps` paths ("" for none)."""
    L = _lib.load()
    h = ctypes.c_void_p()
    _mesh_check(L.ct_mesh_load_obj(str(path).encode(), int(bool(normalize)), ctypes.byref(h)))
    try:
        nv, nt, nm = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        _mesh_check(L.ct_mesh_info(h, ctypes.byref(nv), ctypes.byref(nt), ctypes.byref(nm)))
        out = {"vertices": np.empty((nv.value, 3), np.float32), "normals": np.empty((nv.value, 3), np.float32),
               "texcoords": np.empty((nv.value, 2), np.float32), "indices": np.empty((nt.value, 3), np.uint32),
               "material_idxs": np.empty(nt.value, np.uint32)}
        _mesh_check(L.ct_mesh_arrays(h, *(ptr(out[k]) for k in ("vertices", "normals", "texcoords", "indices",
                                                                 "material_idxs"))))
        mats, dmaps, nmaps = [], [], []
        cap = 4096
        for i in range(nm.value):
            m = _lib.ct_material()
            dbuf, nbuf = ctypes.create_string_buffer(cap), ctypes.create_string_buffer(cap)
            _mesh_check(L.ct_mesh_material(h, i, ctypes.byref(m), ctypes.addressof(dbuf), ctypes.addressof(nbuf),
                                           cap))
            mats.append(Material.from_ct(m))
            dmaps.append(dbuf.value.decode())
            nmaps.append(nbuf.value.decode())
        out.update(materials=mats, diffuse_maps=dmaps, normal_maps=nmaps)
        return out
    finally:
        L.ct_mesh_destroy(h)


def load_image(path: str) -> np.ndarray:
    """An 8-bit TGA as the reference's Surface stores it (src/Utils/Surface.cpp:71-97):
    (height, width, 4) float32, channel/255, alpha 1, row 0 at the bottom."""
    L = _lib.load()
    w, h = ctypes.c_uint32(), ctypes.c_uint32()
    _mesh_check(L.ct_image_load(str(path).encode(), ctypes.byref(w), ctypes.byref(h), None))
    img = np.empty((h.value, w.value, 4), np.float32)
    _mesh_check(L.ct_image_load(str(path).encode(), ctypes.byref(w), ctypes.byref(h), ptr(img)))
    return img


@dataclass
class TriangleList:
    """Host scene container with TriangleList's public vectors (TriangleList.h:59-73).

    force_unit_roughness reproduces addMaterial setting roughness = 1 on every
    material (TriangleList.cpp:56), which is what the reference renders with."""

    force_unit_roughness: bool = True
    vertices: list = field(default_factory=list)
    normals: list = field(default_factory=list)
    center_normals: list = field(default_factory=list)
    texcoords: list = field(default_factory=list)
    indices: list = field(default_factory=list)
    material_idxs: list = field(default_factory=list)
    light_indices: list = field(default_factory=list)
    materials: list = field(default_factory=list)
    textures: list = field(default_factory=list)  # (h, w, 4) float32 arrays
    _arrays: dict = field(default_factory=dict)
    _loaded_textures: dict = field(default_factory=dict)  # m_LoadedTextures: path -> index

    def __post_init__(self):
        # "Have at least 1 material" (TriangleList.cpp:13-15)
        self.add_material(Material.lambertian((1.0, 1.0, 1.0)))

    def add_material(self, mat: Material) -> int:
        m = Material(**mat.__dict__)
        if self.force_unit_roughness:
            m.roughness = 1.0
        self.materials.append(m)
        return len(self.materials) - 1

    def add_triangle(self, p0, p1, p2, n0, n1, n2, mat_idx, t0=(0, 0), t1=(0, 0), t2=(0, 0)):
        """TriangleList::addTriangle (TriangleList.cpp:25-50): stores normalized
        vertex normals, the centre normal from the raw ones, no light entry."""
        f = np.float32
        base = len(self.vertices)
        for p in (p0, p1, p2):
            self.vertices.append(np.asarray(p, f))
        raw = [np.asarray(n, f) for n in (n0, n1, n2)]
        for n in raw:
            self.normals.append(n * (f(1.0) / np.sqrt((n[0] * n[0] + n[1] * n[1]) + n[2] * n[2])))
        self.center_normals.append(((raw[0] + raw[1]) + raw[2]) / f(3.0))
        for t in (t0, t1, t2):
            self.texcoords.append(np.asarray(t, f))
        self.indices.append((base, base + 1, base + 2))
        self.material_idxs.append(int(mat_idx))
        self._arrays.clear()

    def add_mesh(self, vertices, normals, indices, material: int, texcoords=None):
        """The array part of loadModel (TriangleList.cpp:115-146) for an already
        imported mesh: normals kept as given, centre normal = mean of the three
        stored normals, emitters appended to the light list."""
        v = np.asarray(vertices, np.float32).reshape(-1, 3)
        n = np.asarray(normals, np.float32).reshape(-1, 3)
        ix = np.asarray(indices, np.uint32).reshape(-1, 3)
        uv = np.zeros((v.shape[0], 2), np.float32) if texcoords is None else np.asarray(texcoords, np.float32)
        self._flush()
        off = self._arrays["vertices"].shape[0]
        t0 = self._arrays["indices"].shape[0]
        cn = ((n[ix[:, 0]] + n[ix[:, 1]]) + n[ix[:, 2]]) / np.float32(3.0)
        a = self._arrays
        a["vertices"] = np.concatenate([a["vertices"], v])
        a["normals"] = np.concatenate([a["normals"], n])
        a["texcoords"] = np.concatenate([a["texcoords"], uv.reshape(-1, 2)])
        a["indices"] = np.concatenate([a["indices"], ix + np.uint32(off)])
        a["center_normals"] = np.concatenate([a["center_normals"], cn.astype(np.float32)])
        a["material_idxs"] = np.concatenate([a["material_idxs"], np.full(ix.shape[0], material, np.uint32)])
        if self.materials[material].type == MAT_LIGHT:
            a["light_indices"] = np.concatenate(
                [a["light_indices"], np.arange(t0, t0 + ix.shape[0], dtype=np.uint32)])

    def _flush(self):
        if self._arrays:
            return
        f = np.float32
        self._arrays = {
            "vertices": np.asarray(self.vertices, f).reshape(-1, 3),
            "normals": np.asarray(self.normals, f).reshape(-1, 3),
            "texcoords": np.asarray(self.texcoords, f).reshape(-1, 2),
            "indices": np.asarray(self.indices, np.uint32).reshape(-1, 3),
            "center_normals": np.asarray(self.center_normals, f).reshape(-1, 3),
            "material_idxs": np.asarray(self.material_idxs, np.uint32).reshape(-1),
            "light_indices": np.asarray(self.light_indices, np.uint32).reshape(-1),
        }

    def arrays(self) -> dict:
        self._flush()
        return self._arrays

    def load_texture(self, path: str) -> int:
        """TriangleList::loadTexture (TriangleList.cpp:369-387): one texture per
        distinct path; an unreadable file gives -1."""
        loaded = self._loaded_textures
        if path in loaded:
            return loaded[path]
        try:
            img = load_image(path)
        except _lib.CTError:
            return -1
        self.textures.append(img)
        loaded[path] = len(self.textures) - 1
        return loaded[path]

    def load_model(self, path: str, scale: float = 1.0, mat=None, material: int = -1, normalize: bool = True):
        """TriangleList::loadModel (TriangleList.cpp:63-146): import the OBJ,
        add one material per used MTL entry (with its diffuse and normal maps
        loaded) unless `material` >= 0 overrides them, then append
        pos = mat * vec4(p * scale, 1) and norm = mat * vec4(n, 0) in glm's
        float32 evaluation order, texcoords as imported."""
        m = load_obj(path, normalize)
        ids = []
        for i, mt in enumerate(m["materials"]):
            mt = Material(**mt.__dict__)
            if m["diffuse_maps"][i]:
                mt.diffuse_tex = self.load_texture(m["diffuse_maps"][i])
            if m["normal_maps"][i]:
                mt.normal_tex = self.load_texture(m["normal_maps"][i])
            ids.append(self.add_material(mt))
        f = np.float32
        M = np.eye(4, dtype=f) if mat is None else np.asarray(mat, f).reshape(4, 4)

        def xform(v, w):
            # glm mat4 * vec4 (column-major columns M[:, c]): (c0*x + c1*y) + (c2*z + c3*w)
            c = [M[:, k][None, :3] for k in range(4)]
            return ((c[0] * v[:, 0:1] + c[1] * v[:, 1:2]) + (c[2] * v[:, 2:3] + c[3] * f(w))).astype(f)

        pos = xform(m["vertices"] * f(scale), 1.0)
        nrm = xform(m["normals"], 0.0)
        tri_mat = np.asarray(ids, np.uint32)[m["material_idxs"]] if material < 0 else \
            np.full(m["indices"].shape[0], material, np.uint32)
        # one add_mesh per material so emitters land in the light list
        base = len(self.arrays()["vertices"])
        a = self._arrays
        ix = m["indices"] + np.uint32(base)
        cn = ((nrm[m["indices"][:, 0]] + nrm[m["indices"][:, 1]]) + nrm[m["indices"][:, 2]]) / f(3.0)
        t0 = a["indices"].shape[0]
        a["vertices"] = np.concatenate([a["vertices"], pos])
        a["normals"] = np.concatenate([a["normals"], nrm])
        a["texcoords"] = np.concatenate([a["texcoords"], m["texcoords"]])
        a["indices"] = np.concatenate([a["indices"], ix])
        a["center_normals"] = np.concatenate([a["center_normals"], cn.astype(f)])
        a["material_idxs"] = np.concatenate([a["material_idxs"], tri_mat])
        is_light = np.asarray([mm.type == MAT_LIGHT for mm in self.materials], bool)
        lights = np.nonzero(is_light[tri_mat])[0]
        if lights.size:
            a["light_indices"] = np.concatenate([a["light_indices"], (lights + t0).astype(np.uint32)])
        return m

    def get_prim_count(self) -> int:
        return int(self.arrays()["indices"].shape[0])


def scene_desc(arrays: dict, materials, textures=(), skybox_texture=-1):
    """Build a ct_scene_desc over numpy arrays; returns (desc, keepalive)."""
    a = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
    mats = (_lib.ct_material * len(materials))(*[m.to_ct() for m in materials])
    texels = dims = offs = None
    if textures:
        flat, dl, ol, o = [], [], [], 0
        for t in textures:
            t = np.ascontiguousarray(t, np.float32)
            h, w = t.shape[:2]
            flat.append(t.reshape(-1, 4))
            dl += [w, h]
            ol.append(o)
            o += w * h
        texels = np.ascontiguousarray(np.concatenate(flat))
        dims = np.asarray(dl, np.uint32)
        offs = np.asarray(ol, np.uint32)
    d = _lib.ct_scene_desc()
    d.vertices = ptr(a["vertices"])
    d.normals = ptr(a["normals"])
    d.texcoords = ptr(a.get("texcoords"))
    d.vertex_count = a["vertices"].shape[0]
    d.indices = ptr(a["indices"])
    d.center_normals = ptr(a.get("center_normals"))
    d.material_indices = ptr(a.get("material_idxs"))
    d.triangle_count = a["indices"].shape[0]
    d.materials = ctypes.cast(mats, ctypes.c_void_p)
    d.material_count = len(materials)
    li = a.get("light_indices")
    d.light_indices = ptr(li) if li is not None and li.size else None
    d.light_count = 0 if li is None else int(li.size)
    d.texels = ptr(texels)
    d.texel_count = 0 if texels is None else texels.shape[0]
    d.texture_dims = ptr(dims)
    d.texture_offsets = ptr(offs)
    d.texture_count = len(textures)
    d.skybox_texture = skybox_texture
    return d, (a, mats, texels, dims, offs)


class Context:
    """One device context (ct_ctx)."""

    def __init__(self, device: int = 0):
        self.lib = _lib.load()
        h = ctypes.c_void_p()
        check(self.lib.ct_ctx_create(device, ctypes.byref(h)))
        self.h = h

    def close(self):
        if self.h:
            self.lib.ct_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def check(self, stream=None):
        check(self.lib.ct_ctx_check(self.h, _stream(stream)), self.h)

    def set_memory_budget(self, nbytes: int):
        check(self.lib.ct_ctx_set_memory_budget(self.h, int(nbytes)), self.h)

    @property
    def device_bytes(self) -> int:
        return int(self.lib.ct_ctx_device_bytes(self.h))

    def scene(self, arrays: dict, materials, textures=(), skybox_texture=-1) -> "Scene":
        d, keep = scene_desc(arrays, materials, textures, skybox_texture)
        h = ctypes.c_void_p()
        check(self.lib.ct_scene_create(self.h, ctypes.byref(d), ctypes.byref(h)), self.h)
        return Scene(self, h, keep[0]["indices"].shape[0])

    def scene_from_list(self, tl: TriangleList, skybox_texture=-1) -> "Scene":
        return self.scene(tl.arrays(), tl.materials, tl.textures, skybox_texture)


def _stream(s):
    if s is None:
        return None
    if hasattr(s, "cuda_stream"):
        return s.cuda_stream
    return int(s)


class Scene:
    def __init__(self, ctx: Context, h, ntri: int):
        self.ctx, self.h, self.ntri = ctx, h, ntri

    def close(self):
        if self.h:
            self.ctx.lib.ct_scene_destroy(self.ctx.h, self.h)
            self.h = None

    def set_material(self, index: int, m: Material):
        mm = m.to_ct()
        check(self.ctx.lib.ct_scene_set_material(self.ctx.h, self.h, index, ctypes.byref(mm)), self.ctx.h)

    def build_bvh(self, nthreads: int = 0) -> "BVH":
        h = ctypes.c_void_p()
        check(self.ctx.lib.ct_bvh_build(self.ctx.h, self.h, nthreads, ctypes.byref(h)), self.ctx.h)
        return BVH(self, h)

    def build_bvh_fast(self, nthreads: int = 0) -> "BVH":
        """Quad tree built for traversal speed (ct_bvh_build_fast): hits equal the
        reference tree's up to exact t ties; use it for fast-math frames and queries."""
        h = ctypes.c_void_p()
        check(self.ctx.lib.ct_bvh_build_fast(self.ctx.h, self.h, nthreads, ctypes.byref(h)), self.ctx.h)
        return BVH(self, h)

    def build_bvh_device(self, stream=None) -> "BVH":
        """The same SAH tree built on the GPU (ct_bvh_build_device): quad nodes
        equal build_bvh's bit for bit, primitives within a leaf may be reordered."""
        h = ctypes.c_void_p()
        s = None if stream is None else getattr(stream, "cuda_stream", stream)
        check(self.ctx.lib.ct_bvh_build_device(self.ctx.h, self.h, s, ctypes.byref(h)), self.ctx.h)
        return BVH(self, h)

    def build_bvh_fast_device(self, stream=None) -> "BVH":
        """build_bvh_fast's tree built on the GPU (ct_bvh_build_fast_device): the
        same quad nodes and primitive order, byte for byte."""
        h = ctypes.c_void_p()
        s = None if stream is None else getattr(stream, "cuda_stream", stream)
        check(self.ctx.lib.ct_bvh_build_fast_device(self.ctx.h, self.h, s, ctypes.byref(h)), self.ctx.h)
        return BVH(self, h)

    def build_bvh_wide(self, stream=None) -> "BVH":
        """8-wide BVH with 8-bit quantised child bounds for ray queries
        (ct_bvh_build_wide): FP32 watertight tests settled in FP64 where FP32
        cannot decide, so queries return the FP64 closest hit."""
        h = ctypes.c_void_p()
        s = None if stream is None else getattr(stream, "cuda_stream", stream)
        check(self.ctx.lib.ct_bvh_build_wide(self.ctx.h, self.h, s, ctypes.byref(h)), self.ctx.h)
        return BVH(self, h)

    def import_quad(self, nodes: np.ndarray, prims: np.ndarray) -> "BVH":
        nodes = np.ascontiguousarray(nodes)
        prims = np.ascontiguousarray(prims, np.uint32)
        h = ctypes.c_void_p()
        check(self.ctx.lib.ct_bvh_import_quad(self.ctx.h, self.h, ptr(nodes), nodes.nbytes // 128, ptr(prims),
                                              prims.size, ctypes.byref(h)), self.ctx.h)
        return BVH(self, h)

    def import_binary(self, nodes: np.ndarray, prims: np.ndarray) -> "BVH":
        nodes = np.ascontiguousarray(nodes)
        prims = np.ascontiguousarray(prims, np.uint32)
        h = ctypes.c_void_p()
        check(self.ctx.lib.ct_bvh_import_binary(self.ctx.h, self.h, ptr(nodes), nodes.nbytes // 32, ptr(prims),
                                                prims.size, ctypes.byref(h)), self.ctx.h)
        return BVH(self, h)


class BVH:
    def __init__(self, scene: Scene, h):
        self.scene, self.ctx, self.h = scene, scene.ctx, h

    def close(self):
        if self.h:
            self.ctx.lib.ct_bvh_destroy(self.ctx.h, self.h)
            self.h = None

    def info(self) -> dict:
        i = _lib.ct_bvh_info()
        check(self.ctx.lib.ct_bvh_info_get(self.h, ctypes.byref(i)))
        return {k: getattr(i, k) for k, _ in i._fields_}

    def export(self, layout=_lib.CT_BVH_QUAD):
        inf = self.info()
        n = inf["binary_node_count"] if layout == _lib.CT_BVH_BINARY else inf["quad_node_count"]
        rec = {_lib.CT_BVH_BINARY: 32, _lib.CT_BVH_QUAD: 128, _lib.CT_BVH_WIDE8_Q8: 80}[layout]
        nodes = np.zeros(n * rec // 4, np.int32)
        prims = np.zeros(inf["prim_count"], np.uint32)
        check(self.ctx.lib.ct_bvh_export(self.h, layout, ptr(nodes), ptr(prims)))
        return nodes.reshape(n, rec // 4), prims

    def wide_stats(self, reset: bool = False) -> dict:
        """Query counters of a wide BVH: rays, FP64 re-tests (of which only to
        tighten t), full FP64 traversals."""
        a, b, c, d = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint64()
        check(self.ctx.lib.ct_bvh_wide_stats(self.ctx.h, self.h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(c),
                                             ctypes.byref(d), int(reset)), self.ctx.h)
        return {"rays": a.value, "fp64_retests": b.value, "fp64_t_only": c.value, "fp64_full": d.value}

    def trace_closest(self, org, dir, hit=None, t=None, tri_eps=1e-3, stream=None):
        """org/dir: (n,4) float32 CUDA tensors (dir.w = initial t). Returns (hit, t)."""
        import torch

        n = org.shape[0]
        if hit is None:
            hit = torch.empty(n, dtype=torch.int32, device=org.device)
        if t is None:
            t = torch.empty(n, dtype=torch.float32, device=org.device)
        check(self.ctx.lib.ct_trace_closest(self.ctx.h, self.h, ptr(org), ptr(dir), ptr(hit), ptr(t), n, tri_eps,
                                            _stream(stream)), self.ctx.h)
        return hit, t

    def trace_any(self, org, dir, occluded=None, tri_eps=1e-3, stream=None):
        import torch

        n = org.shape[0]
        if occluded is None:
            occluded = torch.empty(n, dtype=torch.uint8, device=org.device)
        check(self.ctx.lib.ct_trace_any(self.ctx.h, self.h, ptr(org), ptr(dir), ptr(occluded), n, tri_eps,
                                        _stream(stream)), self.ctx.h)
        return occluded


def host_bvh_build(vertices: np.ndarray, indices: np.ndarray, nthreads: int = 0, fast: bool = False) -> dict:
    """BVHTree + MBVHTree construction on the host only (no device): returns the
    reference-layout binary nodes (n,8 int32 view), quad nodes (n,32) and prims.
    fast=True builds ct_bvh_build_fast's tree instead (no binary nodes: 0 rows)."""
    lib = _lib.load()
    v = np.ascontiguousarray(vertices, np.float32)
    ix = np.ascontiguousarray(indices, np.uint32)
    h = ctypes.c_void_p()
    fn = lib.ct_host_bvh_build_fast if fast else lib.ct_host_bvh_build
    check(fn(ptr(v), v.shape[0], ptr(ix), ix.shape[0], nthreads, ctypes.byref(h)))
    try:
        nb, nq, npr = ctypes.c_uint32(), ctypes.c_uint32(), ctypes.c_uint32()
        bms, cms = ctypes.c_double(), ctypes.c_double()
        check(lib.ct_host_bvh_counts(h, ctypes.byref(nb), ctypes.byref(nq), ctypes.byref(npr), ctypes.byref(bms),
                                     ctypes.byref(cms)))
        bin_nodes = np.zeros((nb.value, 8), np.int32)
        quad = np.zeros((nq.value, 32), np.int32)
        prims = np.zeros(npr.value, np.uint32)
        if nb.value:
            check(lib.ct_host_bvh_export(h, _lib.CT_BVH_BINARY, ptr(bin_nodes), None))
        check(lib.ct_host_bvh_export(h, _lib.CT_BVH_QUAD, ptr(quad), ptr(prims)))
        return {"binary": bin_nodes, "quad": quad, "prims": prims, "build_ms": bms.value, "collapse_ms": cms.value}
    finally:
        lib.ct_host_bvh_destroy(h)


@dataclass
class Camera:
    """core::Camera: pinhole, forward (0,0,-1) and up (0,1,0) unless set."""

    width: int
    height: int
    fov: float
    position: tuple = (0.0, 0.0, 1.0)
    forward: tuple = (0.0, 0.0, -1.0)
    up: tuple = (0.0, 1.0, 0.0)

    def to_ct(self) -> _lib.ct_camera:
        c = _lib.ct_camera()
        c.position[:] = [float(x) for x in self.position]
        c.forward[:] = [float(x) for x in self.forward]
        c.up[:] = [float(x) for x in self.up]
        c.fov_deg = float(self.fov)
        return c


def default_params(width: int, height: int) -> _lib.ct_render_params:
    p = _lib.ct_render_params()
    _lib.load().ct_render_params_default(ctypes.byref(p))
    p.width, p.height = width, height
    return p


class RenderJob:
    """One render job's resident device state (ray queues + accumulation)."""

    def __init__(self, ctx: Context, width: int, height: int):
        self.ctx, self.width, self.height = ctx, width, height
        h = ctypes.c_void_p()
        check(ctx.lib.ct_render_create(ctx.h, width, height, ctypes.byref(h)), ctx.h)
        self.h = h

    def close(self):
        if self.h:
            self.ctx.lib.ct_render_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def reset(self, stream=None):
        check(self.ctx.lib.ct_render_reset(self.ctx.h, self.h, _stream(stream)), self.ctx.h)

    def accumulate(self, scene: Scene, bvh: BVH, camera: Camera, params, stream=None):
        cam = camera.to_ct()
        check(self.ctx.lib.ct_render_accumulate(self.ctx.h, scene.h, bvh.h, ctypes.byref(cam), ctypes.byref(params),
                                                self.h, _stream(stream)), self.ctx.h)

    def accum_tensor(self):
        """The float4 accumulation buffer as a (h*w, 4) torch view (no copy)."""
        import torch

        p = ctypes.c_void_p()
        check(self.ctx.lib.ct_render_accum(self.h, ctypes.byref(p)))
        return _device_view(p.value, self.width * self.height * 4, torch.float32).view(-1, 4)

    def present(self, samples: float, out, stream=None):
        check(self.ctx.lib.ct_present(self.ctx.h, self.h, float(samples), ptr(out), _stream(stream)), self.ctx.h)

    def stats(self, reset=False, stream=None) -> dict:
        s = _lib.ct_frame_stats()
        check(self.ctx.lib.ct_render_stats(self.ctx.h, self.h, ctypes.byref(s), int(reset), _stream(stream)),
              self.ctx.h)
        return {k: getattr(s, k) for k, _ in s._fields_}


    STAGES = ("raygen", "extend", "shade", "connect")

    def profile(self, enable: bool = True):
        """Bracket every stage launch with CUDA events (see profile_read)."""
        check(self.ctx.lib.ct_render_profile(self.ctx.h, self.h, int(enable)), self.ctx.h)

    def profile_read(self, reset: bool = True) -> dict:
        s = _lib.ct_stage_times()
        check(self.ctx.lib.ct_render_profile_read(self.ctx.h, self.h, ctypes.byref(s), int(reset)), self.ctx.h)
        return {name: {"ms": s.ms[i], "launches": s.launches[i]} for i, name in enumerate(self.STAGES)}


def _device_view(addr: int, numel: int, dtype):
    """Wrap device memory owned by the library as a torch tensor (no copy)."""
    import torch

    class _Holder:
        pass

    holder = _Holder()
    nbytes = numel * torch.empty((), dtype=dtype).element_size()
    holder.__cuda_array_interface__ = {
        "shape": (numel,), "typestr": {torch.float32: "<f4", torch.int32: "<i4"}[dtype],
        "data": (addr, False), "version": 3, "strides": None,
    }
    _ = nbytes
    return torch.as_tensor(holder, device="cuda")


@dataclass
class Params:
    """Params (src/CUDA/Kernel.cuh:23-72): size, sample counter and flags."""

    width: int
    height: int
    samples: int = 0
    camera: Camera | None = None
    max_depth: int = 5
    shadow: bool = True
    indirect: bool = True
    sky: bool = True
    exact_math: int = _lib.CT_MATH_FAST  # CT_MATH_*: False/0 fast, True/1 exact, 2 exact shading + fast traversal
    normal_eps: float = 1e-5
    dist_eps: float = 1e-5
    tri_eps: float = 1e-3
    shading_mode: int = _lib.CT_SHADE_COMPAT
    texture_filter: int = _lib.CT_TEX_NEAREST
    ray_sort: int = _lib.CT_SORT_NONE

    def reset(self, job: RenderJob, stream=None):
        """Params::reset: clear the accumulation buffer and the sample count."""
        job.reset(stream)
        self.samples = 0

    def to_ct(self) -> _lib.ct_render_params:
        p = default_params(self.width, self.height)
        p.max_depth = self.max_depth
        p.frame_index = self.samples
        p.exact_math = int(self.exact_math)
        p.shadow, p.indirect, p.sky = int(self.shadow), int(self.indirect), int(self.sky)
        p.normal_eps, p.dist_eps, p.tri_eps = self.normal_eps, self.dist_eps, self.tri_eps
        p.shading_mode, p.texture_filter = int(self.shading_mode), int(self.texture_filter)
        p.ray_sort = int(self.ray_sort)
        return p


def launch_kernels(job: RenderJob, scene: Scene, bvh: BVH, params: Params, present_out=None, stream=None):
    """launchKernels (src/CUDA/Kernel.cu:355-371): one 1-spp frame seeded with
    params.samples, which then advances by 2 (sample()'s frame++ plus
    launchKernels' samples++); the presented image divides by the new count."""
    job.accumulate(scene, bvh, params.camera, params.to_ct(), stream)
    params.samples += 2
    if present_out is not None:
        job.present(params.samples, present_out, stream)


class Batch:
    """Many render jobs in one queue set (ct_batch_*): every stage is one
    launch over all jobs' rays, iterations replayed from a CUDA graph.

    jobs: sequence of dicts with scene (Scene), bvh (quad BVH), camera
    (Camera), params (ct_render_params, e.g. Params.to_ct()) and spp."""

    def __init__(self, ctx: Context, jobs, exact_math: bool = False):
        self.ctx = ctx
        arr = (_lib.ct_batch_job * len(jobs))()
        self._keep = []
        for k, j in enumerate(jobs):
            a = arr[k]
            a.scene, a.bvh = j["scene"].h, j["bvh"].h
            a.camera = j["camera"].to_ct()
            a.params = j["params"]
            a.spp = int(j["spp"])
            self._keep.append((j["scene"], j["bvh"]))
        self.sizes = [(int(j["params"].width), int(j["params"].height)) for j in jobs]
        self.h = ctypes.c_void_p()
        check(ctx.lib.ct_batch_create(ctx.h, arr, len(jobs), int(exact_math), ctypes.byref(self.h)), ctx.h)

    def close(self):
        if self.h:
            self.ctx.lib.ct_batch_destroy(self.ctx.h, self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def run(self, stream=None):
        check(self.ctx.lib.ct_batch_run(self.ctx.h, self.h, _stream(stream)), self.ctx.h)

    def accum_tensor(self, job: int):
        """Job `job`'s float4 accumulation as a (h*w, 4) torch view (no copy)."""
        import torch

        p, n = ctypes.c_void_p(), ctypes.c_uint32()
        check(self.ctx.lib.ct_batch_accum(self.h, job, ctypes.byref(p), ctypes.byref(n)))
        return _device_view(p.value, n.value * 4, torch.float32).view(-1, 4)

    @property
    def tuning(self) -> dict:
        t = _lib.ct_batch_tuning()
        check(self.ctx.lib.ct_batch_get_tuning(self.h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}

    def set_tuning(self, extend_block=128, connect_block=128, shade_waves=1, use_graph=1, sort_key=0, refill=24):
        t = _lib.ct_batch_tuning(extend_block, connect_block, shade_waves, use_graph, sort_key, refill)
        check(self.ctx.lib.ct_batch_set_tuning(self.ctx.h, self.h, ctypes.byref(t)), self.ctx.h)

    def autotune(self, stream=None) -> tuple[dict, float]:
        t, ms = _lib.ct_batch_tuning(), ctypes.c_double()
        check(self.ctx.lib.ct_batch_autotune(self.ctx.h, self.h, _stream(stream), ctypes.byref(t), ctypes.byref(ms)),
              self.ctx.h)
        return {k: getattr(t, k) for k, _ in t._fields_}, ms.value

    def stats(self, reset=False, stream=None) -> dict:
        s = _lib.ct_frame_stats()
        check(self.ctx.lib.ct_batch_stats(self.ctx.h, self.h, ctypes.byref(s), int(reset), _stream(stream)), self.ctx.h)
        return {k: getattr(s, k) for k, _ in s._fields_}


class Server:
    """The serving loop (ct_server_*): render jobs and ray queries admitted as
    they arrive against an HBM budget, render jobs continuously batched, ray
    queries overlapping on a second stream. Results land in pinned host
    buffers owned here until the request is waited for."""

    def __init__(self, ctx: Context, hbm_budget: int = 0, max_inflight_pixels: int = 1 << 22,
                 exact_math: bool = False, iter_pixels: int = 0):
        self.ctx = ctx
        cfg = _lib.ct_server_config(int(hbm_budget), int(max_inflight_pixels), int(exact_math), int(iter_pixels))
        self.h = ctypes.c_void_p()
        check(ctx.lib.ct_server_create(ctx.h, ctypes.byref(cfg), ctypes.byref(self.h)), ctx.h)
        self._req = {}

    def close(self):
        if self.h:
            self.ctx.lib.ct_server_destroy(self.h)
            self.h = None
            self._req.clear()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @staticmethod
    def _pinned(shape, dtype):
        import torch

        return torch.empty(shape, dtype=dtype, pin_memory=True)

    def submit_render(self, job: dict) -> int:
        import torch

        W, H = int(job["params"].width), int(job["params"].height)
        out = self._pinned((W * H, 4), torch.float32)
        j = _lib.ct_batch_job()
        j.scene, j.bvh = job["scene"].h, job["bvh"].h
        j.camera = job["camera"].to_ct()
        j.params = job["params"]
        j.spp = int(job["spp"])
        rid = ctypes.c_uint64()
        check(self.ctx.lib.ct_server_submit_render(self.h, ctypes.byref(j), out.data_ptr(), ctypes.byref(rid)),
              self.ctx.h)
        self._req[rid.value] = ("render", out, job)
        return rid.value

    def submit_query(self, bvh: "BVH", org: np.ndarray, dir: np.ndarray, any_hit: bool = False,
                     tri_eps: float = 1e-3) -> int:
        import torch

        n = int(org.shape[0])
        o = self._pinned((n, 4), torch.float32)
        d = self._pinned((n, 4), torch.float32)
        o.numpy()[:] = org
        d.numpy()[:] = dir
        rid = ctypes.c_uint64()
        if any_hit:
            occ = self._pinned((n,), torch.uint8)
            check(self.ctx.lib.ct_server_submit_query(self.h, bvh.h, o.data_ptr(), d.data_ptr(), n, float(tri_eps), 1,
                                                      None, None, occ.data_ptr(), ctypes.byref(rid)), self.ctx.h)
            self._req[rid.value] = ("any", (o, d, occ), bvh)
        else:
            hit = self._pinned((n,), torch.int32)
            t = self._pinned((n,), torch.float32)
            check(self.ctx.lib.ct_server_submit_query(self.h, bvh.h, o.data_ptr(), d.data_ptr(), n, float(tri_eps), 0,
                                                      hit.data_ptr(), t.data_ptr(), None, ctypes.byref(rid)),
                  self.ctx.h)
            self._req[rid.value] = ("closest", (o, d, hit, t), bvh)
        return rid.value

    def wait(self, rid: int, timeout: float = -1.0):
        """(info dict, result): result is the (h*w, 4) accumulation, (hit, t)
        or the occlusion flags, as numpy arrays."""
        info = _lib.ct_request_info()
        st = self.ctx.lib.ct_server_wait(self.h, rid, float(timeout), ctypes.byref(info))
        kind, bufs, _ = self._req.pop(rid)
        d = {k: getattr(info, k) for k, _ in info._fields_}
        if st != _lib.CT_OK:
            raise _lib.CTError(st, f"request {rid} failed")
        if kind == "render":
            return d, bufs.numpy().copy()
        if kind == "any":
            return d, bufs[2].numpy().copy()
        return d, (bufs[2].numpy().copy(), bufs[3].numpy().copy())

    def stats(self) -> dict:
        s = _lib.ct_server_stats()
        check(self.ctx.lib.ct_server_get_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in s._fields_}
