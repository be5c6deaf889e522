"""Python access to the CPU oracle (liboracle.so) and the reference build (libctref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py. The product package never imports this module.

  liboracle.so  - oracle/ct_oracle.cpp, a scalar C++ restatement of the
                  reference's hot path (build, traversal, wavefront frame).
  libctref.so   - the reference's own host code (oracle/ref_build.py); only
                  present where the reference sources were staged.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SRC = os.path.join(HERE, "ct_oracle.cpp")
# the reproducible binary32 functions exact-math frames use on both sides
PORTABLE_MATH = os.path.join(os.path.dirname(HERE), "cudatracer_gb300", "csrc", "portable_math.h")
ORACLE_LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libctref.so")
P = ctypes.c_void_p

MAT_DTYPE = np.dtype([
    ("albedo", "<f4", 3), ("refract_idx", "<f4"), ("diffuse_tex", "<i4"), ("normal_tex", "<i4"),
    ("mask_tex", "<i4"), ("displace_tex", "<i4"), ("type", "<i4"), ("roughness", "<f4"), ("absorption", "<f4", 3),
])
assert MAT_DTYPE.itemsize == 52


def _elf_machine(path: str) -> int:
    with open(path, "rb") as f:
        return int.from_bytes(f.read(20)[18:20], "little")


def _native_machine() -> int:
    import platform

    return 62 if platform.machine().lower() in ("x86_64", "amd64") else 183


# The same source built with floating-point contraction (a*b+c fused where the
# compiler finds it, as nvcc does by default): used only to compare with frames
# the reference's own GPU build rendered, whose rounding it follows more closely.
ORACLE_FMA_LIB = os.path.join(HERE, "liboracle_fma.so")


def build_oracle(force: bool = False, contracted: bool = False) -> str:
    out = ORACLE_FMA_LIB if contracted else ORACLE_LIB
    fresh = (os.path.exists(out) and os.path.getmtime(out) >= os.path.getmtime(ORACLE_SRC)
             and os.path.getmtime(out) >= os.path.getmtime(PORTABLE_MATH)
             and _elf_machine(out) == _native_machine())
    if fresh and not force:
        return out
    tmp = out + ".tmp"
    if contracted:
        fp = ["-ffp-contract=fast"] + (["-mfma"] if _native_machine() == 62 else [])
    else:
        fp = ["-ffp-contract=off"]
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", *fp, "-fno-fast-math", "-o", tmp, ORACLE_SRC]
    subprocess.run(cmd, check=True)
    os.replace(tmp, out)
    return out


FP64_SRC = os.path.join(HERE, "ct_fp64.cpp")
FP64_LIB = os.path.join(HERE, "libfp64.so")


def build_fp64(force: bool = False) -> str:
    fresh = (os.path.exists(FP64_LIB) and os.path.getmtime(FP64_LIB) >= os.path.getmtime(FP64_SRC)
             and _elf_machine(FP64_LIB) == _native_machine())
    if fresh and not force:
        return FP64_LIB
    tmp = FP64_LIB + ".tmp"
    subprocess.run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-pthread", "-ffp-contract=off",
                    "-fno-fast-math", "-o", tmp, FP64_SRC], check=True)
    os.replace(tmp, FP64_LIB)
    return FP64_LIB


_fp64 = None


def fp64() -> ctypes.CDLL:
    global _fp64
    if _fp64 is None:
        build_fp64()
        L = ctypes.CDLL(FP64_LIB)
        L.fp64_render.argtypes = [P, P, P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                  ctypes.c_uint64, P, P, ctypes.c_int]
        L.fp64_microfacet.argtypes = [ctypes.c_int, ctypes.c_double, P, ctypes.c_double, ctypes.c_double, P, P, P]
        L.fp64_roughness_to_alpha.restype = ctypes.c_double
        L.fp64_roughness_to_alpha.argtypes = [ctypes.c_double]
        L.fp64_trace.argtypes = [P, P, P, P, P, P, ctypes.c_uint32, ctypes.c_int, P, P, ctypes.c_int]
        _fp64 = L
    return _fp64


def trace_fp64(vertices, indices, quad, prims, org, dir, any_hit: bool = False, nthreads: int = 8):
    """FP64 watertight closest hit (or occlusion) over the padded quad BVH:
    returns (hit int32, t float64); equal t resolves to the lower primitive id."""
    v = np.ascontiguousarray(vertices, np.float32)
    ix = np.ascontiguousarray(indices, np.uint32)
    q = np.ascontiguousarray(quad)
    pr = np.ascontiguousarray(prims, np.uint32)
    o = np.ascontiguousarray(org, np.float32)
    d = np.ascontiguousarray(dir, np.float32)
    n = o.shape[0]
    hit = np.empty(n, np.int32)
    t = np.empty(n, np.float64)
    fp64().fp64_trace(_p(v), _p(ix), _p(q), _p(pr), _p(o), _p(d), n, int(any_hit), _p(hit), _p(t), nthreads)
    return hit, t


def render_fp64(arrays: dict, materials: np.ndarray, quad, prims, camera: dict, width: int, height: int, spp: int,
                depth: int, textures=(), sky_tex: int = -1, sky: bool = True, shadow: bool = True,
                indirect: bool = True, eps=(1e-5, 1e-5, 1e-3), seed: int = 1, nthreads: int = 8,
                tex_filter: int = 0):
    """FP64 Monte Carlo estimate of the full-material image: per-pixel (mean, standard error), (h*w, 3) each."""
    L = fp64()
    a = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
    texels = dims = offs = None
    if textures:
        flat, dl, ol, o = [], [], [], 0
        for tx in textures:
            tx = np.ascontiguousarray(tx, np.float32)
            h, w = tx.shape[:2]
            flat.append(tx.reshape(-1, 4))
            dl += [w, h]
            ol.append(o)
            o += w * h
        texels = np.ascontiguousarray(np.concatenate(flat))
        dims = np.asarray(dl, np.uint32)
        offs = np.asarray(ol, np.uint32)
    li = a.get("light_indices")
    mats = np.ascontiguousarray(materials)
    q = np.ascontiguousarray(quad)
    pr = np.ascontiguousarray(prims, np.uint32)
    d = OrSceneDesc(
        _p(a["vertices"]), _p(a["normals"]), _p(a["center_normals"]), _p(a["texcoords"]), _p(a["indices"]),
        _p(a["material_idxs"]), _p(mats), _p(li) if li is not None and li.size else None,
        0 if li is None else int(li.size), _p(texels), _p(dims), _p(offs), sky_tex,
        int(sky and sky_tex >= 0), int(shadow), int(indirect), eps[0], eps[1], eps[2], _p(q), _p(pr), int(tex_filter))
    hor, ver = camera_basis(camera["forward"], camera["up"], camera["fov"], width, height)
    pos = np.asarray(camera["position"], np.float32)
    fw = np.asarray(camera["forward"], np.float32)
    s = np.zeros((width * height, 3), np.float64)
    s2 = np.zeros((width * height, 3), np.float64)
    L.fp64_render(ctypes.byref(d), _p(pos), _p(fw), _p(hor), _p(ver), width, height, spp, depth, seed, _p(s), _p(s2),
                  nthreads)
    mean = s / spp
    var = np.maximum(s2 / spp - mean * mean, 0.0)
    return mean, np.sqrt(var / spp)


def build(force: bool = False) -> None:
    """Compile the oracle restatement and, where its sources exist, the reference."""
    build_oracle(force)
    build_fp64(force)
    try:
        from . import ref_build  # type: ignore
    except ImportError:
        import importlib.util

        spec = importlib.util.spec_from_file_location("ref_build", os.path.join(HERE, "ref_build.py"))
        ref_build = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(ref_build)
    ref_build.build()


_orc = None
_orc_fma = None
_ref = None


def lib(contracted: bool = False) -> ctypes.CDLL:
    """The oracle library; contracted=True the build with FMA contraction."""
    global _orc, _orc_fma
    if contracted:
        if _orc_fma is None:
            _orc_fma = _bind(ctypes.CDLL(build_oracle(contracted=True)))
        return _orc_fma
    if _orc is None:
        _orc = _bind(ctypes.CDLL(build_oracle()))
    return _orc


def _bind(L: ctypes.CDLL) -> ctypes.CDLL:
    L.or_build.restype = P
    L.or_build.argtypes = [P, P, ctypes.c_int, ctypes.c_int]
    for n in ("or_bvh_count", "or_mbvh_count"):
        getattr(L, n).argtypes = [P]
    L.or_export.argtypes = [P, P, P, P]
    L.or_free.argtypes = [P]
    L.or_trace_closest.argtypes = [P, P, P, P, ctypes.c_float, P, P, ctypes.c_int, P, P, P, ctypes.c_int]
    L.or_trace_any.argtypes = [P, P, P, P, ctypes.c_float, P, P, P, ctypes.c_int, P, ctypes.c_int]
    L.or_trace_closest_binary.argtypes = [P, P, P, P, ctypes.c_float, P, P, ctypes.c_int, P, P, ctypes.c_int]
    L.or_camera_basis.argtypes = [P, P, ctypes.c_float, ctypes.c_int, ctypes.c_int, P, P]
    L.or_render_frame.argtypes = [P, P, P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.c_int,
                                  ctypes.c_int, P, ctypes.c_int, ctypes.c_int, ctypes.c_int]
    L.or_present.argtypes = [P, ctypes.c_int, ctypes.c_float, P]
    L.or_plane_distance.restype = ctypes.c_float
    L.or_plane_distance.argtypes = [ctypes.c_float]
    return L


def ref_available() -> bool:
    return os.path.exists(REF_LIB) and _elf_machine(REF_LIB) == _native_machine()


def ref() -> ctypes.CDLL:
    global _ref
    if _ref is None:
        if not ref_available():
            raise FileNotFoundError("reference host library not built (oracle/ref_build.py)")
        L = ctypes.CDLL(REF_LIB)
        L.ctref_build.restype = P
        L.ctref_build.argtypes = [P, ctypes.c_int, P, ctypes.c_int, ctypes.c_int]
        for n in ("ctref_build_ms", "ctref_mbvh_ms"):
            getattr(L, n).restype = ctypes.c_double
            getattr(L, n).argtypes = [P]
        for n in ("ctref_bvh_count", "ctref_mbvh_count", "ctref_prim_count"):
            getattr(L, n).argtypes = [P]
        L.ctref_export.argtypes = [P, P, P, P]
        L.ctref_trace_mbvh.argtypes = [P, P, P, ctypes.c_int, P, P, ctypes.c_int]
        L.ctref_trace_bvh.argtypes = [P, P, P, ctypes.c_int, P, P, ctypes.c_int]
        L.ctref_free.argtypes = [P]
        L.ctref_camera_rays.argtypes = [P, ctypes.c_float, ctypes.c_int, ctypes.c_int, P, P]
        L.ctref_camera_plane_distance.restype = ctypes.c_float
        L.ctref_camera_plane_distance.argtypes = [ctypes.c_float]
        L.ctref_wang_hash.restype = ctypes.c_uint32
        L.ctref_wang_hash.argtypes = [ctypes.c_uint32]
        L.ctref_random_stream.argtypes = [ctypes.c_uint32, ctypes.c_int, P, P]
        L.ctref_triangle_intersect.argtypes = [P, P, P, P, P, P, ctypes.c_float]
        L.ctref_mbvh_intersect.argtypes = [P, P, P, ctypes.c_float, P, P]
        L.ctref_area.restype = ctypes.c_float
        L.ctref_fresnel_exact.restype = ctypes.c_float
        L.ctref_fresnel_exact.argtypes = [P, P, ctypes.c_float]
        L.ctref_cos_weighted.argtypes = [ctypes.c_float, ctypes.c_float, P]
        L.ctref_roughness_to_alpha.restype = ctypes.c_float
        L.ctref_roughness_to_alpha.argtypes = [ctypes.c_float]
        L.ctref_mf_sample.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_int, P, ctypes.c_float,
                                      ctypes.c_float, P]
        L.ctref_mf_pdf.restype = ctypes.c_float
        L.ctref_mf_pdf.argtypes = [ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_int, P, P, P]
        L.ctref_sample_bsdf.argtypes = [P, ctypes.c_float, ctypes.c_float, P, P, P, P, P, ctypes.c_float,
                                        ctypes.c_float, P, P, P, P]
        _ref = L
    return _ref


def _p(a):
    return None if a is None else a.ctypes.data_as(P)


# ---------------------------------------------------------------- oracle ----
def bvh_build(verts: np.ndarray, idx: np.ndarray, nthreads: int = 8) -> dict:
    L = lib()
    v = np.ascontiguousarray(verts, np.float32)
    ix = np.ascontiguousarray(idx, np.uint32)
    h = L.or_build(_p(v), _p(ix), ix.shape[0], nthreads)
    try:
        nb, nq = L.or_bvh_count(h), L.or_mbvh_count(h)
        b = np.zeros((nb, 8), np.int32)
        q = np.zeros((nq, 32), np.int32)
        pr = np.zeros(ix.shape[0], np.uint32)
        L.or_export(h, _p(b), _p(pr), _p(q))
        return {"binary": b, "quad": q, "prims": pr}
    finally:
        L.or_free(h)


def trace_closest(quad, prims, verts, idx, org, dir, eps=1e-3, nthreads=8, want_deep=False):
    L = lib()
    o = np.ascontiguousarray(org[:, :3], np.float32)
    d = np.ascontiguousarray(dir[:, :3], np.float32)
    n = o.shape[0]
    hit = np.zeros(n, np.int32)
    t = np.zeros(n, np.float32)
    deep = np.zeros(n, np.int32) if want_deep else None
    L.or_trace_closest(_p(np.ascontiguousarray(quad)), _p(np.ascontiguousarray(prims, np.uint32)),
                       _p(np.ascontiguousarray(verts, np.float32)), _p(np.ascontiguousarray(idx, np.uint32)),
                       eps, _p(o), _p(d), n, _p(hit), _p(t), _p(deep), nthreads)
    return (hit, t, deep) if want_deep else (hit, t)


def trace_any(quad, prims, verts, idx, org, dir, tmax, eps=1e-3, nthreads=8):
    L = lib()
    o = np.ascontiguousarray(org[:, :3], np.float32)
    d = np.ascontiguousarray(dir[:, :3], np.float32)
    tm = np.ascontiguousarray(tmax, np.float32)
    n = o.shape[0]
    occ = np.zeros(n, np.uint8)
    L.or_trace_any(_p(np.ascontiguousarray(quad)), _p(np.ascontiguousarray(prims, np.uint32)),
                   _p(np.ascontiguousarray(verts, np.float32)), _p(np.ascontiguousarray(idx, np.uint32)),
                   eps, _p(o), _p(d), _p(tm), n, _p(occ), nthreads)
    return occ


def trace_closest_binary(binary, prims, verts, idx, org, dir, eps=1e-3, nthreads=8):
    L = lib()
    o = np.ascontiguousarray(org[:, :3], np.float32)
    d = np.ascontiguousarray(dir[:, :3], np.float32)
    n = o.shape[0]
    hit = np.zeros(n, np.int32)
    t = np.zeros(n, np.float32)
    L.or_trace_closest_binary(_p(np.ascontiguousarray(binary)), _p(np.ascontiguousarray(prims, np.uint32)),
                              _p(np.ascontiguousarray(verts, np.float32)), _p(np.ascontiguousarray(idx, np.uint32)),
                              eps, _p(o), _p(d), n, _p(hit), _p(t), nthreads)
    return hit, t


class OrSceneDesc(ctypes.Structure):
    _fields_ = [
        ("verts", P), ("normals", P), ("center_normals", P), ("uvs", P), ("idx", P), ("mat_idx", P),
        ("materials", P), ("lights", P), ("light_count", ctypes.c_uint32), ("tex", P), ("tex_dims", P),
        ("tex_offsets", P), ("sky_tex", ctypes.c_int32), ("sky_enabled", ctypes.c_int32), ("shadow", ctypes.c_int32),
        ("indirect", ctypes.c_int32), ("normal_eps", ctypes.c_float), ("dist_eps", ctypes.c_float),
        ("tri_eps", ctypes.c_float), ("qnodes", P), ("prims", P), ("tex_filter", ctypes.c_int32),
    ]


def pack_materials(mats) -> np.ndarray:
    """mats: sequence of objects/dicts with the Material fields."""
    out = np.zeros(len(mats), MAT_DTYPE)
    for i, m in enumerate(mats):
        g = (lambda k: m[k]) if isinstance(m, dict) else (lambda k: getattr(m, k))
        out[i]["albedo"] = g("albedo")
        out[i]["refract_idx"] = g("refract_idx")
        out[i]["diffuse_tex"] = g("diffuse_tex")
        out[i]["normal_tex"] = g("normal_tex")
        out[i]["mask_tex"] = g("mask_tex")
        out[i]["displace_tex"] = g("displace_tex")
        out[i]["type"] = g("type")
        out[i]["roughness"] = g("roughness")
        out[i]["absorption"] = g("absorption")
    return out


def work_read(reset: bool = True) -> dict:
    """Traversal work counted by render_frames since the last reset."""
    L = lib()
    L.or_work_read.argtypes = [P, ctypes.c_int]
    w = np.zeros(6, np.uint64)
    L.or_work_read(_p(w), int(reset))
    keys = ("ext_rays", "ext_nodes", "ext_tris", "shadow_rays", "shadow_nodes", "shadow_tris")
    return {k: int(v) for k, v in zip(keys, w)}


def set_full_sort(on: bool) -> None:
    """Visit quad children in full distance order (as fast-math GPU frames do)
    instead of the reference's partial order; changes work counts only."""
    L = lib()
    L.or_set_full_sort.argtypes = [ctypes.c_int]
    L.or_set_full_sort(int(on))


def camera_basis(forward, up, fov_deg, width, height):
    L = lib()
    fw = np.asarray(forward, np.float32)
    upv = np.asarray(up, np.float32)
    hor = np.zeros(3, np.float32)
    ver = np.zeros(3, np.float32)
    dist = L.or_plane_distance(float(fov_deg))
    L.or_camera_basis(_p(fw), _p(upv), dist, width, height, _p(hor), _p(ver))
    return hor, ver


def _frame_scene(arrays: dict, materials: np.ndarray, quad, prims, camera: dict, width: int, height: int,
                 textures=(), sky_tex: int = -1, sky: bool = True, shadow: bool = True, indirect: bool = True,
                 eps=(1e-5, 1e-5, 1e-3), tex_filter: int = 0):
    """The OrSceneDesc of a frame and the camera vectors, with the arrays they
    point into (keep the returned tuple alive while the pointers are used)."""
    a = {k: np.ascontiguousarray(v) for k, v in arrays.items()}
    texels = dims = offs = None
    if textures:
        flat, dl, ol, o = [], [], [], 0
        for tx in textures:
            tx = np.ascontiguousarray(tx, np.float32)
            h, w = tx.shape[:2]
            flat.append(tx.reshape(-1, 4))
            dl += [w, h]
            ol.append(o)
            o += w * h
        texels = np.ascontiguousarray(np.concatenate(flat))
        dims = np.asarray(dl, np.uint32)
        offs = np.asarray(ol, np.uint32)
    li = a.get("light_indices")
    mats = np.ascontiguousarray(materials)
    q = np.ascontiguousarray(quad)
    pr = np.ascontiguousarray(prims, np.uint32)
    d = OrSceneDesc(
        _p(a["vertices"]), _p(a["normals"]), _p(a["center_normals"]), _p(a["texcoords"]), _p(a["indices"]),
        _p(a["material_idxs"]), _p(mats), _p(li) if li is not None and li.size else None,
        0 if li is None else int(li.size), _p(texels), _p(dims), _p(offs), sky_tex,
        int(sky and sky_tex >= 0), int(shadow), int(indirect), eps[0], eps[1], eps[2], _p(q), _p(pr), int(tex_filter))
    hor, ver = camera_basis(camera["forward"], camera["up"], camera["fov"], width, height)
    pos = np.asarray(camera["position"], np.float32)
    fw = np.asarray(camera["forward"], np.float32)
    keep = (a, texels, dims, offs, mats, q, pr)
    return d, pos, fw, hor, ver, keep


def render_frames(arrays: dict, materials: np.ndarray, quad, prims, camera: dict, width: int, height: int,
                  frames, depth: int, accum: np.ndarray | None = None, exact_math: bool = True,
                  textures=(), sky_tex: int = -1, sky: bool = True, shadow: bool = True, indirect: bool = True,
                  eps=(1e-5, 1e-5, 1e-3), pixels=None, nthreads: int = 8, tex_filter: int = 0,
                  contracted: bool = False) -> np.ndarray:
    """Accumulate 1-spp frames (seed frame indices `frames`) into accum (h*w,4);
    contracted=True renders with the FMA-contracted build of the oracle."""
    L = lib(contracted)
    if accum is None:
        accum = np.zeros((width * height, 4), np.float32)
    d, pos, fw, hor, ver, _keep = _frame_scene(arrays, materials, quad, prims, camera, width, height, textures,
                                               sky_tex, sky, shadow, indirect, eps, tex_filter)
    p0, p1 = (0, width * height) if pixels is None else pixels
    for fr in frames:
        L.or_render_frame(ctypes.byref(d), _p(pos), _p(fw), _p(hor), _p(ver), width, height, int(fr), depth,
                          int(exact_math), _p(accum), p0, p1, nthreads)
    return accum


def render_pixels(arrays: dict, materials: np.ndarray, quad, prims, camera: dict, width: int, height: int,
                  frames, depth: int, pixels, accum: np.ndarray | None = None, exact_math: bool = True,
                  textures=(), sky_tex: int = -1, nthreads: int = 8, **kw) -> np.ndarray:
    """Accumulate 1-spp frames (seed frame indices `frames`, in order) over the
    listed pixel indices into accum (h*w, 4), in one parallel pass."""
    L = lib()
    if accum is None:
        accum = np.zeros((width * height, 4), np.float32)
    d, pos, fw, hor, ver, _keep = _frame_scene(arrays, materials, quad, prims, camera, width, height, textures,
                                               sky_tex, **kw)
    px = np.ascontiguousarray(pixels, np.int32)
    fr = np.ascontiguousarray(frames, np.uint32)
    P = ctypes.c_void_p
    L.or_render_pixels.argtypes = [P, P, P, P, P, ctypes.c_int, ctypes.c_int, P, ctypes.c_int, ctypes.c_int,
                                   ctypes.c_int, P, P, ctypes.c_int, ctypes.c_int]
    L.or_render_pixels(ctypes.byref(d), _p(pos), _p(fw), _p(hor), _p(ver), width, height, _p(fr), int(fr.size), depth,
                       int(exact_math), _p(accum), _p(px), int(px.size), int(nthreads))
    return accum


def path_hits(arrays: dict, materials: np.ndarray, quad, prims, camera: dict, width: int, height: int, frame: int,
              depth: int, pixel: int, exact_math: bool = True, textures=(), sky_tex: int = -1, **kw):
    """Closest hit of each extension pass of one pixel's path: (primitive ids,
    t values), -2 / 0 for passes the path does not reach (or_path_hits)."""
    L = lib()
    d, pos, fw, hor, ver, _keep = _frame_scene(arrays, materials, quad, prims, camera, width, height, textures,
                                               sky_tex, **kw)
    hits = np.zeros(depth, np.int32)
    ts = np.zeros(depth, np.float32)
    P = ctypes.c_void_p
    L.or_path_hits.argtypes = [P, P, P, P, P, ctypes.c_int, ctypes.c_int, ctypes.c_uint32, ctypes.c_int, ctypes.c_int,
                               ctypes.c_int, P, P]
    L.or_path_hits(ctypes.byref(d), _p(pos), _p(fw), _p(hor), _p(ver), width, height, int(frame), depth,
                   int(exact_math), int(pixel), _p(hits), _p(ts))
    return hits, ts
