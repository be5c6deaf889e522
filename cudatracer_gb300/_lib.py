"""ctypes binding of the C ABI declared in include/cudatracer.h.

The shared library is built in-tree (cudatracer_gb300/libcudatracer.so, see
_build.py). Loading fails loudly when it is missing: there is no CPU fallback
for any entry point.
"""
from __future__ import annotations

import ctypes
import os
from ctypes import POINTER, Structure, c_char_p, c_double, c_float, c_int32, c_uint8, c_uint32, c_uint64, c_void_p

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "libcudatracer.so")

CT_OK = 0
STATUS_NAMES = {
    0: "CT_OK", 1: "CT_ERR_INVALID_ARGUMENT", 2: "CT_ERR_OUT_OF_MEMORY", 3: "CT_ERR_CUDA",
    4: "CT_ERR_UNSUPPORTED", 5: "CT_ERR_TIMEOUT", 6: "CT_ERR_STACK_OVERFLOW", 7: "CT_ERR_NO_DEVICE",
}
globals().update({name: code for code, name in STATUS_NAMES.items()})
CT_BVH_BINARY, CT_BVH_QUAD, CT_BVH_WIDE8_Q8 = 0, 1, 2
CT_SHADE_COMPAT, CT_SHADE_FULL = 0, 1
CT_TEX_NEAREST, CT_TEX_BILINEAR = 0, 1
CT_SORT_NONE, CT_SORT_OCTANT, CT_SORT_FACE_CELLS = 0, 1, 2
CT_MATH_FAST, CT_MATH_EXACT, CT_MATH_EXACT_SHADE = 0, 1, 2


class CTError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {message}")
        self.status = status


class ct_material(Structure):
    _fields_ = [
        ("albedo", c_float * 3), ("refract_idx", c_float), ("diffuse_tex", c_int32), ("normal_tex", c_int32),
        ("mask_tex", c_int32), ("displace_tex", c_int32), ("type", c_int32), ("roughness", c_float),
        ("absorption", c_float * 3),
    ]


class ct_scene_desc(Structure):
    _fields_ = [
        ("vertices", c_void_p), ("normals", c_void_p), ("texcoords", c_void_p), ("vertex_count", c_uint32),
        ("indices", c_void_p), ("center_normals", c_void_p), ("material_indices", c_void_p),
        ("triangle_count", c_uint32), ("materials", c_void_p), ("material_count", c_uint32),
        ("light_indices", c_void_p), ("light_count", c_uint32), ("texels", c_void_p), ("texel_count", c_uint64),
        ("texture_dims", c_void_p), ("texture_offsets", c_void_p), ("texture_count", c_uint32),
        ("skybox_texture", c_int32),
    ]


class ct_bvh_info(Structure):
    _fields_ = [
        ("binary_node_count", c_uint32), ("quad_node_count", c_uint32), ("prim_count", c_uint32),
        ("max_leaf_size", c_uint32), ("quad_depth", c_uint32), ("stack_entries", c_uint32),
        ("build_ms", c_double), ("collapse_ms", c_double), ("upload_ms", c_double), ("device_bytes", c_uint64),
    ]


class ct_camera(Structure):
    _fields_ = [("position", c_float * 3), ("forward", c_float * 3), ("up", c_float * 3), ("fov_deg", c_float)]


class ct_render_params(Structure):
    _fields_ = [
        ("width", c_int32), ("height", c_int32), ("max_depth", c_int32), ("frame_index", c_uint32),
        ("shading_mode", c_int32), ("exact_math", c_int32), ("shadow", c_int32), ("indirect", c_int32),
        ("sky", c_int32), ("normal_eps", c_float), ("dist_eps", c_float), ("tri_eps", c_float),
        ("texture_filter", c_int32), ("ray_sort", c_int32),
    ]


class ct_frame_stats(Structure):
    _fields_ = [("extension_rays", c_uint64), ("shadow_rays", c_uint64), ("samples", c_uint64), ("frames", c_uint32)]


class ct_batch_job(Structure):
    _fields_ = [("scene", c_void_p), ("bvh", c_void_p), ("camera", ct_camera), ("params", ct_render_params),
                ("spp", c_uint32)]


class ct_batch_tuning(Structure):
    _fields_ = [("extend_block", c_int32), ("connect_block", c_int32), ("shade_waves", c_int32),
                ("use_graph", c_int32), ("sort_key", c_int32), ("refill", c_int32)]


class ct_server_config(Structure):
    _fields_ = [("hbm_budget", c_uint64), ("max_inflight_pixels", c_uint32), ("exact_math", c_int32),
                ("iter_pixels", c_uint32)]


class ct_request_info(Structure):
    _fields_ = [("status", c_int32), ("kind", c_int32), ("submit_s", c_double), ("admit_s", c_double),
                ("done_s", c_double), ("device_bytes", c_uint64)]


class ct_server_stats(Structure):
    _fields_ = [("submitted", c_uint64), ("completed", c_uint64), ("failed", c_uint64), ("iterations", c_uint64),
                ("peak_bytes", c_uint64), ("extension_rays", c_uint64), ("shadow_rays", c_uint64),
                ("query_rays", c_uint64)]


class ct_stage_times(Structure):
    _fields_ = [("ms", c_double * 4), ("launches", c_uint32 * 4)]


P = c_void_p
PP = POINTER(c_void_p)
# name -> (restype, argtypes)
SIGNATURES = {
    "ct_abi_version": (c_uint32, []),
    "ct_render_params_default": (None, [POINTER(ct_render_params)]),
    "ct_ctx_create": (c_int32, [c_int32, PP]),
    "ct_ctx_destroy": (c_int32, [P]),
    "ct_last_error": (c_char_p, [P]),
    "ct_ctx_set_memory_budget": (c_int32, [P, c_uint64]),
    "ct_ctx_device_bytes": (c_uint64, [P]),
    "ct_ctx_check": (c_int32, [P, P]),
    "ct_scene_create": (c_int32, [P, POINTER(ct_scene_desc), PP]),
    "ct_scene_destroy": (c_int32, [P, P]),
    "ct_scene_set_material": (c_int32, [P, P, c_uint32, POINTER(ct_material)]),
    "ct_bvh_build": (c_int32, [P, P, c_int32, PP]),
    "ct_bvh_build_fast": (c_int32, [P, P, c_int32, PP]),
    "ct_bvh_import_quad": (c_int32, [P, P, P, c_uint32, P, c_uint32, PP]),
    "ct_bvh_import_binary": (c_int32, [P, P, P, c_uint32, P, c_uint32, PP]),
    "ct_bvh_info_get": (c_int32, [P, POINTER(ct_bvh_info)]),
    "ct_bvh_export": (c_int32, [P, c_int32, P, P]),
    "ct_bvh_destroy": (c_int32, [P, P]),
    "ct_host_bvh_build": (c_int32, [P, c_uint32, P, c_uint32, c_int32, PP]),
    "ct_host_bvh_build_fast": (c_int32, [P, c_uint32, P, c_uint32, c_int32, PP]),
    "ct_host_bvh_counts": (c_int32, [P, POINTER(c_uint32), POINTER(c_uint32), POINTER(c_uint32),
                                     POINTER(c_double), POINTER(c_double)]),
    "ct_host_bvh_export": (c_int32, [P, c_int32, P, P]),
    "ct_host_bvh_destroy": (c_int32, [P]),
    "ct_bvh_build_device": (c_int32, [P, P, P, PP]),
    "ct_bvh_build_fast_device": (c_int32, [P, P, P, PP]),
    "ct_bvh_build_wide": (c_int32, [P, P, P, PP]),
    "ct_bvh_wide_stats": (c_int32, [P, P, POINTER(c_uint64), POINTER(c_uint64), POINTER(c_uint64), POINTER(c_uint64),
                                    c_int32]),
    "ct_mesh_load_obj": (c_int32, [c_char_p, c_int32, PP]),
    "ct_mesh_info": (c_int32, [P, POINTER(c_uint32), POINTER(c_uint32), POINTER(c_uint32)]),
    "ct_mesh_arrays": (c_int32, [P, P, P, P, P, P]),
    "ct_mesh_material": (c_int32, [P, c_uint32, POINTER(ct_material), P, P, c_uint32]),
    "ct_mesh_destroy": (c_int32, [P]),
    "ct_image_load": (c_int32, [c_char_p, POINTER(c_uint32), POINTER(c_uint32), P]),
    "ct_mesh_last_error": (c_char_p, []),
    "ct_trace_closest": (c_int32, [P, P, P, P, P, P, c_uint32, c_float, P]),
    "ct_trace_any": (c_int32, [P, P, P, P, P, c_uint32, c_float, P]),
    "ct_render_create": (c_int32, [P, c_int32, c_int32, PP]),
    "ct_render_destroy": (c_int32, [P, P]),
    "ct_render_reset": (c_int32, [P, P, P]),
    "ct_render_accumulate": (c_int32, [P, P, P, POINTER(ct_camera), POINTER(ct_render_params), P, P]),
    "ct_render_accum": (c_int32, [P, PP]),
    "ct_present": (c_int32, [P, P, c_float, P, P]),
    "ct_render_stats": (c_int32, [P, P, POINTER(ct_frame_stats), c_int32, P]),
    "ct_render_profile": (c_int32, [P, P, c_int32]),
    "ct_render_profile_read": (c_int32, [P, P, POINTER(ct_stage_times), c_int32]),
    "ct_render_accumulate_noalloc": (c_int32, [P, P, P, POINTER(ct_camera), POINTER(ct_render_params), P, P]),
    "ct_batch_create": (c_int32, [P, POINTER(ct_batch_job), c_uint32, c_int32, PP]),
    "ct_batch_destroy": (c_int32, [P, P]),
    "ct_batch_run": (c_int32, [P, P, P]),
    "ct_batch_accum": (c_int32, [P, c_uint32, PP, POINTER(c_uint32)]),
    "ct_batch_set_tuning": (c_int32, [P, P, POINTER(ct_batch_tuning)]),
    "ct_batch_get_tuning": (c_int32, [P, POINTER(ct_batch_tuning)]),
    "ct_batch_autotune": (c_int32, [P, P, P, POINTER(ct_batch_tuning), POINTER(c_double)]),
    "ct_batch_stats": (c_int32, [P, P, POINTER(ct_frame_stats), c_int32, P]),
    "ct_server_create": (c_int32, [P, POINTER(ct_server_config), PP]),
    "ct_server_destroy": (c_int32, [P]),
    "ct_server_submit_render": (c_int32, [P, POINTER(ct_batch_job), P, POINTER(c_uint64)]),
    "ct_server_submit_query": (c_int32, [P, P, P, P, c_uint32, c_float, c_int32, P, P, P, POINTER(c_uint64)]),
    "ct_server_wait": (c_int32, [P, c_uint64, c_double, POINTER(ct_request_info)]),
    "ct_server_get_stats": (c_int32, [P, POINTER(ct_server_stats)]),
}

_lib = None


def load(path: str | None = None) -> ctypes.CDLL:
    """Load libcudatracer.so (build it with cudatracer_gb300._build.build())."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = path or LIB_PATH
    if not os.path.exists(p):
        raise ImportError(f"{p} is missing: run `python -m cudatracer_gb300._build` (no CPU fallback exists)")
    lib = ctypes.CDLL(p)
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.ct_abi_version() != 1:
        raise ImportError("libcudatracer ABI version mismatch")
    if path is None:
        _lib = lib
    return lib


def check(status: int, ctx=None) -> None:
    if status != CT_OK:
        msg = ""
        if ctx is not None:
            raw = load().ct_last_error(ctx)
            msg = raw.decode(errors="replace") if raw else ""
        raise CTError(status, msg)


def ptr(a) -> int | None:
    """Raw address of a numpy array or torch tensor (None passes NULL)."""
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return a.ctypes.data


__all__ = [n for n in dir() if n.startswith("ct_") or n.startswith("CT_")] + ["load", "check", "ptr", "CTError"]
_ = (c_uint8,)
