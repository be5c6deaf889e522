"""Record a golden frame rendered by the REFERENCE's own GPU kernels.

The reference's frame composition (generatePrimaryRays, extend, shade, connect
in src/CUDA/Kernel.cu) runs only on a GPU, so the oracle's restatement of it
is otherwise pinned function by function. This script builds the reference's
Kernel.cu (oracle/ref_build.py: compile_gpu_lib, from the patched copy staged
in oracle/_ref/gpu/src; the patches remove the OpenGL presentation and fix the
grid sizes that drop tail rays) with oracle/ref_gpu_harness.cu, and renders the
first frame of a small seeded terrain scene through the reference's own
launchKernels: its own quad BVH (MBVHTree, built by its host code in
oracle/_ref/libctref.so), compat shading, depth 5, no sky and no textures.
Run on a machine with a GB300 and the staged reference sources:

    python tests/golden/make_ref_frame.py [out.npz]

Output (committed as tests/golden/ref_frame_gpu.npz): the float4 accumulation
of the frame and the scene parameters, with a digest of the reference's tree.
The scene's quad depth must keep the reference's 32-entry traversal stack in
bounds (3 x depth + 1 <= 32); the script checks that before it launches.
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

SCENE = dict(grid=32, spheres=3, sky_size=(64, 32))
W, H, DEPTH = 64, 48, 5
EPS = (1e-5, 1e-5, 1e-3)


def quad_depth(quad: np.ndarray) -> int:
    q = np.ascontiguousarray(quad).view(np.int32).reshape(-1, 32)
    childs, counts = q[:, 24:28], q[:, 28:32]
    depth, stack = 0, [(0, 1)]
    while stack:
        n, lv = stack.pop()
        depth = max(depth, lv)
        for k in range(4):
            if counts[n, k] == -1:
                stack.append((int(childs[n, k]), lv + 1))
    return depth


def main(out: str) -> None:
    import oracle
    import ref_build
    from cudatracer_gb300 import scenes

    oracle.build()
    lib_path = ref_build.compile_gpu_lib()
    ts, cam = scenes.terrain_scene(**SCENE)
    arr = scenes.scene_arrays(ts)
    R = oracle.ref()
    P = ctypes.c_void_p
    v, ix = np.ascontiguousarray(ts.vertices), np.ascontiguousarray(ts.indices)
    h = R.ctref_build(v.ctypes.data_as(P), v.shape[0], ix.ctypes.data_as(P), ix.shape[0], os.cpu_count() or 1)
    quad = np.zeros((R.ctref_mbvh_count(h), 32), np.int32)
    prims = np.zeros(ix.shape[0], np.uint32)
    R.ctref_export(h, None, prims.ctypes.data_as(P), quad.ctypes.data_as(P))
    R.ctref_free(h)
    depth = quad_depth(quad)
    if 3 * depth + 1 > 32:
        raise SystemExit(f"quad depth {depth} would overflow the reference's 32-entry traversal stack")
    mats = oracle.pack_materials(ts.materials)
    a = {k: np.ascontiguousarray(arr[k]) for k in ("vertices", "normals", "center_normals", "texcoords", "indices",
                                                   "material_idxs", "light_indices")}
    L = ctypes.CDLL(lib_path)
    L.ctref_gpu_frame.restype = ctypes.c_int
    fp = ctypes.POINTER(ctypes.c_float)
    accum = np.zeros((W * H, 4), np.float32)
    pos = np.asarray(cam["position"], np.float32)
    fw = np.asarray(cam["forward"], np.float32)
    up = np.asarray(cam["up"], np.float32)
    st = L.ctref_gpu_frame(
        a["vertices"].ctypes.data_as(P), v.shape[0], a["normals"].ctypes.data_as(P),
        a["center_normals"].ctypes.data_as(P), a["texcoords"].ctypes.data_as(P), a["indices"].ctypes.data_as(P),
        ix.shape[0], a["material_idxs"].ctypes.data_as(P), mats.ctypes.data_as(P), len(mats),
        a["light_indices"].ctypes.data_as(P), int(a["light_indices"].size), quad.ctypes.data_as(P), quad.shape[0],
        prims.ctypes.data_as(P), prims.size, pos.ctypes.data_as(P), fw.ctypes.data_as(P), up.ctypes.data_as(P),
        ctypes.c_float(cam["fov"]), W, H, ctypes.c_float(EPS[0]), ctypes.c_float(EPS[1]), ctypes.c_float(EPS[2]), 1,
        1, accum.ctypes.data_as(P))
    if st != 0:
        raise SystemExit(f"ctref_gpu_frame failed ({st})")
    np.savez_compressed(out, accum=accum, width=W, height=H, depth=DEPTH, eps=np.asarray(EPS, np.float32),
                        grid=SCENE["grid"], spheres=SCENE["spheres"], quad_depth=depth,
                        quad_sha=hashlib.sha256(quad.tobytes()).hexdigest(),
                        prims_sha=hashlib.sha256(prims.tobytes()).hexdigest())
    print(f"wrote {out}: {int((accum[:, 3] > 0).sum())} of {W * H} pixels with a contribution, quad depth {depth}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(HERE, "ref_frame_gpu.npz"))
