"""Time the REFERENCE's own GPU frame loop against this repository's kernels on
the same frames (run on a machine with a GB300 and the staged reference sources).

TEST INFRASTRUCTURE ONLY (oracle): the reference's src/CUDA/Kernel.cu is built
for sm_103a from the patched copy in oracle/_ref/gpu/src (ref_build.py:
GPU_PATCHES - OpenGL presentation removed, grid sizes rounded up, traversal
stacks of 64 entries instead of 32) with oracle/ref_gpu_harness.cu, whose
ctref_gpu_time runs launchKernels frame after frame between CUDA events.

Workload: the 3,117,066-triangle terrain scene of the benchmark
(scenes.terrain_scene()), 1920x1080, 1 spp per frame, compat shading (the
reference's shade kernel), five passes (the reference's fixed maxPathLength),
the sky off (the reference's sky lookup reads outside its texture for NaN
directions), on the reference's own quad tree (its host BVHTree/MBVHTree
build, libctref). This repository renders the same frames (same seeds) through
its C ABI on the same tree (device build: identical quad nodes) and on
ct_bvh_build_fast_device's tree, in CT_MATH_FAST (CUDA float functions, as the
reference's build) and CT_MATH_EXACT_SHADE. Both accumulate the same frames, so
the two images are compared pixel by pixel (a sanity check that they computed
the same thing: the first frame pixel by pixel, where rounding divergence moves a
few percent of pixels, and the image totals after all frames). After the first
frame the two do not render the same samples per pixel: the reference shifts
the pixel each queue slot starts from by start_position (Kernel.cu:75-86, 227)
while its primary-ray jitter is keyed to the slot, and its frame counter and
start_position are globals that carry over from the earlier call; this
repository keeps the slot = pixel (offset 0). Per-pixel differences of the
accumulations after all frames are reported but are not a parity measure.

    python oracle/ref_gpu_bench.py [--frames 16]

Prints one JSON line."""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

W, H, DEPTH = 1920, 1080, 5
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


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--frames", type=int, default=16)
    args = ap.parse_args()
    import oracle
    import ref_build
    import torch

    from cudatracer_gb300 import _build, api, scenes

    oracle.build()
    lib_path = ref_build.compile_gpu_lib()
    _build.build()
    ts, cam = scenes.terrain_scene()
    arr = scenes.scene_arrays(ts)
    P = ctypes.c_void_p
    R = oracle.ref()
    v, ix = np.ascontiguousarray(ts.vertices), np.ascontiguousarray(ts.indices)
    t0 = time.perf_counter()
    h = R.ctref_build(v.ctypes.data_as(P), v.shape[0], ix.ctypes.data_as(P), ix.shape[0], os.cpu_count() or 1)
    ref_build_ms = (time.perf_counter() - t0) * 1e3
    quad = np.zeros((R.ctref_mbvh_count(h), 32), np.int32)
    prims = np.zeros(ix.shape[0], np.uint32)
    R.ctref_export(h, None, prims.ctypes.data_as(P), quad.ctypes.data_as(P))
    R.ctref_free(h)
    depth = quad_depth(quad)
    if 3 * depth + 1 > 64:
        raise SystemExit(f"quad depth {depth} would overflow the 64-entry traversal stack")
    mats = oracle.pack_materials(ts.materials)
    a = {k: np.ascontiguousarray(arr[k]) for k in ("vertices", "normals", "center_normals", "texcoords", "indices",
                                                   "material_idxs", "light_indices")}
    L = ctypes.CDLL(lib_path)
    L.ctref_gpu_time.restype = ctypes.c_int
    L.ctref_gpu_frame.restype = ctypes.c_int
    pos = np.asarray(cam["position"], np.float32)
    fw = np.asarray(cam["forward"], np.float32)
    up = np.asarray(cam["up"], np.float32)
    ref_acc = np.zeros((W * H, 4), np.float32)
    ms = ctypes.c_float(0.0)
    scene_args = (
        a["vertices"].ctypes.data_as(P), v.shape[0], a["normals"].ctypes.data_as(P),
        a["center_normals"].ctypes.data_as(P), a["texcoords"].ctypes.data_as(P), a["indices"].ctypes.data_as(P),
        ix.shape[0], a["material_idxs"].ctypes.data_as(P), mats.ctypes.data_as(P), len(mats),
        a["light_indices"].ctypes.data_as(P), int(a["light_indices"].size), quad.ctypes.data_as(P), quad.shape[0],
        prims.ctypes.data_as(P), prims.size, pos.ctypes.data_as(P), fw.ctypes.data_as(P), up.ctypes.data_as(P),
        ctypes.c_float(cam["fov"]), W, H, ctypes.c_float(EPS[0]), ctypes.c_float(EPS[1]), ctypes.c_float(EPS[2]), 1, 1)
    ref_first = np.zeros((W * H, 4), np.float32)
    if L.ctref_gpu_frame(*scene_args, ref_first.ctypes.data_as(P)) != 0:
        raise SystemExit("ctref_gpu_frame failed")
    st = L.ctref_gpu_time(*scene_args, args.frames, ctypes.byref(ms), ref_acc.ctypes.data_as(P))
    if st != 0:
        raise SystemExit(f"ctref_gpu_time failed ({st})")
    samples = W * H * args.frames
    out = {"workload": f"terrain {ix.shape[0]:,} triangles, {W}x{H}, 1 spp x {args.frames} frames (after one "
                       f"untimed), depth {DEPTH}, compat shading, sky off",
           "reference_gpu": {"msamples_per_s": samples / (ms.value / 1e3) / 1e6, "ms_per_frame": ms.value / args.frames,
                             "tree": f"the reference's host build ({ref_build_ms:.0f} ms), quad depth {depth}",
                             "build": "src/CUDA/Kernel.cu for sm_103a, oracle/ref_build.py GPU_PATCHES"}}
    ctx = api.Context(0)
    sc = ctx.scene(arr, [api.Material(**m) for m in ts.materials], ts.textures, ts.skybox_texture)
    trees = {"reference_tree": sc.build_bvh_device(), "fast_tree": sc.build_bvh_fast_device()}
    qd = trees["reference_tree"].export()[0]
    out["reference_tree_identical"] = bool(np.array_equal(np.ascontiguousarray(qd).view(np.int32), quad))
    camera = api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"])
    stream = torch.cuda.Stream()
    for tname, tree in trees.items():
        for mname, mode in (("fast", 0), ("exact_shade", 2)):
            job = api.RenderJob(ctx, W, H)
            p = api.Params(W, H, camera=camera, max_depth=DEPTH, exact_math=mode, sky=False, normal_eps=EPS[0],
                           dist_eps=EPS[1], tri_eps=EPS[2])
            p.reset(job, stream)
            api.launch_kernels(job, sc, tree, p, stream=stream)  # the untimed first frame
            stream.synchronize()
            first = job.accum_tensor().cpu().numpy().reshape(-1, 4).copy()
            rel1 = np.abs(first - ref_first) / np.maximum(np.abs(ref_first), 1e-6)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(args.frames):
                api.launch_kernels(job, sc, tree, p, stream=stream)
            e1.record(stream)
            stream.synchronize()
            ctx.check(stream)
            t = e0.elapsed_time(e1)
            acc = job.accum_tensor().cpu().numpy().reshape(-1, 4)
            rel = np.abs(acc - ref_acc) / np.maximum(np.abs(ref_acc), 1e-6)
            out[f"ours_{tname}_{mname}"] = {
                "msamples_per_s": samples / (t / 1e3) / 1e6, "ms_per_frame": t / args.frames,
                "first_frame_pixels_outside_1e-4_of_reference": float((rel1 > 1e-4).any(axis=1).mean()),
                "pixels_outside_1e-4_of_reference_after_all_frames": float((rel > 1e-4).any(axis=1).mean()),
                "total_ratio_vs_reference": float(acc[:, :3].sum() / ref_acc[:, :3].sum())}
            job.close()
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
