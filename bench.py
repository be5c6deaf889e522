#!/usr/bin/env python
"""Benchmark: path-traced Msamples/s of the wavefront tracer on one GB300.

Workload (one step = one 64-frame accumulation: Params::reset, then 64 calls
of the reference's launchKernels, each a 1-spp frame):
  1920x1080, max depth 8, quad BVH, FP32 RGBA accumulation, over a seeded
  fBm-displaced 1024x1024-vertex terrain (2,093,058 triangles) + 200
  icospheres of 5,120 triangles (radii U[0.5,3]) + 4 emissive quads, with a
  2048x1024 FP32 equirect sky (3,117,066 triangles). Synthetic, seeded data.
  Reference shading (compat mode). Math mode (--math): exact-shade (default:
  bit-reproducible ray generation and shading with the fast traversal; whole
  1080p frames within 1e-4 of the oracle per pixel), fast (CUDA float
  transcendentals) or exact (bit-identical to the oracle, frames in sequence).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference] [--math M]

Prints one JSON line (rank 0). `value` is device-resident throughput; `e2e`
is the same through the C ABI with every frame presented and read back to
pinned host memory. Under torchrun each rank renders its own replica (the
tracer does not shard), and value sums all ranks' samples over the slowest
rank's time.
"""
from __future__ import annotations

import argparse
import json
import os
import re
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

W, H, DEPTH = 1920, 1080, 8
FRAMES_PER_STEP = 64  # 1 spp per frame for 64 frames
MATH = {"fast": 0, "exact": 1, "exact-shade": 2}  # CT_MATH_*
METRIC = "Msamples/s path-traced"
UNIT = "Msamples/s"
WORKLOAD = ("wavefront path tracing 1920x1080, 64 frames of 1 spp per step, depth 8, 3.12M-tri fBm terrain + "
            "200 spheres, quad BVH")


def parse_args():
    global W, H, FRAMES_PER_STEP
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10, help="timed steps (64-frame accumulations)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--cpu-seconds", type=float, default=12.0, help="CPU-baseline sample budget")
    ap.add_argument("--math", choices=sorted(MATH), default="exact-shade",
                    help="math mode of the headline frames (CT_MATH_*)")
    ap.add_argument("--frames-per-step", type=int, default=FRAMES_PER_STEP,
                    help="frames accumulated per step (smaller for profiler captures)")
    ap.add_argument("--tree", choices=["fast", "reference"], default="fast",
                    help="tree traced by frames with the fast traversal (exact frames always trace the reference's)")
    ap.add_argument("--width", type=int, default=1920, help="smaller frames for profiler captures")
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--skip-extras", action="store_true",
                    help="only the timed frames: no e2e pass, roofline model, CPU baseline or sphere query")
    ap.add_argument("--case", choices=["soup", "sphere"], default=None,
                    help="profiling case instead of the benchmark: 'soup' builds the quad and the wide BVH of "
                         "a seeded soup and traces incoherent rays twice through each (prints timings); 'sphere' "
                         "runs the closest-hit query on the 81,920-triangle sphere (3 + 10 launches per tree, "
                         "the reference's tree first) and prints its JSON")
    ap.add_argument("--soup-tris", type=int, default=4_000_000)
    ap.add_argument("--soup-rays", type=int, default=2_000_000)
    ap.add_argument("--skip-serving", action="store_true",
                    help="leave out the 256-job batching and the Poisson serving workloads")
    ap.add_argument("--skip-precision", action="store_true",
                    help="leave out the 10M-triangle precision workload (wide vs quad BVH against FP64)")
    args = ap.parse_args()
    W, H, FRAMES_PER_STEP = args.width, args.height, args.frames_per_step
    args.math_mode = MATH[args.math]
    return args


# ------------------------------------------------------------------ common --
def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return world, rank, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device="cuda" if torch.cuda.is_available() else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


class Clocks:
    """nvidia-smi sampling of SM clock and throttle reasons during a region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.12)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(key: str = "dram_bytes_per_extension_ray", summary: str = "extend_terrain_1080p.md"):
    """A figure from a committed ncu summary in profiles/: by default bytes per
    extension ray of the extend kernel (DRAM, or with
    key="l2_bytes_per_extension_ray" L2; keys prefixed "reference_tree_" for
    frames on the reference's tree), or None."""
    path = os.path.join(ROOT, "profiles", summary)
    try:
        txt = open(path).read()
    except OSError:
        return None
    m = re.search(r"(?m)^" + key + r":\s*([0-9.eE+]+)", txt)
    return float(m.group(1)) if m else None


def build_scene():
    from cudatracer_gb300 import scenes

    ts, cam = scenes.terrain_scene()
    return ts, cam, scenes.scene_arrays(ts)


# ---------------------------------------------------------------- our arm --
def cpu_baseline_port(arrays, textures, materials_packed, quad, prims, cam, seconds: float) -> dict:
    """The oracle's restatement of the reference wavefront path (port), all host
    threads, on whole rows of the same frame until `seconds` of CPU time pass."""
    import numpy as np

    import oracle

    threads = os.cpu_count() or 1
    acc = np.zeros((W * H, 4), np.float32)
    rows, samples, frame, t0 = 0, 0, 0, time.perf_counter()
    row_step = 30
    r = 0
    while time.perf_counter() - t0 < seconds:
        oracle.render_frames(arrays, materials_packed, quad, prims, cam, W, H, [2 * frame], DEPTH, accum=acc,
                             exact_math=False, textures=textures, sky_tex=0,
                             pixels=(r * W, (r + row_step) * W), nthreads=threads)
        samples += row_step * W
        rows += row_step
        r += row_step
        if r + row_step > H:
            r, frame = 0, frame + 1
    dt = time.perf_counter() - t0
    return {"value": samples / dt / 1e6, "unit": UNIT, "cores": threads, "kind": "port",
            "sample": f"{samples} paths ({rows} rows, {frame} whole frames, depth {DEPTH}) in {dt:.1f} s; oracle "
                      f"restatement of the reference shade/extend/connect kernels on the host"}


def reference_traversal_baseline() -> dict | None:
    """The reference's own host BVH build + MBVH closest-hit traversal on the
    81,920-triangle sphere and 256x256 pinhole rays (oracle/_ref)."""
    import ctypes

    import numpy as np

    import oracle
    from cudatracer_gb300 import scenes

    if not oracle.ref_available():
        return None
    R = oracle.ref()
    s = scenes.sphere_scene(6)
    v, ix = np.ascontiguousarray(s.vertices), np.ascontiguousarray(s.indices)
    P = ctypes.c_void_p
    threads = os.cpu_count() or 1
    h = R.ctref_build(v.ctypes.data_as(P), v.shape[0], ix.ctypes.data_as(P), ix.shape[0], threads)
    o, d = scenes.pinhole_rays(256, 256, 60.0)
    reps = 20
    O = np.ascontiguousarray(np.tile(o, (reps, 1)))
    D = np.ascontiguousarray(np.tile(d, (reps, 1)))
    hit = np.zeros(O.shape[0], np.int32)
    t = np.zeros(O.shape[0], np.float32)
    t0 = time.perf_counter()
    R.ctref_trace_mbvh(h, O.ctypes.data_as(P), D.ctypes.data_as(P), O.shape[0], hit.ctypes.data_as(P),
                       t.ctypes.data_as(P), threads)
    dt = time.perf_counter() - t0
    out = {"kind": "reference", "cores": threads, "build_ms": R.ctref_build_ms(h), "collapse_ms": R.ctref_mbvh_ms(h),
           "traverse_mrays_per_s": O.shape[0] / dt / 1e6,
           "sample": f"81,920-triangle sphere, {O.shape[0]} primary rays (256x256 x {reps})"}
    R.ctref_free(h)
    return out


def sphere_closest_hit(ctx):
    """Mrays/s of ct_trace_closest on the 81,920-triangle sphere, 256x256 rays x 64."""
    import numpy as np
    import torch

    from cudatracer_gb300 import api, scenes

    s = scenes.sphere_scene(6)
    sc = ctx.scene(scenes.scene_arrays(s), [api.Material()])
    bvh = sc.build_bvh()
    o, d = scenes.pinhole_rays(256, 256, 60.0)
    O = np.zeros((o.shape[0], 4), np.float32)
    O[:, :3] = o
    D = np.zeros_like(O)
    D[:, :3] = d
    D[:, 3] = 1e34
    O = torch.from_numpy(np.tile(O, (64, 1))).cuda()
    D = torch.from_numpy(np.tile(D, (64, 1))).cuda()
    hit = torch.empty(O.shape[0], dtype=torch.int32, device="cuda")
    t = torch.empty(O.shape[0], device="cuda")

    def rate(tree):
        for _ in range(3):
            tree.trace_closest(O, D, hit, t)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(10):
            tree.trace_closest(O, D, hit, t)
        e1.record()
        torch.cuda.synchronize()
        return O.shape[0] / (e0.elapsed_time(e1) / 10) / 1e3

    mrays = rate(bvh)
    fb = sc.build_bvh_fast_device()
    mrays_fast = rate(fb)

    # the query's roofline: its working set (3.2 MB of nodes, 4.3 MB of triangles)
    # stays in L2 while the 4.2 M rays of 40 B stream from HBM, so L2 bounds it;
    # the algorithmic bytes (ray in and out + node visits x 128 + triangle tests
    # x 52, counted by the oracle along the reference's traversal order, which
    # the query kernel follows) are set against measured HBM, and the L2
    # throughput as a share of the chip's L2 peak comes from the committed ncu
    # capture of this kernel (profiles/query_sphere_81920.md)
    import oracle

    oracle.build_oracle()

    def model(tree):
        q, pr = tree.export()
        oracle.work_read(reset=True)
        oracle.trace_closest(q, pr, s.vertices, s.indices, o, d, nthreads=os.cpu_count() or 1)
        w = oracle.work_read(reset=True)
        vn, vt = w["ext_nodes"] / max(1, w["ext_rays"]), w["ext_tris"] / max(1, w["ext_rays"])
        return {"mean_node_visits": vn, "mean_tri_tests": vt, "bytes_per_ray": 40 + 128 * vn + 52 * vt}

    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    hbm = json.load(open(pk)).get("hbm_gbs", 6800.0) if os.path.exists(pk) else 6800.0
    roof = {}
    for name, tree, rate_ in (("reference_tree", bvh, mrays), ("fast_tree", fb, mrays_fast)):
        m = model(tree)
        ach = rate_ * 1e6 * m["bytes_per_ray"] / 1e9
        roof[name] = {**m, "achieved": ach, "unit": "GB/s", "hbm_frac": ach / hbm,
                      "l2_pct_of_peak_ncu": profiled_traffic(name + "_l2_pct_of_peak", "query_sphere_81920.md"),
                      "l2_gbs_ncu": profiled_traffic(name + "_l2_gbs", "query_sphere_81920.md")}
    fb.close()
    sc.close()
    bvh.close()
    return {"mrays_per_s": mrays, "fast_tree_mrays_per_s": mrays_fast, "rays": int(O.shape[0]),
            "workload": "81,920-tri sphere, 256x256 pinhole rays x64, ct_trace_closest (reference's tree; "
                        "fast_tree_mrays_per_s: ct_bvh_build_fast's)",
            "roofline": {"bound": "l2", "hbm_peak": hbm, "peak_source": "HBM: MEASURED_PEAKS.json; L2: ncu "
                         "lts__throughput (share of the chip's L2 peak) in profiles/query_sphere_81920.md", **roof}}


def precision_soup(ctx, ntri: int = 10_000_000, nray: int = 16_000_000, sample_every: int = 8) -> dict:
    """The precision workload: a 10M-triangle seeded soup (centroids U[0,1]^3,
    edges log-uniform 1e-4..1e-2) and 16M incoherent rays. Closest-hit Mrays/s
    of the plain quad BVH (reference Moller-Trumbore, epsilon 1e-12 since the
    reference's 1e-3 culls every soup triangle) on the reference's tree and on
    ct_bvh_build_fast's, and of the 8-wide quantised BVH
    (watertight FP32 + FP64 settlement); ids, lost hits and t error of both
    against the FP64 watertight oracle on every 8th ray."""
    import numpy as np
    import torch

    import oracle
    from cudatracer_gb300 import api, scenes

    s = scenes.soup_scene(ntri, seed=3)
    o, d = scenes.incoherent_rays(nray, seed=5)
    arr = {"vertices": s.vertices, "normals": np.tile(np.array([[0, 0, 1]], np.float32), (s.vertices.shape[0], 1)),
           "indices": s.indices}
    sc = ctx.scene(arr, [api.Material()])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    qb = sc.build_bvh_device()
    q_ms = (time.perf_counter() - t0) * 1e3
    t0 = time.perf_counter()
    wb = sc.build_bvh_wide()
    w_ms = (time.perf_counter() - t0) * 1e3
    org, dirs = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    hit = torch.empty(nray, dtype=torch.int32, device="cuda")
    t = torch.empty(nray, device="cuda")

    def timed(fn, k=5):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(k):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / k

    q_trace = timed(lambda: qb.trace_closest(org, dirs, hit, t, tri_eps=1e-12))
    hq, tq = hit.cpu().numpy().copy(), t.cpu().numpy().copy()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    fb = sc.build_bvh_fast_device()
    f_ms = (time.perf_counter() - t0) * 1e3
    f_trace = timed(lambda: fb.trace_closest(org, dirs, hit, t, tri_eps=1e-12))
    hf, tf = hit.cpu().numpy().copy(), t.cpu().numpy().copy()
    fb.close()
    wb.wide_stats(reset=True)
    w_trace = timed(lambda: wb.trace_closest(org, dirs, hit, t))
    st = wb.wide_stats(reset=True)
    hw, tw = hit.cpu().numpy().copy(), t.cpu().numpy().copy()
    ctx.check()
    quad, prims = qb.export()
    sel = slice(0, nray, sample_every)
    ho, to = oracle.trace_fp64(s.vertices, s.indices, quad, prims, o[sel], d[sel], nthreads=os.cpu_count() or 1)

    def against(h, tt):
        h, tt = h[sel], tt[sel]
        both = (h >= 0) & (h == ho)
        rel = np.abs(tt[both].astype(np.float64) - to[both]) / to[both]
        return {"id_mismatches": int((h != ho).sum()), "lost_hits": int(((ho >= 0) & (h < 0)).sum()),
                "false_hits": int(((ho < 0) & (h >= 0)).sum()), "mismatch_rate": float((h != ho).mean()),
                "max_rel_t_err": float(rel.max()) if rel.size else 0.0}

    out = {
        "workload": f"{ntri:,}-triangle soup, {nray:,} incoherent rays (origins U[0,1]^3, directions uniform)",
        "plain_quad_fp32": {"mrays_per_s": nray / q_trace / 1e3, "build_ms": q_ms, **against(hq, tq)},
        "plain_quad_fp32_fast_tree": {"mrays_per_s": nray / f_trace / 1e3, "build_ms": f_ms, **against(hf, tf)},
        "wide8_q8": {"mrays_per_s": nray / w_trace / 1e3, "build_ms": w_ms, "nodes": wb.info()["quad_node_count"],
                     "node_bytes": 80, "fp64_retest_frac": st["fp64_retests"] / max(1, st["rays"]),
                     "fp64_full_traversals": st["fp64_full"], **against(hw, tw)},
        "oracle_sample": f"FP64 watertight closest hit on every {sample_every}th ray ({ho.shape[0]:,} rays, "
                         f"{int((ho >= 0).sum()):,} hits)",
    }
    out["speedup_wide_vs_plain"] = out["wide8_q8"]["mrays_per_s"] / out["plain_quad_fp32"]["mrays_per_s"]
    out["speedup_wide_vs_plain_fast_tree"] = (out["wide8_q8"]["mrays_per_s"]
                                              / out["plain_quad_fp32_fast_tree"]["mrays_per_s"])
    qb.close()
    wb.close()
    sc.close()
    return out


def batching_jobs(ctx, n_jobs: int = 256, seed: int = 2024, math: int = MATH["exact-shade"]) -> dict:
    """The batching workload: n_jobs render jobs of the terrain-plus-spheres
    kind, triangle counts log-uniform 10k..2M, square resolutions log-uniform
    64..1024, spp log-uniform 1..64, depth uniform 4..12, all in one batch
    (autotuned launch shapes, graph-replayed iterations); against the same
    jobs rendered one after another through the plain per-job path."""
    import numpy as np
    import torch

    from cudatracer_gb300 import api, scenes

    rng = np.random.default_rng(seed)
    jobs, tris = [], 0
    t0 = time.perf_counter()
    for _ in range(n_jobs):
        tri = float(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
        sph = int(rng.integers(2, 40))
        grid = int(max(16, np.sqrt(max(1.0, tri - sph * 5120) / 2) + 1))
        side = int(np.exp(rng.uniform(np.log(64), np.log(1024))))
        spp = int(np.exp(rng.uniform(0.0, np.log(64))))
        depth = int(rng.integers(4, 13))
        ts, cam = scenes.terrain_scene(grid=grid, spheres=sph, seed=int(rng.integers(1, 100000)), extent=200.0,
                                       sky_size=(256, 128))
        sc = ctx.scene(scenes.scene_arrays(ts), [api.Material(**m) for m in ts.materials], ts.textures,
                       ts.skybox_texture)
        p = api.default_params(side, side)
        p.max_depth = depth
        jobs.append(dict(scene=sc, bvh=sc.build_bvh_fast_device(), params=p, spp=spp,
                         camera=api.Camera(side, side, cam["fov"], cam["position"], cam["forward"], cam["up"])))
        tris += ts.indices.shape[0]
    setup_s = time.perf_counter() - t0
    samples = sum(j["spp"] * j["params"].width * j["params"].height for j in jobs)
    b = api.Batch(ctx, jobs, exact_math=math)
    tuning, tune_ms = b.autotune()
    b.run()
    torch.cuda.synchronize()
    b.stats(reset=True)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    b.run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    st = b.stats(reset=True)
    ctx.check()
    b.close()
    # the same jobs, one after another, through ct_render_accumulate (each
    # job's device state is freed after the timed region)
    e0.record()
    done = []
    for j in jobs:
        W, H = j["params"].width, j["params"].height
        rj = api.RenderJob(ctx, W, H)
        pp = api.Params(W, H, camera=j["camera"], max_depth=j["params"].max_depth, exact_math=math)
        pp.reset(rj)
        for _ in range(j["spp"]):
            api.launch_kernels(rj, j["scene"], j["bvh"], pp)
        done.append(rj)
    e1.record()
    torch.cuda.synchronize()
    serial_ms = e0.elapsed_time(e1)
    for rj in done:
        rj.close()
    for j in jobs:
        j["bvh"].close()
        j["scene"].close()
    return {
        "workload": f"{n_jobs} jobs, {tris:,} triangles, {samples:,} samples (res 64..1024, spp 1..64, depth 4..12)",
        "msamples_per_s": samples / ms / 1e3, "mrays_per_s": (st["extension_rays"] + st["shadow_rays"]) / ms / 1e3,
        "ms": ms, "iterations": st["frames"], "tuning": tuning, "autotune_ms_per_iteration": tune_ms,
        "serial_plain_ms": serial_ms, "serial_plain_msamples_per_s": samples / serial_ms / 1e3,
        "speedup_vs_serial": serial_ms / ms, "setup_s": setup_s,
        "tree": "ct_bvh_build_fast_device (the traversal-speed tree built on the GPU; in setup_s)",
        "math": [k for k, v in MATH.items() if v == math][0],
    }


def serving_world(ctx, seed: int = 77) -> dict:
    """The serving workload's resident state: 16 terrain scenes of the batching
    workload's kind (10k..2M triangles) on fast trees, wide BVHs of 10k..10M-
    triangle soups, and a pool of 4M incoherent rays."""
    import numpy as np

    from cudatracer_gb300 import api, scenes

    rng = np.random.default_rng(seed)
    t0 = time.perf_counter()
    rscenes = []
    for k in range(16):
        tri = float(np.exp(rng.uniform(np.log(1e4), np.log(2e6))))
        sph = int(rng.integers(2, 40))
        grid = int(max(16, np.sqrt(max(1.0, tri - sph * 5120) / 2) + 1))
        ts, cam = scenes.terrain_scene(grid=grid, spheres=sph, seed=100 + k, extent=200.0, sky_size=(256, 128))
        sc = ctx.scene(scenes.scene_arrays(ts), [api.Material(**m) for m in ts.materials], ts.textures,
                       ts.skybox_texture)
        rscenes.append((sc, sc.build_bvh_fast_device(), cam))
    qbvhs = []
    for k, ntri in enumerate([10_000, 100_000, 1_000_000, 10_000_000]):
        s = scenes.soup_scene(ntri, seed=200 + k)
        arr = {"vertices": s.vertices, "normals": np.tile(np.array([[0, 0, 1]], np.float32), (s.vertices.shape[0], 1)),
               "indices": s.indices}
        sq = ctx.scene(arr, [api.Material()])
        qbvhs.append((sq, sq.build_bvh_wide()))
    ray_o, ray_d = scenes.incoherent_rays(4_000_000, seed=seed)
    setup_s = time.perf_counter() - t0
    return dict(rscenes=rscenes, qbvhs=qbvhs, ray_o=ray_o, ray_d=ray_d, setup_s=setup_s)


def serving_close(world: dict) -> None:
    for sc, bvh, _ in world["rscenes"]:
        bvh.close()
        sc.close()
    for sq, b in world["qbvhs"]:
        b.close()
        sq.close()


def serving_poisson(ctx, world: dict, rate: float = 100.0, duration_s: float = 5.0, seed: int = 77,
                    iter_pixels: int = 0, math: int = MATH["exact-shade"]) -> dict:
    """The serving workload: a Poisson request stream (rate req/s for
    duration_s) mixing render jobs (the batching workload's job distribution over 16
    resident terrain scenes) and ray queries (10k..4M incoherent rays against resident
    wide BVHs of 10k..10M-triangle soups), through ct_server with a 150 GB
    HBM budget. Latency = completion - submission. Serial plain execution: the
    same requests' service times measured one at a time through the plain
    per-request path, queued FIFO at the same arrival times."""
    import threading

    import numpy as np
    import torch

    from cudatracer_gb300 import api, scenes

    rng = np.random.default_rng(seed)
    rscenes, qbvhs, ray_o, ray_d = world["rscenes"], world["qbvhs"], world["ray_o"], world["ray_d"]
    setup_s = world["setup_s"]
    # the request list
    n_req = int(rate * duration_s)
    arrivals = np.cumsum(rng.exponential(1.0 / rate, n_req))
    reqs = []
    for _ in range(n_req):
        if rng.uniform() < 0.5:
            sc, bvh, cam = rscenes[int(rng.integers(0, len(rscenes)))]
            side = int(np.exp(rng.uniform(np.log(64), np.log(1024))))
            p = api.default_params(side, side)
            p.max_depth = int(rng.integers(4, 13))
            reqs.append(("render", dict(scene=sc, bvh=bvh, params=p, spp=int(np.exp(rng.uniform(0.0, np.log(64)))),
                                        camera=api.Camera(side, side, cam["fov"], cam["position"], cam["forward"],
                                                          cam["up"]))))
        else:
            n = int(np.exp(rng.uniform(np.log(1e4), np.log(4e6))))
            off = int(rng.integers(0, ray_o.shape[0] - n + 1))
            reqs.append(("query", dict(bvh=qbvhs[int(rng.integers(0, len(qbvhs)))][1], n=n, off=off)))

    def submit(srv, kind, r):
        if kind == "render":
            return srv.submit_render(r)
        return srv.submit_query(r["bvh"], ray_o[r["off"]:r["off"] + r["n"]], ray_d[r["off"]:r["off"] + r["n"]])

    srv = api.Server(ctx, hbm_budget=150 << 30, max_inflight_pixels=1 << 24, iter_pixels=iter_pixels,
                     exact_math=math)
    ids = [None] * n_req

    def client():
        start = time.perf_counter()
        for i, (kind, r) in enumerate(reqs):
            delay = arrivals[i] - (time.perf_counter() - start)
            if delay > 0:
                time.sleep(delay)
            ids[i] = submit(srv, kind, r)

    th = threading.Thread(target=client)
    w0 = time.perf_counter()
    th.start()
    th.join()
    infos = []
    for i in range(n_req):
        infos.append(srv.wait(ids[i])[0])
    wall = time.perf_counter() - w0
    st = srv.stats()
    srv.close()
    ctx.check()
    lat = np.array([x["done_s"] - x["submit_s"] for x in infos]) * 1e3
    kinds = np.array([k == "render" for k, _ in reqs])
    rays = st["extension_rays"] + st["shadow_rays"] + st["query_rays"]
    # serial plain execution: each request alone through the plain path
    svc = []
    for kind, r in reqs:
        torch.cuda.synchronize()
        a = time.perf_counter()
        if kind == "render":
            W, H = r["params"].width, r["params"].height
            rj = api.RenderJob(ctx, W, H)
            pp = api.Params(W, H, camera=r["camera"], max_depth=r["params"].max_depth, exact_math=math)
            pp.reset(rj)
            for _ in range(r["spp"]):
                api.launch_kernels(rj, r["scene"], r["bvh"], pp)
            rj.accum_tensor().cpu()
        else:
            o = torch.from_numpy(ray_o[r["off"]:r["off"] + r["n"]]).cuda()
            d = torch.from_numpy(ray_d[r["off"]:r["off"] + r["n"]]).cuda()
            h, t = r["bvh"].trace_closest(o, d)
            h.cpu(), t.cpu()
        torch.cuda.synchronize()
        svc.append(time.perf_counter() - a)
        if kind == "render":
            rj.close()  # outside the service time
    finish, slat = 0.0, []
    for a_t, s_t in zip(arrivals, svc):
        finish = max(finish, a_t) + s_t
        slat.append((finish - a_t) * 1e3)
    slat = np.array(slat)

    def pct(x):
        return {"p50": float(np.percentile(x, 50)), "p95": float(np.percentile(x, 95)),
                "p99": float(np.percentile(x, 99))}

    return {
        "workload": f"Poisson {rate:g} req/s for {duration_s:g} s: {n_req} requests, {int(kinds.sum())} renders "
                    f"(res 64..1024, spp 1..64, depth 4..12 over 16 resident scenes of 10k..2M triangles), "
                    f"{int((~kinds).sum())} closest-hit queries (10k..4M incoherent rays, wide BVHs of 10k..10M "
                    f"triangles); HBM budget 150 GB",
        "latency_ms": pct(lat), "latency_ms_render": pct(lat[kinds]), "latency_ms_query": pct(lat[~kinds]),
        "mrays_per_s": rays / wall / 1e6, "wall_s": wall, "completed": st["completed"], "failed": st["failed"],
        "peak_request_bytes": st["peak_bytes"], "iterations": st["iterations"],
        "serial_plain_latency_ms": pct(slat), "serial_plain_busy_s": float(sum(svc)),
        "iter_pixels": iter_pixels or (1 << 22), "setup_s": setup_s, "render_tree": "ct_bvh_build_fast_device",
        "rate_req_per_s": rate, "seed": seed,
    }


def soup_case(args) -> None:
    """Profiling case: quad and wide BVH of a seeded soup, incoherent closest-hit
    queries traced twice through each (the second launch of each is the one to
    capture)."""
    import numpy as np
    import torch

    from cudatracer_gb300 import _build, api, scenes

    _build.build()
    ctx = api.Context(0)
    s = scenes.soup_scene(args.soup_tris, seed=3)
    o, d = scenes.incoherent_rays(args.soup_rays, seed=5)
    arr = {"vertices": s.vertices, "normals": np.tile(np.array([[0, 0, 1]], np.float32), (s.vertices.shape[0], 1)),
           "indices": s.indices}
    sc = ctx.scene(arr, [api.Material()])
    wb, qb, fb = sc.build_bvh_wide(), sc.build_bvh_device(), sc.build_bvh_fast_device()
    org, dirs = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    out = {}
    for name, fn in (("wide", lambda: wb.trace_closest(org, dirs)),
                     ("quad", lambda: qb.trace_closest(org, dirs, tri_eps=1e-12)),
                     ("quad_fast_tree", lambda: fb.trace_closest(org, dirs, tri_eps=1e-12)),
                     ("wide_any", lambda: wb.trace_any(org, dirs)),
                     ("quad_fast_tree_any", lambda: fb.trace_any(org, dirs, tri_eps=1e-12))):
        for _ in range(2):  # the second launch of each is the one a profiler captures
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
        out[name + "_mrays_per_s"] = args.soup_rays / e0.elapsed_time(e1) / 1e3
    ctx.check()
    print(json.dumps({"case": "soup", "triangles": args.soup_tris, "rays": args.soup_rays, **out}), flush=True)


def run_ours(args, world, rank, local):
    import numpy as np
    import torch

    from cudatracer_gb300 import _build, api

    _build.build()
    torch.cuda.set_device(local)
    ctx = api.Context(local)
    t_setup = time.perf_counter()
    ts, cam, arrays = build_scene()
    sc = ctx.scene(arrays, [api.Material(**m) for m in ts.materials], ts.textures, ts.skybox_texture)
    ref_bvh = sc.build_bvh_device()  # the reference's tree: quad nodes bit-identical to the host SAH build
    info = ref_bvh.info()
    setup_s = time.perf_counter() - t_setup
    dev_build = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sc.build_bvh_device().close()
        dev_build.append((time.perf_counter() - t0) * 1e3)
    # frames with the fast traversal trace the tree built for traversal speed
    # (equal hits up to exact t ties); exact frames keep the reference's tree
    math = args.math_mode
    fast_bvh = None
    fast_build = []
    if not (math == MATH["exact"] or args.tree == "reference"):
        for _ in range(3):
            if fast_bvh is not None:
                fast_bvh.close()
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            fast_bvh = sc.build_bvh_fast_device()  # byte-equal to ct_bvh_build_fast's host build
            fast_build.append((time.perf_counter() - t0) * 1e3)
    bvh = ref_bvh if fast_bvh is None else fast_bvh
    hinfo = fast_host_ms = None
    if rank == 0:
        hb = sc.build_bvh(0)
        hinfo = hb.info()
        hb.close()
        if fast_bvh is not None:
            t0 = time.perf_counter()
            sc.build_bvh_fast().close()
            fast_host_ms = (time.perf_counter() - t0) * 1e3
    job = api.RenderJob(ctx, W, H)
    camera = api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"])
    stream = torch.cuda.Stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def accumulation(tree, mode, frames=None, present=None, host=None):
        """One step: Params::reset, then `frames` launchKernels calls (1-spp
        frames, seeds advancing by 2); with `present`, every frame is presented
        (draw_framebuffer) and read back to pinned host memory."""
        p = api.Params(W, H, camera=camera, max_depth=DEPTH, exact_math=mode)
        p.reset(job, stream)
        for _ in range(FRAMES_PER_STEP if frames is None else frames):
            api.launch_kernels(job, sc, tree, p, present_out=present, stream=stream)
            if host is not None:
                with torch.cuda.stream(stream):
                    host.copy_(present, non_blocking=True)

    def timed(tree, mode, steps, warmup, clocks=None, **kw):
        """CUDA-event time (and host wall time) of `steps` accumulations after
        `warmup` untimed ones, bracketed by barriers and synchronisation."""
        for _ in range(warmup):
            accumulation(tree, mode, **kw)
        stream.synchronize()
        job.stats(reset=True, stream=stream)
        barrier(world)
        torch.cuda.synchronize()
        if clocks is not None:
            clocks.start()
        w0 = time.perf_counter()
        e0.record(stream)
        for _ in range(steps):
            accumulation(tree, mode, **kw)
        e1.record(stream)
        stream.synchronize()
        wall = (time.perf_counter() - w0) * 1e3
        torch.cuda.synchronize()
        barrier(world)
        clk = clocks.stop() if clocks is not None else None
        ctx.check(stream)
        return e0.elapsed_time(e1), wall, clk, job.stats(reset=True, stream=stream)

    clocks = Clocks(local)
    ms, _, clk, st = timed(bvh, math, args.steps, args.warmup, clocks=clocks)
    ms_max = max_over_ranks(ms, world)
    frames = FRAMES_PER_STEP * args.steps
    # stage times: a separate pass with per-launch events, frames one after another
    # (the timed frames overlap on ten streams, where an interval is not one kernel)
    job.profile(True)
    job.profile_read(reset=True)
    prof_frames = 16
    accumulation(bvh, math, frames=prof_frames)
    stream.synchronize()
    prof = job.profile_read(reset=True)
    job.profile(False)
    prof_st = job.stats(reset=True, stream=stream)

    def rate(ms_, steps_):
        return world * W * H * FRAMES_PER_STEP * steps_ / (max_over_ranks(ms_, world) / 1e3) / 1e6

    # every math mode, and the headline mode on the reference's tree, timed the same way
    modes = None
    ref_tree = None
    if not args.skip_extras:
        modes = {}
        for name, mode in MATH.items():
            if mode == math:
                modes[name] = {"value": world * W * H * frames / (ms_max / 1e3) / 1e6, "steps": args.steps}
                continue
            tree = ref_bvh if (mode == MATH["exact"] or fast_bvh is None) else fast_bvh
            m_ms = timed(tree, mode, 2, 1)[0]
            modes[name] = {"value": rate(m_ms, 2), "steps": 2}
        for name, mode in MATH.items():
            modes[name].update({
                "unit": UNIT, "tree": "reference" if (mode == MATH["exact"] or fast_bvh is None) else "ct_bvh_build_fast_device",
                "parity": {"fast": "statistical: a measured fraction of pixels leaves 1e-4 of the oracle "
                                   "(tests/test_gpu_render.py)",
                           "exact": "accumulation bit-identical to the oracle, whole 1080p frames",
                           "exact-shade": "whole 1080p frames within 1e-4 of the oracle per pixel (0 out of band)"}[name]})
        if fast_bvh is not None:
            r_ms = timed(ref_bvh, math, 2, 1)[0]
            job.profile(True)
            job.profile_read(reset=True)
            accumulation(ref_bvh, math, frames=prof_frames)
            stream.synchronize()
            prof_ref = job.profile_read(reset=True)
            job.profile(False)
            job.stats(reset=True, stream=stream)
            ref_tree = {"value": rate(r_ms, 2), "unit": UNIT, "steps": 2, "math": args.math,
                        "stage_ms": {k: v["ms"] for k, v in prof_ref.items()}, "stage_frames": prof_frames,
                        "tree": "the reference's SAH + MergeNodes quad tree (device build)",
                        "quad_nodes": info["quad_node_count"]}
    samples = W * H * frames
    value = world * samples / (ms_max / 1e3) / 1e6
    mrays = world * (st["extension_rays"] + st["shadow_rays"]) / (ms_max / 1e3) / 1e6

    if args.skip_extras:
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                              "ms_per_step": ms_max / args.steps, "mrays_per_s": mrays, "math": args.math,
                              "frames_per_step": FRAMES_PER_STEP,
                              "stage_ms": {k: v["ms"] for k, v in prof.items()}, "stage_frames": prof_frames,
                              "config": {"width": W, "height": H, "max_depth": DEPTH}}), flush=True)
        return

    # ---- e2e: C ABI, every frame presented and copied to pinned host memory
    out_dev = torch.empty((W * H, 4), device="cuda")
    out_host = torch.empty((W * H, 4), pin_memory=True)
    e_ms, e_wall, _, _ = timed(bvh, math, args.steps, args.warmup, present=out_dev, host=out_host)
    e2e_ms = max_over_ranks(max(e_ms, e_wall), world)
    e2e_value = world * samples / (e2e_ms / 1e3) / 1e6
    h2d_bytes = FRAMES_PER_STEP * (40 + 48)  # ct_camera + ct_render_params passed from host memory per frame
    d2h_bytes = FRAMES_PER_STEP * W * H * 16  # every presented frame

    # ---- roofline of the dominant kernel (extend: closest-hit traversal)
    peak, peak_kind = measured_peaks()
    ext = prof["extend"]
    roofline = None
    roofline_sample = None
    cpu_base = None
    work = None
    if rank == 0:
        import oracle

        oracle.build_oracle()
        quad, prims = ref_bvh.export()
        omats = oracle.pack_materials(ts.materials)
        # traversal work on sampled rows (16 rows of the frame), counted by the oracle
        def oracle_work(quad, prims, full_sort):
            oracle.set_full_sort(full_sort)
            oracle.work_read(reset=True)
            acc = np.zeros((W * H, 4), np.float32)
            paths = 0
            for r0 in range(0, H, 135):
                oracle.render_frames(arrays, omats, quad, prims, cam, W, H, [0], DEPTH, accum=acc, exact_math=False,
                                     textures=ts.textures, sky_tex=0, pixels=(r0 * W, (r0 + 2) * W),
                                     nthreads=os.cpu_count() or 1)
                paths += 2 * W
            w = oracle.work_read(reset=True)
            oracle.set_full_sort(False)
            return w, paths

        # the algorithmic bytes follow the reference's traverseMBVH order on the
        # reference's tree; the counts of the traced tree in the order fast-math
        # frames visit children (full distance sort) are reported beside
        work, paths = oracle_work(quad, prims, False)
        work_fast = oracle_work(*bvh.export(), True)[0] if math != MATH["exact"] else work
        v_node = work["ext_nodes"] / max(1, work["ext_rays"])
        v_tri = work["ext_tris"] / max(1, work["ext_rays"])
        b_ray = 32 + v_node * 128 + v_tri * 52
        ext_rays = prof_st["extension_rays"]  # rays of the profiling pass, whose launches ext["ms"] times
        achieved = ext_rays * b_ray / (ext["ms"] / 1e3) / 1e9 if ext["ms"] > 0 else None
        pre = "" if fast_bvh is not None else "reference_tree_"
        tpr = profiled_traffic(pre + "dram_bytes_per_extension_ray")
        l2pr = profiled_traffic(pre + "l2_bytes_per_extension_ray")
        roofline = {
            "kernel": "k_extend (closest-hit quad-BVH traversal)", "bound": "hbm",
            "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak if achieved else None, "peak_source": peak_kind,
            "traffic": (tpr * ext_rays / max(1, ext["launches"])) if tpr else None,
            "l2_traffic": (l2pr * ext_rays / max(1, ext["launches"])) if l2pr else None,
            "algorithmic_bytes_per_ray": b_ray, "mean_node_visits": v_node, "mean_tri_tests": v_tri,
            "traced_tree": {
                "tree": "reference" if fast_bvh is None else "ct_bvh_build_fast",
                "mean_node_visits": work_fast["ext_nodes"] / max(1, work_fast["ext_rays"]),
                "mean_tri_tests": work_fast["ext_tris"] / max(1, work_fast["ext_rays"]),
                "bytes_per_ray": 32 + 128 * work_fast["ext_nodes"] / max(1, work_fast["ext_rays"])
                + 52 * work_fast["ext_tris"] / max(1, work_fast["ext_rays"]),
                "order": "traverseMBVH" if math == MATH["exact"] else "full distance sort"},
            "rays_per_launch": ext_rays / max(1, ext["launches"]),
            "avg_launch_ms": ext["ms"] / max(1, ext["launches"]),
        }
        # the whole path per sample: extension and shadow traversals, the shading gathers
        # of every extension ray (index 12 + positions 36 + normals 36 + uvs 24 + centre
        # normal 12 + material index 4 + material 52 bytes) and the accumulation update
        vs_node = work["shadow_nodes"] / max(1, work["shadow_rays"])
        vs_tri = work["shadow_tris"] / max(1, work["shadow_rays"])
        b_shadow = 28 + vs_node * 128 + vs_tri * 52
        b_sample = (work["ext_rays"] * (b_ray + 176) + work["shadow_rays"] * b_shadow) / max(1, paths) + 32
        ach_sample = b_sample * (value / world) * 1e6 / 1e9  # per GPU
        roofline_sample = {
            "model": "bytes per path-traced sample: extension rays x (B_ray + 176 shading) + shadow rays x "
                     "B_shadow + 32 accumulation, counts from the oracle on 16 rows of the frame",
            "bytes_per_sample": b_sample, "extension_rays_per_sample": work["ext_rays"] / max(1, paths),
            "shadow_rays_per_sample": work["shadow_rays"] / max(1, paths), "shadow_bytes_per_ray": b_shadow,
            "achieved": ach_sample, "peak": peak, "unit": "GB/s", "frac": ach_sample / peak,
        }
        if world == 1 and args.cpu_seconds > 0:
            cpu_base = cpu_baseline_port(arrays, ts.textures, omats, quad, prims, cam, args.cpu_seconds)
            ref_tr = reference_traversal_baseline()
            if ref_tr:
                cpu_base["reference_host_traversal"] = ref_tr
    # ---- the same workload with every material shaded (CT_SHADE_FULL), for context
    from cudatracer_gb300 import _lib

    full_frames = FRAMES_PER_STEP

    def full_accumulation():
        pf = api.Params(W, H, camera=camera, max_depth=DEPTH, exact_math=math)
        pf.reset(job, stream)
        for _ in range(full_frames):
            c = pf.to_ct()
            c.shading_mode = _lib.CT_SHADE_FULL
            job.accumulate(sc, bvh, camera, c, stream)
            pf.samples += 2

    full_accumulation()
    stream.synchronize()
    e0.record(stream)
    full_accumulation()
    e1.record(stream)
    stream.synchronize()
    full_ms = e0.elapsed_time(e1) / full_frames
    full = {"msamples_per_s": W * H / full_ms / 1e3, "ms_per_frame": full_ms, "frames": full_frames,
            "math": args.math, "shading": "full materials (Lambert, mirror, dielectric IOR 1.5, GGX) with MIS"}
    c1 = sphere_closest_hit(ctx) if rank == 0 else None
    c3 = precision_soup(ctx) if (rank == 0 and not args.skip_precision) else None
    c4 = batching_jobs(ctx, math=math) if (rank == 0 and not args.skip_serving) else None
    # the light end of the request-rate range, one where serial execution saturates, and the
    # top of the range (2,000 req/s), where the server saturates too
    c5 = None
    if rank == 0 and not args.skip_serving:
        sw = serving_world(ctx)
        # three 10-s runs at the light end (100 req/s, other arrival seeds), and the two heavy rates
        c5 = [serving_poisson(ctx, sw, duration_s=10.0, seed=sd, math=math) for sd in (77, 78, 79)]
        c5 += [serving_poisson(ctx, sw, rate=400.0, duration_s=2.0, math=math),
               serving_poisson(ctx, sw, rate=2000.0, duration_s=1.0, math=math)]
        serving_close(sw)
    # our kernels in the timed region: per frame raygen + depth x (extend, shade,
    # connect) + the fold of a fast-math frame slot (the launch counts of the
    # stage-timing pass, which has no fold, confirm the per-frame stage count)
    per_frame = sum(v["launches"] for v in prof.values()) / prof_frames + (0 if math == MATH["exact"] else 1)
    launches = int(round(per_frame * frames))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": WORKLOAD, "width": W, "height": H, "max_depth": DEPTH, "triangles": int(ts.ntri),
                   "frames_per_step": FRAMES_PER_STEP, "spp_per_frame": 1, "shading": "compat (reference shade)",
                   "math": args.math,
                   "l2": "inputs larger than L2: 85-94 MB nodes + 150 MB triangles + 150 MB scene arrays + 300 MB queues",
                   "parallelism": f"replicas x{world}"},
        "mrays_per_s": mrays, "rays_per_step": (st["extension_rays"] + st["shadow_rays"]) / args.steps,
        "stage_ms": {k: v["ms"] for k, v in prof.items()}, "stage_frames": prof_frames,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d_bytes, "d2h_bytes_per_step": d2h_bytes},
        "gpu_launches": launches,
        "reference_tree": ref_tree, "math_modes": modes,
        "roofline": roofline, "roofline_sample": roofline_sample, "cpu_baseline": cpu_base, "closest_hit": c1, "precision": c3, "batching": c4, "serving": c5, "full_materials": full, "clocks": clk,
        "setup": {"scene_and_bvh_s": setup_s, "quad_nodes": bvh.info()["quad_node_count"],
                  "bvh_device_build_ms": min(dev_build),
                  "bvh_fast_device_build_ms": min(fast_build) if fast_bvh is not None else None,
                  "bvh_fast_host_build_ms": fast_host_ms,
                  "bvh_host_build_ms": (hinfo["build_ms"] + hinfo["collapse_ms"] + hinfo["upload_ms"]) if hinfo else None,
                  "bvh": ("reference SAH tree, device build (quad nodes bit-identical to the host build)"
                          if fast_bvh is None else "ct_bvh_build_fast_device (the traversal-speed tree built on the "
                          "GPU, byte-equal to ct_bvh_build_fast's host build); the reference's tree is timed beside "
                          "it in reference_tree")},
    }
    if rank == 0:
        print(json.dumps(line), flush=True)


# ---------------------------------------------------------- reference arm --
def run_reference(args, world, rank):
    """The reference's path on the host cores: its own host BVH build
    (oracle/_ref) when available, and the oracle's restatement of its
    wavefront kernels for shading (the reference has no CPU shading path)."""
    if rank != 0:
        return
    import ctypes

    import numpy as np

    import oracle

    oracle.build_oracle()
    ts, cam, arrays = build_scene()
    threads = os.cpu_count() or 1
    kind = "port"
    if oracle.ref_available():
        R = oracle.ref()
        P = ctypes.c_void_p
        v, ix = np.ascontiguousarray(ts.vertices), np.ascontiguousarray(ts.indices)
        h = R.ctref_build(v.ctypes.data_as(P), v.shape[0], ix.ctypes.data_as(P), ix.shape[0], threads)
        quad = np.zeros((R.ctref_mbvh_count(h), 32), np.int32)
        prims = np.zeros(ix.shape[0], np.uint32)
        R.ctref_export(h, None, prims.ctypes.data_as(P), quad.ctypes.data_as(P))
        build_ms = R.ctref_build_ms(h) + R.ctref_mbvh_ms(h)
        R.ctref_free(h)
        bvh_src = "reference host BVHTree+MBVHTree build"
    else:
        t0 = time.perf_counter()
        b = oracle.bvh_build(ts.vertices, ts.indices, threads)
        quad, prims = b["quad"], b["prims"]
        build_ms = (time.perf_counter() - t0) * 1e3
        bvh_src = "oracle restatement of the reference SAH build"
    omats = oracle.pack_materials(ts.materials)
    acc = np.zeros((W * H, 4), np.float32)
    # each step: 16 rows spread evenly over the frame (a different set each step),
    # every frame of the 64-frame accumulation (seeds 0, 2, ..., 126), so a step
    # is about 2 M paths with the workload's mix of sky, terrain and spheres
    rows_per_step = 16
    stride = H // rows_per_step

    seeds = [2 * f for f in range(FRAMES_PER_STEP)]

    def step(s):
        rows = np.arange(rows_per_step) * stride + (s * 7) % stride
        pix = (rows[:, None] * W + np.arange(W)[None, :]).reshape(-1)
        acc[pix] = 0.0  # Params::reset of the sampled rows
        oracle.render_pixels(arrays, omats, quad, prims, cam, W, H, seeds, DEPTH, pix, accum=acc, exact_math=False,
                             textures=ts.textures, sky_tex=0, nthreads=threads)

    for s in range(args.warmup):
        step(s)
    t0 = time.perf_counter()
    for s in range(args.steps):
        step(args.warmup + s)
    dt = time.perf_counter() - t0
    samples = args.steps * rows_per_step * W * FRAMES_PER_STEP
    value = samples / dt / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dt * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": WORKLOAD, "width": W, "height": H, "max_depth": DEPTH, "triangles": int(ts.ntri),
                   "frames_per_step": FRAMES_PER_STEP,
                   "step_sample": f"{rows_per_step} rows (every {stride}th) x {W} px x {FRAMES_PER_STEP} frames per step"},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads, "kind": kind,
                         "sample": f"{rows_per_step * W * FRAMES_PER_STEP} paths per step ({rows_per_step} rows "
                                   f"spread over the frame x {FRAMES_PER_STEP} frames); BVH from the {bvh_src} "
                                   f"({build_ms:.0f} ms)"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    args = parse_args()
    if args.case == "soup":
        soup_case(args)
        return
    if args.case == "sphere":
        from cudatracer_gb300 import _build, api

        _build.build()
        print(json.dumps(sphere_closest_hit(api.Context(0))), flush=True)
        return
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
