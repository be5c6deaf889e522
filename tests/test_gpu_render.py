"""GPU wavefront frames against the CPU oracle's restatement of the reference
kernels (generatePrimaryRays/extend/shade/connect, src/CUDA/Kernel.cu).

Tolerance: 1e-4 relative per pixel channel. With exact_math the GPU and the
oracle evaluate every operation identically and the accumulation buffers are
expected to be bit-identical."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-4


@pytest.fixture(scope="module")
def small(gpu_ctx, orc):
    from cudatracer_gb300 import api, scenes

    ts, cam = scenes.terrain_scene(grid=128, spheres=12, sky_size=(256, 128))
    arr = scenes.scene_arrays(ts)
    mats = [api.Material(**m) for m in ts.materials]
    sc = gpu_ctx.scene(arr, mats, ts.textures, ts.skybox_texture)
    bvh = sc.build_bvh()
    ob = orc.bvh_build(ts.vertices, ts.indices)
    return dict(ts=ts, cam=cam, arr=arr, sc=sc, bvh=bvh, ob=ob, omats=orc.pack_materials(ts.materials))


def _render(gpu_ctx, S, W, H, frames, depth, exact, **kw):
    from cudatracer_gb300 import api

    job = api.RenderJob(gpu_ctx, W, H)
    cam = S["cam"]
    p = api.Params(W, H, camera=api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"]),
                   max_depth=depth, exact_math=exact, **kw)
    p.reset(job)
    for _ in range(frames):
        api.launch_kernels(job, S["sc"], S["bvh"], p)
    gpu_ctx.check()
    acc = job.accum_tensor().cpu().numpy().copy()
    return job, p, acc


def _oracle(orc, S, W, H, frames, depth, exact, **kw):
    return orc.render_frames(S["arr"], S["omats"], S["ob"]["quad"], S["ob"]["prims"], S["cam"], W, H,
                             [2 * f for f in range(frames)], depth, exact_math=exact, textures=S["ts"].textures,
                             sky_tex=0, **kw)


def _bad(a, b):
    rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-6)
    return (rel > RTOL).any(axis=1)


def test_exact_frames_match_oracle(gpu_ctx, orc, small):
    W, H = 96, 64
    _, p, acc = _render(gpu_ctx, small, W, H, 3, 5, True)
    assert p.samples == 6  # launchKernels advances the counter by 2 per frame
    oacc = _oracle(orc, small, W, H, 3, 5, True)
    assert _bad(acc, oacc).sum() == 0
    bit = (acc.view(np.int32) == oacc.view(np.int32)).all(axis=1).mean()
    assert bit >= 0.999
    assert acc[:, 3].max() > 0


@pytest.mark.parametrize("flags", [dict(shadow=False), dict(indirect=False), dict(sky=False)])
def test_exact_frames_flags(gpu_ctx, orc, small, flags):
    W, H = 64, 48
    _, _, acc = _render(gpu_ctx, small, W, H, 1, 8, True, **flags)
    oacc = _oracle(orc, small, W, H, 1, 8, True, **flags)
    assert _bad(acc, oacc).sum() == 0


@pytest.mark.parametrize("exact", [True, False])
def test_ray_sort_keys_do_not_change_frames(gpu_ctx, orc, small, exact):
    """Sorting the bounce queues by direction class changes which rays share a
    warp, never a result: every key gives the same accumulation bit for bit,
    and exact frames still equal the oracle."""
    from cudatracer_gb300 import _lib, api

    W, H = 96, 64
    outs = [_render(gpu_ctx, small, W, H, 3, 5, exact, ray_sort=k)[2]
            for k in (_lib.CT_SORT_NONE, _lib.CT_SORT_OCTANT, _lib.CT_SORT_FACE_CELLS)]
    for o in outs[1:]:
        assert np.array_equal(outs[0].view(np.int32), o.view(np.int32))
    if exact:
        assert _bad(outs[2], _oracle(orc, small, W, H, 3, 5, True)).sum() == 0
    job = api.RenderJob(gpu_ctx, W, H)
    p = api.Params(W, H, camera=api.Camera(W, H, 60.0, (0, 5, 20), (0, 0, -1), (0, 1, 0)), ray_sort=3)
    with pytest.raises(_lib.CTError):
        api.launch_kernels(job, small["sc"], small["bvh"], p)


def _fold_oracle(orc, S, W, H, frames, depth, **kw):
    """The oracle's exact frames, each accumulated into a zeroed buffer and then
    added to the running sum in float32 (round to nearest): the grouping of the
    overlapped GPU frames, whose private buffers k_fold adds into the job's
    buffer in frame order."""
    acc = np.zeros((W * H, 4), np.float32)
    for f in range(frames):
        acc = acc + _oracle_frames(orc, S, W, H, [2 * f], depth, **kw)
    return acc


def _oracle_frames(orc, S, W, H, seeds, depth, **kw):
    return orc.render_frames(S["arr"], S["omats"], S["ob"]["quad"], S["ob"]["prims"], S["cam"], W, H, seeds, depth,
                             exact_math=True, textures=S["ts"].textures, sky_tex=0, **kw)


@pytest.mark.parametrize("tree", ["reference", "fast"])
def test_exact_shade_frames_match_oracle(gpu_ctx, orc, small, tree):
    """CT_MATH_EXACT_SHADE: the bit-reproducible ray generation and shading with
    the fast traversal (fused slab planes, children in full distance order), in
    overlapped frame slots. That traversal returns the reference traversal's
    closest hit (t bit-equal, only an exact tie's winner can differ) and its
    occlusion, on the reference's tree and on the traversal-speed tree, so no
    pixel leaves the 1e-4 band of the oracle's exact frames (the oracle traces
    the reference's tree) and the accumulation equals those frames summed in
    the GPU's grouping bit for bit (ties aside)."""
    from cudatracer_gb300 import _lib

    W, H = 96, 64
    S = dict(small)
    if tree == "fast":
        S["bvh"] = small["sc"].build_bvh_fast()
    _, p, acc = _render(gpu_ctx, S, W, H, 4, 5, _lib.CT_MATH_EXACT_SHADE)
    assert p.samples == 8
    oacc = _fold_oracle(orc, small, W, H, 4, 5)
    assert _bad(acc, oacc).sum() == 0
    bit = (acc.view(np.int32) == oacc.view(np.int32)).all(axis=1).mean()
    assert bit >= 0.999
    assert acc[:, 3].max() > 0


def test_fast_math_frames_close_to_oracle(gpu_ctx, orc, small):
    """CT_MATH_FAST: CUDA's float sin/cos/atan2/acos and contracted multiply-adds
    differ from the exact build by an ulp or so; a path that grazes an edge then
    diverges, so a few pixels leave the 1e-4 band (the fraction at full size is
    measured in test_full_size_frames_against_oracle). The image total stays
    close."""
    W, H = 96, 64
    _, _, acc = _render(gpu_ctx, small, W, H, 4, 5, False)
    oacc = _oracle(orc, small, W, H, 4, 5, True)
    assert _bad(acc, oacc).mean() < 0.10
    assert abs(acc[:, :3].sum() - oacc[:, :3].sum()) / oacc[:, :3].sum() < 0.02


def test_present_matches_draw_framebuffer(gpu_ctx, orc, small):
    import torch

    W, H = 64, 48
    job, p, acc = _render(gpu_ctx, small, W, H, 2, 5, True)
    out = torch.zeros((W * H, 4), device="cuda")
    job.present(p.samples, out)
    rgba = np.zeros((W * H, 4), np.float32)
    L = orc.lib()
    L.or_present(acc.ctypes.data_as(orc.P), W * H, float(p.samples), rgba.ctypes.data_as(orc.P))
    g = out.cpu().numpy()
    assert np.allclose(g, rgba, rtol=2e-6, atol=1e-7)
    assert (g[:, 3] == 1.0).all()


def test_overlapped_fast_frames_are_deterministic(gpu_ctx, small):
    """Fast-math frames run in two private slots on their own streams and are
    folded in frame order. A job created while the legacy stream is still busy
    (its buffers' zero-fill queued behind other work) must produce the same
    accumulation, bit for bit, as a job created on an idle device."""
    import torch

    from cudatracer_gb300 import api

    W, H = 96, 64
    cam = small["cam"]
    camera = api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"])

    def run(job, frames=5):
        p = api.Params(W, H, camera=camera, max_depth=6, exact_math=False)
        p.reset(job)
        for _ in range(frames):
            api.launch_kernels(job, small["sc"], small["bvh"], p)
        torch.cuda.synchronize()
        return job.accum_tensor().cpu().numpy().copy()

    a = run(api.RenderJob(gpu_ctx, W, H))
    busy = api.RenderJob(gpu_ctx, 1024, 1024)
    pb = api.Params(1024, 1024, camera=api.Camera(1024, 1024, cam["fov"], cam["position"], cam["forward"], cam["up"]),
                    max_depth=8, exact_math=True)
    busy.accumulate(small["sc"], small["bvh"], pb.camera, pb.to_ct())  # keeps the legacy stream busy
    b = run(api.RenderJob(gpu_ctx, W, H))
    gpu_ctx.check()
    assert np.array_equal(a.view(np.int32), b.view(np.int32))
    assert a[:, 3].sum() > 0


def test_overlapped_exact_frames_equal_frames_in_sequence(gpu_ctx, small):
    """CT_MATH_EXACT frames overlap in slots and log their per-pixel
    contributions, which are replayed into the job's buffer in frame order; the
    accumulation equals the same frames run one after another (profiling runs
    them so) byte for byte, also when a deeper frame makes the logs grow."""
    import torch

    from cudatracer_gb300 import api

    W, H = 96, 64
    cam = small["cam"]
    camera = api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"])
    outs = []
    for in_sequence in (False, True):
        job = api.RenderJob(gpu_ctx, W, H)
        if in_sequence:
            job.profile(True)
        p = api.Params(W, H, camera=camera, max_depth=4, exact_math=True)
        p.reset(job)
        for _ in range(6):
            api.launch_kernels(job, small["sc"], small["bvh"], p)
        p.max_depth = 9
        for _ in range(5):
            api.launch_kernels(job, small["sc"], small["bvh"], p)
        torch.cuda.synchronize()
        gpu_ctx.check()
        outs.append(job.accum_tensor().cpu().numpy().copy())
        job.close()
    assert np.array_equal(outs[0].view(np.int32), outs[1].view(np.int32))
    assert outs[0][:, 3].sum() > 0


def test_stats_and_validation(gpu_ctx, small):
    from cudatracer_gb300 import _lib, api

    W, H = 32, 16
    job, p, _ = _render(gpu_ctx, small, W, H, 2, 5, False)
    st = job.stats(reset=True)
    assert st["samples"] == 2 * W * H and st["frames"] == 2
    assert W * H * 2 <= st["extension_rays"] <= W * H * 2 * 5
    bad = p.to_ct()
    bad.width = W + 1
    with pytest.raises(_lib.CTError) as e:
        job.accumulate(small["sc"], small["bvh"], p.camera, bad)
    assert e.value.status == 1
    bad = p.to_ct()
    bad.max_depth = 0
    with pytest.raises(_lib.CTError):
        job.accumulate(small["sc"], small["bvh"], p.camera, bad)
    with pytest.raises(_lib.CTError):
        api.RenderJob(gpu_ctx, 0, 10)


def test_scene_validation(gpu_ctx):
    from cudatracer_gb300 import _lib, api

    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    n = np.tile(np.array([[0, 0, 1]], np.float32), (3, 1))
    with pytest.raises(_lib.CTError):
        gpu_ctx.scene({"vertices": v, "normals": n, "indices": np.array([[0, 1, 5]], np.uint32)}, [api.Material()])
    with pytest.raises(_lib.CTError):
        gpu_ctx.scene({"vertices": v, "normals": n, "indices": np.array([[0, 1, 2]], np.uint32),
                       "material_idxs": np.array([3], np.uint32)}, [api.Material()])
    bad = v.copy()
    bad[1, 0] = np.inf
    with pytest.raises(_lib.CTError):
        gpu_ctx.scene({"vertices": bad, "normals": n, "indices": np.array([[0, 1, 2]], np.uint32)}, [api.Material()])
    with pytest.raises(_lib.CTError):
        gpu_ctx.scene({"vertices": v, "normals": n, "indices": np.array([[0, 1, 2]], np.uint32)},
                      [api.Material(diffuse_tex=0)])


def test_memory_budget_refuses_allocation(gpu_ctx):
    from cudatracer_gb300 import _lib, api

    used = gpu_ctx.device_bytes
    gpu_ctx.set_memory_budget(used + (1 << 20))
    try:
        with pytest.raises(_lib.CTError) as e:
            api.RenderJob(gpu_ctx, 1024, 1024)
        assert e.value.status == 2
        assert gpu_ctx.device_bytes == used  # nothing leaked by the failed creation
    finally:
        gpu_ctx.set_memory_budget(0)


# CT_MATH_FAST on the 1920x1080, depth-8 terrain frame (seed frame 0) against
# the oracle's whole frame: 52,687 of 2,073,600 pixels (2.54 %) measured
# outside 1e-4 relative on a GB300; the bound leaves headroom.
FULL_FAST_OUT_OF_BAND_MAX = 0.03


@pytest.fixture(scope="module")
def full(gpu_ctx, orc):
    """The benchmark workload: 3,117,066-triangle terrain scene, its reference
    tree (host build: the same leaves, primitive order included, as the
    oracle's), its traversal-speed tree, and the oracle's build of the
    reference tree."""
    import os

    from cudatracer_gb300 import api, scenes

    ts, cam = scenes.terrain_scene()
    arr = scenes.scene_arrays(ts)
    sc = gpu_ctx.scene(arr, [api.Material(**m) for m in ts.materials], ts.textures, ts.skybox_texture)
    ob = orc.bvh_build(ts.vertices, ts.indices, nthreads=os.cpu_count() or 8)
    return dict(ts=ts, cam=cam, arr=arr, sc=sc, bvh=sc.build_bvh(), fast=sc.build_bvh_fast(), ob=ob,
                omats=orc.pack_materials(ts.materials), threads=os.cpu_count() or 8)


def test_full_size_frames_against_oracle(gpu_ctx, orc, full):
    """The 1920x1080, depth-8 workload, whole frames against the oracle's whole
    frame (reference tree, reference traversal order, exact math):
      * CT_MATH_EXACT on the reference's tree: every channel bit-identical, and
        a second run gives the same bits (compaction order never leaks in);
      * CT_MATH_EXACT_SHADE on the traversal-speed tree (the benchmark's
        headline mode): no pixel outside 1e-4 relative;
      * CT_MATH_FAST on the traversal-speed tree: at most
        FULL_FAST_OUT_OF_BAND_MAX of the pixels outside 1e-4, image total
        within 0.5 %, finite and non-negative.
    Every exact-shade pixel that differs from the oracle's frame must be an
    exact tie: the oracle's own path for that pixel, traced through the
    reference's tree and through the traversal-speed tree, parts at a bounce
    where both trees report the same t bit for bit and another primitive (a
    ray through the edge two triangles share: the first one tested wins, and
    the trees present them in another order). Against the oracle tracing the
    traversal-speed tree itself, no pixel may leave the band. Two frames of the
    exact-shade mode are also compared with the oracle's two frames summed in
    the GPU's grouping."""
    from cudatracer_gb300 import _lib

    W, H = 1920, 1080
    S = dict(full)
    oacc = _oracle_frames(orc, S, W, H, [0], 8, nthreads=S["threads"])
    fq, fp = full["fast"].export()
    S_fast = dict(S, ob={"quad": fq, "prims": fp})
    orc.set_full_sort(True)  # the child order of the fast traversal
    try:
        ofast = _oracle_frames(orc, S_fast, W, H, [0], 8, nthreads=S["threads"])
    finally:
        orc.set_full_sort(False)
    _, _, a1 = _render(gpu_ctx, S, W, H, 1, 8, _lib.CT_MATH_EXACT)
    _, _, a2 = _render(gpu_ctx, S, W, H, 1, 8, _lib.CT_MATH_EXACT)
    assert np.array_equal(a1.view(np.int32), a2.view(np.int32))
    assert np.isfinite(a1).all() and (a1 >= 0).all()
    exact_bits = int((a1.view(np.int32) != oacc.view(np.int32)).any(axis=1).sum())
    S["bvh"] = full["fast"]
    _, _, h1 = _render(gpu_ctx, S, W, H, 1, 8, _lib.CT_MATH_EXACT_SHADE)
    _, _, f1 = _render(gpu_ctx, S, W, H, 1, 8, _lib.CT_MATH_FAST)
    hybrid_diff = np.nonzero((h1.view(np.int32) != oacc.view(np.int32)).any(axis=1))[0]
    hybrid_bad = int(_bad(h1, oacc).sum())
    hybrid_bad_same_tree = int(_bad(h1, ofast).sum())
    fast_bad = float(_bad(f1, oacc).mean())
    print(f"\nfull frame vs oracle: exact differing pixels {exact_bits}; exact-shade out of band {hybrid_bad} "
          f"(not bit-equal {hybrid_diff.size}; against the oracle on the same tree {hybrid_bad_same_tree}); "
          f"fast out of band {fast_bad:.5f} ({int(_bad(f1, oacc).sum())} of {W * H})")
    assert exact_bits == 0
    assert hybrid_bad_same_tree == 0
    assert hybrid_diff.size <= 64
    kw = dict(textures=S["ts"].textures, sky_tex=0)
    for pix in hybrid_diff:
        ha, ta = orc.path_hits(S["arr"], S["omats"], S["ob"]["quad"], S["ob"]["prims"], S["cam"], W, H, 0, 8,
                               int(pix), **kw)
        hb, tb = orc.path_hits(S["arr"], S["omats"], fq, fp, S["cam"], W, H, 0, 8, int(pix), **kw)
        part = int(np.argmax(ha != hb)) if (ha != hb).any() else -1
        assert part >= 0, f"pixel {pix}: the same path on both trees, yet the GPU frame differs"
        assert ta.view(np.int32)[part] == tb.view(np.int32)[part], f"pixel {pix}: trees part at unequal t"
    assert fast_bad <= FULL_FAST_OUT_OF_BAND_MAX
    assert np.isfinite(f1).all() and (f1 >= 0).all()
    assert abs(f1[:, :3].sum() - oacc[:, :3].sum()) / oacc[:, :3].sum() < 0.005
    # two accumulated frames: the second frame's buffer is added into the first
    _, _, h2 = _render(gpu_ctx, S, W, H, 2, 8, _lib.CT_MATH_EXACT_SHADE)
    orc.set_full_sort(True)
    try:
        o2 = ofast + _oracle_frames(orc, S_fast, W, H, [2], 8, nthreads=S["threads"])
    finally:
        orc.set_full_sort(False)
    assert _bad(h2, o2).sum() == 0


def test_loaded_model_frames_match_oracle(gpu_ctx, orc, tmp_path):
    """A scene assembled by TriangleList.load_model from OBJ/MTL/TGA files
    (an icosphere, a textured floor quad and an emitter) renders identically
    on the GPU and in the oracle: the ingest path feeds the same arrays,
    materials and texels to both."""
    import struct

    from cudatracer_gb300 import api, scenes

    v, f = scenes.icosphere(3)
    with open(tmp_path / "ball.obj", "w") as fh:
        fh.write("mtllib ball.mtl\nusemtl paint\n")
        fh.writelines(f"v {x:.7f} {y:.7f} {z:.7f}\n" for x, y, z in v)
        fh.writelines(f"f {a + 1} {c + 1} {b + 1}\n" for a, b, c in f)  # the import reversal restores (a, b, c) order
    with open(tmp_path / "ball.mtl", "w") as fh:
        fh.write("newmtl paint\nKd 0.7 0.3 0.2\nNs 0\n")
    with open(tmp_path / "floor.obj", "w") as fh:
        fh.write("mtllib floor.mtl\nv -4 0 -4\nv 4 0 -4\nv 4 0 4\nv -4 0 4\nvt 0 0\nvt 3 0\nvt 3 3\nvt 0 3\nvn 0 1 0\n"
                 "usemtl tiles\nf 1/1/1 4/4/1 3/3/1 2/2/1\n"
                 "v -1 3 -1\nv 1 3 -1\nv 1 3 1\nv -1 3 1\nvn 0 -1 0\nusemtl lamp\nf 5//2 6//2 7//2 8//2\n")
    with open(tmp_path / "floor.mtl", "w") as fh:
        fh.write("newmtl tiles\nKd 1 1 1\nNs 0\nmap_Kd tiles.tga\nnewmtl lamp\nKe 6 6 5\n")
    rng = np.random.default_rng(5)
    tex = rng.integers(0, 256, (8, 8, 3), dtype=np.uint8)
    with open(tmp_path / "tiles.tga", "wb") as fh:
        fh.write(struct.pack("<BBBHHBHHHHBB", 0, 0, 2, 0, 0, 0, 0, 0, 8, 8, 24, 0) + tex[:, :, ::-1].tobytes())
    tl = api.TriangleList()
    M = np.eye(4, dtype=np.float32)
    M[:3, 3] = (0.0, 1.0, 0.0)
    tl.load_model(str(tmp_path / "ball.obj"), scale=0.9, mat=M)
    tl.load_model(str(tmp_path / "floor.obj"), normalize=False)
    assert len(tl.textures) == 1 and tl.arrays()["light_indices"].size == 2
    arr = tl.arrays()
    sc = gpu_ctx.scene_from_list(tl)
    bvh = sc.build_bvh()
    ob = orc.bvh_build(arr["vertices"], arr["indices"])
    mats = [m.__dict__ for m in tl.materials]
    cam = {"fov": 60.0, "position": (0.0, 1.5, 5.0), "forward": (0.0, -0.15, -1.0), "up": (0.0, 1.0, 0.0)}
    S = dict(ts=type("T", (), {"textures": tl.textures}), cam=cam, arr=arr, sc=sc, bvh=bvh, ob=ob,
             omats=orc.pack_materials(mats))
    W, H = 80, 60
    _, _, acc = _render(gpu_ctx, S, W, H, 2, 5, True, sky=False)
    oacc = orc.render_frames(arr, S["omats"], ob["quad"], ob["prims"], cam, W, H, [0, 2], 5, exact_math=True,
                             textures=tl.textures, sky_tex=-1, sky=False)
    assert _bad(acc, oacc).sum() == 0
    assert acc[:, :3].sum() > 0


@pytest.fixture(scope="module")
def textured(gpu_ctx, orc):
    from cudatracer_gb300 import api, scenes

    ts, cam = scenes.terrain_scene(grid=128, spheres=12, sky_size=(256, 128), ground_textures=(37, 29))
    arr = scenes.scene_arrays(ts)
    sc = gpu_ctx.scene(arr, [api.Material(**m) for m in ts.materials], ts.textures, ts.skybox_texture)
    bvh = sc.build_bvh()
    ob = orc.bvh_build(ts.vertices, ts.indices)
    return dict(ts=ts, cam=cam, arr=arr, sc=sc, bvh=bvh, ob=ob, omats=orc.pack_materials(ts.materials))


@pytest.mark.parametrize("filt", [0, 1])
def test_textured_frames_match_oracle(gpu_ctx, orc, textured, filt):
    """Diffuse texture + normal map on the ground, nearest (the reference's
    lookup) and bilinear: exact frames agree with the oracle within 1e-4."""
    W, H = 96, 64
    _, _, acc = _render(gpu_ctx, textured, W, H, 2, 5, True, texture_filter=filt)
    oacc = _oracle(orc, textured, W, H, 2, 5, True, tex_filter=filt)
    assert _bad(acc, oacc).sum() == 0
    assert (acc.view(np.int32) == oacc.view(np.int32)).all(axis=1).mean() >= 0.999


def test_bilinear_differs_from_nearest(gpu_ctx, textured):
    W, H = 96, 64
    _, _, a = _render(gpu_ctx, textured, W, H, 1, 3, True, texture_filter=0)
    _, _, b = _render(gpu_ctx, textured, W, H, 1, 3, True, texture_filter=1)
    assert not np.array_equal(a, b)
    with pytest.raises(Exception):
        _render(gpu_ctx, textured, W, H, 1, 3, True, texture_filter=7)
