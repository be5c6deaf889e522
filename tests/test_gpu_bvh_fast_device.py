"""The device build of the traversal-speed tree (ct_bvh_build_fast_device)
against its host build (ct_bvh_build_fast): the quad nodes and the primitive
order equal byte for byte, on soups of 1 to 400,000 triangles, the sphere, a
terrain, and inputs that take every branch of the builder — coincident
triangles (no bin split: ranges halved as they lie, in warp-built subtrees and
in level-built nodes), centroids on one plane (an axis without extent), a
binary tree deep enough to reach the depth limit, a scene at the origin (zero
padding, negative zeros), and scenes whose nodes take the exact sweep only."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(gpu_ctx, v, ix):
    from cudatracer_gb300 import api

    v = np.ascontiguousarray(v, np.float32)
    ix = np.ascontiguousarray(ix, np.uint32)
    arr = {"vertices": v, "normals": np.tile(np.array([[0, 0, 1]], np.float32), (v.shape[0], 1)), "indices": ix}
    return gpu_ctx.scene(arr, [api.Material()])


def _compare(gpu_ctx, v, ix):
    sc = _scene(gpu_ctx, v, ix)
    hb, db = sc.build_bvh_fast(), sc.build_bvh_fast_device()
    qh, ph = hb.export()
    qd, pd = db.export()
    assert qd.shape == qh.shape
    assert np.array_equal(qd.view(np.int32), qh.view(np.int32))
    assert np.array_equal(pd, ph)
    ih, id_ = hb.info(), db.info()
    for k in ("quad_node_count", "max_leaf_size", "quad_depth", "stack_entries", "prim_count", "binary_node_count"):
        assert ih[k] == id_[k], k
    return sc, hb, db


@pytest.mark.parametrize("ntri", [1, 2, 3, 4, 5, 16, 17, 128, 129, 300, 5000, 70000, 400000])
def test_soups_match_host_build(gpu_ctx, ntri):
    from cudatracer_gb300 import scenes

    s = scenes.soup_scene(ntri, seed=ntri)
    _compare(gpu_ctx, s.vertices, s.indices)


def test_sphere_and_terrain_match_host_build(gpu_ctx):
    from cudatracer_gb300 import scenes

    s = scenes.sphere_scene(6)
    _compare(gpu_ctx, s.vertices, s.indices)
    ts, _ = scenes.terrain_scene(grid=256, spheres=20, sky_size=(64, 32))
    _compare(gpu_ctx, ts.vertices, ts.indices)


def test_degenerate_inputs_match_host_build(gpu_ctx):
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    # identical triangles: every split halves the range as it lies (warp-built
    # subtrees at 100, level-built nodes at 3,000)
    for n in (100, 3000):
        _compare(gpu_ctx, v, np.tile(np.array([[0, 1, 2]], np.uint32), (n, 1)))
    # two coincident groups and triangles strung along one axis
    x = np.repeat(np.arange(1000, dtype=np.float32) % 7, 3)
    vs = np.stack([x, np.tile([0, 1, 0], 1000).astype(np.float32), np.tile([0, 0, 1], 1000).astype(np.float32)], 1)
    _compare(gpu_ctx, vs, np.arange(3000, dtype=np.uint32).reshape(-1, 3))
    # a flat grid (no extent along y) and a scene at the origin (zero padding)
    rng = np.random.default_rng(7)
    g = rng.uniform(-3, 3, size=(6000, 3)).astype(np.float32)
    g[:, 1] = 0.0
    _compare(gpu_ctx, g, np.arange(6000, dtype=np.uint32).reshape(-1, 3))
    z = np.zeros((30, 3), np.float32)
    z[::2, 0] = -0.0
    _compare(gpu_ctx, z, np.arange(30, dtype=np.uint32).reshape(-1, 3))
    # geometric spacing: a chain of nested splits that reaches the depth limit
    xs = np.float32(2.0) ** -np.arange(90, dtype=np.float32)
    vv = np.zeros((270, 3), np.float32)
    vv[0::3, 0] = xs
    vv[1::3, 0] = xs
    vv[1::3, 1] = xs
    vv[2::3, 0] = xs
    vv[2::3, 2] = xs
    _compare(gpu_ctx, vv, np.arange(270, dtype=np.uint32).reshape(-1, 3))


def test_hits_and_frames_on_device_tree(gpu_ctx):
    """The device-built tree is the host-built tree: queries and frames on it
    give identical bytes."""
    import torch

    from cudatracer_gb300 import api, scenes

    ts, cam = scenes.terrain_scene(grid=128, spheres=12, sky_size=(128, 64))
    arr = scenes.scene_arrays(ts)
    sc = gpu_ctx.scene(arr, [api.Material(**m) for m in ts.materials], ts.textures, ts.skybox_texture)
    hb, db = sc.build_bvh_fast(), sc.build_bvh_fast_device()
    o, d = scenes.incoherent_rays(50000, seed=3)
    lo, hi = arr["vertices"].min(0), arr["vertices"].max(0)
    o[:, :3] = lo + (hi - lo) * o[:, :3]
    og, dg = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    hh, th = hb.trace_closest(og, dg)
    hd, td = db.trace_closest(og, dg)
    assert torch.equal(hh, hd) and torch.equal(th.view(torch.int32), td.view(torch.int32))
    assert int((hh >= 0).sum()) > 1000
    assert torch.equal(hb.trace_any(og, dg), db.trace_any(og, dg))
    W, H = 96, 64
    outs = []
    for b in (hb, db):
        job = api.RenderJob(gpu_ctx, W, H)
        p = api.Params(W, H, camera=api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"]),
                       max_depth=5, exact_math=2)
        p.reset(job)
        for _ in range(3):
            api.launch_kernels(job, sc, b, p)
        torch.cuda.synchronize()
        outs.append(job.accum_tensor().cpu().numpy().copy())
    gpu_ctx.check()
    assert np.array_equal(outs[0].view(np.int32), outs[1].view(np.int32))
    assert outs[0][:, 3].sum() > 0
