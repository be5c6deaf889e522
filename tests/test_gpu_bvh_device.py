"""The device SAH builder (ct_bvh_build_device) against the host build of the
same scene, which is itself pinned to the reference's BVHTree/MBVHTree: quad
nodes bit-identical (bounds, child numbering, leaf ranges), the same
primitives in every leaf, and identical closest hits and frames."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(gpu_ctx, v, ix):
    from cudatracer_gb300 import api

    v = np.ascontiguousarray(v, np.float32)
    ix = np.ascontiguousarray(ix, np.uint32)
    arr = {"vertices": v, "normals": np.tile(np.array([[0, 0, 1]], np.float32), (v.shape[0], 1)), "indices": ix}
    return gpu_ctx.scene(arr, [api.Material()])


def _leaf_sets_equal(q, p_host, p_dev):
    """Every leaf range holds the same primitives (order inside a leaf may differ)."""
    counts, childs = q[:, 28:32], q[:, 24:28]
    for first, cnt in zip(childs[counts > 0], counts[counts > 0]):
        if not np.array_equal(np.sort(p_host[first:first + cnt]), np.sort(p_dev[first:first + cnt])):
            return False
    return np.array_equal(np.sort(p_host), np.sort(p_dev))


def _compare(gpu_ctx, v, ix):
    sc = _scene(gpu_ctx, v, ix)
    hb, db = sc.build_bvh(), sc.build_bvh_device()
    qh, ph = hb.export()
    qd, pd = db.export()
    assert qd.shape == qh.shape
    assert np.array_equal(qd.view(np.int32), qh.view(np.int32))
    assert _leaf_sets_equal(qh, ph, pd)
    ih, id_ = hb.info(), db.info()
    for k in ("quad_node_count", "max_leaf_size", "quad_depth", "stack_entries", "prim_count"):
        assert ih[k] == id_[k], k
    return sc, hb, db


@pytest.mark.parametrize("ntri", [1, 2, 3, 4, 5, 17, 128, 129, 300, 5000, 70000])
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


def test_coincident_and_collinear_inputs(gpu_ctx):
    # identical triangles: every candidate has an empty side, so one big leaf
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    ix = np.tile(np.array([[0, 1, 2]], np.uint32), (300, 1))
    _compare(gpu_ctx, v, ix)
    # triangles strung along one axis, two coincident groups, and a flat grid
    x = np.repeat(np.arange(1000, dtype=np.float32) % 7, 3)
    v = np.stack([x, np.tile([0, 1, 0], 1000).astype(np.float32), np.tile([0, 0, 1], 1000).astype(np.float32)], 1)
    ix = np.arange(3000, dtype=np.uint32).reshape(-1, 3)
    _compare(gpu_ctx, v, ix)


def test_large_soup_hits_and_frame(gpu_ctx, orc):
    """Closest hits through the device-built tree equal the host-built tree's
    (t bit for bit; ids differ only where two triangles of one leaf tie), and
    the tree's exact frames match the oracle traced through the same tree."""
    import torch

    from cudatracer_gb300 import api, scenes

    s = scenes.soup_scene(400000, seed=8)
    sc, hb, db = _compare(gpu_ctx, s.vertices, s.indices)
    o, d = scenes.incoherent_rays(1 << 20, seed=9)
    org, dir_ = torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda()
    # the reference's absolute determinant epsilon (1e-3) culls every soup
    # triangle (edges <= 1e-2), so trace with a tiny one
    h1, t1 = hb.trace_closest(org, dir_, tri_eps=1e-12)
    h2, t2 = db.trace_closest(org, dir_, tri_eps=1e-12)
    gpu_ctx.check()
    t1, t2, h1, h2 = t1.cpu().numpy(), t2.cpu().numpy(), h1.cpu().numpy(), h2.cpu().numpy()
    assert np.array_equal(t1.view(np.int32), t2.view(np.int32))
    assert (h1 >= 0).sum() > 1000
    assert (h1 != h2).mean() < 1e-4


def test_device_tree_renders_like_oracle(gpu_ctx, orc):
    from cudatracer_gb300 import api, scenes

    ts, cam = scenes.terrain_scene(grid=128, spheres=12, sky_size=(256, 128))
    arr = scenes.scene_arrays(ts)
    sc = gpu_ctx.scene(arr, [api.Material(**m) for m in ts.materials], ts.textures, ts.skybox_texture)
    bvh = sc.build_bvh_device()
    q, p = bvh.export()
    W, H = 96, 64
    job = api.RenderJob(gpu_ctx, W, H)
    prm = api.Params(W, H, camera=api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"]),
                     max_depth=5, exact_math=True)
    prm.reset(job)
    for _ in range(2):
        api.launch_kernels(job, sc, bvh, prm)
    gpu_ctx.check()
    acc = job.accum_tensor().cpu().numpy()
    oacc = orc.render_frames(arr, orc.pack_materials(ts.materials), q, p, cam, W, H, [0, 2], 5, exact_math=True,
                             textures=ts.textures, sky_tex=0)
    rel = np.abs(acc - oacc) / np.maximum(np.abs(oacc), 1e-6)
    assert not (rel > 1e-4).any()
    assert (acc.view(np.int32) == oacc.view(np.int32)).all(axis=1).mean() >= 0.999


def test_binary_export_is_unsupported(gpu_ctx):
    from cudatracer_gb300 import _lib, scenes

    s = scenes.soup_scene(1000, seed=1)
    db = _scene(gpu_ctx, s.vertices, s.indices).build_bvh_device()
    with pytest.raises(_lib.CTError):
        db.export(_lib.CT_BVH_BINARY)
