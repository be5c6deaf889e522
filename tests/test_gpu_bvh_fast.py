"""The traversal-speed quad tree (ct_bvh_build_fast) on the GPU: ray queries
bit-exact against the oracle on the same tree and equal in t to the reference
tree's, frames on it against the oracle's frames on it, and fast-math frames
against fast-math frames on the reference tree."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _t4(a, w=None):
    import torch

    b = np.zeros((a.shape[0], 4), np.float32)
    b[:, :3] = a[:, :3]
    if w is not None:
        b[:, 3] = w
    return torch.from_numpy(b).cuda()


@pytest.fixture(scope="module")
def terrain(gpu_ctx):
    from cudatracer_gb300 import api, scenes

    ts, cam = scenes.terrain_scene(grid=128, spheres=12, sky_size=(256, 128))
    arr = scenes.scene_arrays(ts)
    sc = gpu_ctx.scene(arr, [api.Material(**m) for m in ts.materials], ts.textures, ts.skybox_texture)
    return ts, cam, arr, sc


def test_fast_tree_queries(gpu_ctx, orc, terrain):
    from cudatracer_gb300 import api

    ts, cam, _, sc = terrain
    fb = sc.build_bvh_fast()
    q, pr = fb.export()
    host = api.host_bvh_build(ts.vertices, ts.indices, 2, fast=True)
    assert np.array_equal(q, host["quad"]) and np.array_equal(pr, host["prims"])
    info = fb.info()
    assert info["binary_node_count"] == 0 and info["max_leaf_size"] <= 4
    rng = np.random.default_rng(7)
    n = 1 << 16
    lo, hi = ts.vertices.min(0), ts.vertices.max(0)
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    o[: n // 2] = np.asarray(cam["position"], np.float32)
    d = rng.normal(size=(n, 3))
    fw = np.asarray(cam["forward"], np.float64)
    d[: n // 2] = fw / np.linalg.norm(fw) + rng.uniform(-0.6, 0.6, size=(n // 2, 3))
    d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
    hit, t = fb.trace_closest(_t4(o), _t4(d, 1e34))
    gpu_ctx.check()
    hit, t = hit.cpu().numpy(), t.cpu().numpy()
    oh, ot = orc.trace_closest(q, pr, ts.vertices, ts.indices, o, d)
    assert np.array_equal(hit, oh) and np.array_equal(t.view(np.int32), ot.view(np.int32))
    ref = api.host_bvh_build(ts.vertices, ts.indices, 2)
    rh, rt = orc.trace_closest(ref["quad"], ref["prims"], ts.vertices, ts.indices, o, d)
    assert np.array_equal(t.view(np.int32), rt.view(np.int32))
    assert (hit != rh).mean() < 1e-3 and (hit >= 0).sum() > n // 4
    tmax = np.where(ot < 1e30, ot * rng.uniform(0.5, 1.5, size=n), 50.0).astype(np.float32)
    occ = fb.trace_any(_t4(o), _t4(d, tmax))
    gpu_ctx.check()
    assert np.array_equal(occ.cpu().numpy(), orc.trace_any(ref["quad"], ref["prims"], ts.vertices, ts.indices, o, d,
                                                           tmax))


def test_frames_on_the_fast_tree(gpu_ctx, orc, terrain):
    from cudatracer_gb300 import api

    ts, cam, arr, sc = terrain
    fb, rb = sc.build_bvh_fast(), sc.build_bvh_device()
    W, H = 96, 64
    camera = api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"])

    def render(bvh, exact, frames=2):
        job = api.RenderJob(gpu_ctx, W, H)
        p = api.Params(W, H, camera=camera, max_depth=5, exact_math=exact)
        p.reset(job)
        for _ in range(frames):
            api.launch_kernels(job, sc, bvh, p)
        gpu_ctx.check()
        return job.accum_tensor().cpu().numpy().copy()

    # exact-math frames follow the tree they are given: the oracle on the same tree
    q, pr = fb.export()
    a = render(fb, True)
    o = orc.render_frames(arr, orc.pack_materials(ts.materials), q, pr, cam, W, H, [0, 2], 5, exact_math=True,
                          textures=ts.textures, sky_tex=0)
    assert (a.view(np.int32) == o.view(np.int32)).all(axis=1).mean() >= 0.999
    # fast-math frames equal the reference tree's up to exact t ties
    f_f, f_r = render(fb, False), render(rb, False)
    rel = np.abs(f_f - f_r) / np.maximum(np.abs(f_r), 1e-6)
    assert (rel > 1e-4).any(axis=1).mean() < 1e-3
