"""The serving loop (ct_server_*): requests admitted as they arrive against an
HBM budget, render jobs batched continuously, ray queries overlapping.

Each result must be the same alone and in the mix: a request served by
itself and the same request submitted together with many others (renders of
other scenes, sizes, depths and sample counts; closest-hit and any-hit
queries on quad and wide BVHs) give identical bytes."""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def world(gpu_ctx):
    from cudatracer_gb300 import api, scenes

    out = {"render": [], "query": []}
    for k, (grid, spheres, seed) in enumerate([(48, 6, 11), (96, 10, 12), (32, 3, 13)]):
        ts, cam = scenes.terrain_scene(grid=grid, spheres=spheres, seed=seed, extent=60.0, sky_size=(128, 64))
        sc = gpu_ctx.scene(scenes.scene_arrays(ts), [api.Material(**m) for m in ts.materials], ts.textures,
                           ts.skybox_texture)
        out["render"].append(dict(sc=sc, bvh=sc.build_bvh_device(), cam=dict(cam, position=(0.0, 14.0, 34.0))))
    s = scenes.soup_scene(100000, seed=14)
    arr = {"vertices": s.vertices, "normals": np.tile(np.array([[0, 0, 1]], np.float32), (s.vertices.shape[0], 1)),
           "indices": s.indices}
    sq = gpu_ctx.scene(arr, [api.Material()])
    out["query"] = [sq.build_bvh_device(), sq.build_bvh_wide()]
    out["soup_scene"] = sq
    return out


def _render_job(S, W, H, depth, spp, shading=0):
    from cudatracer_gb300 import api

    cam = S["cam"]
    p = api.default_params(W, H)
    p.max_depth, p.shading_mode = depth, shading
    return dict(scene=S["sc"], bvh=S["bvh"], camera=api.Camera(W, H, cam["fov"], cam["position"], cam["forward"],
                                                                cam["up"]), params=p, spp=spp)


def _requests(world):
    from cudatracer_gb300 import scenes

    R = world["render"]
    reqs = [
        ("render", _render_job(R[0], 48, 32, 5, 3)),
        ("render", _render_job(R[1], 64, 64, 8, 6, shading=1)),
        ("render", _render_job(R[2], 20, 30, 4, 9)),
        ("render", _render_job(R[0], 96, 48, 12, 2)),
        ("render", _render_job(R[1], 16, 16, 6, 12)),
    ]
    for k in range(6):
        o, d = scenes.incoherent_rays(5000 * (k + 1), seed=30 + k)
        if k % 2:
            d[:, 3] = 0.05 * (k + 1)
        reqs.append(("query", dict(bvh=world["query"][k % 2], org=o, dir=d, any_hit=bool(k % 2), tri_eps=1e-12)))
    return reqs


def _submit(srv, kind, r):
    if kind == "render":
        return srv.submit_render(r)
    return srv.submit_query(r["bvh"], r["org"], r["dir"], any_hit=r["any_hit"], tri_eps=r["tri_eps"])


def _same(a, b):
    if isinstance(a, tuple):
        return all(_same(x, y) for x, y in zip(a, b))
    return np.array_equal(np.ascontiguousarray(a).view(np.uint8), np.ascontiguousarray(b).view(np.uint8))


@pytest.mark.parametrize("math", [0, 2])  # CT_MATH_FAST, CT_MATH_EXACT_SHADE
def test_each_result_same_alone_and_in_mix(gpu_ctx, world, math):
    from cudatracer_gb300 import api

    reqs = _requests(world)
    srv = api.Server(gpu_ctx, max_inflight_pixels=1 << 16, exact_math=math)
    alone = []
    for kind, r in reqs:
        rid = _submit(srv, kind, r)
        alone.append(srv.wait(rid)[1])
    srv.close()
    # all at once, in a shuffled order, some arriving while others run
    srv = api.Server(gpu_ctx, max_inflight_pixels=1 << 16, exact_math=math)
    order = np.random.default_rng(5).permutation(len(reqs))
    ids = {}
    for k, i in enumerate(order):
        ids[i] = _submit(srv, *reqs[i])
        if k % 3 == 2:
            time.sleep(0.002)
    mixed = {i: srv.wait(ids[i]) for i in order}
    st = srv.stats()
    srv.close()
    gpu_ctx.check()
    for i in range(len(reqs)):
        assert _same(alone[i], mixed[i][1]), i
        info = mixed[i][0]
        assert info["status"] == 0 and info["submit_s"] <= info["admit_s"] <= info["done_s"]
    assert st["completed"] == len(reqs) and st["failed"] == 0
    # small jobs take min(spp, 65536 // pixels) samples per iteration
    assert st["iterations"] >= max(-(-r["spp"] // max(1, min(r["spp"], 65536 // (r["params"].width * r["params"].height))))
                                   for k, r in reqs if k == "render")


def test_render_matches_batch_and_queries_equal_direct_calls(gpu_ctx, world):
    import torch

    from cudatracer_gb300 import api

    reqs = _requests(world)
    srv = api.Server(gpu_ctx)
    ids = [_submit(srv, *r) for r in reqs]
    res = [srv.wait(i)[1] for i in ids]
    srv.close()
    for (kind, r), got in zip(reqs, res):
        if kind == "render":
            b = api.Batch(gpu_ctx, [r])
            b.run()
            torch.cuda.synchronize()
            ref = b.accum_tensor(0).cpu().numpy()
            b.close()
            # small jobs take several samples per iteration into slot buffers
            # added at the end: the same samples, summed in another order
            assert np.allclose(got, ref, rtol=1e-5, atol=1e-6)
            assert np.array_equal(got[:, 3], ref[:, 3])
        else:
            o, d = torch.from_numpy(r["org"]).cuda(), torch.from_numpy(r["dir"]).cuda()
            if r["any_hit"]:
                ref = r["bvh"].trace_any(o, d, tri_eps=r["tri_eps"]).cpu().numpy()
            else:
                h, t = r["bvh"].trace_closest(o, d, tri_eps=r["tri_eps"])
                ref = (h.cpu().numpy(), t.cpu().numpy())
            assert _same(ref, got)


def test_admission_respects_the_budget(gpu_ctx, world):
    from cudatracer_gb300 import _lib, api

    reqs = _requests(world)
    def render_bytes(r):
        px = r["params"].width * r["params"].height
        k = max(1, min(r["spp"], 65536 // px))
        return min(r["spp"], 2 * k) * px * 16  # slot buffers

    def query_bytes(r):  # rays, results, counters; queries on the wide tree add 32 B of records per ray
        return r["org"].shape[0] * (72 if r["bvh"] is world["query"][1] else 40) + 2048

    sizes = [render_bytes(r) if k == "render" else query_bytes(r) for k, r in reqs]
    budget = max(sizes) + 4096
    srv = api.Server(gpu_ctx, hbm_budget=budget, max_inflight_pixels=1 << 16)
    ids = [_submit(srv, *r) for r in reqs]
    for i in ids:
        srv.wait(i)
    st = srv.stats()
    assert 0 < st["peak_bytes"] <= budget and st["completed"] == len(reqs)
    # a request that can never fit fails instead of waiting forever
    big = _render_job(world["render"][0], 512, 512, 4, 1)
    rid = srv.submit_render(big)
    with pytest.raises(_lib.CTError) as e:
        srv.wait(rid, timeout=30.0)
    assert e.value.status == _lib.CT_ERR_OUT_OF_MEMORY
    srv.close()


def test_larger_iterations_same_alone_and_in_mix(gpu_ctx, world):
    """With a larger per-iteration budget every job here takes several samples
    per iteration (k = min(spp, iter_pixels / pixels) slot buffers); results are
    still identical alone and in the mix, and equal ct_batch's up to the
    summation order of the slots."""
    import torch

    from cudatracer_gb300 import api

    R = world["render"]
    reqs = [("render", _render_job(R[0], 160, 120, 6, 5)), ("render", _render_job(R[1], 128, 128, 8, 7, shading=1)),
            ("render", _render_job(R[2], 64, 48, 5, 9))] + [q for q in _requests(world) if q[0] == "query"][:3]
    cfg = dict(max_inflight_pixels=1 << 17, iter_pixels=1 << 16)
    srv = api.Server(gpu_ctx, **cfg)
    alone = [srv.wait(_submit(srv, *r))[1] for r in reqs]
    srv.close()
    srv = api.Server(gpu_ctx, **cfg)
    order = (5, 2, 0, 3, 1, 4)
    ids = [_submit(srv, *reqs[i]) for i in order]
    mixed = dict(zip(order, (srv.wait(i) for i in ids)))
    st = srv.stats()
    srv.close()
    gpu_ctx.check()
    for i in range(len(reqs)):
        assert _same(alone[i], mixed[i][1]), i
    # 160x120 takes 3 samples per iteration (2 iterations), 128x128 4 (2), 64x48 9 (1)
    assert 2 <= st["iterations"] <= 6
    for (kind, r), got in zip(reqs[:3], alone[:3]):
        b = api.Batch(gpu_ctx, [r])
        b.run()
        torch.cuda.synchronize()
        ref = b.accum_tensor(0).cpu().numpy()
        b.close()
        assert np.allclose(got, ref, rtol=1e-5, atol=1e-6)
        assert np.array_equal(got[:, 3], ref[:, 3])
