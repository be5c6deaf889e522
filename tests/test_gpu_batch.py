"""Batches (ct_batch_*): many uneven jobs in one queue set, iterations
replayed from a CUDA graph, launch shapes from the autotuner.

A job's result must not depend on the batch around it: the same job alone
and in a mix of other scenes, sizes, depths, sample counts and shading
modes gives the same accumulation bit for bit; with exact math a batch
reproduces ct_render_accumulate and the CPU oracle."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scenes_(gpu_ctx, orc):
    from cudatracer_gb300 import api, scenes

    out = []
    for k, (grid, spheres, seed) in enumerate([(48, 6, 1), (96, 10, 2), (32, 3, 3), (128, 16, 4)]):
        ts, cam = scenes.terrain_scene(grid=grid, spheres=spheres, seed=seed, extent=60.0, sky_size=(128, 64),
                                       ground_textures=(16, 16) if k == 1 else None)
        arr = scenes.scene_arrays(ts)
        sc = gpu_ctx.scene(arr, [api.Material(**m) for m in ts.materials], ts.textures, ts.skybox_texture)
        cam = dict(cam, position=(0.0, 14.0, 34.0))
        out.append(dict(ts=ts, cam=cam, arr=arr, sc=sc, bvh=sc.build_bvh_device()))
    return out


def _job(S, W, H, depth, spp, shading=0, frame0=0, tex=0):
    from cudatracer_gb300 import api

    cam = S["cam"]
    camera = api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"])
    p = api.default_params(W, H)
    p.max_depth, p.frame_index, p.shading_mode, p.texture_filter = depth, frame0, shading, tex
    return dict(scene=S["sc"], bvh=S["bvh"], camera=camera, params=p, spp=spp)


def _mix(scenes_):
    return [
        _job(scenes_[0], 40, 30, 5, 3),
        _job(scenes_[1], 64, 48, 8, 2, shading=1, tex=1),
        _job(scenes_[2], 17, 23, 4, 5),
        _job(scenes_[3], 96, 64, 12, 1, frame0=6),
        _job(scenes_[0], 33, 33, 6, 4, shading=1),
        _job(scenes_[1], 8, 8, 3, 7),
    ]


def _run(gpu_ctx, jobs, exact=False, tuning=None):
    import torch

    from cudatracer_gb300 import api

    b = api.Batch(gpu_ctx, jobs, exact_math=exact)
    if tuning:
        b.set_tuning(**tuning)
    b.run()
    torch.cuda.synchronize()
    gpu_ctx.check()
    out = [b.accum_tensor(j).cpu().numpy().copy() for j in range(len(jobs))]
    st = b.stats()
    b.close()
    return out, st


def test_job_alone_equals_job_in_mix(gpu_ctx, scenes_):
    jobs = _mix(scenes_)
    mixed, st = _run(gpu_ctx, jobs)
    assert st["frames"] == max(j["spp"] for j in jobs)
    assert st["samples"] == sum(j["spp"] * j["params"].width * j["params"].height for j in jobs)
    for k, j in enumerate(jobs):
        alone, _ = _run(gpu_ctx, [j])
        assert np.array_equal(alone[0].view(np.int32), mixed[k].view(np.int32)), k
        assert alone[0][:, 3].sum() > 0


def test_exact_batch_equals_render_and_oracle(gpu_ctx, orc, scenes_):
    from cudatracer_gb300 import api

    jobs = _mix(scenes_)
    for j in jobs:
        j["params"].shading_mode = 0
        j["params"].texture_filter = 0
    out, _ = _run(gpu_ctx, jobs, exact=True)
    for k in (0, 2, 3):
        j = jobs[k]
        W, H = j["params"].width, j["params"].height
        job = api.RenderJob(gpu_ctx, W, H)
        job.reset()
        for s in range(j["spp"]):
            p = api.default_params(W, H)
            p.max_depth, p.exact_math = j["params"].max_depth, 1
            p.frame_index = j["params"].frame_index + 2 * s
            job.accumulate(j["scene"], j["bvh"], j["camera"], p)
        gpu_ctx.check()
        single = job.accum_tensor().cpu().numpy()
        assert np.array_equal(single.view(np.int32), out[k].view(np.int32)), k
    S, j = scenes_[2], jobs[2]
    q, pr = S["bvh"].export()
    W, H = j["params"].width, j["params"].height
    frames = [j["params"].frame_index + 2 * s for s in range(j["spp"])]
    oacc = orc.render_frames(S["arr"], orc.pack_materials(S["ts"].materials), q, pr, S["cam"], W, H, frames,
                             j["params"].max_depth, exact_math=True, textures=S["ts"].textures, sky_tex=0)
    rel = np.abs(out[2] - oacc) / np.maximum(np.abs(oacc), 1e-6)
    assert not (rel > 1e-4).any()


def test_exact_shade_batch_matches_oracle_and_is_independent_of_the_mix(gpu_ctx, orc, scenes_):
    """CT_MATH_EXACT_SHADE batches (four lanes, fast traversal, reproducible
    shading): a job in the mix equals the job alone bit for bit, and every
    pixel of the accumulated samples stays within 1e-4 of the oracle's exact
    frames traced in the same child order on the same tree."""
    from cudatracer_gb300 import _lib

    jobs = _mix(scenes_)
    for j in jobs:
        j["params"].shading_mode = 0
        j["params"].texture_filter = 0
    out, _ = _run(gpu_ctx, jobs, exact=_lib.CT_MATH_EXACT_SHADE)
    alone, _ = _run(gpu_ctx, [jobs[3]], exact=_lib.CT_MATH_EXACT_SHADE)
    assert np.array_equal(alone[0].view(np.int32), out[3].view(np.int32))
    orc.set_full_sort(True)
    try:
        for k, si in ((0, 0), (2, 2), (3, 3)):
            S, j = scenes_[si], jobs[k]
            q, pr = S["bvh"].export()
            W, H = j["params"].width, j["params"].height
            frames = [j["params"].frame_index + 2 * s for s in range(j["spp"])]
            oacc = orc.render_frames(S["arr"], orc.pack_materials(S["ts"].materials), q, pr, S["cam"], W, H, frames,
                                     j["params"].max_depth, exact_math=True, textures=S["ts"].textures, sky_tex=0)
            rel = np.abs(out[k] - oacc) / np.maximum(np.abs(oacc), 1e-6)
            assert not (rel > 1e-4).any(), k
            assert out[k][:, 3].sum() > 0
    finally:
        orc.set_full_sort(False)


def test_graph_replay_and_tunings_do_not_change_results(gpu_ctx, scenes_):
    jobs = _mix(scenes_)
    ref, _ = _run(gpu_ctx, jobs, tuning=dict(extend_block=128, connect_block=128, shade_waves=1, use_graph=0))
    for t in (dict(extend_block=64, connect_block=256, shade_waves=2, use_graph=1),
              dict(extend_block=256, connect_block=128, shade_waves=1, use_graph=1),
              dict(extend_block=128, connect_block=128, shade_waves=1, use_graph=1, sort_key=1, refill=8),
              dict(extend_block=64, connect_block=128, shade_waves=2, use_graph=0, sort_key=2, refill=16)):
        out, _ = _run(gpu_ctx, jobs, tuning=t)
        for a, b in zip(ref, out):
            assert np.array_equal(a.view(np.int32), b.view(np.int32))


def test_autotune_picks_a_valid_shape(gpu_ctx, scenes_):
    import torch

    from cudatracer_gb300 import api

    jobs = _mix(scenes_)
    b = api.Batch(gpu_ctx, jobs)
    t, ms = b.autotune()
    assert t["extend_block"] in (64, 128, 256) and t["connect_block"] in (64, 128, 256)
    assert t["shade_waves"] in (1, 2) and t["use_graph"] in (0, 1) and t["sort_key"] in (0, 1, 2) and ms > 0
    assert t["refill"] in (8, 16, 24)
    assert b.tuning == t
    b.run()
    torch.cuda.synchronize()
    got = [b.accum_tensor(j).cpu().numpy().copy() for j in range(len(jobs))]
    b.close()
    ref, _ = _run(gpu_ctx, jobs)
    for a, c in zip(ref, got):
        assert np.array_equal(a.view(np.int32), c.view(np.int32))


def test_batch_validation(gpu_ctx, scenes_):
    from cudatracer_gb300 import _lib, api, scenes

    j = _job(scenes_[0], 16, 16, 4, 0)
    with pytest.raises(_lib.CTError):
        api.Batch(gpu_ctx, [j])  # spp 0
    s = scenes.soup_scene(500, seed=2)
    arr = {"vertices": s.vertices, "normals": np.tile(np.array([[0, 0, 1]], np.float32), (s.vertices.shape[0], 1)),
           "indices": s.indices}
    sc = gpu_ctx.scene(arr, [api.Material()])
    j = _job(scenes_[0], 16, 16, 4, 1)
    j["bvh"] = scenes_[0]["sc"].build_bvh_wide()
    with pytest.raises(_lib.CTError):
        api.Batch(gpu_ctx, [j, _job(scenes_[1], 16, 16, 4, 1)])  # quad and wide trees in one batch


def test_wide_batch_job_alone_equals_job_in_mix(gpu_ctx, scenes_):
    """Batches on the quantised trees: the same independence from the mix."""
    jobs = _mix(scenes_)
    wide = {id(S["sc"]): S["sc"].build_bvh_wide() for S in scenes_}
    for j in jobs:
        j["bvh"] = wide[id(j["scene"])]
    mixed, _ = _run(gpu_ctx, jobs)
    for k in (0, 3, 5):
        alone, _ = _run(gpu_ctx, [jobs[k]])
        assert np.array_equal(alone[0].view(np.int32), mixed[k].view(np.int32)), k
    srt, _ = _run(gpu_ctx, jobs, tuning=dict(extend_block=128, connect_block=128, shade_waves=1, use_graph=1,
                                             sort_key=2))
    for a, b in zip(mixed, srt):
        assert np.array_equal(a.view(np.int32), b.view(np.int32))


def test_fast_tree_batch(gpu_ctx, scenes_):
    """Batches on ct_bvh_build_fast's trees: independent of the mix, and equal
    to the same batch on the reference's trees up to exact t ties."""
    jobs = _mix(scenes_)
    ref, _ = _run(gpu_ctx, jobs)
    fast = {id(S["sc"]): S["sc"].build_bvh_fast() for S in scenes_}
    for j in jobs:
        j["bvh"] = fast[id(j["scene"])]
    mixed, _ = _run(gpu_ctx, jobs)
    for k in (0, 3, 5):
        alone, _ = _run(gpu_ctx, [jobs[k]])
        assert np.array_equal(alone[0].view(np.int32), mixed[k].view(np.int32)), k
    for a, b in zip(mixed, ref):
        rel = np.abs(a - b) / np.maximum(np.abs(b), 1e-6)
        assert (rel > 1e-4).any(axis=-1).mean() < 2e-3
