"""Full-material shading (CT_SHADE_FULL) against the FP64 Monte Carlo oracle
(oracle/ct_fp64.cpp): converged images must agree within 3 standard errors.

The GPU estimate and its standard error come from independent batches of
frames (the mean of the batch means and their spread); the oracle reports its
own per-pixel sample variance. Per pixel channel z = (gpu - fp64) / sqrt(se_gpu^2 +
se_fp64^2); for a correct estimator |z| > 3 occurs for ~0.3 % of values (caustic
paths through mirrors and dielectrics make the tails a little heavier, so up to
1 % is accepted), the mean of z is ~0 and the image totals agree within 0.5 %.
Measured on GB300: 0.39 % beyond 3 sigma, mean z +0.012, totals within 0.04 %."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def zoo(gpu_ctx, orc):
    from cudatracer_gb300 import api, scenes

    sc, cam = scenes.material_zoo_scene()
    arr = scenes.scene_arrays(sc)
    s = gpu_ctx.scene(arr, [api.Material(**m) for m in sc.materials], sc.textures, sc.skybox_texture)
    bvh = s.build_bvh()
    return dict(sc=sc, cam=cam, arr=arr, scene=s, bvh=bvh)


def _gpu_batches(gpu_ctx, z, W, H, depth, batches, frames, exact=False, texture_filter=0):
    import torch

    from cudatracer_gb300 import _lib, api

    cam = z["cam"]
    job = api.RenderJob(gpu_ctx, W, H)
    camera = api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"])
    means = []
    for b in range(batches):
        job.reset()
        for f in range(frames):
            p = api.default_params(W, H)
            p.max_depth = depth
            p.frame_index = 2 * (b * frames + f)
            p.shading_mode = _lib.CT_SHADE_FULL
            p.exact_math = int(exact)
            p.texture_filter = texture_filter
            job.accumulate(z["scene"], z["bvh"], camera, p)
        torch.cuda.synchronize()
        means.append(job.accum_tensor().cpu().numpy()[:, :3].astype(np.float64) / frames)
    gpu_ctx.check()
    m = np.stack(means)
    return m.mean(0), m.std(0, ddof=1) / np.sqrt(batches)


def test_full_mode_converges_to_fp64_oracle(gpu_ctx, orc, zoo):
    W, H, depth = 40, 30, 6
    g, g_se = _gpu_batches(gpu_ctx, zoo, W, H, depth, batches=32, frames=32)
    ob = orc.bvh_build(zoo["sc"].vertices, zoo["sc"].indices)
    o, o_se = orc.render_fp64(zoo["arr"], orc.pack_materials(zoo["sc"].materials), ob["quad"], ob["prims"],
                              zoo["cam"], W, H, 1024, depth, textures=zoo["sc"].textures, sky_tex=0, seed=7)
    se = np.sqrt(g_se ** 2 + o_se ** 2)
    live = se > 1e-7
    z = (g - o)[live] / se[live]
    assert np.isfinite(g).all() and (g >= 0).all()
    frac = (np.abs(z) > 3).mean()
    assert frac < 0.01, f"{frac:.4f} of pixel channels beyond 3 sigma"
    assert abs(z.mean()) < 0.1, z.mean()
    assert abs(g.sum() / o.sum() - 1) < 0.005
    dead = ~live  # pixels with no variance on either side must agree exactly in value
    assert np.allclose(g[dead], o[dead], atol=1e-6)


def test_full_mode_flags_and_determinism(gpu_ctx, zoo):
    W, H = 32, 24
    g1, _ = _gpu_batches(gpu_ctx, zoo, W, H, 4, batches=2, frames=2, exact=True)
    g2, _ = _gpu_batches(gpu_ctx, zoo, W, H, 4, batches=2, frames=2, exact=True)
    assert np.array_equal(g1, g2)


@pytest.fixture(scope="module")
def zoo_tex(gpu_ctx):
    from cudatracer_gb300 import api, scenes

    sc, cam = scenes.material_zoo_scene(ground_textures=(48, 40))
    arr = scenes.scene_arrays(sc)
    s = gpu_ctx.scene(arr, [api.Material(**m) for m in sc.materials], sc.textures, sc.skybox_texture)
    return dict(sc=sc, cam=cam, arr=arr, scene=s, bvh=s.build_bvh_device())


def test_full_mode_textured_bilinear_converges(gpu_ctx, orc, zoo_tex):
    """The same 3-sigma bar with a bilinear-filtered diffuse texture and a
    normal map on the ground (FP64 oracle filters in double)."""
    z = zoo_tex
    W, H, depth = 40, 30, 5
    g, g_se = _gpu_batches(gpu_ctx, z, W, H, depth, batches=32, frames=32, texture_filter=1)
    q, p = z["bvh"].export()
    o, o_se = orc.render_fp64(z["arr"], orc.pack_materials(z["sc"].materials), q, p, z["cam"], W, H, 1024, depth,
                              textures=z["sc"].textures, sky_tex=0, seed=11, tex_filter=1)
    se = np.sqrt(g_se ** 2 + o_se ** 2)
    live = se > 1e-7
    zz = (g - o)[live] / se[live]
    assert np.isfinite(g).all() and (g >= 0).all()
    assert (np.abs(zz) > 3).mean() < 0.01
    assert abs(zz.mean()) < 0.1
    assert abs(g.sum() / o.sum() - 1) < 0.005
