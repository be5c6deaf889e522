"""GPU frames through the C ABI against a frame rendered by the REFERENCE's own
GPU kernels (tests/golden/ref_frame_gpu.npz: the reference's Kernel.cu built for
sm_103a and its launchKernels, on its own quad BVH; 64x48, depth 5, compat
shading, no sky, first frame; made by tests/golden/make_ref_frame.py).

CT_MATH_FAST uses nvcc's FMA contraction and CUDA's sinf/cosf like the
reference's build, but its source contracts into other FMAs, so some paths that
graze an edge diverge (45 of 3,072 pixels measured on the reference's tree).
CT_MATH_EXACT is the uncontracted oracle bit for bit (67 pixels, the oracle's
own count); CT_MATH_EXACT_SHADE the same up to exact-t ties. Bounds are about
twice what was measured; the per-pixel band is 1e-4."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-4


@pytest.fixture(scope="module")
def ref_scene(gpu_ctx):
    from cudatracer_gb300 import api, scenes

    from tests.conftest import golden

    g = golden("ref_frame_gpu.npz")
    ts, cam = scenes.terrain_scene(grid=int(g["grid"]), spheres=int(g["spheres"]), sky_size=(64, 32))
    arr = scenes.scene_arrays(ts)
    sc = gpu_ctx.scene(arr, [api.Material(**m) for m in ts.materials], ts.textures, ts.skybox_texture)
    return dict(g=g, cam=cam, sc=sc)


def _frame(gpu_ctx, R, bvh, math):
    from cudatracer_gb300 import api

    g, cam = R["g"], R["cam"]
    W, H = int(g["width"]), int(g["height"])
    eps = [float(x) for x in g["eps"]]
    job = api.RenderJob(gpu_ctx, W, H)
    p = api.Params(W, H, camera=api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"]),
                   max_depth=int(g["depth"]), exact_math=math, sky=False, normal_eps=eps[0], dist_eps=eps[1],
                   tri_eps=eps[2])
    p.reset(job)
    api.launch_kernels(job, R["sc"], bvh, p)
    gpu_ctx.check()
    return job.accum_tensor().cpu().numpy().copy()


@pytest.mark.parametrize("math,tree,max_bad", [(0, "reference", 90), (0, "fast", 90), (1, "reference", 120),
                                               (2, "fast", 120)])
def test_frame_matches_reference_gpu_frame(gpu_ctx, ref_scene, math, tree, max_bad):
    sc = ref_scene["sc"]
    bvh = sc.build_bvh() if tree == "reference" else sc.build_bvh_fast()
    ref = ref_scene["g"]["accum"]
    acc = _frame(gpu_ctx, ref_scene, bvh, math)
    rel = np.abs(acc - ref) / np.maximum(np.abs(ref), 1e-6)
    bad = (rel > RTOL).any(axis=1)
    print(f"math {math} {tree} tree: {int(bad.sum())} of {ref.shape[0]} pixels outside 1e-4, "
          f"contributions {acc[:, 3].sum():.0f} vs {ref[:, 3].sum():.0f}")
    assert bad.sum() <= max_bad
    assert abs(acc[:, :3].sum() - ref[:, :3].sum()) <= 0.01 * ref[:, :3].sum()
    assert abs(acc[:, 3].sum() - ref[:, 3].sum()) <= 0.02 * ref[:, 3].sum()
