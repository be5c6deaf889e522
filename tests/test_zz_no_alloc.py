"""The allocation-free frame entry point (ct_render_accumulate_noalloc).

It exists for hosts that must not let the library allocate device memory
while they render: applications that account for all device memory
themselves, or render threads that must never enter the CUDA allocator
because cudaMalloc/cudaFree can synchronise the device and stall a frame.
Its ray queues live in one static device array inside the library, so a
frame may hold at most CT_NOALLOC_MAX_PIXELS (65,536) paths.

The test calls it through the C ABI and compares what it adds to the caller's
accumulation buffer with what ct_render_accumulate adds to a ct_render's
buffer, for two calls in a row: bit for bit in exact math (both run the same
kernels in the same order on the caller's stream), and at the 1e-4 relative
tolerance the frame tests use in fast math (ct_render_accumulate adds each
overlapped frame's private buffer into the job's, a different summation
grouping). The file is named to be collected last."""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu
RTOL = 1e-4


def test_noalloc_matches_allocating_path_twice(gpu_ctx):
    import torch

    from cudatracer_gb300 import _lib, api, scenes

    lib = gpu_ctx.lib
    ts, cam = scenes.terrain_scene(grid=64, spheres=6, sky_size=(128, 64))
    arr = scenes.scene_arrays(ts)
    sc = gpu_ctx.scene(arr, [api.Material(**m) for m in ts.materials], ts.textures, ts.skybox_texture)
    bvh = sc.build_bvh()
    W, H = 160, 120  # 19,200 paths, under the 65,536 limit
    camera = api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"]).to_ct()
    ref_job = api.RenderJob(gpu_ctx, W, H)
    ref_job.reset()
    accum = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
    for exact in (1, 0):
        ref_job.reset()
        accum.zero_()
        for frame in (0, 2):  # two calls in a row, seeds as launchKernels advances them
            p = api.default_params(W, H)
            p.frame_index = frame
            p.exact_math = exact
            before = gpu_ctx.device_bytes
            st = lib.ct_render_accumulate_noalloc(gpu_ctx.h, sc.h, bvh.h, ctypes.byref(camera), ctypes.byref(p),
                                                  accum.data_ptr(), None)
            _lib.check(st, gpu_ctx.h)
            assert gpu_ctx.device_bytes == before  # nothing allocated by the library
            ref_job.accumulate(sc, bvh, api.Camera(W, H, cam["fov"], cam["position"], cam["forward"], cam["up"]), p)
            torch.cuda.synchronize()
            gpu_ctx.check()
            got = accum.cpu().numpy()
            want = ref_job.accum_tensor().cpu().numpy()
            if exact:
                assert np.array_equal(got.view(np.int32), want.view(np.int32)), (
                    f"{(got.view(np.int32) != want.view(np.int32)).any(axis=1).sum()} pixels differ in exact math")
            rel = np.abs(got - want) / np.maximum(np.abs(want), 1e-6)
            assert (rel <= RTOL).all(), f"{(rel > RTOL).any(axis=1).sum()} pixels differ (exact={exact})"
            assert want[:, 3].sum() > 0


def test_noalloc_rejects_frames_over_the_limit(gpu_ctx):
    import torch

    from cudatracer_gb300 import _lib, api, scenes

    s = scenes.sphere_scene(2)
    sc = gpu_ctx.scene(scenes.scene_arrays(s), [api.Material()])
    bvh = sc.build_bvh()
    W, H = 257, 256  # one column over 256 x 256
    accum = torch.zeros((W * H, 4), dtype=torch.float32, device="cuda")
    p = api.default_params(W, H)
    cam = api.Camera(W, H, 60.0, (0.0, 0.0, 3.0)).to_ct()
    st = gpu_ctx.lib.ct_render_accumulate_noalloc(gpu_ctx.h, sc.h, bvh.h, ctypes.byref(cam), ctypes.byref(p),
                                                  accum.data_ptr(), None)
    assert st == 1  # CT_ERR_INVALID_ARGUMENT
    assert b"65536" in gpu_ctx.lib.ct_last_error(gpu_ctx.h)
    assert float(accum.abs().sum()) == 0.0
