"""The oracle's pixel-list renderer (or_render_pixels, used by the bench's
reference arm to sample rows spread over a frame) gives, for every listed
pixel, the bits the per-frame renderer gives when frames are rendered one
after another, and leaves other pixels untouched."""
import numpy as np


def test_render_pixels_equals_frames(orc):
    from cudatracer_gb300 import scenes

    ts, cam = scenes.terrain_scene(grid=32, spheres=3, sky_size=(64, 32))
    arr = scenes.scene_arrays(ts)
    ob = orc.bvh_build(ts.vertices, ts.indices)
    om = orc.pack_materials(ts.materials)
    W, H, frames = 48, 36, [0, 2, 4]
    rows = np.array([0, 7, 19, 35])
    pix = (rows[:, None] * W + np.arange(W)[None, :]).reshape(-1)
    want = np.zeros((W * H, 4), np.float32)
    for r in rows:
        for f in frames:
            orc.render_frames(arr, om, ob["quad"], ob["prims"], cam, W, H, [f], 5, accum=want, exact_math=True,
                              textures=ts.textures, sky_tex=0, pixels=(r * W, (r + 1) * W), nthreads=3)
    got = orc.render_pixels(arr, om, ob["quad"], ob["prims"], cam, W, H, frames, 5, pix, exact_math=True,
                            textures=ts.textures, sky_tex=0, nthreads=5)
    assert np.array_equal(got.view(np.int32), want.view(np.int32))
    other = np.setdiff1d(np.arange(W * H), pix)
    assert (got[other] == 0).all() and got[pix, 3].sum() > 0
