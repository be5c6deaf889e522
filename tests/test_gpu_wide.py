"""The 8-wide quantised BVH (ct_bvh_build_wide) and its queries.

Structure (exported nodes, checked on the host): every triangle in exactly
one leaf slot, every node reached once, and every dequantised child box
containing all triangles below it (the outward rounding). Queries: closest
hits and occlusion equal the FP64 watertight oracle (oracle/ct_fp64.cpp
fp64_trace) ray for ray — 0 id mismatches, 0 lost hits, t within 1e-5
relative — on incoherent soup rays, rays aimed at vertices and edge
midpoints, rays through the vertices of a closed mesh, and axis-parallel rays."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(gpu_ctx, v, ix):
    from cudatracer_gb300 import api

    v = np.ascontiguousarray(v, np.float32)
    ix = np.ascontiguousarray(ix, np.uint32)
    arr = {"vertices": v, "normals": np.tile(np.array([[0, 0, 1]], np.float32), (v.shape[0], 1)), "indices": ix}
    return gpu_ctx.scene(arr, [api.Material()])


def _decode(nodes):
    b = np.ascontiguousarray(nodes).view(np.uint8).reshape(-1, 80)
    p = b[:, 0:12].copy().view(np.float32).reshape(-1, 3)
    e = b[:, 12:15].astype(np.int64)
    scale = np.ldexp(1.0, e - 127)
    child_base = b[:, 16:20].copy().view(np.uint32).reshape(-1)
    prim_base = b[:, 20:24].copy().view(np.uint32).reshape(-1)
    meta = b[:, 24:32]
    qlo = b[:, 32:56].reshape(-1, 3, 8).astype(np.float64)
    qhi = b[:, 56:80].reshape(-1, 3, 8).astype(np.float64)
    # fma(s, q, p) rounded once: s*q + p is exact in float64 here
    lo = (scale[:, :, None] * qlo + p[:, :, None].astype(np.float64)).astype(np.float32)
    hi = (scale[:, :, None] * qhi + p[:, :, None].astype(np.float64)).astype(np.float32)
    return dict(meta=meta, child_base=child_base, prim_base=prim_base, lo=lo, hi=hi, imask=b[:, 15])


def _check_structure(v, ix, nodes, prims):
    n = ix.shape[0]
    assert np.array_equal(np.sort(prims), np.arange(n))
    D = _decode(nodes)
    nn = nodes.shape[0]
    seen_node = np.zeros(nn, np.int64)
    seen_tri = np.zeros(n, np.int64)
    tri_lo = v[ix].min(axis=1)
    tri_hi = v[ix].max(axis=1)
    # bounds of everything below each node, children before parents
    order, st = [], [0]
    seen_node[0] = 1
    while st:
        k = st.pop()
        order.append(k)
        for i in range(8):
            m = int(D["meta"][k, i])
            if m & 0x80:
                c = int(D["child_base"][k]) + (m & 7)
                assert c < nn
                seen_node[c] += 1
                st.append(c)
                assert D["imask"][k] & (1 << i)
    assert (seen_node == 1).all()
    sub_lo = np.full((nn, 3), np.inf, np.float32)
    sub_hi = np.full((nn, 3), -np.inf, np.float32)
    for k in reversed(order):
        for i in range(8):
            m = int(D["meta"][k, i])
            if m == 0:
                continue
            blo, bhi = D["lo"][k, :, i], D["hi"][k, :, i]
            if m & 0x80:
                c = int(D["child_base"][k]) + (m & 7)
                clo, chi = sub_lo[c], sub_hi[c]
            else:
                cnt, off = m >> 5, m & 31
                assert 1 <= cnt <= 3
                slots = np.arange(cnt) + int(D["prim_base"][k]) + off
                seen_tri[slots] += 1
                pr = prims[slots]
                clo, chi = tri_lo[pr].min(axis=0), tri_hi[pr].max(axis=0)
            assert (blo <= clo).all() and (bhi >= chi).all(), (k, i)
            sub_lo[k] = np.minimum(sub_lo[k], clo)
            sub_hi[k] = np.maximum(sub_hi[k], chi)
    assert (seen_tri == 1).all()


@pytest.mark.parametrize("ntri", [1, 2, 3, 4, 5, 17, 300, 5000, 60000])
def test_wide_structure_soups(gpu_ctx, ntri):
    from cudatracer_gb300 import _lib, scenes

    s = scenes.soup_scene(ntri, seed=100 + ntri)
    b = _scene(gpu_ctx, s.vertices, s.indices).build_bvh_wide()
    nodes, prims = b.export(_lib.CT_BVH_WIDE8_Q8)
    _check_structure(s.vertices, s.indices, nodes, prims)
    inf = b.info()
    assert inf["max_leaf_size"] == 3 and inf["quad_node_count"] == nodes.shape[0]


def test_wide_structure_sphere_and_terrain(gpu_ctx):
    from cudatracer_gb300 import _lib, scenes

    for s in (scenes.sphere_scene(5), scenes.terrain_scene(grid=128, spheres=8, sky_size=(16, 8))[0]):
        b = _scene(gpu_ctx, s.vertices, s.indices).build_bvh_wide()
        nodes, prims = b.export(_lib.CT_BVH_WIDE8_Q8)
        _check_structure(s.vertices, s.indices, nodes, prims)


def _compare_closest(gpu_ctx, orc, v, ix, O, D):
    import torch

    wb = _scene(gpu_ctx, v, ix).build_bvh_wide()
    ob = orc.bvh_build(v, ix)
    h, t = wb.trace_closest(torch.from_numpy(O).cuda(), torch.from_numpy(D).cuda())
    gpu_ctx.check()
    h, t = h.cpu().numpy(), t.cpu().numpy()
    ho, to = orc.trace_fp64(v, ix, ob["quad"], ob["prims"], O, D)
    mism = int((h != ho).sum())
    lost = int(((ho >= 0) & (h < 0)).sum())
    both = (h >= 0) & (h == ho)
    rel = np.abs(t[both].astype(np.float64) - to[both]) / to[both] if both.any() else np.zeros(1)
    return wb, h, ho, mism, lost, float(rel.max())


def test_wide_closest_equals_fp64_oracle(gpu_ctx, orc):
    from cudatracer_gb300 import scenes

    s = scenes.soup_scene(200000, seed=31)
    o, d = scenes.incoherent_rays(1 << 18, seed=32)
    rng = np.random.default_rng(33)
    # rays aimed at vertices and edge midpoints: the near-edge cases
    tri = rng.integers(0, 200000, 20000)
    P = s.vertices[s.indices[tri]]
    w = rng.integers(0, 3, 20000)
    tgt = np.where((w == 0)[:, None], P[:, 0], np.where((w == 1)[:, None], (P[:, 0] + P[:, 1]) * 0.5, P[:, 2]))
    o2 = np.zeros((20000, 4), np.float32)
    o2[:, :3] = rng.uniform(0, 1, (20000, 3))
    d2 = np.zeros((20000, 4), np.float32)
    dv = tgt - o2[:, :3]
    d2[:, :3] = dv / np.linalg.norm(dv, axis=1, keepdims=True)
    d2[:, 3] = 1e34
    O, D = np.concatenate([o, o2]), np.concatenate([d, d2])
    wb, h, ho, mism, lost, rel = _compare_closest(gpu_ctx, orc, s.vertices, s.indices, O, D)
    assert (ho >= 0).sum() > 10000
    assert mism == 0 and lost == 0, (mism, lost)
    assert rel <= 1e-5, rel
    st = wb.wide_stats(reset=True)
    assert st["rays"] == O.shape[0]
    assert st["fp64_retests"] > 0  # the aimed rays do need the FP64 arbiter


def test_wide_any_hit_equals_fp64_oracle(gpu_ctx, orc):
    import torch

    from cudatracer_gb300 import scenes

    s = scenes.soup_scene(100000, seed=41)
    o, d = scenes.incoherent_rays(1 << 17, seed=42)
    ob = orc.bvh_build(s.vertices, s.indices)
    h, t = orc.trace_fp64(s.vertices, s.indices, ob["quad"], ob["prims"], o, d)
    rng = np.random.default_rng(43)
    # finite ranges around the closest hit: just before, just after, and random
    d[:, 3] = np.where(h >= 0, t * rng.choice([0.999999, 1.000001, 3.0], size=h.shape), rng.uniform(0.05, 2.0, h.shape))
    occ_ref, _ = orc.trace_fp64(s.vertices, s.indices, ob["quad"], ob["prims"], o, d, any_hit=True)
    wb = _scene(gpu_ctx, s.vertices, s.indices).build_bvh_wide()
    occ = wb.trace_any(torch.from_numpy(o).cuda(), torch.from_numpy(d).cuda())
    gpu_ctx.check()
    occ = occ.cpu().numpy()
    assert np.array_equal(occ.astype(bool), occ_ref >= 0)
    assert occ.sum() > 100


def test_wide_closed_mesh_is_watertight(gpu_ctx, orc):
    """Rays from inside a closed icosphere through its vertices and edge
    midpoints: every one hits (no crack), and the hit equals FP64's."""
    from cudatracer_gb300 import scenes

    v, f = scenes.icosphere(4)
    v = v.astype(np.float32)
    f = f.astype(np.uint32)
    edges = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]])
    mid = (v[edges[:, 0]] + v[edges[:, 1]]) * 0.5
    tg = np.concatenate([v, mid]).astype(np.float64)
    origins = [np.zeros(3), np.array([0.1, -0.05, 0.02])]
    for c in origins:
        dv = tg - c
        O = np.zeros((tg.shape[0], 4), np.float32)
        O[:, :3] = c
        D = np.zeros_like(O)
        D[:, :3] = dv / np.linalg.norm(dv, axis=1, keepdims=True)
        D[:, 3] = 1e34
        _, h, ho, mism, lost, rel = _compare_closest(gpu_ctx, orc, v, f, O, D)
        assert (h >= 0).all() and (ho >= 0).all()
        assert mism == 0 and rel <= 1e-5


def test_wide_axis_parallel_rays(gpu_ctx, orc):
    from cudatracer_gb300 import scenes

    s = scenes.soup_scene(50000, seed=51)
    rng = np.random.default_rng(52)
    n = 60000
    O = np.zeros((n, 4), np.float32)
    O[:, :3] = rng.uniform(0, 1, (n, 3))
    D = np.zeros((n, 4), np.float32)
    ax = np.arange(n) % 3
    D[np.arange(n), ax] = np.where(np.arange(n) % 2, 1.0, -1.0)
    D[:, 3] = 1e34
    # half of them start exactly on a vertex coordinate plane of some triangle
    tri = rng.integers(0, 50000, n // 2)
    O[: n // 2, (ax[: n // 2] + 1) % 3] = s.vertices[s.indices[tri, 0], (ax[: n // 2] + 1) % 3]
    _, h, ho, mism, lost, rel = _compare_closest(gpu_ctx, orc, s.vertices, s.indices, O, D)
    assert mism == 0 and lost == 0 and rel <= 1e-5


def test_frames_on_the_wide_tree(gpu_ctx, orc):
    """Frames traced through the wide tree use the reference's triangle test:
    with exact math they match the oracle (traced through the quad tree) up to
    exact t ties, and fast-math frames match the quad tree's fast frames."""
    from cudatracer_gb300 import api, scenes

    ts, cam = scenes.terrain_scene(grid=128, spheres=12, sky_size=(256, 128))
    arr = scenes.scene_arrays(ts)
    sc = gpu_ctx.scene(arr, [api.Material(**m) for m in ts.materials], ts.textures, ts.skybox_texture)
    qb, wb = sc.build_bvh_device(), sc.build_bvh_wide()
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

    a = render(wb, True)
    ob = orc.bvh_build(ts.vertices, ts.indices)
    o = orc.render_frames(arr, orc.pack_materials(ts.materials), ob["quad"], ob["prims"], cam, W, H, [0, 2], 5,
                          exact_math=True, textures=ts.textures, sky_tex=0)
    rel = np.abs(a - o) / np.maximum(np.abs(o), 1e-6)
    assert (rel > 1e-4).any(axis=1).mean() < 1e-3
    assert (a.view(np.int32) == o.view(np.int32)).all(axis=1).mean() >= 0.999
    f_w, f_q = render(wb, False), render(qb, False)
    rel = np.abs(f_w - f_q) / np.maximum(np.abs(f_q), 1e-6)
    assert (rel > 1e-4).any(axis=1).mean() < 1e-3
