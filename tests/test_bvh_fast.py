"""The traversal-speed quad tree (ct_host_bvh_build_fast / ct_bvh_build_fast)
on the host, no GPU: structure, thread-count independence, and the oracle's
closest and any hits on it against the oracle on the reference's tree (equal
t bit for bit; another primitive only where two triangles tie at that t)."""
import numpy as np
import pytest


def _fast(v, ix, nthreads=4):
    from cudatracer_gb300 import api

    return api.host_bvh_build(v, ix, nthreads, fast=True)


def _check_structure(q, pr, v, ix, max_leaf=4):
    """Every primitive in exactly one leaf of at most max_leaf, every inner
    node reached once, every slot box holding its triangles / child slots."""
    nq = q.shape[0]
    f = q.view(np.float32)
    lo = np.stack([f[:, 0:4], f[:, 8:12], f[:, 16:20]], 2)   # (n, 4, 3) slot minima
    hi = np.stack([f[:, 4:8], f[:, 12:16], f[:, 20:24]], 2)
    ch, cnt = q[:, 24:28], q[:, 28:32]
    assert np.array_equal(np.sort(pr), np.arange(pr.size))
    inner = cnt == -1
    kids = ch[inner]
    assert (kids > 0).all() and (kids < nq).all()
    assert np.array_equal(np.sort(kids), np.arange(1, nq))  # each non-root node reached once
    assert ((cnt == -1) | (cnt > 0)).sum(1).min() >= 1      # no node without children
    leaf = cnt > 0
    assert cnt[leaf].max() <= max_leaf
    cover = np.zeros(pr.size, np.int32)
    tri = v[ix.astype(np.int64)]  # (ntri, 3, 3)
    for (n, s) in zip(*np.nonzero(leaf)):
        first, c = ch[n, s], cnt[n, s]
        cover[first:first + c] += 1
        pts = tri[pr[first:first + c]].reshape(-1, 3)
        assert (pts >= lo[n, s]).all() and (pts <= hi[n, s]).all()
    assert (cover == 1).all()
    for (n, s) in zip(*np.nonzero(inner)):
        c = ch[n, s]
        used = cnt[c] != 0
        assert (lo[c][used] >= lo[n, s]).all() and (hi[c][used] <= hi[n, s]).all()


def _tie_ok(orc, v, ix, o, d, prim, t, eps):
    """The oracle's triangle test alone on `prim` gives exactly t (one-triangle
    tree from ct_host_bvh_build, whose root leaf stays traceable)."""
    from cudatracer_gb300 import api

    tri = v[ix[prim].astype(np.int64)].astype(np.float32)
    q1 = api.host_bvh_build(tri, np.array([[0, 1, 2]], np.uint32), 1)
    h, t1 = orc.trace_closest(q1["quad"], q1["prims"], tri, np.array([[0, 1, 2]], np.uint32), o[None], d[None],
                              eps=eps)
    return h[0] == 0 and t1.view(np.int32)[0] == np.float32(t).view(np.int32)


def _compare_hits(orc, v, ix, o, d, eps=1e-3, any_hit=True, all_ties=False):
    from cudatracer_gb300 import api

    # the reference's tree (ct_host_bvh_build: equal to the oracle's build except
    # that a root leaf stays traceable where the reference's collapse empties it)
    ref = api.host_bvh_build(v, ix, 4)
    fast = _fast(v, ix)
    rh, rt = orc.trace_closest(ref["quad"], ref["prims"], v, ix, o, d, eps=eps)
    fh, ft = orc.trace_closest(fast["quad"], fast["prims"], v, ix, o, d, eps=eps)
    assert np.array_equal(rt.view(np.int32), ft.view(np.int32))
    diff = np.nonzero(rh != fh)[0]
    if not all_ties:  # in a scene of coincident triangles every hit is a tie
        assert diff.size <= max(8, rh.size // 100)
    for i in diff[:64]:
        assert rh[i] >= 0 and fh[i] >= 0 and _tie_ok(orc, v, ix, o[i, :3], d[i, :3], fh[i], ft[i], eps)
    if any_hit:
        rng = np.random.default_rng(11)
        tmax = np.where(rt < 1e30, rt * rng.uniform(0.5, 1.5, size=rt.size), 50.0).astype(np.float32)
        ra = orc.trace_any(ref["quad"], ref["prims"], v, ix, o, d, tmax, eps=eps)
        fa = orc.trace_any(fast["quad"], fast["prims"], v, ix, o, d, tmax, eps=eps)
        assert np.array_equal(ra, fa)
    return (rh >= 0).sum()


@pytest.fixture(scope="module")
def small_terrain():
    from cudatracer_gb300 import scenes

    return scenes.terrain_scene(grid=128, spheres=12, sky_size=(64, 32))


def _view_rays(cam, n, seed):
    rng = np.random.default_rng(seed)
    fw = np.asarray(cam["forward"], np.float64)
    fw /= np.linalg.norm(fw)
    d = fw[None] + rng.uniform(-0.6, 0.6, size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    o = np.tile(np.asarray(cam["position"], np.float32), (n, 1))
    return o.astype(np.float32), d.astype(np.float32)


def test_fast_tree_structure_and_thread_independence(lib, small_terrain):
    from cudatracer_gb300 import scenes

    ts, _ = small_terrain
    for v, ix in ((ts.vertices, ts.indices), (scenes.soup_scene(5000, seed=2).vertices,
                                               scenes.soup_scene(5000, seed=2).indices)):
        a = _fast(v, ix, 1)
        b = _fast(v, ix, 8)
        assert np.array_equal(a["quad"], b["quad"]) and np.array_equal(a["prims"], b["prims"])
        assert a["binary"].shape[0] == 0
        _check_structure(a["quad"], a["prims"], v, ix)
        ref = _fast(v, ix)  # same tree again: the build is deterministic
        assert np.array_equal(ref["quad"], a["quad"])


def test_fast_tree_hits_equal_reference_tree_terrain(lib, orc, small_terrain):
    from cudatracer_gb300 import scenes

    ts, cam = small_terrain
    o, d = _view_rays(cam, 20000, 3)
    assert _compare_hits(orc, ts.vertices, ts.indices, o, d) > 10000
    # incoherent rays from inside the scene's bounds
    rng = np.random.default_rng(4)
    lo, hi = ts.vertices.min(0), ts.vertices.max(0)
    o2 = rng.uniform(lo, hi, size=(20000, 3)).astype(np.float32)
    d2 = rng.normal(size=(20000, 3))
    d2 = (d2 / np.linalg.norm(d2, axis=1, keepdims=True)).astype(np.float32)
    assert _compare_hits(orc, ts.vertices, ts.indices, o2, d2) > 5000


@pytest.mark.parametrize("seed,ntri", [(1, 7), (2, 300), (3, 5000), (4, 40000)])
def test_fast_tree_hits_equal_reference_tree_soups(lib, orc, seed, ntri):
    from cudatracer_gb300 import scenes

    s = scenes.soup_scene(ntri, seed=seed)
    o, d = scenes.incoherent_rays(4096, seed=seed + 10)
    o, d = o[:, :3].copy(), d[:, :3].copy()
    n = _compare_hits(orc, s.vertices, s.indices, o, d, eps=1e-12)
    assert n > 0 or ntri < 100


def test_fast_tree_degenerate_inputs(lib, orc):
    """One triangle (one leaf slot under the root), coincident triangles (every
    hit a tie), and axis-aligned flat quads hit by axis-parallel rays from
    origins on the quads' planes."""
    v1 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    i1 = np.array([[0, 1, 2]], np.uint32)
    h1 = _fast(v1, i1, 1)
    assert h1["quad"].shape[0] == 1 and h1["quad"][0, 28] == 1 and (h1["quad"][0, 29:32] == 0).all()
    o = np.array([[0.2, 0.2, 1.0], [2.0, 2.0, 1.0]], np.float32)
    d = np.array([[0, 0, -1.0], [0, 0, -1.0]], np.float32)
    # the reference's collapse empties a root leaf (nothing to compare with)
    h, t = orc.trace_closest(h1["quad"], h1["prims"], v1, i1, o, d)
    assert h.tolist() == [0, -1] and t[0] == np.float32(1.0)
    v = np.tile(v1, (192, 1))
    ix = np.arange(v.shape[0], dtype=np.uint32).reshape(-1, 3)
    f = _fast(v, ix, 2)
    _check_structure(f["quad"], f["prims"], v, ix)
    rng = np.random.default_rng(0)
    o2 = np.concatenate([rng.uniform(0, 0.5, size=(256, 2)), np.ones((256, 1))], 1).astype(np.float32)
    d2 = np.tile(np.array([[0, 0, -1.0]], np.float32), (256, 1))
    _compare_hits(orc, v, ix, o2, d2, any_hit=False, all_ties=True)
    # a stack of flat axis-aligned quads, 2 triangles each, at y = k
    quads = []
    for k in range(40):
        x0, z0 = rng.uniform(-5, 5, size=2)
        quads.append([[x0, k, z0], [x0 + 1, k, z0], [x0 + 1, k, z0 + 1], [x0, k, z0 + 1]])
    vq = np.asarray(quads, np.float32).reshape(-1, 3)
    iq = np.concatenate([[[4 * k, 4 * k + 1, 4 * k + 2], [4 * k, 4 * k + 2, 4 * k + 3]] for k in range(40)]).astype(np.uint32)
    n = 4096
    oq = rng.uniform(-5, 6, size=(n, 3)).astype(np.float32)
    oq[:, 1] = rng.integers(0, 40, size=n).astype(np.float32) + np.where(rng.random(n) < 0.5, 0.0, 0.5)
    dq = np.zeros((n, 3), np.float32)
    dq[np.arange(n), rng.integers(0, 3, size=n)] = rng.choice([-1.0, 1.0], size=n)
    dq[: n // 4] = rng.normal(size=(n // 4, 3))
    dq /= np.linalg.norm(dq, axis=1, keepdims=True)
    _compare_hits(orc, vq, iq, oq, dq)


def test_fast_tree_tests_fewer_triangles_per_ray(lib, orc, small_terrain):
    """Fast-math frames on the small terrain: fewer node visits plus triangle
    tests per extension ray on the fast tree, and the same accumulation (the
    hits are equal)."""
    from cudatracer_gb300 import scenes

    ts, cam = small_terrain
    arr = scenes.scene_arrays(ts)
    mats = orc.pack_materials(ts.materials)
    W, H = 160, 96
    out = {}
    for name, tree in (("ref", orc.bvh_build(ts.vertices, ts.indices)), ("fast", _fast(ts.vertices, ts.indices))):
        orc.set_full_sort(True)
        orc.work_read(reset=True)
        acc = orc.render_frames(arr, mats, tree["quad"], tree["prims"], cam, W, H, [0], 5, exact_math=False,
                                textures=ts.textures, sky_tex=0)
        w = orc.work_read(reset=True)
        orc.set_full_sort(False)
        out[name] = (w["ext_nodes"] / w["ext_rays"], w["ext_tris"] / w["ext_rays"], acc)
    # 1.6-unit triangles here, so the reference's fixed box padding costs little;
    # on the 0.2-unit triangles of a 1024-grid terrain the fast tree tests 22 % fewer
    assert out["fast"][1] <= out["ref"][1]
    assert out["fast"][0] + out["fast"][1] < 0.98 * (out["ref"][0] + out["ref"][1])
    a, b = out["ref"][2], out["fast"][2]
    rel = np.abs(a - b) / np.maximum(np.abs(a), 1e-6)
    assert (rel > 1e-4).any(axis=1).mean() < 1e-3


def test_fast_build_rejects_bad_input(lib):
    from cudatracer_gb300 import _lib

    v = np.array([[0, 0, 0], [1, 0, 0], [0, np.nan, 0]], np.float32)
    with pytest.raises(_lib.CTError):
        _fast(v, np.array([[0, 1, 2]], np.uint32))
    v[2, 1] = 1.0
    with pytest.raises(_lib.CTError):
        _fast(v, np.array([[0, 1, 3]], np.uint32))


def _fma_slab_hits(lo, hi, o, d):
    """The fast-math slab test of the traversal kernels for one box per ray:
    inv = 1/d and nox = -o * inv in float32, each plane fmaf(b, inv, nox)
    (emulated: the float64 product is exact, the sum is rounded to float64 and
    then to float32), hit when tmax > 0 and tmin <= tmax."""
    inv = (np.float32(1.0) / d.astype(np.float32)).astype(np.float32)
    nox = (-o.astype(np.float32) * inv).astype(np.float32)
    t1 = (lo.astype(np.float64) * inv + nox).astype(np.float32)
    t2 = (hi.astype(np.float64) * inv + nox).astype(np.float32)
    tmin = np.minimum(t1, t2).max(axis=1)
    tmax = np.maximum(t1, t2).min(axis=1)
    return (tmax > 0) & (tmin <= tmax)


@pytest.mark.parametrize("which", ["terrain", "soup"])
def test_fast_padding_keeps_grazing_hits(lib, small_terrain, which):
    """Rays from origins up to 10 M away (M: largest coordinate magnitude) aimed
    just inside a triangle next to the vertex that defines a face of its box:
    the leaf slot box that holds the triangle passes the kernels' fast-math
    slab test for every ray; without padding the same rays lose boxes."""
    from cudatracer_gb300 import scenes

    if which == "terrain":
        v, ix = small_terrain[0].vertices, small_terrain[0].indices
    else:
        s = scenes.soup_scene(20000, seed=6)
        v, ix = s.vertices, s.indices
    f = _fast(v, ix)
    q, pr = f["quad"], f["prims"]
    qf = q.view(np.float32)
    box_of = np.zeros((pr.size, 2, 3), np.float32)
    for n, sl in zip(*np.nonzero(q[:, 28:32] > 0)):
        first, c = q[n, 24 + sl], q[n, 28 + sl]
        box_of[pr[first:first + c], 0] = qf[n, [sl, 8 + sl, 16 + sl]]
        box_of[pr[first:first + c], 1] = qf[n, [4 + sl, 12 + sl, 20 + sl]]
    M = float(np.abs(v).max())
    rng = np.random.default_rng(8)
    n = 40000
    tri = rng.integers(0, ix.shape[0], size=n)
    P = v[ix[tri].astype(np.int64)].astype(np.float64)  # (n, 3 vertices, 3)
    axis = rng.integers(0, 3, size=n)
    side = rng.integers(0, 2, size=n)
    key = np.where(side[:, None] == 0, P[np.arange(n), :, axis], -P[np.arange(n), :, axis])
    k = key.argmin(axis=1)  # the vertex that defines the box face on (axis, side)
    e = 1e-4
    target = (1 - 2 * e) * P[np.arange(n), k] + e * P[np.arange(n), (k + 1) % 3] + e * P[np.arange(n), (k + 2) % 3]
    for R in (0.5 * M, 2.0 * M, 10.0 * M):
        u = rng.normal(size=(n, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        o = (target + R * u).astype(np.float32)
        d = target - o.astype(np.float64)
        d = (d / np.linalg.norm(d, axis=1, keepdims=True)).astype(np.float32)
        ok = _fma_slab_hits(box_of[tri, 0], box_of[tri, 1], o, d)
        assert ok.all(), (R / M, int((~ok).sum()))
    # the check has teeth: exact (unpadded) triangle boxes lose some of these rays
    lo, hi = P.min(axis=1).astype(np.float32), P.max(axis=1).astype(np.float32)
    assert (~_fma_slab_hits(lo, hi, o, d)).sum() > 0


def test_fast_tree_is_order_deterministic(lib):
    """What lets the device build reproduce the host tree byte for byte: no box
    coordinate is a negative zero (min/max unions then do not depend on the
    order in which boxes meet), and the tree is a function of the input alone:
    the same bytes for every thread count, also for coincident triangles (ranges
    halved as they lie) and for a scene at the origin (no padding)."""
    rng = np.random.default_rng(3)
    z = np.zeros((60, 3), np.float32)
    z[::2, 0] = -0.0
    z[1::3, 1] = -0.0
    v1 = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    soup = rng.normal(size=(3000, 3)).astype(np.float32)
    soup[::5] *= -0.0
    for v, ix in ((z, np.arange(60, dtype=np.uint32).reshape(-1, 3)),
                  (v1, np.tile(np.array([[0, 1, 2]], np.uint32), (300, 1))),
                  (soup, np.arange(3000, dtype=np.uint32).reshape(-1, 3))):
        trees = [_fast(v, ix, t) for t in (1, 3, 8)]
        for t in trees[1:]:
            assert np.array_equal(t["quad"], trees[0]["quad"]) and np.array_equal(t["prims"], trees[0]["prims"])
        bounds = trees[0]["quad"][:, :24].view(np.uint32)
        assert not (bounds == 0x80000000).any(), "a negative zero in a node box"
