"""The CPU oracle against the reference's own answers (tests/golden, made by
tests/golden/make_golden.py from the reference's host code)."""
import ctypes
import hashlib

import numpy as np
import pytest

P = ctypes.c_void_p


def _p(a):
    return a.ctypes.data_as(P)


def test_rng_streams(orc, kat):
    L = orc.lib()
    L.or_wang_hash.restype = ctypes.c_uint32
    L.or_wang_hash.argtypes = [ctypes.c_uint32]
    got = np.array([L.or_wang_hash(int(s)) for s in kat["wang_in"]], np.uint32)
    assert np.array_equal(got, kat["wang_out"])
    L.or_random_stream.argtypes = [ctypes.c_uint32, ctypes.c_int, P, P]
    for s, ii, ff in zip(kat["stream_seeds"], kat["stream_int"], kat["stream_float"]):
        gi = np.zeros(64, np.uint32)
        gf = np.zeros(64, np.float32)
        L.or_random_stream(int(s), 64, _p(gi), _p(gf))
        assert np.array_equal(gi, ii)
        assert np.array_equal(gf.view(np.int32), ff.view(np.int32))


def test_moller_trumbore(orc, kat):
    L = orc.lib()
    L.or_tri_intersect.argtypes = [P, P, P, P, P, P, ctypes.c_float]
    n = kat["mt_hit"].shape[0]
    hits = np.zeros(n, np.int32)
    tout = kat["mt_tin"].copy()
    for i in range(n):
        t = tout[i:i + 1]
        hits[i] = L.or_tri_intersect(_p(kat["mt_org"][i]), _p(kat["mt_dir"][i]), _p(t), _p(kat["mt_p0"][i]),
                                     _p(kat["mt_p1"][i]), _p(kat["mt_p2"][i]), 1e-3)
    assert np.array_equal(hits, kat["mt_hit"])
    assert np.array_equal(tout.view(np.int32), kat["mt_tout"].view(np.int32))
    assert 0 < hits.sum() < n  # both outcomes exercised


def test_quad_slab(orc, kat):
    L = orc.lib()
    L.or_quad_intersect.argtypes = [P, P, P, ctypes.c_float, P, P]
    m = kat["slab_t"].shape[0]
    tm = np.zeros((m, 4), np.int32)
    rs = np.zeros((m, 4), np.int32)
    for i in range(m):
        L.or_quad_intersect(_p(kat["slab_nodes"][i]), _p(kat["slab_org"][i]), _p(kat["slab_inv"][i]),
                            float(kat["slab_t"][i]), _p(tm[i]), _p(rs[i]))
    assert np.array_equal(tm, kat["slab_tmini"])
    assert np.array_equal(rs, kat["slab_res"])


def test_triangle_helpers(orc, kat):
    L = orc.lib()
    L.or_bary.argtypes = [P, P, P, P, P, P]
    L.or_area.restype = ctypes.c_float
    L.or_area.argtypes = [P, P, P]
    L.or_random_point.argtypes = [P, P, P, ctypes.c_float, ctypes.c_float, P]
    k = kat["area_out"].shape[0]
    bo = np.zeros((k, 3), np.float32)
    rp = np.zeros((k, 3), np.float32)
    ar = np.zeros(k, np.float32)
    for i in range(k):
        L.or_bary(_p(kat["bary_p"][i]), _p(kat["bary_n"][i]), _p(kat["tri0"][i]), _p(kat["tri1"][i]),
                  _p(kat["tri2"][i]), _p(bo[i]))
        ar[i] = L.or_area(_p(kat["tri0"][i]), _p(kat["tri1"][i]), _p(kat["tri2"][i]))
        L.or_random_point(_p(kat["tri0"][i]), _p(kat["tri1"][i]), _p(kat["tri2"][i]), float(kat["rp_r1"][i]),
                          float(kat["rp_r2"][i]), _p(rp[i]))
    assert np.array_equal(bo.view(np.int32), kat["bary_out"].view(np.int32))
    assert np.array_equal(ar.view(np.int32), kat["area_out"].view(np.int32), equal_nan=False) or \
        np.allclose(ar, kat["area_out"], equal_nan=True, rtol=0, atol=0)
    assert np.array_equal(rp.view(np.int32), kat["rp_out"].view(np.int32))


def test_frames_and_samples(orc, kat):
    L = orc.lib()
    L.or_tangent2world.argtypes = [P, P, P]
    L.or_local_space.argtypes = [P, P, P]
    L.or_cos_weighted.argtypes = [ctypes.c_float, ctypes.c_float, ctypes.c_int, P]
    k = kat["t2w_out"].shape[0]
    to = np.zeros((k, 3), np.float32)
    lT = np.zeros((k, 3), np.float32)
    lB = np.zeros((k, 3), np.float32)
    cw = np.zeros((k, 3), np.float32)
    for i in range(k):
        L.or_tangent2world(_p(kat["t2w_v"][i]), _p(kat["t2w_n"][i]), _p(to[i]))
        L.or_local_space(_p(kat["t2w_n"][i]), _p(lT[i]), _p(lB[i]))
        L.or_cos_weighted(float(kat["rp_r1"][i]), float(kat["rp_r2"][i]), 0, _p(cw[i]))
    assert np.array_equal(to.view(np.int32), kat["t2w_out"].view(np.int32))
    assert np.array_equal(lT.view(np.int32), kat["ls_T"].view(np.int32))
    assert np.array_equal(lB.view(np.int32), kat["ls_B"].view(np.int32))
    # sin/cos come from the C library on both sides here; allow one ulp
    assert np.allclose(cw, kat["cw_out"], rtol=2e-7, atol=1e-7)


def test_sample_bsdf(orc, kat):
    L = orc.lib()
    L.or_sample_bsdf.argtypes = [P, ctypes.c_float, P, P, P, ctypes.c_float, ctypes.c_float, ctypes.c_int, P, P, P, P]
    k = kat["bsdf_pdf"].shape[0]
    f = np.zeros((k, 3), np.float32)
    wo = np.zeros((k, 3), np.float32)
    pdf = np.zeros(k, np.float32)
    typ = np.zeros(k, np.int32)
    for i in range(k):
        L.or_sample_bsdf(_p(kat["bsdf_col"][i]), float(kat["bsdf_rough"][i]), _p(kat["bsdf_iN"][i]),
                         _p(kat["bsdf_N"][i]), _p(kat["bsdf_wi"][i]), float(kat["rp_r1"][i]), float(kat["rp_r2"][i]),
                         0, _p(f[i]), _p(wo[i]), _p(pdf[i:i + 1]), _p(typ[i:i + 1]))
    assert np.array_equal(typ, kat["bsdf_type"])
    assert np.allclose(pdf, kat["bsdf_pdf"], rtol=1e-6, atol=1e-7)
    assert np.allclose(wo, kat["bsdf_wo"], rtol=1e-6, atol=1e-6)
    assert np.allclose(f, kat["bsdf_f"], rtol=1e-6, atol=1e-7)
    mirror = kat["bsdf_rough"] < 0.1
    # the mirror branch has no transcendental: bit exact
    assert np.array_equal(wo[mirror].view(np.int32), kat["bsdf_wo"][mirror].view(np.int32))


def test_camera_rays(orc, kat):
    from cudatracer_gb300 import scenes

    hor, ver = orc.camera_basis((0, 0, -1), (0, 1, 0), float(kat["cam_fov"]), int(kat["cam_w"]), int(kat["cam_h"]))
    L = orc.lib()
    assert np.float32(L.or_plane_distance(float(kat["cam_fov"]))) == kat["cam_plane"]
    # pinhole_rays restates Camera::generateRay (square-aspect form is exact)
    o, d = scenes.pinhole_rays(int(kat["cam_w"]), int(kat["cam_h"]), float(kat["cam_fov"]), tuple(kat["cam_pos"]))
    assert np.array_equal(o, kat["cam_org"])
    assert np.array_equal(d.view(np.int32), kat["cam_dir"].view(np.int32))


def test_bvh_matches_reference(orc):
    """Byte-identical quad tree, primitive order and binary topology."""
    from cudatracer_gb300 import scenes
    from tests.golden.make_golden import canonical_binary

    for name in ("sphere_s5.npz", "sphere_c1.npz"):
        from tests.conftest import golden

        g = golden(name)
        s = scenes.sphere_scene(int(g["subdivisions"]))
        v = g["vertices"] if "vertices" in g else s.vertices
        if "vertices_sha" in g:
            assert hashlib.sha256(v.tobytes()).hexdigest() == str(g["vertices_sha"])
        b = orc.bvh_build(v, s.indices)
        assert b["quad"].shape[0] == int(g["quad_count"])
        assert hashlib.sha256(b["quad"].tobytes()).hexdigest() == str(g["quad_sha"])
        assert hashlib.sha256(b["prims"].tobytes()).hexdigest() == str(g["prims_sha"])
        assert hashlib.sha256(canonical_binary(b["binary"])).hexdigest() == str(g["binary_canonical_sha"])


def test_traversal_matches_reference(orc, c1):
    g = c1["g"]
    b = orc.bvh_build(c1["vertices"], c1["indices"])
    o = np.zeros_like(g["cam_dirs"])
    o[:, 2] = 3.0
    hit, t = orc.trace_closest(b["quad"], b["prims"], c1["vertices"], c1["indices"], o, g["cam_dirs"])
    assert np.array_equal(hit, g["hit"])
    assert np.array_equal(t.view(np.int32), g["t"].view(np.int32))
    hit, t = orc.trace_closest(b["quad"], b["prims"], c1["vertices"], c1["indices"], g["inc_org"], g["inc_dir"])
    assert np.array_equal(hit, g["inc_hit"])
    assert np.array_equal(t.view(np.int32), g["inc_t"].view(np.int32))
    # the reference's binary traversal finds the same closest hits up to exact ties
    hb, tb = orc.trace_closest_binary(b["binary"], b["prims"], c1["vertices"], c1["indices"], o, g["cam_dirs"])
    assert np.array_equal(tb.view(np.int32), g["t"].view(np.int32))
    assert (hb != g["hit"]).sum() <= 8


def test_fp64_microfacet_matches_reference(orc, kat):
    """The FP64 oracle's microfacet sampling and Smith G1 against the reference's
    Material::sample / Material::evaluate (src/Core/Material.cuh:175-215) for
    isotropic alphas: visible-normal sampling for Beckmann/GGX, full-distribution
    sampling for Trowbridge-Reitz, and G1(Lambda(wo)) as the visible-mode pdf."""
    L = orc.fp64()
    tv, al, inp, out, pdf = (kat["mf_type_vis"], kat["mf_alpha"], kat["mf_in"], kat["mf_out"], kat["mf_pdf"])
    m = np.zeros(3, np.float64)
    g1 = np.zeros(1, np.float64)
    checked_m = checked_g = 0
    for (typ, vis), (ax, ay), row, ref_m, ref_pdf in zip(tv, al, inp, out, pdf):
        if ax != ay:
            continue
        wi = np.ascontiguousarray(row[0:3], np.float32)
        wo = np.ascontiguousarray(row[5:8], np.float32)
        L.fp64_microfacet(int(typ), float(ax), _p(wi), float(row[3]), float(row[4]), _p(wo), _p(m), _p(g1))
        if vis == 1 or typ in (6, 9):
            assert np.allclose(m, ref_m, rtol=2e-3, atol=2e-3), (typ, vis, m, ref_m)
            checked_m += 1
        if vis == 1:
            assert abs(g1[0] - ref_pdf) <= 1e-5 * max(1.0, abs(ref_pdf)), (typ, g1[0], ref_pdf)
            checked_g += 1
    assert checked_m >= 100 and checked_g >= 60
    for r, a in zip(kat["r2a_in"], kat["r2a_out"]):
        assert abs(L.fp64_roughness_to_alpha(float(r)) - a) <= 1e-5


@pytest.mark.parametrize("w,h", [(16, 12)])
def test_frame_oracle_runs_and_is_deterministic(orc, w, h):
    from cudatracer_gb300 import scenes

    ts, cam = scenes.terrain_scene(grid=32, spheres=3, sky_size=(64, 32))
    a = scenes.scene_arrays(ts)
    b = orc.bvh_build(ts.vertices, ts.indices)
    mats = orc.pack_materials(ts.materials)
    acc1 = orc.render_frames(a, mats, b["quad"], b["prims"], cam, w, h, [0, 2], 5, textures=ts.textures, sky_tex=0)
    acc2 = orc.render_frames(a, mats, b["quad"], b["prims"], cam, w, h, [0, 2], 5, textures=ts.textures, sky_tex=0,
                             nthreads=1)
    assert np.array_equal(acc1, acc2)
    assert np.isfinite(acc1).all() and acc1[:, 3].min() >= 0
    assert acc1[:, :3].sum() > 0


def test_full_sort_child_order_changes_work_not_results(orc):
    """The roofline counts traversal work in the child order fast-math GPU frames
    use (a full distance sort instead of the reference's partial network). The
    order must not change a frame (the nearest hit does not depend on it here),
    only the node-visit and triangle-test counts."""
    from cudatracer_gb300 import scenes

    ts, cam = scenes.terrain_scene(grid=96, spheres=12, sky_size=(64, 32))
    a = scenes.scene_arrays(ts)
    b = orc.bvh_build(ts.vertices, ts.indices)
    mats = orc.pack_materials(ts.materials)
    out = {}
    try:
        for full in (False, True):
            orc.set_full_sort(full)
            orc.work_read(reset=True)
            acc = orc.render_frames(a, mats, b["quad"], b["prims"], cam, 48, 32, [0], 6, textures=ts.textures,
                                    sky_tex=0)
            out[full] = (acc, orc.work_read(reset=True))
    finally:
        orc.set_full_sort(False)
    (a0, w0), (a1, w1) = out[False], out[True]
    assert np.array_equal(a0.view(np.int32), a1.view(np.int32))
    assert w0["ext_rays"] == w1["ext_rays"] > 0
    assert (w0["ext_nodes"], w0["ext_tris"]) != (w1["ext_nodes"], w1["ext_tris"])
