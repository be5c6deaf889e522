"""Generate the golden fixtures in tests/golden/ from the REFERENCE's own code.

The reference (meirbon/CudaTracer) ships no tests, fixtures or known answers,
so the pins are produced here by running its host code, compiled from its
sources by oracle/ref_build.py (oracle/_ref/libctref.so). Run in a checkout
where the reference is available:

    python tests/golden/make_golden.py

Outputs (small .npz files, committed):
  kat_math.npz   per-function known answers: WangHash/xorshift streams,
                 Moller-Trumbore, the quad-node slab test, barycentrics, area,
                 light-sample points, Tangent2World, cosine-weighted samples,
                 SampleBSDF, FresnelDielectricExact, RoughnessToAlpha,
                 microfacet sample/pdf, Camera::generateRay rays.
  sphere_c1.npz  the 81,920-triangle sphere (vertices as generated) with the
                 reference's quad-BVH digest, binary-tree digest and its
                 closest hits (ids, t) for the 256x256 pinhole rays and 4,096
                 incoherent rays.
  sphere_s5.npz  the same for the 20,480-triangle sphere (digests only).
"""
from __future__ import annotations

import ctypes
import hashlib
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import oracle  # noqa: E402
from cudatracer_gb300 import scenes  # noqa: E402

P = ctypes.c_void_p


def _p(a):
    return a.ctypes.data_as(P)


def canonical_binary(nodes: np.ndarray) -> bytes:
    """Binary BVH bytes renumbered in depth-first pair order (the reference's
    thread-pool build numbers nodes by thread timing; topology is fixed)."""
    f = nodes.view(np.float32)
    out = []

    def rec(i):
        n = nodes[i]
        if n[7] > -1:
            out.append(np.concatenate([f[i, 0:3], f[i, 4:7]]).tobytes() + n[[3, 7]].tobytes())
            return
        out.append(np.concatenate([f[i, 0:3], f[i, 4:7]]).tobytes() + b"inner")
        rec(int(n[3]))
        rec(int(n[3]) + 1)

    sys.setrecursionlimit(100000)
    rec(0)
    return b"".join(out)


def digest(b: bytes) -> str:
    return hashlib.sha256(b).hexdigest()


def ref_build(verts, idx, nthreads=8):
    R = oracle.ref()
    h = R.ctref_build(_p(verts), verts.shape[0], _p(idx), idx.shape[0], nthreads)
    nb, nq = R.ctref_bvh_count(h), R.ctref_mbvh_count(h)
    b = np.zeros((nb, 8), np.int32)
    q = np.zeros((nq, 32), np.int32)
    pr = np.zeros(idx.shape[0], np.uint32)
    R.ctref_export(h, _p(b), _p(pr), _p(q))
    return h, b, q, pr


def ref_trace(h, o, d, nthreads=8):
    R = oracle.ref()
    o = np.ascontiguousarray(o[:, :3], np.float32)
    d = np.ascontiguousarray(d[:, :3], np.float32)
    hit = np.zeros(o.shape[0], np.int32)
    t = np.zeros(o.shape[0], np.float32)
    R.ctref_trace_mbvh(h, _p(o), _p(d), o.shape[0], _p(hit), _p(t), nthreads)
    return hit, t


def sphere_fixture(sub: int, path: str, with_hits: bool) -> None:
    s = scenes.sphere_scene(sub)
    v = np.ascontiguousarray(s.vertices)
    ix = np.ascontiguousarray(s.indices)
    h, b, q, pr = ref_build(v, ix)
    rec = dict(
        subdivisions=sub, indices_sha=digest(ix.tobytes()), quad_sha=digest(q.tobytes()),
        prims_sha=digest(pr.tobytes()), binary_canonical_sha=digest(canonical_binary(b)),
        quad_count=q.shape[0], binary_count=b.shape[0],
    )
    if with_hits:
        o, d = scenes.pinhole_rays(256, 256, 60.0)
        ro = np.zeros((65536, 3), np.float32)
        rd = np.zeros((65536, 3), np.float32)
        pos = np.array([0, 0, 3], np.float32)
        oracle.ref().ctref_camera_rays(_p(pos), 60.0, 256, 256, _p(ro), _p(rd))
        assert np.array_equal(ro, o) and np.array_equal(rd, d), "pinhole_rays differs from Camera::generateRay"
        hit, t = ref_trace(h, ro, rd)
        io, idr = scenes.incoherent_rays(4096, seed=11)
        io[:, :3] = io[:, :3] * 2.4 - 1.2
        ihit, it = ref_trace(h, io, idr)
        rec.update(vertices=v, cam_dirs=rd, hit=hit, t=t, inc_org=io, inc_dir=idr, inc_hit=ihit, inc_t=it)
    else:
        rec.update(vertices_sha=digest(v.tobytes()))
    oracle.ref().ctref_free(h)
    np.savez_compressed(path, **rec)


def kat_fixture(path: str) -> None:
    R = oracle.ref()
    rng = np.random.default_rng(2024)
    out = {}
    seeds = rng.integers(0, 2**32, size=512, dtype=np.uint64).astype(np.uint32)
    out["wang_in"] = seeds
    out["wang_out"] = np.array([R.ctref_wang_hash(int(s)) for s in seeds], np.uint32)
    streams_i, streams_f = [], []
    for s in seeds[:32]:
        ii = np.zeros(64, np.uint32)
        ff = np.zeros(64, np.float32)
        R.ctref_random_stream(int(s), 64, _p(ii), _p(ff))
        streams_i.append(ii)
        streams_f.append(ff)
    out["stream_seeds"] = seeds[:32]
    out["stream_int"] = np.stack(streams_i)
    out["stream_float"] = np.stack(streams_f)
    # Moller-Trumbore: random + near-degenerate triangles, rays through/near them
    n = 4000
    p0 = rng.normal(size=(n, 3)).astype(np.float32)
    e1 = rng.normal(size=(n, 3)).astype(np.float32) * np.exp(rng.uniform(-8, 1, size=(n, 1))).astype(np.float32)
    e2 = rng.normal(size=(n, 3)).astype(np.float32) * np.exp(rng.uniform(-8, 1, size=(n, 1))).astype(np.float32)
    p1 = (p0 + e1).astype(np.float32)
    p2 = (p0 + e2).astype(np.float32)
    bary = rng.uniform(-0.1, 1.1, size=(n, 3)).astype(np.float32)
    target = (p0 * bary[:, :1] + p1 * bary[:, 1:2] + p2 * bary[:, 2:3]) / np.maximum(bary.sum(1, keepdims=True), 0.1)
    org = (rng.normal(size=(n, 3)) * 4).astype(np.float32)
    dirs = (target - org)
    dirs = (dirs / np.linalg.norm(dirs, axis=1, keepdims=True)).astype(np.float32)
    tin = np.where(rng.uniform(size=n) < 0.5, 1e34, rng.uniform(0.5, 6.0, size=n)).astype(np.float32)
    hitv = np.zeros(n, np.int32)
    tout = tin.copy()
    for i in range(n):
        t = np.array([tin[i]], np.float32)
        hitv[i] = R.ctref_triangle_intersect(_p(org[i]), _p(dirs[i]), _p(t), _p(p0[i]), _p(p1[i]), _p(p2[i]),
                                             ctypes.c_float(1e-3))
        tout[i] = t[0]
    out.update(mt_org=org, mt_dir=dirs, mt_p0=p0, mt_p1=p1, mt_p2=p2, mt_tin=tin, mt_hit=hitv, mt_tout=tout)
    # quad-node slab test
    m = 2000
    lo = rng.normal(size=(m, 3, 4)).astype(np.float32)
    hi = (lo + np.abs(rng.normal(size=(m, 3, 4))).astype(np.float32)).astype(np.float32)
    nodes = np.zeros((m, 32), np.int32)
    nf = nodes.view(np.float32)
    for a in range(3):
        nf[:, 8 * a:8 * a + 4] = lo[:, a]
        nf[:, 8 * a + 4:8 * a + 8] = hi[:, a]
    so = (rng.normal(size=(m, 3)) * 3).astype(np.float32)
    sd = rng.normal(size=(m, 3)).astype(np.float32)
    sd[rng.uniform(size=(m, 3)) < 0.05] = 0.0
    sinv = (np.float32(1.0) / sd).astype(np.float32)
    st = np.where(rng.uniform(size=m) < 0.5, 1e34, rng.uniform(0.1, 5.0, size=m)).astype(np.float32)
    tmini = np.zeros((m, 4), np.int32)
    res = np.zeros((m, 4), np.int32)
    with np.errstate(divide="ignore"):
        for i in range(m):
            R.ctref_mbvh_intersect(_p(nodes[i]), _p(so[i]), _p(sinv[i]), float(st[i]), _p(tmini[i]), _p(res[i]))
    out.update(slab_nodes=nodes, slab_org=so, slab_inv=sinv, slab_t=st, slab_tmini=tmini, slab_res=res)
    # barycentrics / area / light-sample point
    k = 500
    bp = rng.normal(size=(k, 3)).astype(np.float32)
    bn = rng.normal(size=(k, 3)).astype(np.float32)
    b0, b1, b2 = (rng.normal(size=(k, 3)).astype(np.float32) for _ in range(3))
    bo = np.zeros((k, 3), np.float32)
    ar = np.zeros(k, np.float32)
    r1 = rng.uniform(size=k).astype(np.float32)
    r2 = rng.uniform(size=k).astype(np.float32)
    rp = np.zeros((k, 3), np.float32)
    R.ctref_area.argtypes = [P, P, P]
    R.ctref_bary.argtypes = [P, P, P, P, P, P]
    R.ctref_random_point.argtypes = [P, P, P, ctypes.c_float, ctypes.c_float, P]
    R.ctref_tangent2world.argtypes = [P, P, P]
    R.ctref_local_space.argtypes = [P, P, P]
    for i in range(k):
        R.ctref_bary(_p(bp[i]), _p(bn[i]), _p(b0[i]), _p(b1[i]), _p(b2[i]), _p(bo[i]))
        ar[i] = R.ctref_area(_p(b0[i]), _p(b1[i]), _p(b2[i]))
        R.ctref_random_point(_p(b0[i]), _p(b1[i]), _p(b2[i]), float(r1[i]), float(r2[i]), _p(rp[i]))
    out.update(bary_p=bp, bary_n=bn, tri0=b0, tri1=b1, tri2=b2, bary_out=bo, area_out=ar, rp_r1=r1, rp_r2=r2,
               rp_out=rp)
    # Tangent2World, convertToLocalSpace, cosine-weighted sample, Fresnel
    tv = rng.normal(size=(k, 3)).astype(np.float32)
    tn = rng.normal(size=(k, 3)).astype(np.float32)
    to = np.zeros((k, 3), np.float32)
    lT = np.zeros((k, 3), np.float32)
    lB = np.zeros((k, 3), np.float32)
    cw = np.zeros((k, 3), np.float32)
    fr = np.zeros(k, np.float32)
    eta = rng.uniform(0.8, 2.5, size=k).astype(np.float32)
    for i in range(k):
        R.ctref_tangent2world(_p(tv[i]), _p(tn[i]), _p(to[i]))
        R.ctref_local_space(_p(tn[i]), _p(lT[i]), _p(lB[i]))
        R.ctref_cos_weighted(float(r1[i]), float(r2[i]), _p(cw[i]))
        fr[i] = R.ctref_fresnel_exact(_p(tv[i]), _p(tn[i]), float(eta[i]))
    out.update(t2w_v=tv, t2w_n=tn, t2w_out=to, ls_T=lT, ls_B=lB, cw_out=cw, fr_eta=eta, fr_out=fr)
    # SampleBSDF (diffuse and mirror branches)
    col = rng.uniform(size=(k, 3)).astype(np.float32)
    rough = np.where(rng.uniform(size=k) < 0.3, 0.05, 1.0).astype(np.float32)
    iN = tn / np.linalg.norm(tn, axis=1, keepdims=True)
    iN = (iN * rng.uniform(0.8, 1.2, size=(k, 1))).astype(np.float32)
    Ng = (iN + rng.normal(size=(k, 3)) * 0.1).astype(np.float32)
    wi = rng.normal(size=(k, 3)).astype(np.float32)
    wi = (wi / np.linalg.norm(wi, axis=1, keepdims=True)).astype(np.float32)
    sf = np.zeros((k, 3), np.float32)
    swo = np.zeros((k, 3), np.float32)
    spdf = np.zeros(k, np.float32)
    stype = np.zeros(k, np.int32)
    for i in range(k):
        R.ctref_sample_bsdf(_p(col[i]), float(rough[i]), 1.0, _p(iN[i]), _p(Ng[i]), _p(lT[i]), _p(lB[i]), _p(wi[i]),
                            float(r1[i]), float(r2[i]), _p(sf[i]), _p(swo[i]), _p(spdf[i:i + 1]), _p(stype[i:i + 1]))
    out.update(bsdf_col=col, bsdf_rough=rough, bsdf_iN=iN, bsdf_N=Ng, bsdf_wi=wi, bsdf_f=sf, bsdf_wo=swo,
               bsdf_pdf=spdf, bsdf_type=stype)
    # microfacet distributions through Material::sample / evaluate
    rr = rng.uniform(0.0, 1.0, size=64).astype(np.float32)
    out["r2a_in"] = rr
    out["r2a_out"] = np.array([R.ctref_roughness_to_alpha(float(x)) for x in rr], np.float32)
    mts, mins, mr, mout, mpdf = [], [], [], [], []
    for typ in range(4, 10):
        for vis in (0, 1):
            for _ in range(40):
                ax = float(np.float32(rng.uniform(0.05, 0.9)))
                ay = ax if rng.uniform() < 0.5 else float(np.float32(rng.uniform(0.05, 0.9)))
                w = rng.normal(size=3)
                w[2] = abs(w[2]) + 0.05
                w = (w / np.linalg.norm(w)).astype(np.float32)
                q1, q2 = (float(np.float32(x)) for x in rng.uniform(0.01, 0.99, size=2))
                o3 = np.zeros(3, np.float32)
                R.ctref_mf_sample(typ, ax, ay, vis, _p(w), q1, q2, _p(o3))
                wo = rng.normal(size=3)
                wo[2] = abs(wo[2]) + 0.05
                wo = (wo / np.linalg.norm(wo)).astype(np.float32)
                pdf = R.ctref_mf_pdf(typ, ax, ay, vis, _p(wo), _p(o3), _p(w))
                mts.append([typ, vis])
                mins.append([ax, ay])
                mr.append(np.concatenate([w, [q1, q2], wo]))
                mout.append(o3)
                mpdf.append(pdf)
    out.update(mf_type_vis=np.array(mts, np.int32), mf_alpha=np.array(mins, np.float32),
               mf_in=np.array(mr, np.float32), mf_out=np.array(mout, np.float32), mf_pdf=np.array(mpdf, np.float32))
    # camera
    ro = np.zeros((64 * 48, 3), np.float32)
    rd = np.zeros((64 * 48, 3), np.float32)
    pos = np.array([0.5, -1.0, 4.0], np.float32)
    R.ctref_camera_rays(_p(pos), 70.0, 64, 48, _p(ro), _p(rd))
    out.update(cam_pos=pos, cam_fov=np.float32(70.0), cam_w=64, cam_h=48, cam_org=ro, cam_dir=rd,
               cam_plane=np.float32(R.ctref_camera_plane_distance(70.0)))
    np.savez_compressed(path, **out)


if __name__ == "__main__":
    oracle.build()
    if not oracle.ref_available():
        sys.exit("the reference host library is not available (oracle/ref_build.py needs the reference sources)")
    kat_fixture(os.path.join(HERE, "kat_math.npz"))
    sphere_fixture(5, os.path.join(HERE, "sphere_s5.npz"), with_hits=False)
    sphere_fixture(6, os.path.join(HERE, "sphere_c1.npz"), with_hits=True)
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))
