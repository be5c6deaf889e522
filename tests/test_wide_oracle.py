"""The FP64 watertight oracle of the wide-BVH queries (oracle/ct_fp64.cpp
fp64_trace) against a brute-force numpy evaluation of the same test over
every triangle (no BVH), on soups with near-edge and axis-aligned rays."""
import numpy as np
import pytest


def _wt_bruteforce(v, ix, o, d):
    """Watertight test (Woop, Benthin, Wald 2013) in float64 over all triangles."""
    n = o.shape[0]
    hit = np.full(n, -1, np.int64)
    tb = d[:, 3].astype(np.float64).copy()
    P = v[ix].astype(np.float64)  # (T,3,3)
    for i in range(n):
        dd = d[i, :3]
        ad = np.abs(dd)
        kz = (0 if ad[0] > ad[2] else 2) if ad[0] > ad[1] else (1 if ad[1] > ad[2] else 2)
        kx = 0 if kz == 2 else kz + 1
        ky = 0 if kx == 2 else kx + 1
        if dd[kz] < 0:
            kx, ky = ky, kx
        dkz = np.float64(dd[kz])
        Sx, Sy, Sz = np.float64(dd[kx]) / dkz, np.float64(dd[ky]) / dkz, 1.0 / dkz
        oo = o[i, :3].astype(np.float64)
        A, B, C = P[:, 0] - oo, P[:, 1] - oo, P[:, 2] - oo
        Ax, Ay = A[:, kx] - Sx * A[:, kz], A[:, ky] - Sy * A[:, kz]
        Bx, By = B[:, kx] - Sx * B[:, kz], B[:, ky] - Sy * B[:, kz]
        Cx, Cy = C[:, kx] - Sx * C[:, kz], C[:, ky] - Sy * C[:, kz]
        U = Cx * By - Cy * Bx
        V = Ax * Cy - Ay * Cx
        W = Bx * Ay - By * Ax
        neg = (U < 0) | (V < 0) | (W < 0)
        pos = (U > 0) | (V > 0) | (W > 0)
        det = (U + V) + W
        with np.errstate(divide="ignore", invalid="ignore"):
            T = ((U * (Sz * A[:, kz])) + (V * (Sz * B[:, kz]))) + (W * (Sz * C[:, kz]))
            t = T / det
        ok = ~(neg & pos) & (det != 0) & (t > 0) & (t < tb[i])
        if ok.any():
            cand = np.nonzero(ok)[0]
            tmin = t[cand].min()
            win = cand[t[cand] == tmin].min()
            hit[i], tb[i] = win, tmin
    return hit, tb


def test_fp64_trace_matches_bruteforce(orc):
    from cudatracer_gb300 import scenes

    s = scenes.soup_scene(3000, seed=21)
    rng = np.random.default_rng(4)
    o, d = scenes.incoherent_rays(300, seed=6)
    # rays aimed at triangle vertices and edge midpoints (near-edge hits)
    tri = rng.integers(0, 3000, 100)
    P = s.vertices[s.indices[tri]]
    tgt = np.concatenate([P[:50, 0], (P[50:, 0] + P[50:, 1]) * 0.5])
    o2 = np.zeros((100, 4), np.float32)
    o2[:, :3] = rng.uniform(0, 1, (100, 3))
    d2 = np.zeros((100, 4), np.float32)
    dv = tgt - o2[:, :3]
    d2[:, :3] = dv / np.linalg.norm(dv, axis=1, keepdims=True)
    d2[:, 3] = 1e34
    # axis-aligned rays
    o3 = o[:40].copy()
    d3 = np.zeros((40, 4), np.float32)
    d3[np.arange(40), np.arange(40) % 3] = np.where(np.arange(40) % 2, 1.0, -1.0)
    d3[:, 3] = 1e34
    O = np.concatenate([o, o2, o3])
    D = np.concatenate([d, d2, d3])
    ob = orc.bvh_build(s.vertices, s.indices)
    h, t = orc.trace_fp64(s.vertices, s.indices, ob["quad"], ob["prims"], O, D)
    hb, tb = _wt_bruteforce(s.vertices, s.indices, O, D)
    assert np.array_equal(h, hb)
    assert np.array_equal(t[h >= 0], tb[hb >= 0])
    assert (h[300:400] >= 0).sum() >= 25  # rays aimed at vertices and edge midpoints: about half hit
    # occlusion agrees with the closest-hit result for finite ranges
    D4 = D.copy()
    D4[:, 3] = np.where(h >= 0, t * 1.5, 0.3).astype(np.float32)
    occ, _ = orc.trace_fp64(s.vertices, s.indices, ob["quad"], ob["prims"], O, D4, any_hit=True)
    ref, _ = _wt_bruteforce(s.vertices, s.indices, O, D4)
    assert np.array_equal(occ >= 0, ref >= 0)
