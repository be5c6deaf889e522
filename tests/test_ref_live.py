"""The oracle against the reference's own host code run live (only where the
reference was compiled, see oracle/ref_build.py): random soups, spheres and
rays beyond the committed fixtures."""
import ctypes

import numpy as np
import pytest

P = ctypes.c_void_p


@pytest.fixture(scope="module")
def ref(orc):
    if not orc.ref_available():
        pytest.skip("reference host library not built here")
    return orc.ref()


def _p(a):
    return a.ctypes.data_as(P)


def _ref_build(R, v, ix, nthreads=4):
    v = np.ascontiguousarray(v, np.float32)
    ix = np.ascontiguousarray(ix, np.uint32)
    h = R.ctref_build(_p(v), v.shape[0], _p(ix), ix.shape[0], nthreads)
    q = np.zeros((R.ctref_mbvh_count(h), 32), np.int32)
    pr = np.zeros(ix.shape[0], np.uint32)
    R.ctref_export(h, None, _p(pr), _p(q))
    return h, q, pr


@pytest.mark.parametrize("seed,ntri", [(11, 100), (12, 3000), (13, 30000)])
def test_soup_build_and_trace(ref, orc, seed, ntri):
    from cudatracer_gb300 import scenes

    s = scenes.soup_scene(ntri, seed=seed)
    h, q, pr = _ref_build(ref, s.vertices, s.indices)
    try:
        o = orc.bvh_build(s.vertices, s.indices)
        assert np.array_equal(o["quad"], q) and np.array_equal(o["prims"], pr)
        ro, rd = scenes.incoherent_rays(20000, seed=seed)
        hit = np.zeros(20000, np.int32)
        t = np.zeros(20000, np.float32)
        oo = np.ascontiguousarray(ro[:, :3])
        dd = np.ascontiguousarray(rd[:, :3])
        ref.ctref_trace_mbvh(h, _p(oo), _p(dd), 20000, _p(hit), _p(t), 4)
        oh, ot = orc.trace_closest(o["quad"], o["prims"], s.vertices, s.indices, ro, rd)
        assert np.array_equal(oh, hit)
        assert np.array_equal(ot.view(np.int32), t.view(np.int32))
    finally:
        ref.ctref_free(h)
