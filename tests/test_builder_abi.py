"""Host-side checks that need no GPU: the C ABI surface and the product's host
BVH builder (ct_host_bvh_build) against the reference's trees."""
import ctypes
import hashlib
import os
import re

import numpy as np
import pytest

from tests.conftest import ROOT, golden


def header_functions():
    src = open(os.path.join(ROOT, "include", "cudatracer.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(ct_[a-z0-9_]+)\s*\(", src)))


def test_library_exports_every_declared_symbol(lib):
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    from cudatracer_gb300 import _lib

    assert set(names) == set(_lib.SIGNATURES), set(names) ^ set(_lib.SIGNATURES)


def test_abi_structs_match_reference_layouts(lib):
    from cudatracer_gb300 import _lib

    assert ctypes.sizeof(_lib.ct_material) == 52  # reference Material
    assert lib.ct_abi_version() == 1
    p = _lib.ct_render_params()
    lib.ct_render_params_default(ctypes.byref(p))
    assert (p.max_depth, p.shadow, p.indirect, p.sky) == (5, 1, 1, 1)
    assert np.float32(p.normal_eps) == np.float32(1e-5) and np.float32(p.tri_eps) == np.float32(1e-3)


def test_host_build_matches_reference_trees(lib):
    from cudatracer_gb300 import api, scenes
    from tests.golden.make_golden import canonical_binary

    for name in ("sphere_s5.npz", "sphere_c1.npz"):
        g = golden(name)
        s = scenes.sphere_scene(int(g["subdivisions"]))
        v = g["vertices"] if "vertices" in g else s.vertices
        for nthreads in (1, 4):
            h = api.host_bvh_build(v, s.indices, nthreads)
            assert hashlib.sha256(h["quad"].tobytes()).hexdigest() == str(g["quad_sha"])
            assert hashlib.sha256(h["prims"].tobytes()).hexdigest() == str(g["prims_sha"])
            assert hashlib.sha256(canonical_binary(h["binary"])).hexdigest() == str(g["binary_canonical_sha"])


@pytest.mark.parametrize("seed,ntri", [(1, 7), (2, 300), (3, 5000), (4, 40000)])
def test_host_build_matches_oracle_on_soups(lib, orc, seed, ntri):
    from cudatracer_gb300 import api, scenes

    s = scenes.soup_scene(ntri, seed=seed)
    h = api.host_bvh_build(s.vertices, s.indices, 4)
    o = orc.bvh_build(s.vertices, s.indices)
    assert np.array_equal(h["prims"], o["prims"])
    assert np.array_equal(h["binary"], o["binary"])
    if o["binary"][0, 7] > -1:  # root leaf: the reference leaves an empty quad root
        assert h["quad"][0, 28] == o["binary"][0, 7]
    else:
        assert np.array_equal(h["quad"], o["quad"])


def test_host_build_degenerate_inputs(lib, orc):
    """Coincident triangles (no useful split) and a single triangle."""
    from cudatracer_gb300 import api

    v = np.tile(np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32), (64, 1))
    ix = np.arange(v.shape[0], dtype=np.uint32).reshape(-1, 3)
    h = api.host_bvh_build(v, ix, 2)
    o = orc.bvh_build(v, ix)
    assert np.array_equal(h["binary"], o["binary"]) and np.array_equal(h["prims"], o["prims"])
    h1 = api.host_bvh_build(v[:3], ix[:1], 1)
    assert h1["quad"].shape[0] == 1 and h1["quad"][0, 28] == 1  # root leaf kept as child 0


def test_host_build_rejects_bad_input(lib):
    from cudatracer_gb300 import _lib, api

    v = np.array([[0, 0, 0], [1, 0, 0], [0, np.nan, 0]], np.float32)
    with pytest.raises(_lib.CTError) as e:
        api.host_bvh_build(v, np.array([[0, 1, 2]], np.uint32))
    assert e.value.status == 1
    v[2, 1] = 1.0
    with pytest.raises(_lib.CTError):
        api.host_bvh_build(v, np.array([[0, 1, 3]], np.uint32))


def test_context_without_device_fails_cleanly(lib):
    import torch

    if torch.cuda.is_available():
        pytest.skip("a device is present")
    h = ctypes.c_void_p()
    assert lib.ct_ctx_create(0, ctypes.byref(h)) == 7  # CT_ERR_NO_DEVICE
    assert lib.ct_ctx_destroy(None) == 1
