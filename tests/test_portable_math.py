"""Accuracy of the reproducible binary32 sin, cos, atan2 and acos
(cudatracer_gb300/csrc/portable_math.h) that exact-math frames use on the GPU
and in the oracle. Evaluated through the oracle library (the same header
compiled for the host) against float64 references; the error is in units of
the spacing of the correctly rounded float result (a correctly rounded
function scores at most 0.5)."""
import ctypes

import numpy as np
import pytest

TWO_PI_F = np.float32(6.28318530717958647692528676655900576)


@pytest.fixture(scope="module")
def pm(orc):
    L = orc.lib()
    P = ctypes.c_void_p
    L.or_pm_eval.argtypes = [P, P, ctypes.c_int, P, P, P, P]

    def ev(x, y=None):
        x = np.ascontiguousarray(x, np.float32)
        n = x.size
        y = np.ascontiguousarray(np.zeros(n, np.float32) if y is None else y, np.float32)
        out = [np.zeros(n, np.float32) for _ in range(4)]
        L.or_pm_eval(x.ctypes.data_as(P), y.ctypes.data_as(P), n, *[o.ctypes.data_as(P) for o in out])
        return out

    return ev


def ulp_error(got, ref64):
    sp = np.spacing(np.abs(ref64.astype(np.float32))).astype(np.float64)
    return np.abs(got.astype(np.float64) - ref64) / sp


def test_sin_cos_on_shading_angles(pm):
    """The angles the cosine-weighted sample takes: 2 pi r, r from the
    reference's RandomFloat grid (a 32-bit integer times 2^-32), plus the
    floats next to k pi / 2, where the reduced argument is smallest."""
    rng = np.random.default_rng(11)
    r = rng.integers(0, 2**32, 1_000_000, dtype=np.uint64).astype(np.uint32).astype(np.float32)
    th = TWO_PI_F * (r * np.float32(2.3283064365387e-10))
    near = []
    for k in range(5):
        v = np.float32(k * np.pi / 2)
        for _ in range(64):
            near.append(v)
            v = np.nextafter(v, np.float32(10))
    th = np.concatenate([th, np.array(near, np.float32), np.array([0.0, TWO_PI_F], np.float32)])
    s, c, _, _ = pm(th)
    x = th.astype(np.float64)
    assert ulp_error(s, np.sin(x)).max() <= 2.0
    assert ulp_error(c, np.cos(x)).max() <= 2.0
    assert s[-2] == 0.0 and c[-2] == 1.0


def test_sin_cos_wide_range(pm):
    x = np.random.default_rng(12).uniform(-1024, 1024, 500_000).astype(np.float32)
    s, c, _, _ = pm(x)
    assert ulp_error(s, np.sin(x.astype(np.float64))).max() <= 3.0
    assert ulp_error(c, np.cos(x.astype(np.float64))).max() <= 3.0


def test_atan2_and_acos_on_directions(pm):
    """The sky lookup's arguments: atan2(d.x, -d.z) and acos(d.y) of unit
    directions, plus acos over [-1, 1] and its end points."""
    rng = np.random.default_rng(13)
    d = rng.normal(size=(3, 500_000))
    d = (d / np.linalg.norm(d, axis=0)).astype(np.float32)
    _, _, a, _ = pm(-d[2], d[0])
    assert ulp_error(a, np.arctan2(d[0].astype(np.float64), -d[2].astype(np.float64))).max() <= 3.0
    xs = np.concatenate([d[1], rng.uniform(-1, 1, 500_000).astype(np.float32),
                         np.array([1, -1, 0, 0.5, -0.5, 1 - 2**-24, -1 + 2**-24], np.float32)])
    _, _, _, ac = pm(xs)
    assert ulp_error(ac, np.arccos(xs.astype(np.float64))).max() <= 3.0
    _, _, _, ac = pm(np.array([np.nextafter(np.float32(1), np.float32(2)), -1.0000001, np.nan], np.float32))
    assert np.isnan(ac).all()  # outside [-1, 1], as the C library's acos


def test_atan2_special_values(pm):
    """Signed zeros and infinities follow the C library's atan2."""
    inf = np.inf
    cases = [(0.0, 1.0), (0.0, -1.0), (-0.0, -1.0), (1.0, 0.0), (-1.0, -0.0), (0.0, 0.0), (0.0, -0.0),
             (-0.0, -0.0), (inf, 1.0), (inf, inf), (inf, -inf), (-inf, -inf), (3.0, -inf), (-3.0, inf)]
    y = np.array([c[0] for c in cases], np.float32)
    x = np.array([c[1] for c in cases], np.float32)
    _, _, a, _ = pm(x, y)
    want = np.arctan2(y, x)
    assert np.array_equal(np.signbit(a), np.signbit(want))
    assert ulp_error(a, want.astype(np.float64)).max() <= 1.0
    _, _, a, _ = pm(np.array([np.nan, 1.0], np.float32), np.array([1.0, np.nan], np.float32))
    assert np.isnan(a).all()
