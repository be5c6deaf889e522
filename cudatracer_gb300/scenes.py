"""Seeded synthetic scenes for the tracer's workloads (no datasets are involved).

Every generator returns plain numpy arrays laid out like the reference's host
scene container (TriangleList public vectors, src/Core/TriangleList.h:59-73):
float32 vertices/normals (n,3), float32 texcoords (n,2), uint32 indices (m,3),
uint32 per-triangle material index (m,). The same arrays feed the CUDA path and
the CPU oracle, so both always see bit-identical input.

Workloads (sizes as used by the tests and bench):
  * sphere scene   - icosahedron subdivided 6x (81,920 triangles), each vertex
                     radius scaled by U[0.95, 1.05]; 256x256 pinhole rays, FOV 60,
                     camera at (0,0,3) looking down -z.
  * terrain scene  - fBm-displaced 1024x1024 vertex grid (2,093,058 triangles)
                     plus 200 icospheres of 5,120 triangles, radii U[0.5, 3];
                     materials 40% Lambertian, 20% specular, 10% dielectric
                     (IOR 1.5), 30% GGX; 4 emissive quads (8 triangles,
                     radiance U[10, 50]); 2048x1024 FP32 equirect sky gradient.
  * triangle soup  - centroids U[0,1]^3, edge lengths log-uniform [1e-4, 1e-2],
                     with incoherent rays (origins U[0,1]^3, directions on S^2).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# Material type codes, same values as the reference MaterialType enum
# (src/Core/Material.cuh:13-27).
MAT_LIGHT, MAT_SPECULAR, MAT_FRESNEL, MAT_LAMBERTIAN = 0, 1, 2, 3
MAT_BECKMANN, MAT_GGX, MAT_TROWBRIDGE = 4, 5, 6
MAT_FRESNEL_BECKMANN, MAT_FRESNEL_GGX, MAT_FRESNEL_TROWBRIDGE = 7, 8, 9


@dataclass
class Scene:
    vertices: np.ndarray  # (nv, 3) float32
    normals: np.ndarray  # (nv, 3) float32, per vertex
    texcoords: np.ndarray  # (nv, 2) float32
    indices: np.ndarray  # (nt, 3) uint32
    mat_idx: np.ndarray  # (nt,) uint32
    materials: list = field(default_factory=list)  # list of dicts (see Material in api.py)
    light_indices: np.ndarray | None = None  # (nl,) uint32
    textures: list = field(default_factory=list)  # list of (h, w, 4) float32
    skybox_texture: int = -1

    @property
    def ntri(self) -> int:
        return int(self.indices.shape[0])


def icosphere(subdivisions: int) -> tuple[np.ndarray, np.ndarray]:
    """Unit icosphere: float64 vertices on the sphere and uint32 triangles.

    20 * 4**subdivisions triangles; edge midpoints are shared so the mesh is
    watertight and per-vertex displacement keeps it closed."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array(
        [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
         [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]],
        dtype=np.float64,
    )
    f = np.array(
        [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11], [1, 5, 9], [5, 11, 4],
         [11, 10, 2], [10, 7, 6], [7, 1, 8], [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8],
         [3, 8, 9], [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]],
        dtype=np.int64,
    )
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(subdivisions):
        a, b, c = f[:, 0], f[:, 1], f[:, 2]
        edges = np.concatenate([np.stack([a, b], 1), np.stack([b, c], 1), np.stack([c, a], 1)])
        key = np.sort(edges, axis=1)
        uniq, inv = np.unique(key, axis=0, return_inverse=True)
        inv = inv.reshape(-1)
        mid = v[uniq[:, 0]] + v[uniq[:, 1]]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        base = v.shape[0]
        v = np.concatenate([v, mid])
        n = f.shape[0]
        ab, bc, ca = inv[:n] + base, inv[n:2 * n] + base, inv[2 * n:] + base
        f = np.concatenate([
            np.stack([a, ab, ca], 1), np.stack([b, bc, ab], 1),
            np.stack([c, ca, bc], 1), np.stack([ab, bc, ca], 1),
        ])
    return v, f.astype(np.uint32)


def _default_material() -> dict:
    return dict(albedo=(1.0, 1.0, 1.0), refract_idx=1.0, diffuse_tex=-1, normal_tex=-1, mask_tex=-1, displace_tex=-1,
                type=MAT_LAMBERTIAN, roughness=1.0, absorption=(0.0, 0.0, 0.0))


def sphere_scene(subdivisions: int = 6, seed: int = 1234, jitter: float = 0.05) -> Scene:
    """Icosphere with each vertex radius scaled by U[1-jitter, 1+jitter]."""
    v, f = icosphere(subdivisions)
    rng = np.random.default_rng(seed)
    r = rng.uniform(1.0 - jitter, 1.0 + jitter, size=(v.shape[0], 1))
    verts = (v * r).astype(np.float32)
    normals = v.astype(np.float32)
    uv = np.zeros((v.shape[0], 2), np.float32)
    return Scene(verts, normals, uv, f, np.zeros(f.shape[0], np.uint32), [_default_material()])


def _value_noise_fbm(n: int, rng: np.random.Generator, octaves: int = 6) -> np.ndarray:
    """fBm of bilinear value noise on an n x n grid, range roughly [-1, 1]."""
    out = np.zeros((n, n), np.float64)
    amp, total = 1.0, 0.0
    for o in range(octaves):
        cells = 4 * (2 ** o)
        g = rng.uniform(-1.0, 1.0, size=(cells + 1, cells + 1))
        x = np.linspace(0.0, cells, n, endpoint=False)
        i0 = np.floor(x).astype(np.int64)
        fx = x - i0
        fx = fx * fx * (3.0 - 2.0 * fx)
        a = g[i0][:, i0] * (1 - fx)[None, :] + g[i0][:, i0 + 1] * fx[None, :]
        b = g[i0 + 1][:, i0] * (1 - fx)[None, :] + g[i0 + 1][:, i0 + 1] * fx[None, :]
        out += amp * (a * (1 - fx)[:, None] + b * fx[:, None])
        total += amp
        amp *= 0.5
    return out / total


def sky_gradient(width: int = 2048, height: int = 1024) -> np.ndarray:
    """Procedural FP32 equirect sky: horizon-to-zenith blue gradient, (h, w, 4)."""
    v = (np.arange(height, dtype=np.float32) + 0.5) / height  # 0 = zenith row... 1 = nadir
    up = np.clip(1.0 - 2.0 * v, -1.0, 1.0)[:, None]
    zen = np.array([0.25, 0.45, 0.95], np.float32)
    hor = np.array([0.85, 0.9, 1.0], np.float32)
    gnd = np.array([0.3, 0.28, 0.25], np.float32)
    t = np.clip(up, 0.0, 1.0)[..., None]
    col = np.where(up[..., None] >= 0, hor * (1 - t) + zen * t, gnd)
    u = (np.arange(width, dtype=np.float32) + 0.5) / width
    tint = (1.0 + 0.05 * np.sin(2 * np.pi * u))[None, :, None]
    img = np.ones((height, width, 4), np.float32)
    img[..., :3] = (np.broadcast_to(col, (height, 1, 3)) * tint).astype(np.float32)
    return img


def terrain_scene(grid: int = 1024, spheres: int = 200, seed: int = 7, extent: float = 200.0,
                  sky_size=(2048, 1024), ground_textures: tuple | None = None) -> tuple[Scene, dict]:
    """fBm terrain + icospheres + four emissive quads + sky.

    ground_textures=(w, h) also gives the ground a seeded diffuse texture and a
    tangent-space normal map of that size (textures 1 and 2; the uv span is
    tiled 4x so the wrap is exercised). Returns (scene, camera) where camera =
    dict(position, forward, up, fov)."""
    rng = np.random.default_rng(seed)
    h = _value_noise_fbm(grid, rng) * 12.0
    xs = np.linspace(-extent / 2, extent / 2, grid)
    X, Z = np.meshgrid(xs, xs)
    tv = np.stack([X, h, Z], -1).reshape(-1, 3)
    gy, gx = np.gradient(h, xs[1] - xs[0])
    tn = np.stack([-gx, np.ones_like(h), -gy], -1).reshape(-1, 3)
    tn /= np.linalg.norm(tn, axis=1, keepdims=True)
    r_, c_ = np.meshgrid(np.arange(grid - 1), np.arange(grid - 1), indexing="ij")
    v00 = (r_ * grid + c_).reshape(-1)
    v01, v10, v11 = v00 + 1, v00 + grid, v00 + grid + 1
    tf = np.concatenate([np.stack([v00, v10, v01], 1), np.stack([v01, v10, v11], 1)])
    tuv = np.stack([X / extent + 0.5, Z / extent + 0.5], -1).reshape(-1, 2)
    materials = [dict(type=MAT_LAMBERTIAN, albedo=(0.55, 0.5, 0.42), refract_idx=1.0, roughness=1.0)]
    mat_idx = [np.zeros(tf.shape[0], np.int64)]
    verts, norms, uvs, faces = [tv], [tn], [tuv], [tf]
    base = tv.shape[0]
    sv, sf = icosphere(4)
    for _ in range(spheres):
        r = rng.uniform(0.5, 3.0)
        cx, cz = rng.uniform(-extent * 0.3, extent * 0.3, size=2)
        gi = int(np.clip((cz + extent / 2) / extent * (grid - 1), 0, grid - 1))
        gj = int(np.clip((cx + extent / 2) / extent * (grid - 1), 0, grid - 1))
        cy = h[gi, gj] + r * 0.8
        u = rng.uniform()
        if u < 0.4:
            m = dict(type=MAT_LAMBERTIAN, albedo=tuple(rng.uniform(0.1, 0.9, 3)), refract_idx=1.0, roughness=1.0)
        elif u < 0.6:
            m = dict(type=MAT_SPECULAR, albedo=tuple(rng.uniform(0.6, 0.95, 3)), refract_idx=1.0, roughness=0.0001)
        elif u < 0.7:
            m = dict(type=MAT_FRESNEL, albedo=(0.95, 0.95, 0.95), refract_idx=1.5, roughness=0.0)
        else:
            m = dict(type=MAT_GGX, albedo=tuple(rng.uniform(0.3, 0.9, 3)), refract_idx=1.0,
                     roughness=float(rng.uniform(0.05, 0.8)))
        materials.append(m)
        verts.append(sv * r + np.array([cx, cy, cz]))
        norms.append(sv)
        uvs.append(np.zeros((sv.shape[0], 2)))
        faces.append(sf.astype(np.int64) + base)
        mat_idx.append(np.full(sf.shape[0], len(materials) - 1))
        base += sv.shape[0]
    light_tris = []
    for k in range(4):
        e = rng.uniform(10.0, 50.0)
        materials.append(dict(type=MAT_LIGHT, albedo=(e, e, e), refract_idx=1.0, roughness=0.0))
        cx, cz = (-40.0 + 80.0 * (k % 2)), (-40.0 + 80.0 * (k // 2))
        y, s = 70.0, 6.0
        qv = np.array([[cx - s, y, cz - s], [cx + s, y, cz - s], [cx + s, y, cz + s], [cx - s, y, cz + s]])
        qf = np.array([[0, 1, 2], [0, 2, 3]]) + base
        verts.append(qv)
        norms.append(np.tile([0.0, -1.0, 0.0], (4, 1)))
        uvs.append(np.zeros((4, 2)))
        t0 = sum(f.shape[0] for f in faces)
        faces.append(qf)
        mat_idx.append(np.full(2, len(materials) - 1))
        light_tris += [t0, t0 + 1]
        base += 4
    full = []
    for m in materials:
        d = dict(albedo=(1.0, 1.0, 1.0), refract_idx=1.0, diffuse_tex=-1, normal_tex=-1, mask_tex=-1,
                 displace_tex=-1, type=MAT_LAMBERTIAN, roughness=1.0, absorption=(0.0, 0.0, 0.0))
        d.update(m)
        d["albedo"] = tuple(float(c) for c in d["albedo"])
        full.append(d)
    textures = [sky_gradient(*sky_size)]
    if ground_textures is not None:
        tw, th = ground_textures
        trng = np.random.default_rng(seed + 100)
        yy, xx = np.mgrid[0:th, 0:tw]
        check = ((xx // max(1, tw // 8) + yy // max(1, th // 8)) % 2).astype(np.float32)
        diff = np.empty((th, tw, 4), np.float32)
        diff[..., 0] = 0.35 + 0.4 * check + 0.1 * trng.uniform(size=(th, tw))
        diff[..., 1] = 0.3 + 0.3 * check + 0.1 * trng.uniform(size=(th, tw))
        diff[..., 2] = 0.25 + 0.2 * (1 - check) + 0.1 * trng.uniform(size=(th, tw))
        diff[..., 3] = 1.0
        nrm = np.empty((th, tw, 4), np.float32)
        bump = trng.normal(scale=0.25, size=(th, tw, 2))
        nrm[..., 0], nrm[..., 1], nrm[..., 2], nrm[..., 3] = bump[..., 0], bump[..., 1], 1.0, 1.0
        textures += [diff, nrm]
        full[0]["diffuse_tex"], full[0]["normal_tex"] = 1, 2
        uvs[0] = uvs[0] * 4.0
    sc = Scene(
        np.concatenate(verts).astype(np.float32), np.concatenate(norms).astype(np.float32),
        np.concatenate(uvs).astype(np.float32), np.concatenate(faces).astype(np.uint32),
        np.concatenate(mat_idx).astype(np.uint32), full, np.asarray(light_tris, np.uint32), textures, 0)
    cam = dict(position=(0.0, 35.0, 95.0), forward=_unit((0.0, -0.32, -1.0)), up=(0.0, 1.0, 0.0), fov=60.0)
    return sc, cam


def material_zoo_scene(grid: int = 48, spheres: int = 27, seed: int = 11,
                       ground_textures: tuple | None = None) -> tuple[Scene, dict]:
    """A small terrain scene whose spheres cycle through every non-emitter
    material type (Lambertian, specular, Fresnel, Beckmann, GGX, Trowbridge and
    the three rough dielectrics), for checking the full-material mode."""
    sc, cam = terrain_scene(grid=grid, spheres=spheres, seed=seed, extent=60.0, sky_size=(256, 128),
                            ground_textures=ground_textures)
    kinds = [MAT_LAMBERTIAN, MAT_SPECULAR, MAT_FRESNEL, MAT_BECKMANN, MAT_GGX, MAT_TROWBRIDGE,
             MAT_FRESNEL_BECKMANN, MAT_FRESNEL_GGX, MAT_FRESNEL_TROWBRIDGE]
    rng = np.random.default_rng(seed + 1)
    for k in range(spheres):
        m = sc.materials[1 + k]
        m["type"] = kinds[k % len(kinds)]
        m["roughness"] = float(rng.uniform(0.15, 0.6))
        m["refract_idx"] = 1.5
        m["albedo"] = tuple(float(c) for c in rng.uniform(0.4, 0.95, 3))
    cam = dict(position=(0.0, 14.0, 34.0), forward=_unit((0.0, -0.35, -1.0)), up=(0.0, 1.0, 0.0), fov=60.0)
    return sc, cam


def _unit(v):
    v = np.asarray(v, np.float64)
    v = v / np.linalg.norm(v)
    return tuple(float(np.float32(c)) for c in v)


def scene_arrays(sc: Scene) -> dict:
    """The SceneData arrays (centre normals as loadModel computes them)."""
    n = sc.normals
    ix = sc.indices
    cn = ((n[ix[:, 0]] + n[ix[:, 1]]) + n[ix[:, 2]]) / np.float32(3.0)
    return {
        "vertices": sc.vertices, "normals": sc.normals, "texcoords": sc.texcoords, "indices": sc.indices,
        "center_normals": cn.astype(np.float32), "material_idxs": sc.mat_idx,
        "light_indices": sc.light_indices if sc.light_indices is not None else np.zeros(0, np.uint32),
    }


def soup_scene(ntri: int, seed: int = 3) -> Scene:
    """Random triangle soup: centroids U[0,1]^3, edge lengths log-uniform [1e-4, 1e-2]."""
    rng = np.random.default_rng(seed)
    c = rng.uniform(0.0, 1.0, size=(ntri, 1, 3))
    L = np.exp(rng.uniform(np.log(1e-4), np.log(1e-2), size=(ntri, 1, 1)))
    d = rng.normal(size=(ntri, 3, 3))
    d /= np.linalg.norm(d, axis=2, keepdims=True)
    v = (c + d * L).reshape(-1, 3).astype(np.float32)
    f = np.arange(3 * ntri, dtype=np.uint32).reshape(-1, 3)
    e1 = v[f[:, 1]] - v[f[:, 0]]
    e2 = v[f[:, 2]] - v[f[:, 0]]
    n = np.cross(e1, e2)
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    nv = np.repeat(n, 3, axis=0).astype(np.float32)
    return Scene(v, nv, np.zeros((v.shape[0], 2), np.float32), f, np.zeros(ntri, np.uint32), [_default_material()])


def incoherent_rays(n: int, seed: int = 5) -> tuple[np.ndarray, np.ndarray]:
    """Origins U[0,1]^3, directions uniform on the sphere; (n,4) float32 each, dir.w = 1e34."""
    rng = np.random.default_rng(seed)
    o = np.zeros((n, 4), np.float32)
    o[:, :3] = rng.uniform(0.0, 1.0, size=(n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    dd = np.zeros((n, 4), np.float32)
    dd[:, :3] = d
    dd[:, 3] = 1e34
    return o, dd


def pinhole_rays(width: int, height: int, fov_deg: float, pos=(0.0, 0.0, 3.0)) -> tuple[np.ndarray, np.ndarray]:
    """Primary rays through integer pixel coordinates for a camera looking down
    -z with up +y, restating Camera::generateRay (src/Core/Camera.cpp:19-37) in
    float32 with the reference's operation order. Returns (origins, dirs) (n,3)."""
    f32 = np.float32
    dist = f32(np.tan(f32(f32(fov_deg) * f32(0.5)) * f32(0.01745329251994329576923690768489)))
    aspect = f32(width) / f32(height)
    # u = normalize(cross(w, up)) = (1,0,0); v = normalize(cross(u, w)) = (0,1,0)
    hor = np.array([f32(1.0) * dist * aspect, f32(0.0), f32(0.0)], f32)
    ver = np.array([f32(0.0), f32(1.0) * dist, f32(0.0)], f32)
    w = np.array([0.0, 0.0, -1.0], f32)
    ys, xs = np.meshgrid(np.arange(height, dtype=f32), np.arange(width, dtype=f32), indexing="ij")
    sx = f32(2.0) * (xs.reshape(-1) * (f32(1.0) / f32(width))) - f32(1.0)
    sy = f32(1.0) - f32(2.0) * (ys.reshape(-1) * (f32(1.0) / f32(height)))
    p = w[None, :] + hor[None, :] * sx[:, None]
    p = p + ver[None, :] * sy[:, None]
    d2 = (p[:, 0] * p[:, 0] + p[:, 1] * p[:, 1]) + p[:, 2] * p[:, 2]
    inv = f32(1.0) / np.sqrt(d2)
    d = (p * inv[:, None]).astype(f32)
    o = np.broadcast_to(np.array(pos, f32), d.shape).copy()
    return o, d
