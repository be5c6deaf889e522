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
    return dict(type=MAT_LAMBERTIAN, albedo=(1.0, 1.0, 1.0), refract_idx=1.0, roughness=1.0)


def sphere_scene(subdivisions: int = 6, seed: int = 1234, jitter: float = 0.05) -> Scene:
    """Icosphere with each vertex radius scaled by U[1-jitter, 1+jitter]."""
    v, f = icosphere(subdivisions)
    rng = np.random.default_rng(seed)
    r = rng.uniform(1.0 - jitter, 1.0 + jitter, size=(v.shape[0], 1))
    verts = (v * r).astype(np.float32)
    normals = v.astype(np.float32)
    uv = np.zeros((v.shape[0], 2), np.float32)
    return Scene(verts, normals, uv, f, np.zeros(f.shape[0], np.uint32), [_default_material()])


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
