"""Scene description for the path tracer (PathTracer, src/pathtracer.cpp) and the
Cornell box it is used with.

The reference builds its scene from a COLLADA file: triangle meshes with one BSDF
each, lights and a camera placed by target / angles / distance (Camera::place,
src/camera.cpp:33-46). Here a scene is plain arrays: triangles with vertex normals, a
material index per triangle, the materials and the lights. The fluid's surface is
added by the renderer itself (DiffuseBSDF(0.1, 0.1, 0.8) as Particles::updateSurface,
src/particles.cpp:392-401).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

# BSDF kinds (src/bsdf.h)
DIFFUSE, MIRROR, GLASS, REFRACTION, EMISSION = 0, 1, 2, 3, 4
# light kinds (src/static_scene/light.h)
DIRECTIONAL, HEMISPHERE, POINT, AREA = 0, 1, 2, 3

FLUID_ALBEDO = (0.1, 0.1, 0.8)  # src/particles.cpp:398


@dataclass
class Material:
    """kind DIFFUSE: c1 = albedo; MIRROR: c1 = reflectance; GLASS: c1 = transmittance,
    c2 = reflectance, ior; REFRACTION: c1 = transmittance, ior (the reference's
    RefractionBSDF::sample_f returns black); EMISSION: c1 = radiance."""
    kind: int
    c1: tuple = (0.0, 0.0, 0.0)
    c2: tuple = (0.0, 0.0, 0.0)
    ior: float = 1.0


@dataclass
class Light:
    """DIRECTIONAL: direction of travel; HEMISPHERE: radiance only; POINT: position;
    AREA: centre position, direction of emission (a point p is lit where
    dot(light point - p, direction) < 0), edge vectors dim_x and dim_y."""
    kind: int
    radiance: tuple
    position: tuple = (0.0, 0.0, 0.0)
    direction: tuple = (0.0, 0.0, 0.0)
    dim_x: tuple = (0.0, 0.0, 0.0)
    dim_y: tuple = (0.0, 0.0, 0.0)


@dataclass
class CameraDesc:
    """Camera::configure (fields of view in degrees, clip distances) and Camera::place
    (target, polar angle phi from +y, azimuth theta, distance r clamped to [min_r, max_r])."""
    hfov: float
    vfov: float
    nclip: float
    fclip: float
    target: tuple
    phi: float
    theta: float
    r: float
    min_r: float = 0.0
    max_r: float = 1e9


@dataclass
class RenderScene:
    tri: np.ndarray            # (T, 3, 3) vertices
    nrm: np.ndarray            # (T, 3, 3) vertex normals
    tri_mat: np.ndarray        # (T,) material index
    materials: list = field(default_factory=list)
    lights: list = field(default_factory=list)

    def __post_init__(self):
        self.tri = np.ascontiguousarray(self.tri, dtype=np.float64).reshape(-1, 3, 3)
        self.nrm = np.ascontiguousarray(self.nrm, dtype=np.float64).reshape(-1, 3, 3)
        self.tri_mat = np.ascontiguousarray(self.tri_mat, dtype=np.int64).reshape(-1)
        if not (len(self.tri) == len(self.nrm) == len(self.tri_mat)):
            raise ValueError("tri, nrm and tri_mat differ in length")
        if len(self.tri_mat) and (self.tri_mat.min() < 0 or self.tri_mat.max() >= len(self.materials)):
            raise ValueError("material index out of range")


def _quad(a, b, c, d, n):
    """Two triangles (a, b, c), (a, c, d) with the vertex normal n."""
    t = np.array([[a, b, c], [a, c, d]], dtype=np.float64)
    return t, np.broadcast_to(np.asarray(n, dtype=np.float64), (2, 3, 3)).copy()


def cornell_box(lo=(0.0, 0.0, 0.0), hi=(1.0, 1.0, 1.0), *, light: float = 5.0, open_front: bool = True,
                glass_block: bool = False):
    """A Cornell box on [lo, hi] (floor y = lo, ceiling y = hi, front face z = hi open):
    white floor, ceiling and back wall, red left wall, blue right wall (the albedos of the
    reference's dae/sky/CBempty.dae), a 0.4 x 0.3 area light of radiance `light` just
    under the ceiling, and a camera in front of the open face. Returns (RenderScene,
    CameraDesc)."""
    lo = np.asarray(lo, dtype=np.float64)
    hi = np.asarray(hi, dtype=np.float64)
    x0, y0, z0 = lo
    x1, y1, z1 = hi
    mats = [Material(DIFFUSE, (0.6, 0.6, 0.6)), Material(DIFFUSE, (0.6, 0.2, 0.2)),
            Material(DIFFUSE, (0.2, 0.2, 0.6))]
    tris, nrms, ids = [], [], []

    def add(q, m):
        tris.append(q[0])
        nrms.append(q[1])
        ids.extend([m, m])

    add(_quad((x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1), (0, 1, 0)), 0)   # floor
    add(_quad((x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (x1, y1, z0), (0, -1, 0)), 0)  # ceiling
    add(_quad((x0, y0, z0), (x0, y1, z0), (x1, y1, z0), (x1, y0, z0), (0, 0, 1)), 0)   # back
    add(_quad((x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0), (1, 0, 0)), 1)   # left (red)
    add(_quad((x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1), (-1, 0, 0)), 2)  # right (blue)
    if not open_front:
        add(_quad((x0, y0, z1), (x0, y1, z1), (x1, y1, z1), (x1, y0, z1), (0, 0, -1)), 0)
    if glass_block:
        mats.append(Material(GLASS, (1.0, 1.0, 1.0), (1.0, 1.0, 1.0), 1.5))
        mats.append(Material(MIRROR, (0.9, 0.9, 0.9)))
        s = 0.15 * (x1 - x0)
        cx, cz = x0 + 0.3 * (x1 - x0), z0 + 0.35 * (z1 - z0)
        add(_quad((cx - s, y0 + 2 * s, cz - s), (cx - s, y0 + 2 * s, cz + s), (cx + s, y0 + 2 * s, cz + s),
                  (cx + s, y0 + 2 * s, cz - s), (0, 1, 0)), len(mats) - 2)
        mx = x0 + 0.75 * (x1 - x0)
        add(_quad((mx, y0, z0 + 0.1), (mx, y0, z0 + 0.5), (mx, y0 + 0.5 * (y1 - y0), z0 + 0.5),
                  (mx, y0 + 0.5 * (y1 - y0), z0 + 0.1), (-1, 0, 0)), len(mats) - 1)
    scene = RenderScene(np.concatenate(tris), np.concatenate(nrms), np.array(ids), mats,
                        [Light(AREA, (light, light, light), position=((x0 + x1) / 2, y1 - 0.01 * (y1 - y0), (z0 + z1) / 2),
                               direction=(0.0, -1.0, 0.0), dim_x=(0.4 * (x1 - x0), 0.0, 0.0),
                               dim_y=(0.0, 0.0, 0.3 * (z1 - z0)))])
    size = float(max(x1 - x0, y1 - y0))
    # aimed slightly off the box's centre, so that no camera ray meets a box edge exactly
    # (on an exact tie between two triangles the closest hit depends on traversal order)
    cam = CameraDesc(hfov=49.13434, vfov=38.0, nclip=0.1 * size, fclip=100.0 * size,
                     target=((x0 + x1) / 2 + 0.0123 * size, (y0 + y1) / 2 + 0.0371 * size, (z0 + z1) / 2),
                     phi=np.pi / 2 - 0.013, theta=0.011, r=2.1 * size, min_r=0.0, max_r=1e9)
    return scene, cam
