"""Seeded synthetic PBF scenes (the five workload configurations) and the particle XML format.

All randomness comes from a project-owned counter-based splitmix64 stream, so a scene
is a pure function of (name, seed) on every machine. Positions and velocities are
FP64 here; the CUDA path receives them rounded to FP32.

Mass convention. The reference step has implicit unit particle mass
(src/particles.cpp:185-204 sums W without a mass factor and without the self term).
A scene quoted with a physical rest density and lattice spacing s is expressed in the
reference's formulas by ``physical_params``: the rest density is the lattice's own
density, and the dimensional constants the reference tuned at H = 0.3 are carried to
the scene's resolution (see ``physical_params``).
"""
from __future__ import annotations

import math
import xml.etree.ElementTree as ET
from dataclasses import dataclass, field

import numpy as np

from .params import PbfParams, decimal_square

_GAMMA = np.uint64(0x9E3779B97F4A7C15)
_M1 = np.uint64(0xBF58476D1CE4E5B9)
_M2 = np.uint64(0x94D049BB133111EB)


def splitmix64(seed: int, count: int, stream: int = 0) -> np.ndarray:
    """``count`` outputs of splitmix64 started at ``seed + stream * 2**32`` (uint64)."""
    with np.errstate(over="ignore"):
        base = np.uint64((seed + (stream << 32)) & 0xFFFFFFFFFFFFFFFF)
        k = np.arange(1, count + 1, dtype=np.uint64)
        z = base + k * _GAMMA
        z = (z ^ (z >> np.uint64(30))) * _M1
        z = (z ^ (z >> np.uint64(27))) * _M2
        return z ^ (z >> np.uint64(31))


def uniform(seed: int, count: int, lo: float = 0.0, hi: float = 1.0, stream: int = 0) -> np.ndarray:
    u = (splitmix64(seed, count, stream) >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)
    return lo + (hi - lo) * u


def normal(seed: int, count: int, sd: float = 1.0, stream: int = 0) -> np.ndarray:
    """Box-Muller pairs from the uniform stream."""
    m = (count + 1) // 2
    u = uniform(seed, 2 * m, stream=stream)
    u1 = np.maximum(u[0::2], 1e-300)
    u2 = u[1::2]
    r = np.sqrt(-2.0 * np.log(u1))
    z = np.concatenate([r * np.cos(2 * np.pi * u2), r * np.sin(2 * np.pi * u2)])
    return sd * z[:count]


def lattice(nx: int, ny: int, nz: int, spacing: float, corner=(0.0, 0.0, 0.0)) -> np.ndarray:
    """Points (i+1/2)*s from ``corner``, x fastest then y then z."""
    i = np.arange(nx)
    j = np.arange(ny)
    k = np.arange(nz)
    kk, jj, ii = np.meshgrid(k, j, i, indexing="ij")
    pts = np.stack([ii.ravel(), jj.ravel(), kk.ravel()], axis=1).astype(np.float64)
    return (pts + 0.5) * spacing + np.asarray(corner, dtype=np.float64)


def lattice_density(h: float, h2: float, spacing: float) -> float:
    """Density the reference's formula gives a particle inside a perfect cubic lattice.

    particles.cpp:185-204 sums poly6 over neighbours only (no self term), so a lattice of
    spacing s has density sum_{j != i} W(x_i - x_j) = 0.814/s^3 for h = 2s, not 1/s^3.
    """
    m = int(math.ceil(h / spacing)) + 1
    r = np.arange(-m, m + 1) * spacing
    X, Y, Z = np.meshgrid(r, r, r, indexing="ij")
    r2 = X * X + Y * Y + Z * Z
    r2[m, m, m] = np.inf
    w = np.where(r2 < h2, 1.56668147106 * (h2 - r2) ** 3 / h ** 9, 0.0)
    return float(w.sum())


REFERENCE_H = 0.3   # particles.cpp:26: the resolution the reference's constants were tuned at
PAPER_H = 0.1       # Macklin & Mueller (2013) scenes, where tensile k = 0.1 is quoted


def physical_params(h: float, spacing: float, scale: str = "mass", *, xsph_c: float = 0.001,
                    vort_eps: float = 0.001, epsilon: float = 2.0, scorr_k: float = 0.0001,
                    scorr_k_h: float = REFERENCE_H, **kw) -> PbfParams:
    """Reference-formula parameters for a fluid sampled at lattice spacing ``spacing``.

    The reference's formulas are kept exactly; only the constants are chosen here.
    ``scale="mass"`` transfers the reference's dimensional constants to resolution h:
    rest density = the lattice's own density (the configured fluid starts at rest),
    EPSILON (units of |grad C|^2 ~ 1/h^2) times (0.3/h)^2, the tensile K (added to
    lambda ~ h^2) times (h/h_K)^2 where h_K is the resolution K was quoted at, and the
    XSPH / vorticity coefficients (multiplying sums of W ~ number density) divided by
    the rest density. ``scale="ref"`` uses the raw constants with rest density 1/s^3.
    Unspecified parameters take the reference defaults except g = -9.8 y, dt = 1/60
    and a [0,1]^3 collider box.
    """
    h2 = decimal_square(h)
    base = dict(h=h, h2=h2, iters=4, dt=1.0 / 60.0, gravity=(0.0, -9.8, 0.0),
                box_lo=(0.0, 0.0, 0.0), box_hi=(1.0, 1.0, 1.0))
    if scale == "mass":
        rho0 = lattice_density(h, h2, spacing)
        base.update(rest_density=rho0, epsilon=epsilon * (REFERENCE_H / h) ** 2,
                    scorr_k=scorr_k * (h / scorr_k_h) ** 2, xsph_c=xsph_c / rho0, vort_eps=vort_eps / rho0)
    elif scale == "ref":
        base.update(rest_density=1.0 / spacing ** 3, epsilon=epsilon, scorr_k=scorr_k, xsph_c=xsph_c,
                    vort_eps=vort_eps)
    else:
        raise ValueError(f"unknown scale {scale!r}")
    base.update(kw)
    return PbfParams(**base)


@dataclass
class Scene:
    name: str
    pos: np.ndarray            # (N, 3) float64
    vel: np.ndarray            # (N, 3) float64
    params: PbfParams
    steps: int
    seed: int
    counts: list = field(default_factory=list)  # batched scenes: particles per scene
    boxes: list = field(default_factory=list)   # batched scenes: (lo, hi) per scene
    notes: str = ""

    @property
    def n(self) -> int:
        return self.pos.shape[0]


def block4096(seed: int = 1, scale: str = "mass") -> Scene:
    """16^3 lattice, s = 0.05 from the (0,0,0) corner, jitter U(+-0.001), h = 0.1, 60 steps."""
    s = 0.05
    p = lattice(16, 16, 16, s)
    p += uniform(seed, p.size, -0.001, 0.001).reshape(p.shape)
    return Scene("block4096", p, np.zeros_like(p), physical_params(0.1, s, scale=scale), 60, seed,
                 notes=f"xsph/vorticity scale={scale}")


def dam_break_262k(seed: int = 2) -> Scene:
    """64^3 lattice, s = h/2 = 0.0125 (0.8 m cube against the x=0 wall), jitter U(+-1e-4), h = 0.025."""
    h = 0.025
    s = h / 2
    p = lattice(64, 64, 64, s)
    p += uniform(seed, p.size, -1e-4, 1e-4).reshape(p.shape)
    prm = physical_params(h, s, xsph_c=0.01, vort_eps=1e-4)
    return Scene("dam_break_262k", p, np.zeros_like(p), prm, 300, seed,
                 notes="0.8 m cube: the lattice cannot fit an x<0.4 slab at this spacing")


def colliding_blocks_1m(seed: int = 3) -> Scene:
    """Two 64x128x64 lattices (x, y, z), s = h/2 = 0.00625, h = 0.0125, v_x = +-1 + N(0, 0.01^2)."""
    h = 0.0125
    s = h / 2
    a = lattice(64, 128, 64, s, corner=(0.0, 0.0, 0.3))
    b = lattice(64, 128, 64, s, corner=(0.6, 0.0, 0.3))
    p = np.concatenate([a, b])
    p += uniform(seed, p.size, -0.008 * s, 0.008 * s).reshape(p.shape)
    v = normal(seed, p.size, 0.01, stream=1).reshape(p.shape)
    v[: a.shape[0], 0] += 1.0
    v[a.shape[0]:, 0] -= 1.0
    prm = physical_params(h, s, scorr_k=0.1, scorr_k_h=PAPER_H, scorr_n=4)
    return Scene("colliding_blocks_1m", p, v, prm, 200, seed,
                 notes="blocks 0.4x0.8x0.4 m at x in [0,0.4) and [0.6,1.0); position jitter +-0.8% of s")


def _block_of(count: int, s: float, corner_sel: int, box=(0.0, 1.0)) -> np.ndarray:
    side = int(math.ceil(count ** (1.0 / 3.0)))
    p = lattice(side, side, side, s)[:count]
    ext = side * s
    lo, hi = box
    corner = [hi - ext if (corner_sel >> a) & 1 else lo for a in range(3)]
    corner[1] = lo  # blocks rest on the floor corner of their box
    return p + np.asarray(corner)


def batched_counts(seed: int = 4, n_scenes: int = 256, lo: int = 2048, hi: int = 32768) -> list:
    """Particle counts of the batched workload's scenes: log-uniform in [lo, hi]."""
    u = uniform(seed, n_scenes, math.log(lo), math.log(hi))
    return [int(round(math.exp(x))) for x in u]


def batched_256(seed: int = 4, n_scenes: int = 256, lo: int = 2048, hi: int = 32768) -> Scene:
    """256 independent [0,1]^3 scenes, counts log-uniform in [2k, 32k], h = 0.05, s = 0.025."""
    h = 0.05
    s = h / 2
    counts = batched_counts(seed, n_scenes, lo, hi)
    corners = (splitmix64(seed, n_scenes, stream=2) >> np.uint64(61)).astype(int)
    vels = uniform(seed, 3 * n_scenes, -0.5, 0.5, stream=3).reshape(n_scenes, 3)
    jit_total = sum(counts) * 3
    jit = uniform(seed, jit_total, -0.008 * s, 0.008 * s, stream=4)
    ps, vs = [], []
    off = 0
    for i, c in enumerate(counts):
        p = _block_of(c, s, int(corners[i]), (0.0, 1.0))
        p += jit[off: off + 3 * c].reshape(c, 3)
        off += 3 * c
        ps.append(p)
        vs.append(np.broadcast_to(vels[i], (c, 3)).copy())
    prm = physical_params(h, s)
    boxes = [((0.0, 0.0, 0.0), (1.0, 1.0, 1.0))] * n_scenes
    return Scene("batched_256", np.concatenate(ps), np.concatenate(vs), prm, 120, seed,
                 counts=counts, boxes=boxes,
                 notes="per-scene block velocity; block at a random box corner on the floor")


def adjoint_32k(seed: int = 5) -> Scene:
    """32^3 lattice, s = 0.025, h = 0.05, 30 steps, zero initial velocity.

    Four Jacobi iterations cannot hold the 0.8 m column up: it compresses to ~3.3x the
    rest density by step 30 (the FP64 restatement does the same), with up to ~230
    neighbours per particle, so the neighbour capacity is 512."""
    h = 0.05
    s = h / 2
    p = lattice(32, 32, 32, s, corner=(0.1, 0.0, 0.1))
    p += uniform(seed, p.size, -0.008 * s, 0.008 * s).reshape(p.shape)
    return Scene("adjoint_32k", p, np.zeros_like(p), physical_params(h, s, max_neighbors=512), 30, seed,
                 notes="column compresses under 4 Jacobi iterations; max_neighbors 512")


SCENES = {
    "block4096": block4096,
    "dam_break_262k": dam_break_262k,
    "colliding_blocks_1m": colliding_blocks_1m,
    "batched_256": batched_256,
    "adjoint_32k": adjoint_32k,
}


# ---------------------------------------------------------------------------
# Particle XML (the format of Application::load_particles, application.cpp:302-344)
# ---------------------------------------------------------------------------

def write_xml(path, pos: np.ndarray, vel: np.ndarray, rest_density: float, params: PbfParams | None = None) -> None:
    """Write ``<particles><density/><ps><particle><pos/><v/>...``.

    Optional ``<params>`` children (h, h2, iters, dt, ...) are an extension that the
    reference loader ignores; the C++ loader reads them when present.
    """
    root = ET.Element("particles")
    ET.SubElement(root, "density").text = repr(float(rest_density))
    if params is not None:
        pe = ET.SubElement(root, "params")
        for key in ("h", "h2", "iters", "scorr_n", "epsilon", "scorr_k", "scorr_dq",
                    "vort_eps", "xsph_c", "dt"):
            ET.SubElement(pe, key).text = repr(float(getattr(params, key))) if key != "iters" and key != "scorr_n" \
                else str(int(getattr(params, key)))
        ET.SubElement(pe, "gravity").text = " ".join(repr(float(x)) for x in params.gravity)
        ET.SubElement(pe, "box_lo").text = " ".join(repr(float(x)) for x in params.box_lo)
        ET.SubElement(pe, "box_hi").text = " ".join(repr(float(x)) for x in params.box_hi)
    ps = ET.SubElement(root, "ps")
    for p, v in zip(np.asarray(pos, dtype=np.float64).tolist(), np.asarray(vel, dtype=np.float64).tolist()):
        pe = ET.SubElement(ps, "particle")
        ET.SubElement(pe, "pos").text = f"{p[0]!r} {p[1]!r} {p[2]!r}"
        ET.SubElement(pe, "v").text = f"{v[0]!r} {v[1]!r} {v[2]!r}"
    ET.SubElement(root, "fs")
    ET.ElementTree(root).write(path)
