"""PBF step parameters, mirroring ``struct pbf_params`` in ``include/pbf.h``.

Defaults are the reference's compile-time constants (src/particles.cpp:20-44, the
gravity literal at :180, the clip planes at :57-74 and the clamp box at :81-83).
The reference has implicit unit particle mass: ``rest_density`` here is the value the
reference formulas use (for a physical rest density rho0 and lattice spacing s the
mass-consistent value is ``1/s**3``, see :func:`fluid_gb300.scenes.physical_params`).
"""
from __future__ import annotations

import ctypes
from dataclasses import dataclass, field, replace

PBF_FLAG_STATS = 1
PBF_FLAG_GRAPH = 2
PBF_FLAG_KEEP_PREDICTED = 4


class CParams(ctypes.Structure):
    """ctypes image of ``struct pbf_params`` (include/pbf.h)."""

    _fields_ = [
        ("h", ctypes.c_double),
        ("h2", ctypes.c_double),
        ("iters", ctypes.c_int32),
        ("scorr_n", ctypes.c_int32),
        ("epsilon", ctypes.c_double),
        ("scorr_k", ctypes.c_double),
        ("scorr_dq", ctypes.c_double),
        ("vort_eps", ctypes.c_double),
        ("xsph_c", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("gravity", ctypes.c_double * 3),
        ("rest_density", ctypes.c_double),
        ("box_lo", ctypes.c_double * 3),
        ("box_hi", ctypes.c_double * 3),
        ("box_open_mask", ctypes.c_int32),
        ("n_clip", ctypes.c_int32),
        ("clip_axis", ctypes.c_int32 * 2),
        ("clip_value", ctypes.c_double * 2),
        ("clamp_lo", ctypes.c_double * 3),
        ("clamp_hi", ctypes.c_double * 3),
        ("max_neighbors", ctypes.c_int32),
        ("flags", ctypes.c_int32),
    ]


def decimal_square(h: float) -> float:
    """h*h written the way the reference writes H2 (a decimal literal, 0.09 for 0.3)."""
    return float(f"{h * h:.12g}")


@dataclass(frozen=True)
class PbfParams:
    h: float = 0.3                      # H, particles.cpp:26
    h2: float = 0.09                    # H2, particles.cpp:28
    iters: int = 12                     # NEWTON_NUM_STEPS, particles.cpp:34
    scorr_n: int = 4                    # N, particles.cpp:40
    epsilon: float = 2.0                # EPSILON, particles.cpp:36
    scorr_k: float = 0.0001             # K, particles.cpp:38
    scorr_dq: float = 0.1               # delta q / H, particles.cpp:151
    vort_eps: float = 0.001             # VORTICITY_EPSILON, particles.cpp:42
    xsph_c: float = 0.001               # C, particles.cpp:44
    dt: float = 0.016                   # DEFAULT_DELTA_T, particles.cpp:24
    gravity: tuple = (0.0, -10.0, 0.0)  # particles.cpp:180
    rest_density: float = 1000.0        # Particles(double rest_density = 1000.0), particles.h:112
    box_lo: tuple = (-1.0, 0.0, -1.0)   # collider walls (the Cornell box of dae/sky)
    box_hi: tuple = (1.0, 1.5, 1.0)
    box_open_mask: int = 0
    clip_planes: tuple = ((2, 1.0), (1, 1.49))     # particles.cpp:57-74
    clamp_lo: tuple = (-1.0, 0.0, -1.0)            # particles.cpp:81-83
    clamp_hi: tuple = (1.0, 1.49, 1.0)
    max_neighbors: int = 128
    flags: int = PBF_FLAG_STATS

    def with_(self, **kw) -> "PbfParams":
        return replace(self, **kw)

    def to_c(self) -> CParams:
        c = CParams()
        c.h, c.h2, c.iters, c.scorr_n = self.h, self.h2, self.iters, self.scorr_n
        c.epsilon, c.scorr_k, c.scorr_dq = self.epsilon, self.scorr_k, self.scorr_dq
        c.vort_eps, c.xsph_c, c.dt = self.vort_eps, self.xsph_c, self.dt
        c.gravity[:] = list(self.gravity)
        c.rest_density = self.rest_density
        c.box_lo[:] = list(self.box_lo)
        c.box_hi[:] = list(self.box_hi)
        c.box_open_mask = self.box_open_mask
        c.n_clip = len(self.clip_planes)
        for i, (axis, value) in enumerate(self.clip_planes):
            c.clip_axis[i] = axis
            c.clip_value[i] = value
        c.clamp_lo[:] = list(self.clamp_lo)
        c.clamp_hi[:] = list(self.clamp_hi)
        c.max_neighbors = self.max_neighbors
        c.flags = self.flags
        return c


REFERENCE_DEFAULTS = PbfParams()
