"""Python binding of the C ABI (include/pbf.h) over ctypes.

``Simulator`` mirrors the reference's ``Particles`` (src/particles.h:105-140): construct
from positions/velocities and a parameter set, ``time_step(dt)``, position / velocity /
density accessors, ``estimate_densities()`` and ``estimate_density_at()``. Every call
goes to libpbf.so; there is no Python or CPU fallback, and loading fails loudly when
the library has not been built.
"""
from __future__ import annotations

import ctypes
import os
from pathlib import Path

import numpy as np

from .params import CParams, PbfParams

# PBF_LIB, when set, names another build of the library (for comparing builds)
LIB_PATH = Path(os.environ.get("PBF_LIB") or Path(__file__).resolve().parent / "_lib" / "libpbf.so")

PBF_OK = 0
ABI_VERSION = 4  # PBF_ABI_VERSION of include/pbf.h that these declarations follow
STATUS = {0: "PBF_OK", 1: "PBF_ERR_INVALID", 2: "PBF_ERR_CUDA", 3: "PBF_ERR_TIMEOUT",
          4: "PBF_ERR_NONFINITE", 5: "PBF_ERR_CAPACITY", 6: "PBF_ERR_NOMEM"}


class PbfError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class CTuning(ctypes.Structure):
    _fields_ = [("block_predict", ctypes.c_int32), ("block_nbr", ctypes.c_int32),
                ("block_solve", ctypes.c_int32), ("block_misc", ctypes.c_int32)]


class CStats(ctypes.Structure):
    _fields_ = [
        ("steps", ctypes.c_uint64),
        ("mean_density_iter0", ctypes.c_double),
        ("mean_density", ctypes.c_double),
        ("max_density_error", ctypes.c_double),
        ("mean_density_error", ctypes.c_double),
        ("min_neighbors", ctypes.c_uint32),
        ("max_neighbors", ctypes.c_uint32),
        ("mean_neighbors", ctypes.c_double),
        ("low_neighbor_count", ctypes.c_uint64),
        ("error_flags", ctypes.c_uint32),
    ]


_lib = None
P = ctypes.c_void_p


def _declare(L):
    st = ctypes.c_int
    sz = ctypes.c_size_t
    sigs = {
        "pbf_params_default": (None, [P]),
        "pbf_abi_version": (ctypes.c_int, []),
        "pbf_create": (st, [P, sz, P, P, ctypes.c_int, P]),
        "pbf_batch_create": (st, [P, ctypes.c_int, P, P, P, P, P, ctypes.c_int, P]),
        "pbf_destroy": (st, [P]),
        "pbf_step": (st, [P, ctypes.c_double, ctypes.c_int]),
        "pbf_step_async": (st, [P, ctypes.c_double, ctypes.c_int]),
        "pbf_sync": (st, [P]),
        "pbf_stream": (P, [P]),
        "pbf_get_positions": (st, [P, P]),
        "pbf_get_velocities": (st, [P, P]),
        "pbf_get_densities": (st, [P, P]),
        "pbf_set_state": (st, [P, P, P]),
        "pbf_set_state_device": (st, [P, P, P, P]),
        "pbf_get_state_device": (st, [P, P, P, P, P]),
        "pbf_estimate_densities": (st, [P, P]),
        "pbf_estimate_density_at": (st, [P, sz, P, P]),
        "pbf_get_stats": (st, [P, P]),
        "pbf_get_neighbors": (st, [P, P, P, sz, P]),
        "pbf_get_cells": (st, [P, P]),
        "pbf_get_predicted": (st, [P, P]),
        "pbf_get_tuning": (st, [P, P]),
        "pbf_set_tuning": (st, [P, P]),
        "pbf_autotune": (st, [P, ctypes.c_double, ctypes.c_int, P]),
        "pbf_sort": (st, [P]),
        "pbf_snapshot": (st, [P]),
        "pbf_restore": (st, [P]),
        "pbf_set_profiling": (st, [P, ctypes.c_int]),
        "pbf_get_phase_times": (st, [P, P, P, ctypes.c_int]),
        "pbf_reset_phase_times": (st, [P]),
        "pbf_num_phases": (ctypes.c_int, []),
        "pbf_phase_name": (ctypes.c_char_p, [ctypes.c_int]),
        "pbf_density_noalloc": (st, [P, sz, P, P, P]),
        "pbf_adjoint_step_device": (st, [P, ctypes.c_double, P, P, P, P, P, P, P, P, P, P]),
        "pbf_surface": (st, [P, ctypes.c_double, ctypes.c_double, P, P, P, P, sz, P]),
        "pbf_mc_table": (None, [P, P, P]),
        "pbf_set_collider_mesh": (st, [P, sz, P]),
        "pbf_size": (sz, [P]),
        "pbf_num_scenes": (ctypes.c_int, [P]),
        "pbf_last_error": (ctypes.c_char_p, [P]),
    }
    for name, (res, args) in sigs.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    return L


def lib():
    """Load libpbf.so (built by ``fluid_gb300.build``); raise if it is missing."""
    global _lib
    if _lib is None:
        if not LIB_PATH.exists():
            raise FileNotFoundError(
                f"{LIB_PATH} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
        L = _declare(ctypes.CDLL(str(LIB_PATH)))
        if L.pbf_abi_version() != ABI_VERSION:
            raise ImportError(f"{LIB_PATH} has ABI version {L.pbf_abi_version()}, expected {ABI_VERSION}: rebuild it")
        _lib = L
    return _lib


def mc_table():
    """The marching-cubes triangulation table of pbf_surface: (edges[256] u16, ntri[256] u8,
    tri[256, 15] i8 as edge triples)."""
    edges = np.zeros(256, dtype=np.uint16)
    ntri = np.zeros(256, dtype=np.uint8)
    tri = np.zeros((256, 15), dtype=np.int8)
    lib().pbf_mc_table(_ptr(edges), _ptr(ntri), _ptr(tri))
    return edges, ntri, tri


def default_params_c() -> CParams:
    c = CParams()
    lib().pbf_params_default(ctypes.byref(c))
    return c


def _f32(a, shape_last=3):
    a = np.ascontiguousarray(a, dtype=np.float32)
    if a.ndim != 2 or a.shape[1] != shape_last:
        raise ValueError(f"expected an (n, {shape_last}) array")
    return a


def _ptr(a):
    return None if a is None else a.ctypes.data_as(P)


class Simulator:
    """A GPU PBF simulator over one scene or a batch of independent scenes."""

    def __init__(self, pos, vel=None, params: PbfParams | None = None, device: int = 0,
                 counts=None, boxes=None):
        L = lib()
        self._h = P()
        self.params = params or PbfParams()
        cp = self.params.to_c()
        pos = _f32(pos)
        vel = None if vel is None else _f32(vel)
        if vel is not None and vel.shape != pos.shape:
            raise ValueError("vel must match pos")
        self.n = pos.shape[0]
        if counts is None:
            rc = L.pbf_create(ctypes.byref(cp), self.n, _ptr(pos), _ptr(vel), device, ctypes.byref(self._h))
        else:
            cnt = np.ascontiguousarray(counts, dtype=np.uint64)
            if int(cnt.sum()) != self.n:
                raise ValueError("counts must sum to the number of particles")
            lo = hi = None
            if boxes is not None:
                lo = np.ascontiguousarray([b[0] for b in boxes], dtype=np.float32)
                hi = np.ascontiguousarray([b[1] for b in boxes], dtype=np.float32)
            rc = L.pbf_batch_create(ctypes.byref(cp), len(cnt), _ptr(cnt), _ptr(lo), _ptr(hi), _ptr(pos),
                                    _ptr(vel), device, ctypes.byref(self._h))
        if rc != PBF_OK:
            raise PbfError(rc, L.pbf_last_error(None).decode())

    # -- lifetime ---------------------------------------------------------------
    def close(self):
        if self._h:
            lib().pbf_destroy(self._h)
            self._h = P()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _check(self, rc):
        if rc != PBF_OK:
            raise PbfError(rc, lib().pbf_last_error(self._h).decode())

    # -- stepping -----------------------------------------------------------------
    def time_step(self, dt: float = 0.0, steps: int = 1):
        """Particles::timeStep(dt) (particles.cpp:250-297); dt <= 0 uses params.dt."""
        self._check(lib().pbf_step(self._h, float(dt), int(steps)))

    def step_async(self, dt: float = 0.0, steps: int = 1):
        self._check(lib().pbf_step_async(self._h, float(dt), int(steps)))

    def sync(self):
        self._check(lib().pbf_sync(self._h))

    @property
    def stream(self) -> int:
        return lib().pbf_stream(self._h) or 0

    # -- accessors ------------------------------------------------------------------
    def positions(self) -> np.ndarray:
        out = np.empty((self.n, 3), dtype=np.float32)
        self._check(lib().pbf_get_positions(self._h, _ptr(out)))
        return out

    def velocities(self) -> np.ndarray:
        out = np.empty((self.n, 3), dtype=np.float32)
        self._check(lib().pbf_get_velocities(self._h, _ptr(out)))
        return out

    def densities(self) -> np.ndarray:
        out = np.empty(self.n, dtype=np.float32)
        self._check(lib().pbf_get_densities(self._h, _ptr(out)))
        return out

    def set_state(self, pos, vel=None):
        pos = _f32(pos)
        vel = None if vel is None else _f32(vel)
        self._check(lib().pbf_set_state(self._h, _ptr(pos), _ptr(vel)))

    def set_state_device(self, pos_ptr: int, vel_ptr: int | None, stream: int = 0):
        self._check(lib().pbf_set_state_device(self._h, P(pos_ptr), P(vel_ptr) if vel_ptr else None,
                                               P(stream) if stream else None))

    def get_state_device(self, pos_ptr: int | None, vel_ptr: int | None, rho_ptr: int | None,
                         stream: int = 0):
        self._check(lib().pbf_get_state_device(self._h, P(pos_ptr) if pos_ptr else None,
                                               P(vel_ptr) if vel_ptr else None,
                                               P(rho_ptr) if rho_ptr else None, P(stream) if stream else None))

    def adjoint_step_device(self, dt: float, pos_ptr: int | None, vel_ptr: int | None,
                            gx_out_ptr: int | None, gv_out_ptr: int | None, gx_in_ptr: int, gv_in_ptr: int,
                            g_rho0_ptr: int, pos_out_ptr: int | None = None, vel_out_ptr: int | None = None,
                            stream: int = 0):
        """pbf_adjoint_step_device: one recorded step from (pos, vel) and its reverse mode.

        All pointers are device addresses of (n, 3) float32 arrays in original order
        (``g_rho0_ptr``: one float64). ``pos_ptr`` None steps from the current state.
        """
        def opt(q):
            return P(q) if q else None
        self._check(lib().pbf_adjoint_step_device(
            self._h, dt, opt(pos_ptr), opt(vel_ptr), opt(gx_out_ptr), opt(gv_out_ptr), P(gx_in_ptr),
            P(gv_in_ptr), P(g_rho0_ptr), opt(pos_out_ptr), opt(vel_out_ptr), opt(stream)))

    def set_collider_mesh(self, tri=None):
        """Collider triangles besides the box walls: (m, 9) p1 p2 p3 (None or empty removes them)."""
        if tri is None or len(tri) == 0:
            self._check(lib().pbf_set_collider_mesh(self._h, 0, None))
            return
        t = np.ascontiguousarray(tri, dtype=np.float32).reshape(-1, 9)
        self._check(lib().pbf_set_collider_mesh(self._h, t.shape[0], _ptr(t)))

    def surface(self, iso: float | None = None, step: float | None = None, lo=None, hi=None):
        """Particles::getSurfacePrims (particles.cpp:352-385) on the current state: the
        marching-cubes surface of the density field as (xyz, nrm), each (T, 3, 3) float32.
        Defaults are updateSurface's (iso 0.95 rest density, step 0.5 h) and the
        reference's fixed bounds [-1, 1] x [0, 1.5] x [-1, 1]."""
        iso = 0.95 * self.params.rest_density if iso is None else float(iso)
        step = 0.5 * self.params.h if step is None else float(step)
        lo_a = None if lo is None else np.ascontiguousarray(lo, dtype=np.float64)
        hi_a = None if hi is None else np.ascontiguousarray(hi, dtype=np.float64)
        count = ctypes.c_size_t(0)
        self._check(lib().pbf_surface(self._h, iso, step, _ptr(lo_a), _ptr(hi_a), None, None, 0,
                                      ctypes.byref(count)))
        t = count.value
        xyz = np.zeros((max(t, 1), 3, 3), dtype=np.float32)
        nrm = np.zeros((max(t, 1), 3, 3), dtype=np.float32)
        self._check(lib().pbf_surface(self._h, iso, step, _ptr(lo_a), _ptr(hi_a), _ptr(xyz), _ptr(nrm), t,
                                      ctypes.byref(count)))
        return xyz[:t], nrm[:t]

    def estimate_densities(self) -> np.ndarray:
        """Particles::estimateDensities (particles.cpp:440-444): self term included."""
        out = np.empty(self.n, dtype=np.float32)
        self._check(lib().pbf_estimate_densities(self._h, _ptr(out)))
        return out

    def estimate_density_at(self, pts) -> np.ndarray:
        """Particles::estimateDensityAt (particles.cpp:446-453) at each row of pts."""
        pts = _f32(pts)
        out = np.empty(pts.shape[0], dtype=np.float32)
        self._check(lib().pbf_estimate_density_at(self._h, pts.shape[0], _ptr(pts), _ptr(out)))
        return out

    def stats(self) -> dict:
        s = CStats()
        self._check(lib().pbf_get_stats(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in CStats._fields_}

    def neighbors(self):
        """Neighbour sets of the last step in original ids: (offsets[n+1], ids), ascending."""
        counts = np.zeros(self.n, dtype=np.uint32)
        total = ctypes.c_size_t(0)
        self._check(lib().pbf_get_neighbors(self._h, _ptr(counts), None, 0, ctypes.byref(total)))
        ids = np.zeros(max(total.value, 1), dtype=np.uint32)
        self._check(lib().pbf_get_neighbors(self._h, _ptr(counts), _ptr(ids), ids.size, ctypes.byref(total)))
        off = np.zeros(self.n + 1, dtype=np.int64)
        off[1:] = np.cumsum(counts)
        return off, ids[: total.value]

    def cells(self) -> np.ndarray:
        out = np.zeros(self.n, dtype=np.uint32)
        self._check(lib().pbf_get_cells(self._h, _ptr(out)))
        return out

    def tuning(self) -> dict:
        t = CTuning()
        self._check(lib().pbf_get_tuning(self._h, ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in CTuning._fields_}

    def set_tuning(self, **kw):
        cur = self.tuning()
        cur.update(kw)
        t = CTuning(**cur)
        self._check(lib().pbf_set_tuning(self._h, ctypes.byref(t)))

    def autotune(self, dt: float = 0.0, reps: int = 3) -> dict:
        """Pick the fastest launch shape per kernel family on the current state."""
        t = CTuning()
        self._check(lib().pbf_autotune(self._h, float(dt), int(reps), ctypes.byref(t)))
        return {k: getattr(t, k) for k, _ in CTuning._fields_}

    def sort(self):
        self._check(lib().pbf_sort(self._h))

    def snapshot(self):
        self._check(lib().pbf_snapshot(self._h))

    def restore(self):
        self._check(lib().pbf_restore(self._h))

    def set_profiling(self, on: bool = True):
        self._check(lib().pbf_set_profiling(self._h, 1 if on else 0))

    def reset_phase_times(self):
        self._check(lib().pbf_reset_phase_times(self._h))

    def phase_times(self) -> dict:
        """{phase: (device ms, kernel launches)} accumulated since the last reset."""
        k = lib().pbf_num_phases()
        ms = np.zeros(k, dtype=np.float64)
        cnt = np.zeros(k, dtype=np.uint64)
        self._check(lib().pbf_get_phase_times(self._h, _ptr(ms), _ptr(cnt), k))
        return {lib().pbf_phase_name(q).decode(): (float(ms[q]), int(cnt[q])) for q in range(k)}

    def predicted(self) -> np.ndarray:
        out = np.empty((self.n, 3), dtype=np.float32)
        self._check(lib().pbf_get_predicted(self._h, _ptr(out)))
        return out
