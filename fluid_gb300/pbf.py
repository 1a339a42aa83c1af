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
ABI_VERSION = 6  # PBF_ABI_VERSION of include/pbf.h that these declarations follow
STATUS = {0: "PBF_OK", 1: "PBF_ERR_INVALID", 2: "PBF_ERR_CUDA", 3: "PBF_ERR_TIMEOUT",
          4: "PBF_ERR_NONFINITE", 5: "PBF_ERR_CAPACITY", 6: "PBF_ERR_NOMEM"}


class PbfError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class CTuning(ctypes.Structure):
    _fields_ = [("block_predict", ctypes.c_int32), ("block_nbr", ctypes.c_int32),
                ("block_solve", ctypes.c_int32), ("block_misc", ctypes.c_int32),
                ("gather_depth", ctypes.c_int32), ("list_stream", ctypes.c_int32)]


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


class CMaterial(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32), ("c1", ctypes.c_float * 3), ("c2", ctypes.c_float * 3),
                ("ior", ctypes.c_float)]


class CLight(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_uint32)] + [(k, ctypes.c_float * 3) for k in
                                              ("radiance", "position", "direction", "dim_x", "dim_y")]


class CCameraDesc(ctypes.Structure):
    _fields_ = [("hfov", ctypes.c_double), ("vfov", ctypes.c_double), ("nclip", ctypes.c_double),
                ("fclip", ctypes.c_double), ("target", ctypes.c_double * 3), ("phi", ctypes.c_double),
                ("theta", ctypes.c_double), ("r", ctypes.c_double), ("min_r", ctypes.c_double),
                ("max_r", ctypes.c_double)]


class CCamera(ctypes.Structure):
    _fields_ = [("position", ctypes.c_double * 3), ("c2w", ctypes.c_double * 9), ("hfov", ctypes.c_double),
                ("vfov", ctypes.c_double), ("nclip", ctypes.c_double), ("fclip", ctypes.c_double)]


class CRenderParams(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("ns_aa", ctypes.c_uint32),
                ("max_ray_depth", ctypes.c_uint32), ("ns_area_light", ctypes.c_uint32),
                ("fluid_surface", ctypes.c_uint32), ("surface_bounds", ctypes.c_uint32), ("path_buffer_mib", ctypes.c_uint32),
                ("seed", ctypes.c_uint64), ("isolevel", ctypes.c_double), ("step", ctypes.c_double),
                ("surface_lo", ctypes.c_double * 3), ("surface_hi", ctypes.c_double * 3),
                ("fluid_albedo", ctypes.c_float * 3), ("ray_eps", ctypes.c_float)]


class CRenderStats(ctypes.Structure):
    _fields_ = [("triangles", ctypes.c_uint64), ("surface_triangles", ctypes.c_uint64),
                ("ms_surface", ctypes.c_double), ("ms_bvh", ctypes.c_double), ("ms_trace", ctypes.c_double),
                ("ms_total", ctypes.c_double)]


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
        "pbf_set_collider_spheres": (st, [P, sz, P]),
        "pbf_get_state": (st, [P, P, P, P]),
        "pbf_render_params_default": (None, [P]),
        "pbf_camera_frame": (st, [P, ctypes.c_uint32, ctypes.c_uint32, P]),
        "pbf_render_set_scene": (st, [P, P, P, P, sz, P, sz, P, sz]),
        "pbf_render": (st, [P, P, P, P, P, P]),
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


def camera_frame(cam, width: int, height: int) -> CCamera:
    """Camera::configure + Camera::place of a fluid_gb300.render.CameraDesc (no GPU)."""
    d = CCameraDesc(cam.hfov, cam.vfov, cam.nclip, cam.fclip, (ctypes.c_double * 3)(*cam.target), cam.phi,
                    cam.theta, cam.r, cam.min_r, cam.max_r)
    out = CCamera()
    if lib().pbf_camera_frame(ctypes.byref(d), width, height, ctypes.byref(out)) != PBF_OK:
        raise PbfError(1, "pbf_camera_frame: bad camera")
    return out


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

    def set_collider_spheres(self, xyzr=None):
        """Collider spheres: (m, 4) centre x, y, z and radius (None or empty removes them)."""
        if xyzr is None or len(xyzr) == 0:
            self._check(lib().pbf_set_collider_spheres(self._h, 0, None))
            return
        q = np.ascontiguousarray(xyzr, dtype=np.float32).reshape(-1, 4)
        self._check(lib().pbf_set_collider_spheres(self._h, q.shape[0], _ptr(q)))

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

    def set_render_scene(self, scene):
        """The scene the fluid is rendered in (a fluid_gb300.render.RenderScene)."""
        tri = np.ascontiguousarray(scene.tri, dtype=np.float32).reshape(-1, 9)
        nrm = np.ascontiguousarray(scene.nrm, dtype=np.float32).reshape(-1, 9)
        ids = np.ascontiguousarray(scene.tri_mat, dtype=np.uint32)
        mats = (CMaterial * max(len(scene.materials), 1))(*[
            CMaterial(m.kind, (ctypes.c_float * 3)(*m.c1), (ctypes.c_float * 3)(*m.c2), m.ior)
            for m in scene.materials])
        lights = (CLight * max(len(scene.lights), 1))(*[
            CLight(l.kind, *[(ctypes.c_float * 3)(*getattr(l, k)) for k in
                             ("radiance", "position", "direction", "dim_x", "dim_y")]) for l in scene.lights])
        self._check(lib().pbf_render_set_scene(self._h, _ptr(tri), _ptr(nrm), _ptr(ids), tri.shape[0],
                                               ctypes.cast(mats, P), len(scene.materials), ctypes.cast(lights, P),
                                               len(scene.lights)))

    def render(self, cam, width: int, height: int, ns_aa: int = 1, max_depth: int = 1, ns_area_light: int = 1,
               seed: int = 1, fluid_surface: bool = True, fluid_albedo=(0.1, 0.1, 0.8), ray_eps: float = 0.0,
               hdr: bool = True, rgba: bool = True, lo=None, hi=None, iso: float = 0.0, step: float = 0.0,
               path_buffer_mib: int = 0) -> dict:
        """One frame of PathTracer::render_to_file: ``hdr`` (H, W, 3) float32 with row 0 the
        bottom row, ``rgba`` (H, W, 4) uint8 with the top row first (the reference's PNG),
        ``stats`` (triangles and device milliseconds per phase). ``cam`` is a CameraDesc or
        a CCamera from camera_frame. ``lo`` / ``hi``: the surface grid's bounds (default the
        reference's fixed bounds); ``iso`` / ``step`` <= 0: updateSurface's."""
        frame = cam if isinstance(cam, CCamera) else camera_frame(cam, width, height)
        p = CRenderParams()
        lib().pbf_render_params_default(ctypes.byref(p))
        p.width, p.height, p.ns_aa, p.max_ray_depth, p.ns_area_light = width, height, ns_aa, max_depth, ns_area_light
        p.fluid_surface, p.seed, p.ray_eps = int(bool(fluid_surface)), seed, ray_eps
        p.fluid_albedo = (ctypes.c_float * 3)(*fluid_albedo)
        p.isolevel, p.step = iso, step
        p.path_buffer_mib = path_buffer_mib
        if lo is not None:
            p.surface_bounds = 1
            p.surface_lo = (ctypes.c_double * 3)(*lo)
            p.surface_hi = (ctypes.c_double * 3)(*hi)
        h = np.zeros((height, width, 3), dtype=np.float32) if hdr else None
        c = np.zeros((height, width, 4), dtype=np.uint8) if rgba else None
        st = CRenderStats()
        self._check(lib().pbf_render(self._h, ctypes.byref(frame), ctypes.byref(p), _ptr(h), _ptr(c),
                                     ctypes.byref(st)))
        return {"hdr": h, "rgba": c, "stats": {k: getattr(st, k) for k, _ in CRenderStats._fields_}}

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
