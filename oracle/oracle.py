"""ctypes wrapper of the FP64 restatement oracle (oracle/pbf_oracle.c).

TEST INFRASTRUCTURE (the oracle): imported only by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, as the values results are compared with or the timed CPU baseline. ``build()``
compiles the restatement with ``-ffp-contract=off`` so that x86-64 and aarch64 round
identically; it is called by ``__graft_entry__.build()``.
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent
SRC = HERE / "pbf_oracle.c"
LIB = HERE / "_build" / "libpbf_oracle.so"
LIB32 = HERE / "_build" / "libpbf_oracle_fp32.so"
SRC_ADJ = HERE / "pbf_oracle_adj.c"
LIB_ADJ = HERE / "_build" / "libpbf_oracle_adj.so"
SRC_PT = HERE / "pbf_oracle_pt.c"
LIB_PT = HERE / "_build" / "libpbf_oracle_pt.so"

if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from fluid_gb300.params import PbfParams  # noqa: E402


def build(force: bool = False) -> Path:
    """Build the FP64 restatement, its FP32 twin (same source, -DORC_FLOAT) and the
    FP64 reference gradient (pbf_oracle_adj.c, which includes the restatement) and the
    path tracer's restatement (pbf_oracle_pt.c)."""
    LIB.parent.mkdir(parents=True, exist_ok=True)
    for out, src, extra in ((LIB, SRC, []), (LIB32, SRC, ["-DORC_FLOAT"]), (LIB_ADJ, SRC_ADJ, []),
                            (LIB_PT, SRC_PT, [])):
        newest = src.stat().st_mtime if src == SRC_PT else max(SRC.stat().st_mtime, src.stat().st_mtime)
        if not force and out.exists() and out.stat().st_mtime >= newest:
            continue
        cmd = ["gcc", "-O2", "-std=c11", "-fopenmp", "-ffp-contract=off", "-fno-fast-math",
               "-fPIC", "-shared", "-Wall", *extra, "-o", str(out), str(src), "-lm"]
        subprocess.run(cmd, check=True)
    return LIB


_libs = {}


def lib(fp32: bool = False, adjoint: bool = False):
    path = LIB_ADJ if adjoint else (LIB32 if fp32 else LIB)
    if path not in _libs:
        if not path.exists():
            build()
        L = ctypes.CDLL(str(path))
        P = ctypes.c_void_p
        if adjoint:
            L.orc_step_adjoint.argtypes = [P, ctypes.c_int64, P, P, ctypes.c_double, P, P, P, P, P, P, P,
                                           P, P, P, ctypes.c_int]
            L.orc_step_adjoint.restype = ctypes.c_int
        L.orc_step.argtypes = [P, ctypes.c_int64, P, P, P, ctypes.c_int, ctypes.c_double,
                               P, P, ctypes.c_int64, P, P, ctypes.c_int]
        L.orc_step.restype = ctypes.c_int
        L.orc_step2.argtypes = [P, ctypes.c_int64, P, P, P, ctypes.c_int, ctypes.c_double,
                                P, P, ctypes.c_int64, P, P, P, P, ctypes.c_int]
        L.orc_step2.restype = ctypes.c_int
        L.orc_estimate_densities.argtypes = [P, ctypes.c_int64, P, P, ctypes.c_int]
        L.orc_estimate_densities.restype = ctypes.c_int
        L.orc_estimate_density_at.argtypes = [P, ctypes.c_int64, P, ctypes.c_int64, P, P, ctypes.c_int]
        L.orc_estimate_density_at.restype = ctypes.c_int
        L.orc_max_threads.restype = ctypes.c_int
        L.orc_set_mesh.argtypes = [ctypes.c_int64, P]
        L.orc_set_mesh.restype = ctypes.c_int
        L.orc_set_spheres.argtypes = [ctypes.c_int64, P]
        L.orc_set_spheres.restype = ctypes.c_int
        L.orc_surface.argtypes = [P, ctypes.c_int64, P, ctypes.c_double, ctypes.c_double, P, P, P, P, P, P, P,
                                  ctypes.c_int64, ctypes.c_int]
        L.orc_surface.restype = ctypes.c_int64
        L.orc_nbr_check_fp32.argtypes = [ctypes.c_int64, P, ctypes.c_float, P, P, P, P, P, P, ctypes.c_int]
        L.orc_nbr_check_fp32.restype = ctypes.c_int
        _libs[path] = L
    return _libs[path]


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def step(pos, vel, params: PbfParams, steps: int = 1, dt: float | None = None,
         neighbors: bool = False, predicted: bool = False, threads: int = 0,
         given_neighbors=None, fp32: bool = False) -> dict:
    """``steps`` FP64 steps from (pos, vel); returns pos, vel, density (+ neighbour CSR).

    ``given_neighbors=(offsets, ids)`` replaces the first step's neighbour search;
    ``fp32`` runs the FP32 twin of the restatement (a statistical comparator only).
    """
    L = lib(fp32)
    pos = np.array(pos, dtype=np.float64, order="C", copy=True)
    vel = np.array(vel, dtype=np.float64, order="C", copy=True)
    n = pos.shape[0]
    rho = np.zeros(n, dtype=np.float64)
    cp = params.to_c()
    rho0 = np.zeros(max(steps, 1), dtype=np.float64)
    pred = np.zeros((n, 3), dtype=np.float64) if predicted else None
    off = np.zeros(n + 1, dtype=np.int64) if neighbors else None
    cap = 64 * n if neighbors else 0
    idx = np.zeros(max(cap, 1), dtype=np.int64) if neighbors else None
    dtv = params.dt if dt is None else dt
    pos0, vel0 = pos.copy(), vel.copy()
    g_off = g_idx = None
    if given_neighbors is not None:
        g_off = np.ascontiguousarray(given_neighbors[0], dtype=np.int64)
        g_idx = np.ascontiguousarray(given_neighbors[1], dtype=np.int64)
        if g_idx.size == 0:
            g_idx = np.zeros(1, dtype=np.int64)

    def call():
        return L.orc_step2(ctypes.byref(cp), n, _ptr(pos), _ptr(vel), _ptr(rho), steps, dtv,
                           _ptr(off), _ptr(idx), cap, _ptr(pred), _ptr(rho0), _ptr(g_off), _ptr(g_idx),
                           threads)

    rc = call()
    if rc == 1 and neighbors:  # rerun with the exact capacity the last step needed
        cap = int(off[-1])
        idx = np.zeros(max(cap, 1), dtype=np.int64)
        pos, vel = pos0, vel0.copy()
        rc = call()
    if rc != 0:
        raise RuntimeError(f"orc_step failed: {rc}")
    out = {"pos": pos, "vel": vel, "density": rho, "mean_density_iter0": rho0[:steps]}
    if neighbors:
        out["nbr_offsets"] = off
        out["nbr_idx"] = idx[: off[-1]].copy()
    if predicted:
        out["pred"] = pred
    return out


def check_neighbors_fp32(xs32, h2: float, off, ids, threads: int = 0) -> dict:
    """Compares ascending CSR neighbour lists (``off[n+1]``, ``ids``) with the sets the FP32
    predicate fl32(|x_i - x_j|^2) <= fl32(h2) gives on the FP32 positions ``xs32``.

    Returns the number of particles whose sets differ (``bad``), the pairs the lists miss
    (``missing``) and hold in excess (``extra``), and the first differing particle
    (``first``, -1 if none)."""
    xs = np.ascontiguousarray(xs32, dtype=np.float32).reshape(-1, 3)
    off = np.ascontiguousarray(off, dtype=np.int64)
    ids = np.ascontiguousarray(ids, dtype=np.uint32)
    if ids.size == 0:
        ids = np.zeros(1, dtype=np.uint32)
    if off.shape[0] != xs.shape[0] + 1:
        raise ValueError("offsets must have n + 1 entries")
    out = [ctypes.c_int64(0) for _ in range(4)]
    rc = lib().orc_nbr_check_fp32(xs.shape[0], _ptr(xs), float(np.float32(h2)), _ptr(off), _ptr(ids),
                                  *(ctypes.byref(o) for o in out), threads)
    if rc:
        raise RuntimeError(f"orc_nbr_check_fp32 failed: {rc}")
    return dict(zip(("bad", "missing", "extra", "first"), (o.value for o in out)))


def estimate_densities(pos, params: PbfParams, threads: int = 0) -> np.ndarray:
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    out = np.zeros(pos.shape[0], dtype=np.float64)
    cp = params.to_c()
    rc = lib().orc_estimate_densities(ctypes.byref(cp), pos.shape[0], _ptr(pos), _ptr(out), threads)
    if rc:
        raise RuntimeError(f"orc_estimate_densities failed: {rc}")
    return out


def estimate_density_at(pos, pts, params: PbfParams, threads: int = 0) -> np.ndarray:
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    pts = np.ascontiguousarray(pts, dtype=np.float64)
    out = np.zeros(pts.shape[0], dtype=np.float64)
    cp = params.to_c()
    rc = lib().orc_estimate_density_at(ctypes.byref(cp), pos.shape[0], _ptr(pos), pts.shape[0],
                                       _ptr(pts), _ptr(out), threads)
    if rc:
        raise RuntimeError(f"orc_estimate_density_at failed: {rc}")
    return out


def step_adjoint(pos, vel, params: PbfParams, gx, gv, dt: float | None = None,
                 given_neighbors=None, threads: int = 0) -> dict:
    """One FP64 step and its reverse mode (oracle/pbf_oracle_adj.c).

    ``gx``/``gv``: adjoints of the step's output positions / velocities. Returns the
    adjoints of the inputs (``gx``, ``gv``, ``grho0``) and the step's outputs
    (``pos``, ``vel``) and ``kinds``, the census of collision kinds (not moved, free,
    stop, stop + slide, stop + slide + stop) of the prediction (0-4) and of the Jacobi
    iterations (5-9). ``given_neighbors=(offsets, ids)`` fixes the neighbour sets.
    """
    L = lib(adjoint=True)
    f64 = lambda a: np.ascontiguousarray(a, dtype=np.float64)  # noqa: E731
    pos, vel, gx, gv = f64(pos), f64(vel), f64(gx), f64(gv)
    n = pos.shape[0]
    out = {k: np.zeros((n, 3), dtype=np.float64) for k in ("gx", "gv", "pos", "vel")}
    g0 = ctypes.c_double(0.0)
    kinds = np.zeros(10, dtype=np.int64)
    g_off = g_idx = None
    if given_neighbors is not None:
        g_off = np.ascontiguousarray(given_neighbors[0], dtype=np.int64)
        g_idx = np.ascontiguousarray(given_neighbors[1], dtype=np.int64)
        if g_idx.size == 0:
            g_idx = np.zeros(1, dtype=np.int64)
    cp = params.to_c()
    rc = L.orc_step_adjoint(ctypes.byref(cp), n, _ptr(pos), _ptr(vel), params.dt if dt is None else dt,
                            _ptr(g_off), _ptr(g_idx), _ptr(gx), _ptr(gv), _ptr(out["gx"]), _ptr(out["gv"]),
                            ctypes.byref(g0), _ptr(out["pos"]), _ptr(out["vel"]), _ptr(kinds), threads)
    if rc:
        raise RuntimeError(f"orc_step_adjoint failed: {rc}")
    out["grho0"] = g0.value
    out["kinds"] = kinds
    return out


def rollout_adjoint(pos, vel, params: PbfParams, steps: int, gx, gv, dt: float | None = None,
                    threads: int = 0) -> dict:
    """Reverse mode of ``steps`` FP64 steps: checkpoints (x, v) per step on the way
    forward, recomputes each step's forward inside its reverse call (neighbour sets
    searched again from the checkpoint, as in the forward)."""
    xs, vs = [np.array(pos, dtype=np.float64)], [np.array(vel, dtype=np.float64)]
    for _ in range(steps):
        o = step(xs[-1], vs[-1], params, 1, dt=dt, threads=threads)
        xs.append(o["pos"])
        vs.append(o["vel"])
    gx = np.array(gx, dtype=np.float64)
    gv = np.array(gv, dtype=np.float64)
    g0 = 0.0
    for s in range(steps - 1, -1, -1):
        a = step_adjoint(xs[s], vs[s], params, gx, gv, dt=dt, threads=threads)
        gx, gv, g0 = a["gx"], a["gv"], g0 + a["grho0"]
    return {"gx": gx, "gv": gv, "grho0": g0, "pos": xs[-1], "vel": vs[-1]}


def set_mesh(tri=None, fp32: bool = False) -> None:
    """Collider triangles besides the box walls ((m, 9) p1 p2 p3, None to clear) for the
    following calls (process-wide in the restatement)."""
    L = lib(fp32)
    if tri is None or len(tri) == 0:
        L.orc_set_mesh(0, None)
        return
    t = np.ascontiguousarray(tri, dtype=np.float64).reshape(-1, 9)
    if L.orc_set_mesh(t.shape[0], _ptr(t)) != 0:
        raise ValueError("at most 65536 collider triangles")


def set_spheres(xyzr=None, fp32: bool = False) -> None:
    """Collider spheres ((m, 4) centre and radius, None to clear) for the following calls
    (process-wide in the restatement, like the mesh)."""
    L = lib(fp32)
    if xyzr is None or len(xyzr) == 0:
        L.orc_set_spheres(0, None)
        return
    q = np.ascontiguousarray(xyzr, dtype=np.float64).reshape(-1, 4)
    if L.orc_set_spheres(q.shape[0], _ptr(q)) != 0:
        raise ValueError("at most 1024 collider spheres")


def surface(pos, params: PbfParams, ntri, tri, iso: float | None = None, step: float | None = None,
            lo=(-1.0, 0.0, -1.0), hi=(1.0, 1.5, 1.0), threads: int = 0) -> dict:
    """FP64 Particles::getSurfacePrims (particles.cpp:352-385) with the given triangulation
    table (ntri[256], tri[256 * 15]); defaults are updateSurface's (iso 0.95 rest
    density, step 0.5 h) and the reference's fixed bounds. Returns xyz / nrm (T, 3, 3)
    and the cube index of every triangle."""
    L = lib()
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    iso = 0.95 * params.rest_density if iso is None else iso
    step = 0.5 * params.h if step is None else step
    lo = np.ascontiguousarray(lo, dtype=np.float64)
    hi = np.ascontiguousarray(hi, dtype=np.float64)
    ntri = np.ascontiguousarray(ntri, dtype=np.uint8)
    tri = np.ascontiguousarray(tri, dtype=np.int8)
    cp = params.to_c()

    def run(cap):
        xyz = np.zeros((max(cap, 1), 3, 3))
        nrm = np.zeros((max(cap, 1), 3, 3))
        cube = np.zeros(max(cap, 1), dtype=np.int64)
        total = L.orc_surface(ctypes.byref(cp), pos.shape[0], _ptr(pos), iso, step, _ptr(lo), _ptr(hi), _ptr(ntri),
                              _ptr(tri), _ptr(xyz), _ptr(nrm), _ptr(cube), cap, threads)
        if total < 0:
            raise RuntimeError("orc_surface failed")
        return total, xyz, nrm, cube

    total, *_ = run(0)
    total, xyz, nrm, cube = run(int(total))
    return {"xyz": xyz[:total], "nrm": nrm[:total], "cube": cube[:total]}


class OrcMat(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int64), ("c1", ctypes.c_double * 3), ("c2", ctypes.c_double * 3),
                ("ior", ctypes.c_double)]


class OrcLight(ctypes.Structure):
    _fields_ = [("kind", ctypes.c_int64)] + [(k, ctypes.c_double * 3) for k in
                                             ("radiance", "position", "direction", "dim_x", "dim_y")]


class OrcCam(ctypes.Structure):
    _fields_ = [("pos", ctypes.c_double * 3), ("c2w", ctypes.c_double * 9), ("hfov", ctypes.c_double),
                ("vfov", ctypes.c_double), ("nclip", ctypes.c_double), ("fclip", ctypes.c_double)]


RNG_STD, RNG_COUNTER = 0, 1


def _pt_lib():
    if LIB_PT not in _libs:
        if not LIB_PT.exists():
            build()
        L = ctypes.CDLL(str(LIB_PT))
        P = ctypes.c_void_p
        L.orc_camera_frame.argtypes = [ctypes.c_double] * 4 + [P] + [ctypes.c_double] * 5 + [ctypes.c_int64] * 2 + [P]
        L.orc_camera_frame.restype = None
        L.orc_render.argtypes = [P, P, P, ctypes.c_int64, P, P, ctypes.c_int64, P, ctypes.c_int64, ctypes.c_int64,
                                 ctypes.c_int64, ctypes.c_int64, ctypes.c_int64, ctypes.c_int, ctypes.c_uint64, P, P,
                                 ctypes.c_int]
        L.orc_render.restype = ctypes.c_int
        _libs[LIB_PT] = L
    return _libs[LIB_PT]


def camera_frame(cam, width: int, height: int) -> dict:
    """Camera::configure + Camera::place (camera.cpp:15-46, 92-111): position, c2w
    columns (3, 3), the adjusted fields of view and the clip distances."""
    L = _pt_lib()
    out = OrcCam()
    tgt = np.ascontiguousarray(cam.target, dtype=np.float64)
    L.orc_camera_frame(cam.hfov, cam.vfov, cam.nclip, cam.fclip, _ptr(tgt), cam.phi, cam.theta, cam.r, cam.min_r,
                       cam.max_r, width, height, ctypes.byref(out))
    return {"pos": np.array(out.pos[:]), "c2w": np.array(out.c2w[:]).reshape(3, 3), "hfov": out.hfov,
            "vfov": out.vfov, "nclip": out.nclip, "fclip": out.fclip, "_c": out}


def render(scene, cam, surface_xyz, surface_nrm, width: int, height: int, ns_aa: int = 1, max_depth: int = 1,
           ns_area_light: int = 1, rng: int = RNG_STD, seed: int = 1, threads: int = 0) -> dict:
    """One frame of the restated path tracer over the scene's triangles plus the fluid
    surface triangles (DiffuseBSDF(0.1, 0.1, 0.8)). Returns ``hdr`` (H, W, 3) float32 with
    row 0 at y = 0 (the bottom, as the reference's sample buffer) and ``rgba`` (H, W, 4)
    uint8 in PNG row order (top first)."""
    from fluid_gb300 import render as R

    L = _pt_lib()
    sx = np.asarray(surface_xyz, dtype=np.float64).reshape(-1, 3, 3)
    sn = np.asarray(surface_nrm, dtype=np.float64).reshape(-1, 3, 3)
    mats = list(scene.materials) + [R.Material(R.DIFFUSE, R.FLUID_ALBEDO)]
    tri = np.ascontiguousarray(np.concatenate([scene.tri, sx]))
    nrm = np.ascontiguousarray(np.concatenate([scene.nrm, sn]))
    tri_mat = np.ascontiguousarray(np.concatenate([scene.tri_mat, np.full(len(sx), len(mats) - 1, np.int64)]))
    cm = (OrcMat * len(mats))(*[OrcMat(m.kind, (ctypes.c_double * 3)(*m.c1), (ctypes.c_double * 3)(*m.c2), m.ior)
                                for m in mats])
    cl = (OrcLight * max(len(scene.lights), 1))(*[OrcLight(l.kind, *[(ctypes.c_double * 3)(*getattr(l, k)) for k in
                                                                     ("radiance", "position", "direction", "dim_x",
                                                                      "dim_y")]) for l in scene.lights])
    fr = camera_frame(cam, width, height)
    hdr = np.zeros((height, width, 3), dtype=np.float32)
    rgba = np.zeros((height, width, 4), dtype=np.uint8)
    rc = L.orc_render(_ptr(tri), _ptr(nrm), _ptr(tri_mat), len(tri), ctypes.cast(cm, ctypes.c_void_p),
                      ctypes.cast(cl, ctypes.c_void_p), len(scene.lights), ctypes.byref(fr["_c"]), width, height,
                      ns_aa, max_depth, ns_area_light, rng, seed, _ptr(hdr), _ptr(rgba), threads)
    if rc != 0:
        raise ValueError("orc_render: bad arguments")
    return {"hdr": hdr, "rgba": rgba, "frame": fr}


def max_threads() -> int:
    return int(lib().orc_max_threads())


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
