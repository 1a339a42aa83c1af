"""Run the reference's own PBF step (oracle/_ref/pbf_ref_driver) on numpy inputs.

Test infrastructure only (the oracle): tests, the fixture generator and bench.py's
CPU-baseline leg call this; the product path never does. The driver binary is built by
oracle/ref/build_ref.py from the reference's sources; its I/O format is described in
oracle/ref/ref_driver.cpp.
"""
from __future__ import annotations

import os
import struct
import subprocess
import tempfile
from pathlib import Path

import numpy as np

DRIVER = Path(__file__).resolve().parent / "_ref" / "pbf_ref_driver"


def available() -> bool:
    return DRIVER.is_file() and os.access(DRIVER, os.X_OK)


def run(pos, vel, params, steps: int = 1, mode: str = "jacobi", neighbors: bool = False,
        load_density: bool = False, restart: bool = False, timeout: float | None = None,
        surface: bool = False, mesh=None) -> dict:
    """Run ``steps`` reference steps. ``params`` is a fluid_gb300.params.PbfParams.

    ``restart``: every step starts again from (pos, vel); ``seconds`` then times
    ``steps`` steps of the same input. ``surface``: also the triangles of the
    reference's surface after the steps (Particles::getSurfacePrims with
    updateSurface's arguments): ``surf_xyz`` / ``surf_nrm`` (T, 3, 3), ``surf_cube``.
    ``mesh``: (m, 9) collider triangles added to the box (the reference's BVH holds them
    as MarchingTriangles with the normal ((p2 - p1) x (p3 - p1)).unit()).

    The reference hard-codes gravity on -y, the clip planes z=1 / y=1.49 and the
    clamp box (particles.cpp:57-83, 180); params that disagree are rejected.
    """
    if not available():
        raise FileNotFoundError(f"reference driver not built: {DRIVER}")
    g = params.gravity
    if g[0] != 0.0 or g[2] != 0.0:
        raise ValueError("the reference applies gravity on y only")
    if tuple(params.clip_planes) != ((2, 1.0), (1, 1.49)):
        raise ValueError("the reference's clip planes are fixed at z=1 and y=1.49")
    if tuple(params.clamp_lo) != (-1.0, 0.0, -1.0) or tuple(params.clamp_hi) != (1.0, 1.49, 1.0):
        raise ValueError("the reference's clamp box is fixed")
    if params.scorr_n != 4:
        raise ValueError("the reference's tensile exponent N is a template argument fixed at 4")
    if abs(params.scorr_dq - 0.1) > 0:
        raise ValueError("the reference's delta q is fixed at 0.1 H")
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    vel = np.ascontiguousarray(vel, dtype=np.float64)
    n = pos.shape[0]
    flags = ((2 if neighbors else 0) | (4 if load_density else 0) | (8 if restart else 0) | (16 if surface else 0)
             | (32 if mesh is not None else 0))
    with tempfile.TemporaryDirectory() as td:
        fin = Path(td) / "in.bin"
        fout = Path(td) / "out.bin"
        with open(fin, "wb") as f:
            f.write(b"PBFREFI1")
            f.write(struct.pack("<6q", n, steps, 0 if mode == "literal" else 1, params.iters,
                                flags, params.box_open_mask))
            f.write(struct.pack("<9d", params.h, params.h2, params.dt, -g[1], params.rest_density,
                                params.epsilon, params.scorr_k, params.vort_eps, params.xsph_c))
            f.write(struct.pack("<3d", *params.box_lo))
            f.write(struct.pack("<3d", *params.box_hi))
            f.write(pos.tobytes())
            f.write(vel.tobytes())
            if mesh is not None:
                m = np.ascontiguousarray(mesh, dtype=np.float64).reshape(-1, 9)
                f.write(struct.pack("<q", m.shape[0]))
                f.write(m.tobytes())
        subprocess.run([str(DRIVER), str(fin), str(fout)], check=True, timeout=timeout)
        buf = fout.read_bytes()
    assert buf[:8] == b"PBFREFO1"
    off = 8
    (n2,) = struct.unpack_from("<q", buf, off)
    off += 8
    assert n2 == n

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(buf, dtype=dtype, count=count, offset=off).copy()
        off += a.nbytes
        return a

    out = {
        "pos": take(np.float64, 3 * n).reshape(n, 3),
        "vel": take(np.float64, 3 * n).reshape(n, 3),
        "density": take(np.float64, n),
        "load_density": take(np.float64, n),
    }
    (nnz,) = struct.unpack_from("<q", buf, off)
    off += 8
    out["nbr_offsets"] = take(np.int64, n + 1)
    out["nbr_idx"] = take(np.int64, nnz)
    (out["seconds"],) = struct.unpack_from("<d", buf, off)
    off += 8
    if surface:
        (nt,) = struct.unpack_from("<q", buf, off)
        off += 8
        out["surf_xyz"] = take(np.float64, 9 * nt).reshape(nt, 3, 3)
        out["surf_nrm"] = take(np.float64, 9 * nt).reshape(nt, 3, 3)
        out["surf_cube"] = take(np.int64, nt)
    return out
