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
        surface: bool = False, mesh=None, spheres=None) -> dict:
    """Run ``steps`` reference steps. ``params`` is a fluid_gb300.params.PbfParams.

    ``restart``: every step starts again from (pos, vel); ``seconds`` then times
    ``steps`` steps of the same input. ``surface``: also the triangles of the
    reference's surface after the steps (Particles::getSurfacePrims with
    updateSurface's arguments): ``surf_xyz`` / ``surf_nrm`` (T, 3, 3), ``surf_cube``.
    ``mesh``: (m, 9) collider triangles added to the box (the reference's BVH holds them
    as MarchingTriangles with the normal ((p2 - p1) x (p3 - p1)).unit()). ``spheres``:
    (m, 4) centres and radii, the reference's Sphere primitives in the same BVH.

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
             | (32 if mesh is not None else 0) | (64 if spheres is not None else 0))
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
            if spheres is not None:
                q = np.ascontiguousarray(spheres, dtype=np.float64).reshape(-1, 4)
                f.write(struct.pack("<q", q.shape[0]))
                f.write(q.tobytes())
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


RENDER = Path(__file__).resolve().parent / "_ref" / "pbf_ref_render"


def read_png(path) -> np.ndarray:
    """A non-interlaced PNG as lodepng::encode writes it (it picks the smallest colour
    type: grey, RGB, palette or RGBA) -> (H, W, 4) uint8 RGBA."""
    import zlib

    data = Path(path).read_bytes()
    assert data[:8] == b"\x89PNG\r\n\x1a\n", "not a PNG"
    off, idat, w, h, depth, ctype, plte, trns = 8, b"", 0, 0, 8, 6, None, None
    while off < len(data):
        (ln,) = struct.unpack_from(">I", data, off)
        kind = data[off + 4:off + 8]
        body = data[off + 8:off + 8 + ln]
        off += 12 + ln
        if kind == b"IHDR":
            w, h, depth, ctype, _, _, interlace = struct.unpack(">IIBBBBB", body)
            assert interlace == 0 and (depth == 8 or ctype in (0, 3)), "unsupported PNG"
        elif kind == b"PLTE":
            plte = np.frombuffer(body, dtype=np.uint8).reshape(-1, 3)
        elif kind == b"tRNS":
            trns = np.frombuffer(body, dtype=np.uint8)
        elif kind == b"IDAT":
            idat += body
        elif kind == b"IEND":
            break
    chans = {0: 1, 2: 3, 3: 1, 4: 2, 6: 4}[ctype]
    stride = (w * chans * depth + 7) // 8
    bpp = max(1, chans * depth // 8)
    raw = np.frombuffer(zlib.decompress(idat), dtype=np.uint8).reshape(h, 1 + stride)
    rows = np.zeros((h, stride), dtype=np.int32)
    for y in range(h):
        ft, line = raw[y, 0], raw[y, 1:].astype(np.int32)
        prev = rows[y - 1] if y else np.zeros(stride, dtype=np.int32)
        cur = np.zeros(stride, dtype=np.int32)
        for x in range(stride):
            a = cur[x - bpp] if x >= bpp else 0
            b = prev[x]
            c = prev[x - bpp] if x >= bpp else 0
            if ft == 0:
                p = 0
            elif ft == 1:
                p = a
            elif ft == 2:
                p = b
            elif ft == 3:
                p = (a + b) // 2
            else:
                pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                p = a if (pa <= pb and pa <= pc) else (b if pb <= pc else c)
            cur[x] = (line[x] + p) & 255
        rows[y] = cur
    rows = rows.astype(np.uint8)
    if depth < 8:
        bits = np.unpackbits(rows, axis=1).reshape(h, -1, depth)
        vals = np.zeros(bits.shape[:2], dtype=np.int32)
        for k in range(depth):
            vals = vals * 2 + bits[:, :, k]
        samples = vals[:, :w * chans].astype(np.uint8)
    else:
        samples = rows[:, :w * chans]
    px = samples.reshape(h, w, chans)
    out = np.full((h, w, 4), 255, dtype=np.uint8)
    if ctype == 3:
        out[..., :3] = plte[px[..., 0]]
        if trns is not None:
            alpha = np.full(len(plte), 255, dtype=np.uint8)
            alpha[:len(trns)] = trns
            out[..., 3] = alpha[px[..., 0]]
    elif ctype in (0, 4):
        g = px[..., 0] * (255 // ((1 << depth) - 1)) if depth < 8 else px[..., 0]
        out[..., 0] = out[..., 1] = out[..., 2] = g
        if ctype == 4:
            out[..., 3] = px[..., 1]
    else:
        out[..., :chans] = px
    return out


def render_available() -> bool:
    return RENDER.is_file() and os.access(RENDER, os.X_OK)


def render(scene, cam, pos, params, width: int, height: int, ns_aa: int = 1, max_depth: int = 1,
           ns_area_light: int = 1, seed: int = 1, timeout: float | None = None) -> dict:
    """One frame of the reference's PathTracer::render_to_file over ``scene`` (a
    fluid_gb300.render.RenderScene) plus the surface of particles ``pos``, camera ``cam``
    (CameraDesc), random numbers from srand(seed). Returns ``rgba`` (H, W, 4) from the
    PNG, the camera's ``position`` / ``up`` / ``vfov`` after configure + place, the fluid
    surface triangles ``surf_xyz`` / ``surf_nrm`` (T, 3, 3) and ``seconds``."""
    if not render_available():
        raise FileNotFoundError(f"reference renderer not built: {RENDER}")
    pos = np.ascontiguousarray(pos, dtype=np.float64)
    with tempfile.TemporaryDirectory() as td:
        fin, fpng, fout = Path(td) / "in.bin", Path(td) / "out.png", Path(td) / "out.bin"
        with open(fin, "wb") as f:
            f.write(b"PBFRNDI1")
            f.write(struct.pack("<10q", len(pos), width, height, ns_aa, max_depth, ns_area_light, seed,
                                len(scene.tri), len(scene.materials), len(scene.lights)))
            f.write(struct.pack("<3d", params.h, params.h2, params.rest_density))
            f.write(pos.tobytes())
            f.write(np.ascontiguousarray(scene.tri, dtype=np.float64).tobytes())
            f.write(np.ascontiguousarray(scene.nrm, dtype=np.float64).tobytes())
            f.write(np.ascontiguousarray(scene.tri_mat, dtype=np.int64).tobytes())
            for m in scene.materials:
                f.write(struct.pack("<q7d", m.kind, *m.c1, *m.c2, m.ior))
            for l in scene.lights:
                f.write(struct.pack("<q15d", l.kind, *l.radiance, *l.position, *l.direction, *l.dim_x, *l.dim_y))
            f.write(struct.pack("<12d", cam.hfov, cam.vfov, cam.nclip, cam.fclip, *cam.target, cam.phi, cam.theta,
                                cam.r, cam.min_r, cam.max_r))
        subprocess.run([str(RENDER), str(fin), str(fpng), str(fout)], check=True, timeout=timeout,
                       stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
        rgba = read_png(fpng)
        buf = fout.read_bytes()
    assert buf[:8] == b"PBFRNDO1"
    off = 8
    position = np.frombuffer(buf, np.float64, 3, off); off += 24
    up = np.frombuffer(buf, np.float64, 3, off); off += 24
    (vfov,) = struct.unpack_from("<d", buf, off); off += 8
    (nt,) = struct.unpack_from("<q", buf, off); off += 8
    sxyz = np.frombuffer(buf, np.float64, 9 * nt, off).reshape(nt, 3, 3); off += 72 * nt
    snrm = np.frombuffer(buf, np.float64, 9 * nt, off).reshape(nt, 3, 3); off += 72 * nt
    (seconds,) = struct.unpack_from("<d", buf, off)
    return {"rgba": rgba, "position": position.copy(), "up": up.copy(), "vfov": vfov, "surf_xyz": sxyz.copy(),
            "surf_nrm": snrm.copy(), "seconds": seconds}
