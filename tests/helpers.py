"""Host-side checkers shared by the tests (CPU only, numpy)."""
from __future__ import annotations

import math

import numpy as np


def rel_err(a, b) -> float:
    """Normwise relative error ||a - b|| / ||b||."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def elem_rel(a, b, floor: float) -> np.ndarray:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor)


def scene_grid(params, lo, hi):
    """Mirror of make_scene() in fluid_gb300/csrc/pbf_api.cu: origin (f32), inv_cell (f32), dims."""
    cell = math.sqrt(params.h2) * 1.001
    origin, dims = [], []
    for a in range(3):
        e0, e1 = float(lo[a]), float(hi[a])
        if params.box_open_mask & (1 << (2 * a)):
            e0 = min(e0, params.clamp_lo[a])
        if params.box_open_mask & (1 << (2 * a + 1)):
            e1 = max(e1, params.clamp_hi[a])
        origin.append(np.float32(e0 - cell))
        dims.append(int(math.ceil((e1 - e0) / cell) + 2))
    return np.array(origin, dtype=np.float32), np.float32(1.0 / cell), dims


def cells_fp32(xs32, params, lo=None, hi=None, cell_off=0):
    """Linear cell ids of FP32 positions, evaluated as the kernel does (IEEE round-to-nearest)."""
    lo = params.box_lo if lo is None else lo
    hi = params.box_hi if hi is None else hi
    origin, inv, dims = scene_grid(params, np.float32(lo), np.float32(hi))
    xs32 = np.asarray(xs32, dtype=np.float32)
    c = np.floor((xs32 - origin) * inv)
    c = np.clip(c, 0, np.array(dims) - 1).astype(np.int64)
    return cell_off + (c[:, 2] * dims[1] + c[:, 1]) * dims[0] + c[:, 0]


def neighbor_sets_fp32(xs32, h2):
    """N(i) = {j != i : fl32(|x_i - x_j|^2) <= fl32(H2)} with no contraction, as CSR ascending.

    Brute force over a coarse grid of the same FP32 positions (exact predicate; the grid
    is only a pruning device, wide enough that no candidate within sqrt(h2) is missed).
    """
    x = np.asarray(xs32, dtype=np.float32)
    n = x.shape[0]
    h2f = np.float32(h2)
    cell = 1.01 * math.sqrt(float(h2))
    key = np.floor((x.astype(np.float64) - x.min(0)) / cell).astype(np.int64)
    dims = key.max(0) + 1
    lin = (key[:, 2] * dims[1] + key[:, 1]) * dims[0] + key[:, 0]
    order = np.argsort(lin, kind="stable")
    sorted_lin = lin[order]
    lists = [[] for _ in range(n)]
    offs = [(dx, dy, dz) for dz in (-1, 0, 1) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]
    for dx, dy, dz in offs:
        nb = key + np.array([dx, dy, dz])
        ok = np.all((nb >= 0) & (nb < dims), axis=1)
        nl = (nb[:, 2] * dims[1] + nb[:, 1]) * dims[0] + nb[:, 0]
        lo_i = np.searchsorted(sorted_lin, nl, "left")
        hi_i = np.searchsorted(sorted_lin, nl, "right")
        for i in np.nonzero(ok & (hi_i > lo_i))[0]:
            js = order[lo_i[i]:hi_i[i]]
            d = x[i] - x[js]                     # float32 elementwise, round to nearest
            r2 = (d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2]
            sel = js[(r2 <= h2f) & (js != i)]
            lists[i].extend(sel.tolist())
    off = np.zeros(n + 1, dtype=np.int64)
    idx = []
    for i in range(n):
        lst = sorted(lists[i])
        idx.extend(lst)
        off[i + 1] = off[i] + len(lst)
    return off, np.asarray(idx, dtype=np.int64)


def csr_sets(off, idx):
    return [set(idx[off[i]:off[i + 1]].tolist()) for i in range(len(off) - 1)]


# ---------------------------------------------------------------------------
# small scenes for the adjoint checks (h = 0.05, s = 0.025, [0,1]^3 box)
# ---------------------------------------------------------------------------

def adjoint_fall_scene(m: int = 6, seed: int = 7):
    """m^3 jittered lattice on the floor with random velocities and a downward push:
    floor stops in the prediction and in the Jacobi iterations."""
    from fluid_gb300.scenes import lattice, physical_params, uniform

    s = 0.025
    p = lattice(m, m, m, s, corner=(0.4, 0.0, 0.4))
    p += uniform(seed, p.size, -0.2 * s, 0.2 * s).reshape(p.shape)
    v = uniform(seed, p.size, -0.3, 0.3, stream=1).reshape(p.shape)
    v[:, 1] -= 0.5
    return p, v, physical_params(0.05, s)


def adjoint_corner_scene(seed: int = 3):
    """5^3 lattice in the x = 0, y = 0 corner moving into it with a z component:
    wall stops, slides along a wall and second stops on the other wall."""
    from fluid_gb300.scenes import lattice, physical_params, uniform

    s = 0.025
    p = lattice(5, 5, 5, s, corner=(0.0, 0.0, 0.3))
    p += uniform(seed, p.size, -0.2 * s, 0.2 * s).reshape(p.shape)
    p = np.clip(p, 0.002, None)
    v = np.tile([-1.5, -1.5, 0.8], (p.shape[0], 1)) + uniform(seed + 1, p.size, -0.2, 0.2).reshape(p.shape)
    return p, v, physical_params(0.05, s)


def adjoint_free_scene(m: int = 8, seed: int = 5):
    """m^3 jittered lattice at rest, far from every wall (a [0,3]^3 box without clip
    planes): no collision for several steps, so the rollout is a smooth map."""
    from fluid_gb300.scenes import lattice, physical_params, uniform

    s = 0.025
    p = lattice(m, m, m, s, corner=(1.0, 2.0, 1.0))
    p += uniform(seed, p.size, -0.008 * s, 0.008 * s).reshape(p.shape)
    prm = physical_params(0.05, s, box_lo=(0.0, 0.0, 0.0), box_hi=(3.0, 3.0, 3.0), clip_planes=(),
                          clamp_lo=(0.0, 0.0, 0.0), clamp_hi=(3.0, 3.0, 3.0))
    return p, np.zeros_like(p), prm
