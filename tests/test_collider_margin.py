"""The collider's shortcut (pbf_device.cuh clear_move): a move that starts and ends inside
the scene's interior box (the closed walls and the clamp box shrunk by 1e-4 of the largest
coordinate among them) and keeps that margin from every clip plane is added unchanged,
without the general path's stop distances. That is only right if the general path, in FP32,
would find no wall and no plane within the move and clamp nothing. This checks it with the
general path's FP32 arithmetic (numpy float32: IEEE rounding of each operation) on random
moves and on moves that end exactly at the margin, for the default scene and a batched one.
"""
from __future__ import annotations

import numpy as np

F = np.float32
MARGIN = 1e-4  # kInteriorMargin


def interior_box(lo, hi, clamp_lo, clamp_hi, open_mask=0):
    scale = max([1.0] + [abs(float(v)) for v in (*lo, *hi, *clamp_lo, *clamp_hi)])
    m = MARGIN * scale
    ilo, ihi = [], []
    for a in range(3):
        l, h = float(clamp_lo[a]), float(clamp_hi[a])
        if not open_mask & (1 << (2 * a)):
            l = max(l, float(lo[a]))
        if not open_mask & (1 << (2 * a + 1)):
            h = min(h, float(hi[a]))
        ilo.append(F(l + m))
        ihi.append(F(h - m))
    return np.array(ilo, F), np.array(ihi, F)


def general_path_is_free(p, delta, lo, hi, clamp_lo, clamp_hi, clips):
    """collide()'s general path in FP32 (slide or not does not matter when nothing is hit):
    True when no clip plane or wall stops the move and the clamp box changes nothing."""
    s2 = F(F(F(delta[0] * delta[0]) + F(delta[1] * delta[1])) + F(delta[2] * delta[2]))
    l = F(np.sqrt(s2))
    if not l > F(1e-11):
        return True
    inv = F(F(1.0) / l)
    d = (delta * inv).astype(F)
    for axis, value in clips:
        if d[axis] != 0:
            pt = F(F(F(value) - p[axis]) / d[axis])
            if F(0) < pt < l:
                return False
    for a in range(3):
        if d[a] < 0:
            tt = max(F(F(F(lo[a]) - p[a]) / d[a]), F(0))
            if tt <= l:
                return False
        elif d[a] > 0:
            tt = max(F(F(F(hi[a]) - p[a]) / d[a]), F(0))
            if tt <= l:
                return False
    q = (p + delta).astype(F)
    return bool(np.all(q >= np.asarray(clamp_lo, F)) and np.all(q <= np.asarray(clamp_hi, F)))


def shortcut_accepts(p, delta, ilo, ihi, clips, clip_margin):
    s2 = F(F(F(delta[0] * delta[0]) + F(delta[1] * delta[1])) + F(delta[2] * delta[2]))
    if not s2 > F(1e-22) * F(1.001):
        return False
    e = (p + delta).astype(F)
    if not (np.all(np.minimum(p, e) > ilo) and np.all(np.maximum(p, e) < ihi)):
        return False
    for axis, value in clips:
        u, w = p[axis], e[axis]
        if not (min(u, w) > F(value) + clip_margin or max(u, w) < F(value) - clip_margin):
            return False
    return True


def _check(lo, hi, clamp_lo, clamp_hi, clips, seed):
    ilo, ihi = interior_box(lo, hi, clamp_lo, clamp_hi)
    clip_margin = F(MARGIN * max([1.0] + [abs(v) for _, v in clips]))
    rng = np.random.default_rng(seed)
    accepted = 0
    for k in range(20000):
        p = rng.uniform(ilo, ihi).astype(F)
        length = 10.0 ** rng.uniform(-9, -0.5)
        u = rng.normal(size=3)
        delta = (u / np.linalg.norm(u) * length).astype(F)
        if k % 4 == 0:  # end the move exactly at the interior box, on a random axis and side
            a = int(rng.integers(3))
            target = ihi[a] if rng.random() < 0.5 else ilo[a]
            delta[a] = F(target - p[a])
            delta[a] = np.nextafter(delta[a], F(0))  # just inside
        if shortcut_accepts(p, delta, ilo, ihi, clips, clip_margin):
            accepted += 1
            assert general_path_is_free(p, delta, lo, hi, clamp_lo, clamp_hi, clips), (p, delta)
    assert accepted > 5000


def test_default_scene_shortcut_is_exact():
    """The reference's Cornell box with its clip planes at z = 1 and y = 1.49."""
    _check((-1.0, 0.0, -1.0), (1.0, 1.5, 1.0), (-1.0, 0.0, -1.0), (1.0, 1.49, 1.0), [(2, 1.0), (1, 1.49)], 1)


def test_unit_box_shortcut_is_exact():
    """The unit box of the benchmark scenes, with the default clip planes on its faces."""
    _check((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), (-1.0, 0.0, -1.0), (1.0, 1.49, 1.0), [(2, 1.0), (1, 1.49)], 2)
