// Device-side building blocks of the PBF step: vector helpers, the SPH
// kernels of the reference, the box collider and the compressed neighbour
// iteration. Included by every PBF translation unit.
#pragma once

#include <cstdint>

#include "pbf_internal.h"

namespace pbf {

__device__ __forceinline__ float3 f3(const float4& a) { return make_float3(a.x, a.y, a.z); }
__device__ __forceinline__ float3 operator+(float3 a, float3 b) { return make_float3(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ float3 operator-(float3 a, float3 b) { return make_float3(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ float3 operator*(float3 a, float c) { return make_float3(a.x * c, a.y * c, a.z * c); }
__device__ __forceinline__ float3 operator*(float c, float3 a) { return make_float3(a.x * c, a.y * c, a.z * c); }
__device__ __forceinline__ float dot3(float3 a, float3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float3 cross3(float3 u, float3 v) {
  return make_float3(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
}
__device__ __forceinline__ float cmp3(const float3& v, int a) { return a == 0 ? v.x : (a == 1 ? v.y : v.z); }
__device__ __forceinline__ void set3(float3& v, int a, float x) {
  if (a == 0) v.x = x; else if (a == 1) v.y = x; else v.z = x;
}

// Exactly rounded |a - b|^2 with no contraction: the neighbour predicate of
// particles.cpp:260 evaluated in FP32 (a host check can repeat it bit for bit).
__device__ __forceinline__ float dist2_rn(const float4& a, const float4& b) {
  const float dx = __fsub_rn(a.x, b.x), dy = __fsub_rn(a.y, b.y), dz = __fsub_rn(a.z, b.z);
  return __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
}

// Cell of x* within its scene's grid: floor((x - origin) * inv_cell), clamped.
struct CellCoord {
  int x, y, z;
};
__device__ __forceinline__ CellCoord cell_of(const float3 p, const SceneDesc& sc, float inv_cell) {
  float c[3] = {p.x, p.y, p.z};
  int out[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    float f = floorf(__fmul_rn(__fsub_rn(c[a], sc.origin[a]), inv_cell));
    f = fminf(fmaxf(f, 0.0f), static_cast<float>(sc.dim[a] - 1));
    out[a] = static_cast<int>(f);
  }
  return CellCoord{out[0], out[1], out[2]};
}
__device__ __forceinline__ uint32_t cell_key(const CellCoord& c, const SceneDesc& sc) {
  return sc.cell_off + static_cast<uint32_t>((c.z * sc.dim[1] + c.y) * sc.dim[0] + c.x);
}
__device__ __forceinline__ uint32_t pack_coord(const CellCoord& c) {
  return static_cast<uint32_t>(c.x) | (static_cast<uint32_t>(c.y) << 10) |
         (static_cast<uint32_t>(c.z) << 21);
}

// ---- collider ------------------------------------------------------------------
// Nearest wall of the scene box hit by the segment p + t*dir, t in [0, l]
// (walls facing the motion only; a point already outside a wall it moves
// away from is stopped at once). Returns t; *wall = 2*axis+side or -1.
__device__ __forceinline__ float wall_hit(const float3 p, const float3 dir, float l,
                                          const SceneDesc& sc, int open_mask, int* wall) {
  float t = l;
  int w = -1;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float da = cmp3(dir, a);
    const float pa = cmp3(p, a);
    if (da < 0.0f) {
      if (!(open_mask & (1 << (2 * a)))) {
        const float tt = fmaxf((sc.lo[a] - pa) / da, 0.0f);
        if (tt <= t) { t = tt; w = 2 * a; }
      }
    } else if (da > 0.0f) {
      if (!(open_mask & (1 << (2 * a + 1)))) {
        const float tt = fmaxf((sc.hi[a] - pa) / da, 0.0f);
        if (tt <= t) { t = tt; w = 2 * a + 1; }
      }
    }
  }
  *wall = w;
  return t;
}

__device__ __forceinline__ float wall_value(const SceneDesc& sc, int wall) {
  return (wall & 1) ? sc.hi[wall >> 1] : sc.lo[wall >> 1];
}

// applyForceVelocity (particles.cpp:180, v += g dt) and the predicted move v dt.
__device__ __forceinline__ float3 predict_delta(const float4& v4, const DevParams& P, float dt) {
  const float3 v = make_float3(v4.x + P.g[0] * dt, v4.y + P.g[1] * dt, v4.z + P.g[2] * dt);
  return v * dt;
}

// Moller-Trumbore test of triangle m (MarchingTriangle::intersect,
// static_scene/marching_triangle.cpp:21-45) against p + s dir, s in [0, t]: on a hit
// (s <= t) sets t = s, *best = the triangle's index as given and *nrm its normal. Of
// hits at the same s the one with the larger index wins, which is what a scan of the
// triangles in index order that keeps the last hit with s <= t gives.
__device__ __forceinline__ void tri_test(int m, const float3 p, const float3 dir, const DevParams& P, float& t,
                                         int& best, float3* nrm) {
  const float4 a = __ldg(&P.mesh[4 * m]), b = __ldg(&P.mesh[4 * m + 1]), c = __ldg(&P.mesh[4 * m + 2]);
  const float3 e1 = f3(b), e2 = f3(c), sv = p - f3(a);
  const float3 s1 = cross3(dir, e2), s2 = cross3(sv, e1);
  const float den = dot3(s1, e1);
  if (den == 0.0f) return;
  const float tt = dot3(s2, e2) / den;
  if (tt < 0.0f || tt > t) return;
  const float u = dot3(s1, sv) / den, v = dot3(s2, dir) / den, w = 1.0f - u - v;
  if (u < 0.0f || u > 1.0f || v < 0.0f || v > 1.0f || w < 0.0f || w > 1.0f) return;
  const float4 nn = __ldg(&P.mesh[4 * m + 3]);
  const int idx = __float_as_int(nn.w);
  if (tt == t && idx < best) return;
  t = tt;
  best = idx;
  *nrm = f3(nn);
}

// Whether the segment p + s dir, s in [0, t], meets the box [lo, hi] (slab test; boxes are
// stored widened, so rounding here never drops a triangle the exact test would hit).
__device__ __forceinline__ bool seg_box(const float3 p, const float3 dir, float t, const float4 lo, const float4 hi) {
  float t0 = 0.0f, t1 = t;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float o = cmp3(p, a), d = cmp3(dir, a);
    const float l = a == 0 ? lo.x : (a == 1 ? lo.y : lo.z), h = a == 0 ? hi.x : (a == 1 ? hi.y : hi.z);
    if (d == 0.0f) {
      if (o < l || o > h) return false;
    } else {
      const float inv = 1.0f / d;
      float ta = (l - o) * inv, tb = (h - o) * inv;
      if (ta > tb) {
        const float x = ta;
        ta = tb;
        tb = x;
      }
      t0 = fmaxf(t0, ta);
      t1 = fminf(t1, tb);
      if (t0 > t1) return false;
    }
  }
  return true;
}

// Nearest collider-mesh triangle hit by p + s dir, s in [0, tmax]: a walk of the
// hierarchy (one stack entry per level, its depth bounded by the build) testing the
// triangles of the leaves the segment meets, with the same per-triangle arithmetic and
// the same winner as a scan of all triangles. Returns s, or tmax when nothing is hit.
__device__ __forceinline__ float mesh_hit(const float3 p, const float3 dir, float tmax, const DevParams& P,
                                          float3* nrm, bool* hit) {
  float t = tmax;
  int best = -1;
  int stack[kMeshMaxDepth];
  int sp = 0, node = 0;
  for (;;) {
    const float4 lo = __ldg(&P.mesh_nodes[2 * node]), hi = __ldg(&P.mesh_nodes[2 * node + 1]);
    if (seg_box(p, dir, t, lo, hi)) {
      const int a = __float_as_int(lo.w), b = __float_as_int(hi.w);
      if (b < 0) {
        for (int m = a; m < a - b; ++m) tri_test(m, p, dir, P, t, best, nrm);
      } else {
        if (sp < kMeshMaxDepth) stack[sp++] = b;
        node = a;
        continue;
      }
    }
    if (sp == 0) break;
    node = stack[--sp];
  }
  *hit = best >= 0;
  return t;
}

// Nearest collider sphere hit by p + s dir, s in [0, tmax] (Sphere::test and
// Sphere::intersect, static_scene/sphere.cpp:10-72: the nearer root in range, else the
// farther; the normal points from the centre to the hit point). Returns s, or tmax.
__device__ __forceinline__ float sphere_hit(const float3 p, const float3 dir, float tmax, const DevParams& P,
                                            float3* nrm, bool* hit) {
  float t = tmax;
  *hit = false;
  for (int k = 0; k < P.n_sph; ++k) {
    const float4 c4 = __ldg(&P.sph[k]);
    const float3 m = p - f3(c4);
    const float a = dot3(dir, dir);
    const float b = 2.0f * dot3(m, dir);
    const float c = dot3(m, m) - c4.w * c4.w;
    const float delta = b * b - 4.0f * a * c;
    if (delta < 0.0f) continue;
    const float sq = sqrtf(delta);
    float tt = (-b - sq) / (2.0f * a);
    if (!(tt >= 0.0f && tt <= t)) {
      tt = (-b + sq) / (2.0f * a);
      if (!(tt >= 0.0f && tt <= t)) continue;
    }
    t = tt;
    *hit = true;
    const float3 q = (p + dir * tt) - f3(c4);
    *nrm = q * rsqrtf(dot3(q, q));
  }
  return t;
}

// The nearest of the collider's mesh triangles and spheres (on equal distance the
// triangle); returns s, or tmax when neither is hit.
__device__ __forceinline__ float prim_hit(const float3 p, const float3 dir, float tmax, const DevParams& P,
                                          float3* nrm, bool* hit) {
  float t = tmax;
  *hit = false;
  if (P.n_sph > 0) t = sphere_hit(p, dir, t, P, nrm, hit);
  if (P.n_mesh > 0) {
    float3 mn;
    bool mh;
    const float tm = mesh_hit(p, dir, t, P, &mn, &mh);
    if (mh) {
      t = tm;
      *nrm = mn;
      *hit = true;
    }
  }
  return t;
}

// Distance to keep from a collider triangle or sphere after a stop (the reference backs off by EPS_D =
// 1e-11 in FP64, below FP32 resolution): 4 ulps of the point's largest coordinate.
__device__ __forceinline__ float mesh_backoff(const float3 p) {
  return 4.0f * 1.1920929e-7f * fmaxf(1.0f, fmaxf(fabsf(p.x), fmaxf(fabsf(p.y), fabsf(p.z))));
}

// Collision record (written by the recording forward of the adjoint): the branch
// collide() took, enough to apply its reverse with the active set fixed.
//   bits 0-2  kind: 0 no move (|delta| <= EPS_D), 1 free, 2 stop, 3 stop + slide,
//             4 stop + slide + second stop
//   bit 3     the stop is a clip plane (else a wall)
//   bits 4-6  wall index (2 axis + side) or clip plane index of the stop
//   bit 7     the stop distance was clamped to 0 (the point was already past the wall)
//   bits 8-10 wall index of the second stop
//   bit 11    the second stop distance was clamped to 0
//   bits 12-14 coordinates pinned by the clamp box
constexpr uint32_t kCollNone = 0u, kCollFree = 1u, kCollStop = 2u, kCollSlide = 3u, kCollSlideStop = 4u;
constexpr uint32_t kCollClipBit = 1u << 3, kCollTau0Bit = 1u << 7, kCollTau2Bit = 1u << 11;
__device__ __forceinline__ uint32_t coll_kind(uint32_t c) { return c & 7u; }
__device__ __forceinline__ uint32_t coll_index(uint32_t c) { return (c >> 4) & 7u; }
__device__ __forceinline__ uint32_t coll_wall2(uint32_t c) { return (c >> 8) & 7u; }
__device__ __forceinline__ uint32_t coll_clamped(uint32_t c) { return (c >> 12) & 7u; }

// Shortcut of collide(): a move longer than EPS_D (by 0.1%, so the rounding of sqrt cannot
// decide it) that starts and ends inside the scene's interior box and keeps clip_margin
// from every clip plane meets no wall and no plane and leaves every coordinate inside the
// clamp box: the general path would add delta unchanged, which the shortcut does without
// the stop distances' divisions. The margins are about 1,000 ulps of the coordinates' scale, far
// above the rounding of those distances, so the two paths give the same bits. NaN or
// infinite coordinates fail the comparisons and take the general path.
template <bool MESH>
__device__ __forceinline__ bool clear_move(const float3 p, const float3 delta, float s2, const SceneDesc& sc,
                                           const DevParams& P) {
  if (MESH && (P.n_mesh > 0 || P.n_sph > 0)) return false;
  if (!(s2 > kEps * kEps * 1.001f)) return false;
  const float3 e = p + delta;
  bool ok = fminf(p.x, e.x) > sc.in_lo[0] && fmaxf(p.x, e.x) < sc.in_hi[0] &&
            fminf(p.y, e.y) > sc.in_lo[1] && fmaxf(p.y, e.y) < sc.in_hi[1] &&
            fminf(p.z, e.z) > sc.in_lo[2] && fmaxf(p.z, e.z) < sc.in_hi[2];
  for (int c = 0; c < P.n_clip; ++c) {
    const int a = P.clip_axis[c];
    const float u = cmp3(p, a), w = cmp3(e, a), v = P.clip_value[c];
    ok = ok && (fminf(u, w) > v + P.clip_margin || fmaxf(u, w) < v - P.clip_margin);
  }
  return ok;
}

// Move x* = x + d by `delta` against the collider, in displacement form: d is
// updated, x is fixed. Follows clamp (slide = false, particles.cpp:51-84) and
// clamp_response (slide = true, particles.cpp:87-132): clip planes first, the
// nearest wall stops the move (the stopped coordinate is placed exactly on
// the wall), the predict move slides once along the wall for half the
// remaining length unless a clip plane was crossed, then the clamp box.
// REC additionally writes the collision record to *code (same arithmetic).
// MESH = false compiles the collider-triangle tests out (for launches with no triangles:
// they hold registers a neighbour pass would otherwise spend on occupancy).
// Moves that clear_move accepts take its shortcut.
template <bool REC = false, bool MESH = true>
__device__ __forceinline__ void collide(const float3 x, float3& d, const float3 delta, bool slide,
                                        const SceneDesc& sc, const DevParams& P, uint32_t* code = nullptr) {
  const float3 p = x + d;
  const float s2 = delta.x * delta.x + delta.y * delta.y + delta.z * delta.z;
  if (clear_move<MESH>(p, delta, s2, sc, P)) {
    d = d + delta;
    if (REC) *code = kCollFree;
    return;
  }
  float l = sqrtf(s2);
  if (!(l > kEps)) {  // particles.cpp:53-55 / 90-92: no move, no clamp
    if (REC) *code = kCollNone;
    return;
  }
  const float3 dir = delta * (1.0f / l);
  const float total = l;
  bool intersect = false;
  int clip = 0;
  for (int c = 0; c < P.n_clip; ++c) {
    const int a = P.clip_axis[c];
    const float da = cmp3(dir, a);
    if (da != 0.0f) {
      const float pt = (P.clip_value[c] - cmp3(p, a)) / da;
      if (pt > 0.0f && pt < l) { l = pt; intersect = true; clip = c; }
    }
  }
  uint32_t rc = kCollFree;
  int wall;
  const float t = wall_hit(p, dir, l, sc, P.open_mask, &wall);
  if (MESH && (P.n_mesh > 0 || P.n_sph > 0)) {  // a collider triangle or sphere nearer than the wall or
                                                  // clip plane stops the move instead
    float3 mn;
    bool mh;
    const float tm = prim_hit(p, dir, t, P, &mn, &mh);
    if (mh && tm < t) {
      float3 nd = d + dir * fmaxf(tm - mesh_backoff(p), 0.0f);
      // slide as clamp_response does (particles.cpp:118-124): half the remaining length along
      // the triangle, unless a clip plane was crossed
      if (slide && !intersect && dot3(dir, mn) > -1.0f) {
        const float3 tan = delta - mn * dot3(delta, mn);
        const float tl = sqrtf(dot3(tan, tan));
        if (tl > 0.0f) {
          const float3 dir2 = tan * (1.0f / tl);
          const float l2 = (total - tm) * 0.5f;
          const float3 p1 = x + nd;
          int wall2;
          const float t2 = wall_hit(p1, dir2, l2, sc, P.open_mask, &wall2);
          float3 mn2;
          bool mh2;
          const float tm2 = prim_hit(p1, dir2, t2, P, &mn2, &mh2);
          if (mh2 && tm2 < t2) {
            nd = nd + dir2 * fmaxf(tm2 - mesh_backoff(p1), 0.0f);
          } else {
            nd = nd + dir2 * t2;
            if (wall2 >= 0) set3(nd, wall2 >> 1, wall_value(sc, wall2) - cmp3(x, wall2 >> 1));
          }
        }
      }
      d = nd;
      const float3 q = x + d;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float qa = cmp3(q, a);
        if (qa < P.clamp_lo[a]) set3(d, a, P.clamp_lo[a] - cmp3(x, a));
        else if (qa > P.clamp_hi[a]) set3(d, a, P.clamp_hi[a] - cmp3(x, a));
      }
      if (REC) *code = kCollNone;  // not recorded: the adjoint takes box colliders only
      return;
    }
  }
  if (wall >= 0 || intersect) {
    float3 nd = d + dir * t;
    if (REC) {
      rc = kCollStop;
      if (wall >= 0) {
        const int a = wall >> 1;
        rc |= static_cast<uint32_t>(wall) << 4;
        if ((wall_value(sc, wall) - cmp3(p, a)) / cmp3(dir, a) < 0.0f) rc |= kCollTau0Bit;
      } else {
        rc |= kCollClipBit | (static_cast<uint32_t>(clip) << 4);
      }
    }
    if (wall >= 0) set3(nd, wall >> 1, wall_value(sc, wall) - cmp3(x, wall >> 1));
    if (slide && wall >= 0 && !intersect) {
      const int a = wall >> 1;
      const float n_dot = (wall & 1) ? -cmp3(dir, a) : cmp3(dir, a);  // dot(dir, inward normal)
      if (n_dot > -1.0f) {
        float3 tan = delta;
        set3(tan, a, 0.0f);
        const float tl = sqrtf(dot3(tan, tan));
        if (tl > 0.0f) {
          const float3 dir2 = tan * (1.0f / tl);
          const float l2 = (total - t) * 0.5f;
          int wall2;
          const float3 p1 = x + nd;
          const float t2 = wall_hit(p1, dir2, l2, sc, P.open_mask, &wall2);
          if (MESH && (P.n_mesh > 0 || P.n_sph > 0)) {  // the slide stops at a collider triangle or
                                                        // sphere before the wall
            float3 mn2;
            bool mh2;
            const float tm2 = prim_hit(p1, dir2, t2, P, &mn2, &mh2);
            if (mh2 && tm2 < t2) {
              d = nd + dir2 * fmaxf(tm2 - mesh_backoff(p1), 0.0f);
              if (REC) *code = kCollNone;  // not recorded: the adjoint takes box colliders only
              const float3 q = x + d;
#pragma unroll
              for (int a = 0; a < 3; ++a) {
                const float qa = cmp3(q, a);
                if (qa < P.clamp_lo[a]) set3(d, a, P.clamp_lo[a] - cmp3(x, a));
                else if (qa > P.clamp_hi[a]) set3(d, a, P.clamp_hi[a] - cmp3(x, a));
              }
              return;
            }
          }
          nd = nd + dir2 * t2;
          if (REC) {
            rc = (rc & ~7u) | kCollSlide;
            if (wall2 >= 0) {
              const int a2 = wall2 >> 1;
              rc = (rc & ~7u) | kCollSlideStop | (static_cast<uint32_t>(wall2) << 8);
              if ((wall_value(sc, wall2) - cmp3(p1, a2)) / cmp3(dir2, a2) < 0.0f) rc |= kCollTau2Bit;
            }
          }
          if (wall2 >= 0) set3(nd, wall2 >> 1, wall_value(sc, wall2) - cmp3(x, wall2 >> 1));
        }
      }
    }
    d = nd;
  } else {
    d = d + delta;
  }
  const float3 q = x + d;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float qa = cmp3(q, a);
    if (qa < P.clamp_lo[a]) {
      set3(d, a, P.clamp_lo[a] - cmp3(x, a));
      if (REC) rc |= 1u << (12 + a);
    } else if (qa > P.clamp_hi[a]) {
      set3(d, a, P.clamp_hi[a] - cmp3(x, a));
      if (REC) rc |= 1u << (12 + a);
    }
  }
  if (REC) *code = rc;
}

// Reverse of a recorded collision with its active set fixed. p = x* before the move,
// D = the requested displacement, g = adjoint of x* after the move; returns the
// adjoints of p (*pb) and of D (*db). A stop moves p to p1 = p + tau D with
// tau = (c - p[a]) / D[a] (p1[a] = c); tau is 0 when the stop distance was clamped.
// The slide adds kappa tan, tan = D without its a component, T = |tan|,
// kappa = |D| (1 - tau) / (2 T); a second stop on axis a2 at c2 instead adds sigma tan
// with sigma = (c2 - p1[a2]) / tan[a2] and puts p2[a2] = c2. Coordinates the clamp
// box pinned pass no adjoint.
__device__ __forceinline__ void collide_reverse(uint32_t code, const float3 p, const float3 D, float3 g,
                                                const SceneDesc& sc, const DevParams& P, float3* pb,
                                                float3* db) {
  const uint32_t cl = coll_clamped(code);
#pragma unroll
  for (int a = 0; a < 3; ++a)
    if (cl & (1u << a)) set3(g, a, 0.0f);
  const uint32_t kind = coll_kind(code);
  if (kind == kCollNone) {
    *pb = g;
    *db = make_float3(0.f, 0.f, 0.f);
    return;
  }
  if (kind == kCollFree) {
    *pb = g;
    *db = g;
    return;
  }
  const uint32_t idx = coll_index(code);
  int a;
  float c;
  if (code & kCollClipBit) {
    a = P.clip_axis[idx];
    c = P.clip_value[idx];
  } else {
    a = static_cast<int>(idx >> 1);
    c = wall_value(sc, static_cast<int>(idx));
  }
  const bool tau0 = (code & kCollTau0Bit) != 0u;
  const float Da = cmp3(D, a);
  const float tau = tau0 ? 0.0f : (c - cmp3(p, a)) / Da;
  float3 g1 = g, dbar = make_float3(0.f, 0.f, 0.f);
  float taub = 0.0f;
  if (kind >= kCollSlide) {
    float3 tan = D;
    set3(tan, a, 0.0f);
    const float T = sqrtf(dot3(tan, tan));
    float3 tanb;
    if (kind == kCollSlide) {
      const float L = sqrtf(dot3(D, D));
      const float kappa = L * (1.0f - tau) / (2.0f * T);
      const float kb = dot3(g, tan);
      tanb = g * kappa;
      const float Lb = kb * (1.0f - tau) / (2.0f * T);
      taub -= kb * L / (2.0f * T);
      const float Tb = -kb * kappa / T;
      tanb = tanb + tan * (Tb / T);
      dbar = dbar + D * (Lb / L);
    } else {
      const int w2 = static_cast<int>(coll_wall2(code));
      const int a2 = w2 >> 1;
      set3(g1, a2, 0.0f);
      tanb = make_float3(0.f, 0.f, 0.f);
      if (!(code & kCollTau2Bit)) {
        const float ta2 = cmp3(tan, a2);
        const float p1a2 = cmp3(p, a2) + tau * cmp3(D, a2);
        const float sigma = (wall_value(sc, w2) - p1a2) / ta2;
        float3 gm = g;
        set3(gm, a2, 0.0f);
        const float sb = dot3(gm, tan);
        tanb = gm * sigma;
        set3(g1, a2, -sb / ta2);
        set3(tanb, a2, -sb * sigma / ta2);
      }
    }
    set3(tanb, a, 0.0f);
    dbar = dbar + tanb;
  }
  // p1 = p + tau D, p1[a] = c
  float3 pbar = g1;
  set3(pbar, a, 0.0f);
  if (!tau0) {
    float3 gm = g1;
    set3(gm, a, 0.0f);
    dbar = dbar + gm * tau;
    taub += dot3(gm, D);
    set3(pbar, a, -taub / Da);
    set3(dbar, a, cmp3(dbar, a) - taub * tau / Da);
  }
  *pb = pbar;
  *db = dbar;
}

// ---- neighbour lists -----------------------------------------------------------
// A particle's neighbours lie in 3 z-slabs (dz = -1, 0, 1) of its cell; inside a slab
// they lie in the rows dy = -1..1 of cells cx-1..cx+1, all within 2*nx+3 cells after the
// slab's first candidate cell, i.e. a short slot range of the cell-sorted arrays. A
// neighbour is stored as a u16 entry (slab << 14 | slot offset from the slab's first
// candidate slot), two entries per u32 word, word-major ([word][N]) so a warp's loads of
// one word index coalesce. hdr = {slab base -1, slab base 0, slab base +1, count}.
constexpr int kOffsetBits = 14;
constexpr uint32_t kOffsetMask = (1u << kOffsetBits) - 1u;

__device__ __forceinline__ int nbr_total(const uint4& h) { return static_cast<int>(h.w); }

// A list entry is a 2-bit slab tag g over a 14-bit offset into slab g's three rows. The
// header holds slab 0's first slot in x and, in y and z, slab 1's and slab 2's first slots
// less slab 0's and less the tag bits (g << 14), all modulo 2^32, so the slot is
// x + entry + (0, y or z by tag): the entry needs no masking.
// Two forms of the same decode (slab tags are 0, 1 and 2, so both give the same slot).
// The compiler schedules a pass's gathers differently around them; every pass measured
// fastest with kBits on the 1M colliding blocks (ms per step, kBits / kCompare): lambda
// 0.238 / 0.256 and delta-p 0.282 / 0.315 with word-major lists, XSPH 0.084 / 0.100 with
// the grouped list words.
enum class Decode { kBits, kCompare };

template <Decode DC = Decode::kBits>
__device__ __forceinline__ uint32_t nbr_decode(const uint4& h, uint32_t e) {
  uint32_t adj;
  if (DC == Decode::kBits) {
    adj = (e & (2u << kOffsetBits)) ? h.z : ((e & (1u << kOffsetBits)) ? h.y : 0u);
  } else {
    const uint32_t g = e >> kOffsetBits;
    adj = g == 0u ? 0u : (g == 1u ? h.y : h.z);
  }
  return h.x + e + adj;
}

// List words are grouped by four: word w of slot i is words[list_word(i, n, w)], i.e. the
// layout is [W/4][N][4] (W = words per slot rounded up to 4). One 16-byte load brings a
// slot 8 entries, the 32 slots of a warp read 512 contiguous bytes, and consecutive warps
// read consecutive lines.
__device__ __forceinline__ size_t list_word(int i, int n, int w) {
  return static_cast<size_t>(w >> 2) * (4 * static_cast<size_t>(n)) + 4 * static_cast<size_t>(i) +
         static_cast<uint32_t>(w & 3);
}

// Calls f(j) for every neighbour slot j of slot i, ascending.
template <typename F>
__device__ __forceinline__ void for_each_neighbor(int i, int n, const uint4 h,
                                                  const uint32_t* __restrict__ words, F&& f) {
  const int total = nbr_total(h);
  for (int k = 0; k < total; k += 2) {
    const uint32_t w = __ldg(&words[list_word(i, n, k >> 1)]);
    f(nbr_decode(h, w & 0xffffu));
    if (k + 1 < total) f(nbr_decode(h, w >> 16));
  }
}

// As for_each_neighbor, with each neighbour's data gathered ahead of the computation:
// load(j) returns what f needs of neighbour j; per round D list entries are decoded and
// their loads issued before f runs on any of them, so every thread keeps D independent
// gathers in flight. A round of 8 entries is one 16-byte group of list words; with D = 8
// the next group is loaded before this round's computation, so its latency overlaps it.
// The last group, with fewer than 8 entries left, is taken from the same registers. Calls
// f(j, load(j)) in the same (ascending) order. D = 4 or 8; DC picks the decode form.
// List words are read once per pass: ST = true loads them with the streaming policy
// (ld.global.cs, evict-first in L1 and L2), so they displace less of the neighbours' x*
// that the pass gathers repeatedly.
template <bool ST>
__device__ __forceinline__ uint4 ld_quad(const uint4* p) {
  return ST ? __ldcs(p) : __ldg(p);
}
template <bool ST>
__device__ __forceinline__ uint4 ld_hdr(const uint4* p) {
  return ST ? __ldcs(p) : __ldg(p);
}

template <int D, Decode DC = Decode::kBits, bool ST = false, typename L, typename F>
__device__ __forceinline__ void for_each_neighbor_pf(int i, int n, const uint4 h,
                                                     const uint32_t* __restrict__ words, L&& load, F&& f) {
  static_assert(D == 4 || D == 8, "gather depth 4 or 8");
  const int total = nbr_total(h);
  if (total <= 0) return;
  const size_t sn = static_cast<size_t>(n);
  const uint4* qp = reinterpret_cast<const uint4*>(words) + i;
  uint4 q = ld_quad<ST>(qp);
  int k = 0;
  for (; k + 7 < total; k += 8) {
    qp += sn;
    uint4 nq = make_uint4(0u, 0u, 0u, 0u);
    if (D == 8 && k + 8 < total) nq = ld_quad<ST>(qp);
    const uint32_t j0 = nbr_decode<DC>(h, q.x & 0xffffu), j1 = nbr_decode<DC>(h, q.x >> 16);
    const uint32_t j2 = nbr_decode<DC>(h, q.y & 0xffffu), j3 = nbr_decode<DC>(h, q.y >> 16);
    if (D == 8) {
      const uint32_t j4 = nbr_decode<DC>(h, q.z & 0xffffu), j5 = nbr_decode<DC>(h, q.z >> 16);
      const uint32_t j6 = nbr_decode<DC>(h, q.w & 0xffffu), j7 = nbr_decode<DC>(h, q.w >> 16);
      const auto a0 = load(j0);
      const auto a1 = load(j1);
      const auto a2 = load(j2);
      const auto a3 = load(j3);
      const auto a4 = load(j4);
      const auto a5 = load(j5);
      const auto a6 = load(j6);
      const auto a7 = load(j7);
      f(j0, a0);
      f(j1, a1);
      f(j2, a2);
      f(j3, a3);
      f(j4, a4);
      f(j5, a5);
      f(j6, a6);
      f(j7, a7);
      q = nq;
    } else {
      const auto a0 = load(j0);
      const auto a1 = load(j1);
      const auto a2 = load(j2);
      const auto a3 = load(j3);
      f(j0, a0);
      f(j1, a1);
      f(j2, a2);
      f(j3, a3);
      const uint32_t j4 = nbr_decode<DC>(h, q.z & 0xffffu), j5 = nbr_decode<DC>(h, q.z >> 16);
      const uint32_t j6 = nbr_decode<DC>(h, q.w & 0xffffu), j7 = nbr_decode<DC>(h, q.w >> 16);
      const auto a4 = load(j4);
      const auto a5 = load(j5);
      const auto a6 = load(j6);
      const auto a7 = load(j7);
      f(j4, a4);
      f(j5, a5);
      f(j6, a6);
      f(j7, a7);
      if (k + 8 < total) q = ld_quad<ST>(qp);
    }
  }
  // fewer than 8 entries left, all in q
  if (k + 3 < total) {
    const uint32_t j0 = nbr_decode<DC>(h, q.x & 0xffffu), j1 = nbr_decode<DC>(h, q.x >> 16);
    const uint32_t j2 = nbr_decode<DC>(h, q.y & 0xffffu), j3 = nbr_decode<DC>(h, q.y >> 16);
    const auto a0 = load(j0);
    const auto a1 = load(j1);
    const auto a2 = load(j2);
    const auto a3 = load(j3);
    f(j0, a0);
    f(j1, a1);
    f(j2, a2);
    f(j3, a3);
    k += 4;
    q.x = q.z;
    q.y = q.w;
  }
  if (k + 1 < total) {
    const uint32_t j0 = nbr_decode<DC>(h, q.x & 0xffffu), j1 = nbr_decode<DC>(h, q.x >> 16);
    const auto a0 = load(j0);
    const auto a1 = load(j1);
    f(j0, a0);
    f(j1, a1);
    k += 2;
    q.x = q.y;
  }
  if (k < total) {
    const uint32_t j0 = nbr_decode<DC>(h, q.x & 0xffffu);
    f(j0, load(j0));
  }
}

// The common case: the neighbours' x* (NC: through the read-only path, for buffers no
// thread writes during the kernel), four in flight; calls f(j, x_j).
template <bool NC, typename F>
__device__ __forceinline__ void for_each_neighbor_x(int i, int n, const uint4 h,
                                                    const uint32_t* __restrict__ words,
                                                    const float4* xs, F&& f) {
  for_each_neighbor_pf<4>(i, n, h, words, [&](uint32_t j) -> float4 { return NC ? __ldg(&xs[j]) : xs[j]; }, f);
}

// Pair geometry shared by every neighbour pass, branch-free:
//   r = x_i - x_j, r2 = |r|^2,
//   q = max(h2 - r2, 0)       so W = poly6_c * q^3     (particles.cpp:134-141)
//   s = (h - |r|)^2 / |r| on [EPS_D, h), else 0, so grad W = spiky_c * s * r (:143-149)
struct Pair {
  float3 r;
  float r2, q, s;
};
// FTZ selects the flush-to-zero form of the approximate reciprocal square root, which
// needs no rescaling of subnormal inputs. The two forms differ only for a subnormal r2,
// far below EPS_D^2, where s is 0 either way (and both give +inf at r2 = 0, where hr is 0),
// so the pair values are the same. Every pass uses it: measured with the current kernels on
// the 1M colliding blocks, lambda 0.222 against 0.235 ms a step, delta-p 0.274 against
// 0.279, XSPH 0.090 against 0.093 (the vorticity pass already used it).
// Every rounding is explicit (_rn intrinsics, fused where written as an fma), so the
// compiler cannot contract differently in differently unrolled loops: every form of a
// neighbour pass gives the same bits.
template <bool FTZ = true>
__device__ __forceinline__ Pair pair_of(const float4& xi, const float4& xj, float h, float h2) {
  Pair p;
  p.r = make_float3(__fsub_rn(xi.x, xj.x), __fsub_rn(xi.y, xj.y), __fsub_rn(xi.z, xj.z));
  p.r2 = __fmaf_rn(p.r.z, p.r.z, __fmaf_rn(p.r.y, p.r.y, __fmul_rn(p.r.x, p.r.x)));
  p.q = fmaxf(__fsub_rn(h2, p.r2), 0.0f);
  float rinv;
  if (FTZ)
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(rinv) : "f"(p.r2));
  else
    rinv = rsqrtf(p.r2);
  const float hr = fmaxf(__fmaf_rn(-p.r2, rinv, h), 0.0f);
  p.s = p.r2 >= kEps * kEps ? __fmul_rn(__fmul_rn(hr, hr), rinv) : 0.0f;
  return p;
}

// acc + a * c per component, one rounding each
__device__ __forceinline__ float3 fma3(const float3 a, float c, const float3 acc) {
  return make_float3(__fmaf_rn(a.x, c, acc.x), __fmaf_rn(a.y, c, acc.y), __fmaf_rn(a.z, c, acc.z));
}
__device__ __forceinline__ float dot3_rn(const float3 a, const float3 b) {
  return __fmaf_rn(a.z, b.z, __fmaf_rn(a.y, b.y, __fmul_rn(a.x, b.x)));
}

// Spiky gradient factor s with grad W(r) = spiky_c * s * r (particles.cpp:143-149);
// returns false outside [EPS_D, h).
__device__ __forceinline__ bool spiky_s(float r2, float h, float* s) {
  const float rinv = rsqrtf(r2);
  const float rl = r2 * rinv;
  if (!(rl < h && rl >= kEps)) return false;
  const float hr = h - rl;
  *s = hr * hr * rinv;
  return true;
}

// Particles::estimateDensityAt (particles.cpp:446-453): sum of poly6 over all particles
// (self included for a particle's own position), gathered from the 27 cells of size
// >= h around p in the cell order of `pos` (cell_start of that order). As in the
// neighbour build, a row of cells farther than h in y/z is skipped and the others are
// trimmed in x to the cells that reach [x - w, x + w], w = sqrt(h^2 - d_yz^2), with a
// margin of 1e-3 cell: only particles that add nothing are left out, so the sum (same
// rows, same slot order) is the same.
__device__ __forceinline__ float density_at_point(const float3 p, const float4* __restrict__ pos,
                                                  const uint32_t* __restrict__ cell_start, const SceneDesc& sc,
                                                  const DevParams& P) {
  const CellCoord cc = cell_of(p, sc, P.inv_cell);
  const float m = 1e-3f;
  const float reach = sqrtf(P.h2) * P.inv_cell + m;
  const float reach2 = reach * reach;
  const float ux = (p.x - sc.origin[0]) * P.inv_cell, uy = (p.y - sc.origin[1]) * P.inv_cell,
              uz = (p.z - sc.origin[2]) * P.inv_cell;
  float qsum = 0.f;
  for (int r = 0; r < 9; ++r) {
    const int z = cc.z + r / 3 - 1, y = cc.y + r % 3 - 1;
    if (z < 0 || z >= sc.dim[2] || y < 0 || y >= sc.dim[1]) continue;
    // distance in cells from p to the row's y and z extents, less the margin
    const float dy = fmaxf(fmaxf(static_cast<float>(y) - uy, uy - static_cast<float>(y + 1)) - m, 0.f);
    const float dz = fmaxf(fmaxf(static_cast<float>(z) - uz, uz - static_cast<float>(z + 1)) - m, 0.f);
    const float w2 = reach2 - (dy * dy + dz * dz);
    if (w2 < 0.f) continue;
    const float w = sqrtf(w2);
    const int xa = max(max(static_cast<int>(floorf(ux - w)), cc.x - 1), 0);
    const int xb = min(min(static_cast<int>(floorf(ux + w)), cc.x + 1), sc.dim[0] - 1);
    if (xa > xb) continue;
    const uint32_t row = sc.cell_off + static_cast<uint32_t>((z * sc.dim[1] + y) * sc.dim[0]);
    const uint32_t e = __ldg(&cell_start[row + xb + 1]);
    for (uint32_t j = __ldg(&cell_start[row + xa]); j < e; ++j) {
      const float4 xj = __ldg(&pos[j]);
      const float3 d = make_float3(xj.x - p.x, xj.y - p.y, xj.z - p.z);
      const float r2 = dot3(d, d);
      if (r2 < P.h2) {
        const float q = P.h2 - r2;
        qsum += q * q * q;
      }
    }
  }
  return P.poly6_c * qsum;
}

__device__ __forceinline__ unsigned lane_id() { return threadIdx.x & 31u; }

// Instantiates a neighbour-pass kernel launch for the tuned block size.
#define PBF_BLOCK_SWITCH(block, ...)                          \
  switch (block) {                                            \
    case 64: { constexpr int BLOCK = 64; __VA_ARGS__; } break;   \
    case 128: { constexpr int BLOCK = 128; __VA_ARGS__; } break; \
    case 512: { constexpr int BLOCK = 512; __VA_ARGS__; } break; \
    default: { constexpr int BLOCK = 256; __VA_ARGS__; } break;  \
  }


}  // namespace pbf
