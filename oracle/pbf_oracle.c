/*
 * pbf_oracle.c — FP64 CPU restatement of the reference's PBF step.
 *
 * TEST INFRASTRUCTURE (the oracle). Only tests/, __graft_entry__.smoke() and
 * bench.py's CPU-baseline leg load this library, and only as the values results are compared with or
 * the timed CPU baseline; the product path never calls it.
 *
 * It restates src/particles.cpp of the reference with the same floating-point
 * operation order (Vector3D ops of CGL/include/CGL/vector3D.h, intpow of
 * src/bsdf.h:49-57), so that with -ffp-contract=off it reproduces the
 * reference's "jacobi" sequence bit for bit. Differences from the reference,
 * each deliberate:
 *   - neighbour search uses a uniform grid instead of the all-pairs loop
 *     (particles.cpp:258-265); lists are sorted by index, which is the order
 *     the all-pairs loop produces, so every sum runs in the same order;
 *   - the XSPH/vorticity pass (particles.cpp:285-288) is order-independent:
 *     every particle sees its neighbours' pre-XSPH velocity;
 *   - the collider is the reference's triangle box (12 triangles, inward
 *     normals, built like oracle/ref/ref_driver.cpp) intersected with
 *     Moller-Trumbore (src/static_scene/marching_triangle.cpp:21-45) by a
 *     linear scan for the NEAREST hit in both clamp and clamp_response. The
 *     reference's clamp (particles.cpp:76) uses BVHAccel::intersect(const
 *     Ray&), which returns the first hit in BVH order (src/bvh.cpp:142-160);
 *     the two differ only when one displacement crosses two walls.
 *   - collider spheres (orc_set_spheres) are the reference's Sphere primitives
 *     (src/static_scene/sphere.cpp:10-72), tested after the triangles in the same
 *     nearest-hit scan;
 *   - gravity is a 3-vector applied per non-zero component (the reference
 *     subtracts 10*dt from v.y, particles.cpp:180).
 * Parallel over particles with OpenMP; every phase is order-independent so the
 * result does not depend on the thread count.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/pbf.h"

#define EPS_D (0.00000000001) /* CGL/include/CGL/misc.h:11 */

/* Scalar type of the restatement: double (the reference's type) unless built with
 * -DORC_FLOAT, which gives an FP32 comparator for statistics of long rollouts. */
#ifdef ORC_FLOAT
typedef float real;
#else
typedef double real;
#endif

typedef struct { real x, y, z; } v3;

static inline v3 V(real x, real y, real z) { v3 r = {x, y, z}; return r; }
static inline v3 vadd(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 vsub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
/* Vector3D * real and real * Vector3D: component products. */
static inline v3 vscale(v3 a, real c) { return V(a.x * c, a.y * c, a.z * c); }
static inline v3 svmul(real c, v3 a) { return V(c * a.x, c * a.y, c * a.z); }
/* Vector3D / real: multiply by the reciprocal (vector3D.h operator/). */
static inline v3 vdiv(v3 a, real c) { const real rc = 1.0 / c; return V(rc * a.x, rc * a.y, rc * a.z); }
static inline real norm2(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline real vnorm(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline v3 unit(v3 a) { real r = 1. / sqrt(a.x * a.x + a.y * a.y + a.z * a.z); return V(r * a.x, r * a.y, r * a.z); }
static inline real dot(v3 u, v3 v) { return u.x * v.x + u.y * v.y + u.z * v.z; }
static inline v3 cross(v3 u, v3 v) {
  return V(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
}
static inline real comp(v3 a, int k) { return k == 0 ? a.x : (k == 1 ? a.y : a.z); }
static inline void setcomp(v3* a, int k, real v) { if (k == 0) a->x = v; else if (k == 1) a->y = v; else a->z = v; }
/* std::max / std::min as <algorithm> defines them. */
static inline real smax(real a, real b) { return (a < b) ? b : a; }
static inline real smin(real a, real b) { return (b < a) ? b : a; }

/* intpow<e>(b) = intpow<e-1>(b) * b, intpow<0> = 1 (src/bsdf.h:49-57). */
static inline real intpow(real b, int e) {
  real r = 1;
  for (int i = 0; i < e; i++) r = r * b;
  return r;
}

#define ORC_MAX_MESH 65536
#define ORC_MAX_TRI (12 + ORC_MAX_MESH)
#define ORC_MAX_SPH 1024

typedef struct {
  real h, h2, h6, h9, tis;
  real epsilon, k, vort_eps, xsph_c, rest_density;
  int iters, scorr_n;
  v3 gravity;
  real clamp_lo[3], clamp_hi[3];
  int n_clip, clip_axis[2];
  real clip_value[2];
  int ntri;
  v3 tp[ORC_MAX_TRI][3];  /* the box walls (up to 12), then the collider mesh */
  v3 tn[ORC_MAX_TRI];
  int nsph;
  v3 so[ORC_MAX_SPH];     /* collider spheres: centre, radius */
  real sr[ORC_MAX_SPH];
} ctx_t;

/* poly6_kernel, particles.cpp:134-141 */
static inline real poly6(const ctx_t* c, v3 r) {
  real r_l_2 = norm2(r);
  if (r_l_2 >= c->h2) return 0.0;
  real temp = c->h2 - r_l_2;
  return 1.56668147106 * intpow(temp, 3) / c->h9;
}

/* grad_spiky_kernel, particles.cpp:143-149 */
static inline v3 spiky(const ctx_t* c, v3 r) {
  real r_l = vnorm(r);
  if (r_l >= c->h || r_l < EPS_D) return V(0, 0, 0);
  const real k0 = -3 * 4.774648292756860;
  return vdiv(svmul(k0 * intpow(c->h - r_l, 2), r), c->h6 * r_l);
}

/* ---- collider: triangle box + Moller-Trumbore ------------------------------ */

static void build_box(ctx_t* c, const double lo[3], const double hi[3], int open_mask) {
  c->ntri = 0;
  for (int axis = 0; axis < 3; axis++) {
    for (int side = 0; side < 2; side++) {
      if (open_mask & (1 << (2 * axis + side))) continue;
      int u = (axis + 1) % 3, w = (axis + 2) % 3;
      real cc = side ? hi[axis] : lo[axis];
      real us[4] = {lo[u], hi[u], hi[u], lo[u]};
      real vs[4] = {lo[w], lo[w], hi[w], hi[w]};
      v3 corner[4];
      for (int k = 0; k < 4; k++) {
        corner[k] = V(0, 0, 0);
        setcomp(&corner[k], axis, cc);
        setcomp(&corner[k], u, us[k]);
        setcomp(&corner[k], w, vs[k]);
      }
      v3 n = V(0, 0, 0);
      setcomp(&n, axis, side ? -1.0 : 1.0);
      int t = c->ntri;
      c->tp[t][0] = corner[0]; c->tp[t][1] = corner[1]; c->tp[t][2] = corner[2]; c->tn[t] = n;
      c->tp[t + 1][0] = corner[0]; c->tp[t + 1][1] = corner[2]; c->tp[t + 1][2] = corner[3]; c->tn[t + 1] = n;
      c->ntri += 2;
    }
  }
}

typedef struct { v3 o, d; real min_t, max_t; } ray_t;

/* MarchingTriangle::intersect(const Ray&, Intersection*) arithmetic. */
static int tri_hit(const ctx_t* c, int t, ray_t* r, v3* nrm) {
  v3 p1 = c->tp[t][0], p2 = c->tp[t][1], p3 = c->tp[t][2];
  v3 e1 = vsub(p2, p1), e2 = vsub(p3, p1), s = vsub(r->o, p1);
  v3 s1 = cross(r->d, e2), s2 = cross(s, e1);
  real d = dot(s1, e1);
  if (d == 0) return 0;
  real tt = dot(s2, e2) / d;
  if ((tt < r->min_t) || (tt > r->max_t)) return 0;
  real u = dot(s1, s) / d;
  real v = dot(s2, r->d) / d;
  real w = 1 - u - v;
  if ((u < 0) || (u > 1) || (v < 0) || (v > 1) || (w < 0) || (w > 1)) return 0;
  r->max_t = tt;
  if (nrm) {
    v3 n = c->tn[t];
    *nrm = vadd(vadd(svmul(w, n), svmul(u, n)), svmul(v, n));
  }
  return 1;
}

/* Sphere::test and Sphere::intersect(const Ray&, Intersection*), static_scene/sphere.cpp:10-72:
 * the nearer root if it lies in [min_t, max_t], else the farther; the normal is the unit
 * vector from the centre to the hit point. */
static int sph_hit(const ctx_t* c, int s, ray_t* r, v3* nrm) {
  const v3 o = c->so[s];
  const real r2 = c->sr[s] * c->sr[s];
  real a = dot(r->d, r->d);
  v3 m = vsub(r->o, o);
  real b = 2 * dot(m, r->d);
  real cc = dot(m, m) - r2;
  real delta = b * b - 4 * a * cc;
  if (delta < 0) return 0;
  real t1;
  real t = (-b - sqrt(delta)) / (2 * a);
  if ((t >= r->min_t) && (t <= r->max_t)) {
    t1 = t;
  } else {
    t = (-b + sqrt(delta)) / (2 * a);
    if ((t >= r->min_t) && (t <= r->max_t)) {
      t1 = t;
    } else {
      return 0;
    }
  }
  r->max_t = t1;
  if (nrm) *nrm = unit(vsub(vadd(r->o, svmul(t1, r->d)), o));
  return 1;
}

/* Nearest hit over all triangles, then all spheres; updates r->max_t, *nrm. */
static int scene_hit(const ctx_t* c, ray_t* r, v3* nrm) {
  int hit = 0;
  for (int t = 0; t < c->ntri; t++) hit |= tri_hit(c, t, r, nrm);
  for (int s = 0; s < c->nsph; s++) hit |= sph_hit(c, s, r, nrm);
  return hit;
}

static inline void clamp_box(const ctx_t* c, v3* p) {
  p->x = smax(c->clamp_lo[0] + EPS_D, smin(c->clamp_hi[0] - EPS_D, p->x));
  p->y = smax(c->clamp_lo[1] + EPS_D, smin(c->clamp_hi[1] - EPS_D, p->y));
  p->z = smax(c->clamp_lo[2] + EPS_D, smin(c->clamp_hi[2] - EPS_D, p->z));
}

static inline int clip_planes(const ctx_t* c, v3 p, v3 d, real* l) {
  int intersect = 0;
  for (int i = 0; i < c->n_clip; i++) {
    int a = c->clip_axis[i];
    real da = comp(d, a);
    if (da != 0.0) {
      real pt = (c->clip_value[i] - comp(p, a)) / da;
      if (pt > 0.0 && pt < *l) {
        *l = pt;
        intersect = 1;
      }
    }
  }
  return intersect;
}

/* clamp, particles.cpp:51-84 */
static void clamp_move(const ctx_t* c, v3* p, v3 delta_p) {
  real l = vnorm(delta_p);
  if (l <= EPS_D) return;
  v3 d = vdiv(delta_p, l);
  int intersect = clip_planes(c, *p, d, &l);
  ray_t r = {*p, d, 0.0, l};
  if (scene_hit(c, &r, NULL) || intersect) {
    *p = vadd(*p, svmul(r.max_t - EPS_D, d));
  } else {
    *p = vadd(*p, delta_p);
  }
  clamp_box(c, p);
}

/* clamp_response, particles.cpp:87-132 */
static void clamp_response(const ctx_t* c, v3* p, v3 v, real dt) {
  v3 delta_p = vscale(v, dt);
  real total_l = vnorm(delta_p), l = total_l;
  if (l <= EPS_D) return;
  v3 d = vdiv(delta_p, l);
  int intersect = clip_planes(c, *p, d, &l);
  ray_t r = {*p, d, 0.0, l};
  v3 n = V(0, 0, 0);
  if (scene_hit(c, &r, &n) || intersect) {
    *p = vadd(*p, svmul(r.max_t - EPS_D, d));
    if (dot(d, n) > -1 && !intersect) {
      d = unit(vsub(delta_p, svmul(dot(delta_p, n), n)));
      ray_t r2 = {*p, d, 0.0, (total_l - r.max_t) * 0.5};
      v3 n2 = V(0, 0, 0);
      scene_hit(c, &r2, &n2);
      *p = vadd(*p, svmul(r2.max_t - EPS_D, d));
    }
  } else {
    *p = vadd(*p, delta_p);
  }
  clamp_box(c, p);
}

/* ---- neighbour search: uniform grid, lists ascending by index -------------- */

typedef struct {
  int64_t* off;  /* n+1 */
  int64_t* idx;  /* off[n] */
} nbrs_t;

static int cmp_i64(const void* a, const void* b) {
  int64_t x = *(const int64_t*)a, y = *(const int64_t*)b;
  return (x > y) - (x < y);
}

/* N(i) = { j != i : |x*_i - x*_j|^2 <= H2 } (particles.cpp:258-265). */
static int find_neighbors(const ctx_t* c, int64_t n, const v3* xs, nbrs_t* out) {
  out->off = (int64_t*)calloc((size_t)n + 1, sizeof(int64_t));
  out->idx = NULL;
  if (!out->off) return -1;
  if (n == 0) return 0;
  real lo[3] = {xs[0].x, xs[0].y, xs[0].z}, hi[3] = {lo[0], lo[1], lo[2]};
  for (int64_t i = 1; i < n; i++)
    for (int k = 0; k < 3; k++) {
      real v = comp(xs[i], k);
      if (v < lo[k]) lo[k] = v;
      if (v > hi[k]) hi[k] = v;
    }
  const real cell = sqrt(c->h2) * (1.0 + 1e-6);
  int64_t dim[3];
  for (int k = 0; k < 3; k++) {
    if (!(hi[k] - lo[k] < 1e6 * cell)) return -2; /* non-finite or absurd extent */
    dim[k] = (int64_t)floor((hi[k] - lo[k]) / cell) + 1;
  }
  int64_t ncell = dim[0] * dim[1] * dim[2];
  if (ncell > ((int64_t)1 << 31)) return -2;
  int64_t* cell_of = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
  int64_t* start = (int64_t*)calloc((size_t)ncell + 1, sizeof(int64_t));
  int64_t* sorted = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
  if (!cell_of || !start || !sorted) return -1;
  for (int64_t i = 0; i < n; i++) {
    int64_t ci[3];
    for (int k = 0; k < 3; k++) {
      ci[k] = (int64_t)floor((comp(xs[i], k) - lo[k]) / cell);
      if (ci[k] < 0) ci[k] = 0;
      if (ci[k] >= dim[k]) ci[k] = dim[k] - 1;
    }
    cell_of[i] = (ci[2] * dim[1] + ci[1]) * dim[0] + ci[0];
    start[cell_of[i] + 1]++;
  }
  for (int64_t q = 0; q < ncell; q++) start[q + 1] += start[q];
  {
    int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncell);
    if (!fill) return -1;
    memcpy(fill, start, sizeof(int64_t) * (size_t)ncell);
    for (int64_t i = 0; i < n; i++) sorted[fill[cell_of[i]]++] = i; /* ascending within a cell */
    free(fill);
  }
  for (int pass = 0; pass < 2; pass++) {
#pragma omp parallel for schedule(dynamic, 256)
    for (int64_t i = 0; i < n; i++) {
      int64_t q = cell_of[i];
      int64_t cx = q % dim[0], cy = (q / dim[0]) % dim[1], cz = q / (dim[0] * dim[1]);
      int64_t cnt = 0;
      int64_t* dst = pass ? out->idx + out->off[i] : NULL;
      for (int64_t z = cz - 1; z <= cz + 1; z++) {
        if (z < 0 || z >= dim[2]) continue;
        for (int64_t y = cy - 1; y <= cy + 1; y++) {
          if (y < 0 || y >= dim[1]) continue;
          for (int64_t x = cx - 1; x <= cx + 1; x++) {
            if (x < 0 || x >= dim[0]) continue;
            int64_t qq = (z * dim[1] + y) * dim[0] + x;
            for (int64_t s = start[qq]; s < start[qq + 1]; s++) {
              int64_t j = sorted[s];
              if (j == i) continue;
              v3 a = xs[i < j ? i : j], b = xs[i < j ? j : i];
              if (norm2(vsub(a, b)) <= c->h2) {
                if (dst) dst[cnt] = j;
                cnt++;
              }
            }
          }
        }
      }
      if (pass == 0) {
        out->off[i + 1] = cnt;
      } else {
        qsort(dst, (size_t)cnt, sizeof(int64_t), cmp_i64);
      }
    }
    if (pass == 0) {
      for (int64_t i = 0; i < n; i++) out->off[i + 1] += out->off[i];
      out->idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)(out->off[n] > 0 ? out->off[n] : 1));
      if (!out->idx) return -1;
    }
  }
  free(cell_of);
  free(start);
  free(sorted);
  return 0;
}

/* Collider triangles besides the box walls (orc_set_mesh), as the reference's BVH holds
 * the scene's triangles: each a MarchingTriangle with the normal unit((p2 - p1) x (p3 - p1))
 * at all three vertices. Process-wide: set it before the calls that should see it. */
static int64_t g_mesh_n = 0;
static double g_mesh[9 * ORC_MAX_MESH];

int orc_set_mesh(int64_t n, const double* tri) {
  if (n < 0 || n > ORC_MAX_MESH) return -1;
  g_mesh_n = n;
  if (n) memcpy(g_mesh, tri, sizeof(double) * 9 * (size_t)n);
  return 0;
}

/* Collider spheres (orc_set_spheres): the reference's Sphere primitives in the same BVH.
 * Process-wide, like the mesh. */
static int64_t g_sph_n = 0;
static double g_sph[4 * ORC_MAX_SPH];

int orc_set_spheres(int64_t n, const double* xyzr) {
  if (n < 0 || n > ORC_MAX_SPH) return -1;
  g_sph_n = n;
  if (n) memcpy(g_sph, xyzr, sizeof(double) * 4 * (size_t)n);
  return 0;
}

static void add_mesh(ctx_t* c) {
  c->nsph = (int)g_sph_n;
  for (int64_t s = 0; s < g_sph_n; s++) {
    c->so[s] = V(g_sph[4 * s], g_sph[4 * s + 1], g_sph[4 * s + 2]);
    c->sr[s] = g_sph[4 * s + 3];
  }
  for (int64_t m = 0; m < g_mesh_n; m++) {
    const double* q = g_mesh + 9 * m;
    v3 p1 = V(q[0], q[1], q[2]), p2 = V(q[3], q[4], q[5]), p3 = V(q[6], q[7], q[8]);
    int t = c->ntri++;
    c->tp[t][0] = p1;
    c->tp[t][1] = p2;
    c->tp[t][2] = p3;
    c->tn[t] = unit(cross(vsub(p2, p1), vsub(p3, p1)));
  }
}

/* ---- the step ---------------------------------------------------------------- */

static void make_ctx(ctx_t* c, const pbf_params* p) {
  memset(c, 0, sizeof(*c));
  c->h = p->h;
  c->h2 = p->h2;
  c->h6 = intpow(p->h, 6);
  c->h9 = intpow(p->h, 9);
  c->epsilon = p->epsilon;
  c->k = p->scorr_k;
  c->vort_eps = p->vort_eps;
  c->xsph_c = p->xsph_c;
  c->rest_density = p->rest_density;
  c->iters = p->iters;
  c->scorr_n = p->scorr_n;
  c->gravity = V(p->gravity[0], p->gravity[1], p->gravity[2]);
  for (int k = 0; k < 3; k++) {
    c->clamp_lo[k] = p->clamp_lo[k];
    c->clamp_hi[k] = p->clamp_hi[k];
  }
  c->n_clip = p->n_clip < 0 ? 0 : (p->n_clip > 2 ? 2 : p->n_clip);
  for (int i = 0; i < c->n_clip; i++) {
    c->clip_axis[i] = p->clip_axis[i];
    c->clip_value[i] = p->clip_value[i];
  }
  build_box(c, p->box_lo, p->box_hi, p->box_open_mask);
  add_mesh(c);
  /* Particle::tensile_instability_scale, particles.cpp:151 */
  c->tis = 1.0 / poly6(c, V(0, 0, p->scorr_dq * p->h));
}

typedef struct {
  double density_iter0_sum;
} step_info_t;

/*
 * One step, "jacobi" form (see file comment). pos/vel/rho: n entries (v3 / real).
 * nb receives the neighbour lists of this step (caller frees).
 */
static int step_once(const ctx_t* c, int64_t n, v3* x, v3* v, real* rho, real dt,
                     nbrs_t* nb, const nbrs_t* given, v3* pred_out, step_info_t* info) {
  v3* xs = (v3*)malloc(sizeof(v3) * (size_t)(n ? n : 1));
  real* lam = (real*)malloc(sizeof(real) * (size_t)(n ? n : 1));
  v3* vort = (v3*)malloc(sizeof(v3) * (size_t)(n ? n : 1));
  v3* vnew = (v3*)malloc(sizeof(v3) * (size_t)(n ? n : 1));
  if (!xs || !lam || !vort || !vnew) return -1;

  /* applyForceVelocity, particles.cpp:175-183 */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    if (c->gravity.x != 0.0) v[i].x -= (-c->gravity.x) * dt;
    if (c->gravity.y != 0.0) v[i].y -= (-c->gravity.y) * dt;
    if (c->gravity.z != 0.0) v[i].z -= (-c->gravity.z) * dt;
    xs[i] = x[i];
    clamp_response(c, &xs[i], v[i], dt);
  }
  if (pred_out) memcpy(pred_out, xs, sizeof(v3) * (size_t)n);

  int rc = 0;
  if (given) {
    /* caller-supplied neighbour sets (ascending per particle) replace the search */
    nb->off = (int64_t*)malloc(sizeof(int64_t) * (size_t)(n + 1));
    nb->idx = (int64_t*)malloc(sizeof(int64_t) * (size_t)(given->off[n] > 0 ? given->off[n] : 1));
    if (!nb->off || !nb->idx) return -1;
    memcpy(nb->off, given->off, sizeof(int64_t) * (size_t)(n + 1));
    if (given->off[n] > 0) memcpy(nb->idx, given->idx, sizeof(int64_t) * (size_t)given->off[n]);
  } else {
    rc = find_neighbors(c, n, xs, nb);
    if (rc) return rc;
  }
  const int64_t* off = nb->off;
  const int64_t* idx = nb->idx;
  int64_t nnz = off[n];
  real* scorr = (real*)malloc(sizeof(real) * (size_t)(nnz ? nnz : 1));
  v3* gw = (v3*)malloc(sizeof(v3) * (size_t)(nnz ? nnz : 1));
  if (!scorr || !gw) return -1;

  for (int it = 0; it < c->iters; it++) {
    /* newtonStepCalculateLambda, particles.cpp:185-204 */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      real density = 0.0, denom = 0.0;
      v3 grad_i_c_i = V(0, 0, 0);
      for (int64_t e = off[i]; e < off[i + 1]; e++) {
        v3 r = vsub(xs[i], xs[idx[e]]);
        real w = poly6(c, r);
        v3 g = spiky(c, r);
        density += w;
        scorr[e] = -c->k * intpow(w * c->tis, c->scorr_n);
        gw[e] = g;
        g = svmul(1. / c->rest_density, g);
        grad_i_c_i = vadd(grad_i_c_i, g);
        denom += norm2(g);
      }
      real c_i = density / c->rest_density - 1.0;
      denom += norm2(grad_i_c_i);
      lam[i] = -c_i / (denom + c->epsilon);
      rho[i] = density;
    }
    if (it == 0 && info) {
      double s = 0.0;
      for (int64_t i = 0; i < n; i++) s += rho[i];
      info->density_iter0_sum = s;
    }
    /* newtonStepUpdatePosition, particles.cpp:206-213 */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      v3 delta_p = V(0, 0, 0);
      for (int64_t e = off[i]; e < off[i + 1]; e++) {
        delta_p = vadd(delta_p, svmul(lam[i] + lam[idx[e]] + scorr[e], gw[e]));
      }
      delta_p = svmul(1. / c->rest_density, delta_p);
      clamp_move(c, &xs[i], delta_p);
    }
  }

  /* updateVelocity, particles.cpp:215-217 */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) v[i] = vdiv(vsub(xs[i], x[i]), dt);

  /* calculateVorticityApplyXSPHViscosity, particles.cpp:219-234 (pre-XSPH neighbour velocities) */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    v3 w_acc = V(0, 0, 0), visc = V(0, 0, 0);
    real density = 0.0;
    for (int64_t e = off[i]; e < off[i + 1]; e++) {
      int64_t j = idx[e];
      v3 v_i_n = vsub(v[j], v[i]);
      v3 r = vsub(xs[i], xs[j]);
      v3 g = spiky(c, r);
      w_acc = vadd(w_acc, cross(v_i_n, g));
      real w = poly6(c, r);
      visc = vadd(visc, vscale(v_i_n, w));
      gw[e] = g;
      density += w;
    }
    vort[i] = w_acc;
    rho[i] = density;
    vnew[i] = vadd(v[i], svmul(c->xsph_c, visc));
  }

  /* applyVorticity + updatePosition, particles.cpp:236-248, 289-294 */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    v3 gv = V(0, 0, 0);
    for (int64_t e = off[i]; e < off[i + 1]; e++) {
      gv = vadd(gv, svmul(vnorm(vort[idx[e]]), gw[e]));
    }
    v3 vi = vnew[i];
    if (vnorm(gv) > EPS_D) {
      vi = vadd(vi, svmul(dt * c->vort_eps, cross(unit(gv), vort[i])));
    }
    v[i] = vi;
    x[i] = xs[i];
  }
  free(xs);
  free(lam);
  free(vort);
  free(vnew);
  free(scorr);
  free(gw);
  return 0;
}

/* double (n,3) arrays <-> v3 of real (a copy also when real is double) */
static v3* to_v3(const double* a, int64_t n) {
  v3* r = (v3*)malloc(sizeof(v3) * (size_t)(n ? n : 1));
  if (r && a)
    for (int64_t i = 0; i < n; i++) r[i] = V((real)a[3 * i], (real)a[3 * i + 1], (real)a[3 * i + 2]);
  return r;
}
static void from_v3(double* a, const v3* r, int64_t n) {
  for (int64_t i = 0; i < n; i++) {
    a[3 * i] = r[i].x;
    a[3 * i + 1] = r[i].y;
    a[3 * i + 2] = r[i].z;
  }
}

/* ---- exported ---------------------------------------------------------------- */

static void set_threads(int nthreads) {
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#else
  (void)nthreads;
#endif
}

int orc_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

/*
 * nsteps steps in place on pos/vel ((n,3) float64); rho[n] receives the
 * reported densities. If nbr_off (n+1) is given, the last step's neighbour
 * lists are written to nbr_off / nbr_idx (capacity nbr_cap); returns 1 if the
 * capacity was too small (nbr_off[n] then holds the needed count). pred
 * ((n,3) or NULL) receives x* after the last prediction; rho_iter0 (nsteps or
 * NULL) the mean density after each step's first lambda pass. orc_step2 also takes
 * the first step's neighbour sets from in_off/in_idx (ascending lists) instead of
 * searching, so an FP32 implementation can be compared on identical sets.
 */
int orc_step2(const pbf_params* prm, int64_t n, double* pos, double* vel, double* rho,
              int nsteps, double dt, int64_t* nbr_off, int64_t* nbr_idx, int64_t nbr_cap,
              double* pred, double* rho_iter0, const int64_t* in_off, const int64_t* in_idx,
              int nthreads) {
  set_threads(nthreads);
  ctx_t* c = (ctx_t*)malloc(sizeof(ctx_t));
  v3* x = to_v3(pos, n);
  v3* v = to_v3(vel, n);
  v3* pr = pred ? to_v3(NULL, n) : NULL;
  real* rr = (real*)malloc(sizeof(real) * (size_t)(n ? n : 1));
  if (!c || !x || !v || !rr || (pred && !pr)) return -1;
  make_ctx(c, prm);
  int rc = 0;
  for (int s = 0; s < nsteps && rc == 0; s++) {
    nbrs_t nb = {NULL, NULL};
    step_info_t info = {0};
    nbrs_t given = {(int64_t*)in_off, (int64_t*)in_idx};
    rc = step_once(c, n, x, v, rr, (real)dt, &nb, (in_off && s == 0) ? &given : NULL,
                   (pred && s == nsteps - 1) ? pr : NULL, &info);
    if (rc == 0 && rho_iter0) rho_iter0[s] = n ? info.density_iter0_sum / (double)n : 0.0;
    if (rc == 0 && s == nsteps - 1 && nbr_off) {
      memcpy(nbr_off, nb.off, sizeof(int64_t) * (size_t)(n + 1));
      if (nb.off[n] > nbr_cap) {
        rc = 1;
      } else if (nb.off[n] > 0) {
        memcpy(nbr_idx, nb.idx, sizeof(int64_t) * (size_t)nb.off[n]);
      }
    }
    free(nb.off);
    free(nb.idx);
  }
  from_v3(pos, x, n);
  from_v3(vel, v, n);
  if (pred) from_v3(pred, pr, n);
  for (int64_t i = 0; i < n; i++) rho[i] = rr[i];
  free(x);
  free(v);
  free(pr);
  free(rr);
  free(c);
  return rc;
}

int orc_step(const pbf_params* prm, int64_t n, double* pos, double* vel, double* rho,
             int nsteps, double dt, int64_t* nbr_off, int64_t* nbr_idx, int64_t nbr_cap,
             double* pred, double* rho_iter0, int nthreads) {
  return orc_step2(prm, n, pos, vel, rho, nsteps, dt, nbr_off, nbr_idx, nbr_cap, pred, rho_iter0,
                   NULL, NULL, nthreads);
}

/* Particles::estimateDensities, particles.cpp:440-444: self included, sum in index order. */
int orc_estimate_densities(const pbf_params* prm, int64_t n, const double* pos, double* out,
                           int nthreads) {
  set_threads(nthreads);
  ctx_t* c = (ctx_t*)malloc(sizeof(ctx_t));
  if (!c) return -1;
  make_ctx(c, prm);
  v3* x = to_v3(pos, n);
  if (!x) return -1;
  nbrs_t nb = {NULL, NULL};
  int rc = find_neighbors(c, n, x, &nb);
  if (rc == 0) {
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      real d = 0.0;
      int self_done = 0;
      for (int64_t e = nb.off[i]; e < nb.off[i + 1]; e++) {
        int64_t j = nb.idx[e];
        if (!self_done && j > i) {
          d += poly6(c, vsub(x[i], x[i]));
          self_done = 1;
        }
        d += poly6(c, vsub(x[j], x[i]));
      }
      if (!self_done) d += poly6(c, vsub(x[i], x[i]));
      out[i] = d;
    }
  }
  free(nb.off);
  free(nb.idx);
  free(x);
  free(c);
  return rc;
}

/* Particles::estimateDensityAt, particles.cpp:446-453, brute force in index order. */
int orc_estimate_density_at(const pbf_params* prm, int64_t n, const double* pos, int64_t m,
                            const double* pts, double* out, int nthreads) {
  set_threads(nthreads);
  ctx_t* c = (ctx_t*)malloc(sizeof(ctx_t));
  if (!c) return -1;
  make_ctx(c, prm);
  v3* x = to_v3(pos, n);
  v3* q = to_v3(pts, m);
  if (!x || !q) return -1;
#pragma omp parallel for schedule(static)
  for (int64_t k = 0; k < m; k++) {
    real d = 0.0;
    for (int64_t i = 0; i < n; i++) d += poly6(c, vsub(x[i], q[k]));
    out[k] = d;
  }
  free(x);
  free(q);
  free(c);
  return 0;
}

/* ---- neighbour sets under the FP32 predicate ------------------------------------ */

typedef struct {
  int64_t* a;
  int64_t n, cap;
} i64buf_t;

static int buf_push(i64buf_t* b, int64_t v) {
  if (b->n == b->cap) {
    int64_t nc = b->cap ? 2 * b->cap : 256;
    int64_t* na = (int64_t*)realloc(b->a, sizeof(int64_t) * (size_t)nc);
    if (!na) return -1;
    b->a = na;
    b->cap = nc;
  }
  b->a[b->n++] = v;
  return 0;
}

/*
 * The neighbour relation of particles.cpp:258-265, N(i) = { j != i : |x_i - x_j|^2 <= H2 },
 * evaluated in FP32 on FP32 positions exactly as an FP32 implementation must round it:
 * dx = fl(x_i - x_j) per axis, r2 = fl(fl(fl(dx dx) + fl(dy dy)) + fl(dz dz)), r2 <= h2
 * (this file is built with -ffp-contract=off, so nothing is fused). A uniform grid of
 * cell 1.01 sqrt(h2) (pruning only) lists the candidates; the sets are compared with the
 * given ascending CSR lists (off[n+1], ids). Returns 0 and writes the number of
 * particles whose sets differ, the pairs the given lists miss and the pairs they hold
 * in excess, and the first differing particle (-1 if none); -1 when out of memory,
 * -2 for a non-finite or absurd extent.
 */
int orc_nbr_check_fp32(int64_t n, const float* xs, float h2, const int64_t* off, const uint32_t* ids,
                       int64_t* bad, int64_t* missing, int64_t* extra, int64_t* first_bad, int nthreads) {
  set_threads(nthreads);
  *bad = *missing = *extra = 0;
  *first_bad = -1;
  if (n == 0) return 0;
  double lo[3] = {xs[0], xs[1], xs[2]}, hi[3] = {lo[0], lo[1], lo[2]};
  for (int64_t i = 1; i < n; i++)
    for (int k = 0; k < 3; k++) {
      const double v = xs[3 * i + k];
      if (v < lo[k]) lo[k] = v;
      if (v > hi[k]) hi[k] = v;
    }
  const double cell = 1.01 * sqrt((double)h2);
  int64_t dim[3];
  for (int k = 0; k < 3; k++) {
    if (!(hi[k] - lo[k] < 1e6 * cell)) return -2;
    dim[k] = (int64_t)floor((hi[k] - lo[k]) / cell) + 1;
  }
  const int64_t ncell = dim[0] * dim[1] * dim[2];
  if (ncell > ((int64_t)1 << 31)) return -2;
  int64_t* cell_of = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
  int64_t* start = (int64_t*)calloc((size_t)ncell + 1, sizeof(int64_t));
  int64_t* sorted = (int64_t*)malloc(sizeof(int64_t) * (size_t)n);
  int64_t* fill = (int64_t*)malloc(sizeof(int64_t) * (size_t)ncell);
  if (!cell_of || !start || !sorted || !fill) return -1;
  for (int64_t i = 0; i < n; i++) {
    int64_t ci[3];
    for (int k = 0; k < 3; k++) {
      ci[k] = (int64_t)floor(((double)xs[3 * i + k] - lo[k]) / cell);
      if (ci[k] < 0) ci[k] = 0;
      if (ci[k] >= dim[k]) ci[k] = dim[k] - 1;
    }
    cell_of[i] = (ci[2] * dim[1] + ci[1]) * dim[0] + ci[0];
    start[cell_of[i] + 1]++;
  }
  for (int64_t q = 0; q < ncell; q++) start[q + 1] += start[q];
  memcpy(fill, start, sizeof(int64_t) * (size_t)ncell);
  for (int64_t i = 0; i < n; i++) sorted[fill[cell_of[i]]++] = i;
  free(fill);
  int64_t nbad = 0, nmiss = 0, nextra = 0, first = -1;
  int oom = 0;
#pragma omp parallel reduction(+ : nbad, nmiss, nextra)
  {
    i64buf_t b = {NULL, 0, 0};
    int64_t my_first = -1;
#pragma omp for schedule(dynamic, 1024)
    for (int64_t i = 0; i < n; i++) {
      const int64_t q = cell_of[i];
      const int64_t cx = q % dim[0], cy = (q / dim[0]) % dim[1], cz = q / (dim[0] * dim[1]);
      const float xi = xs[3 * i], yi = xs[3 * i + 1], zi = xs[3 * i + 2];
      b.n = 0;
      for (int64_t z = cz - 1; z <= cz + 1; z++) {
        if (z < 0 || z >= dim[2]) continue;
        for (int64_t y = cy - 1; y <= cy + 1; y++) {
          if (y < 0 || y >= dim[1]) continue;
          for (int64_t x = cx - 1; x <= cx + 1; x++) {
            if (x < 0 || x >= dim[0]) continue;
            const int64_t qq = (z * dim[1] + y) * dim[0] + x;
            for (int64_t s = start[qq]; s < start[qq + 1]; s++) {
              const int64_t j = sorted[s];
              if (j == i) continue;
              const float dx = xi - xs[3 * j], dy = yi - xs[3 * j + 1], dz = zi - xs[3 * j + 2];
              const float ax = dx * dx, ay = dy * dy, az = dz * dz;
              const float sxy = ax + ay;
              const float r2 = sxy + az;
              if (r2 <= h2 && buf_push(&b, j) != 0) oom = 1;
            }
          }
        }
      }
      qsort(b.a, (size_t)b.n, sizeof(int64_t), cmp_i64);
      /* merge the expected set b with the given list */
      int64_t u = 0, e = off[i], ee = off[i + 1], m = 0, x = 0;
      while (u < b.n || e < ee) {
        if (e >= ee || (u < b.n && b.a[u] < (int64_t)ids[e])) {
          m++;
          u++;
        } else if (u >= b.n || (int64_t)ids[e] < b.a[u]) {
          x++;
          e++;
        } else {
          u++;
          e++;
        }
      }
      if (m || x) {
        nbad++;
        nmiss += m;
        nextra += x;
        if (my_first < 0 || i < my_first) my_first = i;
      }
    }
#pragma omp critical
    {
      if (my_first >= 0 && (first < 0 || my_first < first)) first = my_first;
    }
    free(b.a);
  }
  free(cell_of);
  free(start);
  free(sorted);
  if (oom) return -1;
  *bad = nbad;
  *missing = nmiss;
  *extra = nextra;
  *first_bad = first;
  return 0;
}

/* ---- surface (Particles::getSurfacePrims, particles.cpp:352-385) ------------------- */

/* estimateDensityAt, particles.cpp:446-453: poly6 summed over every particle in index order */
static real density_at(const ctx_t* c, int64_t n, const v3* x, v3 p) {
  real d = 0.0;
  for (int64_t i = 0; i < n; i++) d += poly6(c, vsub(x[i], p));
  return d;
}

/* vertexInterp (marching.cpp) */
static v3 vertex_interp(real iso, v3 p1, v3 p2, real v1, real v2) {
  if (fabs(iso - v1) < 0.00001) return p1;
  if (fabs(iso - v2) < 0.00001) return p2;
  if (fabs(v1 - v2) < 0.00001) return p1;
  real mu = (iso - v1) / (v2 - v1);
  return V(p1.x + mu * (p2.x - p1.x), p1.y + mu * (p2.y - p1.y), p1.z + mu * (p2.z - p1.z));
}

/* getVertexNormal, particles.cpp:399-412 (GRADIENT_EPS = 0.001, :16) */
static v3 vertex_normal(const ctx_t* c, int64_t n, const v3* x, v3 p) {
  const real e = 0.001;
  v3 g = V(density_at(c, n, x, V(p.x - e, p.y, p.z)) - density_at(c, n, x, V(p.x + e, p.y, p.z)),
           density_at(c, n, x, V(p.x, p.y - e, p.z)) - density_at(c, n, x, V(p.x, p.y + e, p.z)),
           density_at(c, n, x, V(p.x, p.y, p.z - e)) - density_at(c, n, x, V(p.x, p.y, p.z + e)));
  if (vnorm(g) > 0) return unit(g);
  return g;
}

/*
 * The surface of the density field of `pos` with the caller's triangulation table
 * (ntri[256], tri[256 * 15] as edge triples; corners and edges numbered as
 * generateGridCell, particles.cpp:309-323, and polygonise, marching.cpp). The loops,
 * corner points (x2 = min(hi, x1 + step)), corner values and edge vertices follow the
 * reference; cubes in its order (x outer, y, z inner). Writes the first `cap`
 * triangles (9 doubles of vertices and 9 of normals each) and the cube index of each
 * (ix * ncy + iy) * ncz + iz; returns the total count, or -1 when out of memory.
 */
int64_t orc_surface(const pbf_params* prm, int64_t n, const double* pos, double iso, double step, const double* lo,
                    const double* hi, const uint8_t* ntri, const int8_t* tri, double* xyz, double* nrm, int64_t* cube,
                    int64_t cap, int nthreads) {
  set_threads(nthreads);
  ctx_t* c = (ctx_t*)malloc(sizeof(ctx_t));
  v3* x = to_v3(pos, n);
  if (!c || !x) return -1;
  make_ctx(c, prm);
  int steps[3], nc[3];
  for (int a = 0; a < 3; a++) {
    steps[a] = (int)((hi[a] - lo[a]) / step);
    nc[a] = steps[a] + 1;
  }
  const int64_t ncubes = (int64_t)nc[0] * nc[1] * nc[2];
  int* cnt = (int*)malloc(sizeof(int) * (size_t)(ncubes ? ncubes : 1));
  int* cfg = (int*)malloc(sizeof(int) * (size_t)(ncubes ? ncubes : 1));
  double* vals = (double*)malloc(sizeof(double) * 8 * (size_t)(ncubes ? ncubes : 1));
  v3* pts = (v3*)malloc(sizeof(v3) * 8 * (size_t)(ncubes ? ncubes : 1));
  if (!cnt || !cfg || !vals || !pts) return -1;
  static const int corner[8][3] = {{0, 0, 0}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0},
                                   {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {1, 0, 1}};
#pragma omp parallel for schedule(dynamic, 16)
  for (int64_t q = 0; q < ncubes; q++) {
    const int iz = (int)(q % nc[2]), iy = (int)((q / nc[2]) % nc[1]), ix = (int)(q / ((int64_t)nc[2] * nc[1]));
    const real x1 = lo[0] + ix * step, y1 = lo[1] + iy * step, z1 = lo[2] + iz * step;
    const real x2 = smin(hi[0], x1 + step), y2 = smin(hi[1], y1 + step), z2 = smin(hi[2], z1 + step);
    const real xs[2] = {x1, x2}, ys[2] = {y1, y2}, zs[2] = {z1, z2};
    int ci = 0;
    for (int k = 0; k < 8; k++) {
      v3 p = V(xs[corner[k][0]], ys[corner[k][1]], zs[corner[k][2]]);
      pts[8 * q + k] = p;
      vals[8 * q + k] = density_at(c, n, x, p);
      if (vals[8 * q + k] < iso) ci |= 1 << k;
    }
    cfg[q] = ci;
    cnt[q] = ntri[ci];
  }
  static const int edge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                  {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};
  int64_t total = 0;
  for (int64_t q = 0; q < ncubes; q++) {
    for (int t = 0; t < cnt[q]; t++, total++) {
      if (total >= cap) continue;
      for (int v = 0; v < 3; v++) {
        const int e = tri[15 * cfg[q] + 3 * t + v];
        const int a = edge[e][0], b = edge[e][1];
        v3 p = vertex_interp(iso, pts[8 * q + a], pts[8 * q + b], vals[8 * q + a], vals[8 * q + b]);
        v3 m = vertex_normal(c, n, x, p);
        xyz[9 * total + 3 * v] = p.x;
        xyz[9 * total + 3 * v + 1] = p.y;
        xyz[9 * total + 3 * v + 2] = p.z;
        nrm[9 * total + 3 * v] = m.x;
        nrm[9 * total + 3 * v + 1] = m.y;
        nrm[9 * total + 3 * v + 2] = m.z;
      }
      if (cube) cube[total] = q;
    }
  }
  free(cnt);
  free(cfg);
  free(vals);
  free(pts);
  free(x);
  free(c);
  return total;
}
