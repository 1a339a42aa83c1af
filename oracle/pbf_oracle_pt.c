/* CPU restatement of the reference's path tracer (TEST INFRASTRUCTURE: the oracle of
 * the renderer; only tests/ and the fixture generators call it).
 *
 * Follows src/pathtracer.cpp:483-632 (estimate_direct_lighting,
 * estimate_indirect_lighting, trace_ray, raytrace_pixel), src/bsdf.cpp (make_coord_space
 * and the BSDFs), src/static_scene/light.cpp (sample_L), src/sampler.cpp, src/camera.cpp
 * (configure, place, compute_position, generate_ray), src/static_scene/marching_triangle.cpp
 * (ray-triangle test) and src/image.h:49-58, 174-189 (toColor and the 8-bit packing), with
 * the reference's own arithmetic types: geometry in double (CGL Vector3D, Matrix3x3),
 * radiance in float (CGL Spectrum), a double multiplied into a Spectrum is first rounded
 * to float. The scene's BVH (src/bvh.cpp) is replaced by a test of every triangle in
 * index order; the closest hit is the same except on exact ties of t.
 *
 * Two sources of random numbers:
 *  - ORC_RNG_STD: the reference's random_uniform() = rand() / RAND_MAX
 *    (src/random_util.h) after srand(seed), pixels in the order of the reference's single
 *    render thread: 32x32 tiles in queue order (rows of tiles from y = 0), each tile row
 *    by row (src/pathtracer.cpp:205-210, 590-608). Serial.
 *  - ORC_RNG_COUNTER: the draws of the GPU renderer: draw k of sample s of pixel p is
 *    the top 24 bits of splitmix64(key(p, s) + k * golden gamma) times 2^-24 (a float
 *    that is the same number in FP32 and FP64). Pixels in parallel.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_RNG_STD 0
#define ORC_RNG_COUNTER 1

#define EPS_D 0.00000000001
#define PI_D 3.14159265358979323846

enum { MAT_DIFFUSE = 0, MAT_MIRROR = 1, MAT_GLASS = 2, MAT_REFRACTION = 3, MAT_EMISSION = 4 };
enum { LIGHT_DIRECTIONAL = 0, LIGHT_HEMISPHERE = 1, LIGHT_POINT = 2, LIGHT_AREA = 3 };

typedef struct { double x, y, z; } v3;
typedef struct { float r, g, b; } sp;

typedef struct {
  int64_t kind;
  double c1[3], c2[3];
  double ior;
} orc_mat_t;

typedef struct {
  int64_t kind;
  double radiance[3], position[3], direction[3], dim_x[3], dim_y[3];
} orc_light_t;

/* camera frame after Camera::configure + place: position, c2w columns, fields of view
 * (degrees), clip distances */
typedef struct {
  double pos[3];
  double c2w[9];
  double hfov, vfov, nclip, fclip;
} orc_cam_t;

/* ---- CGL vector and spectrum arithmetic (vector3D.h, spectrum.h) ---------------- */
static inline v3 V(double x, double y, double z) { v3 r = {x, y, z}; return r; }
static inline v3 add(v3 a, v3 b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3 sub(v3 a, v3 b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3 mul(v3 a, double c) { return V(a.x * c, a.y * c, a.z * c); }      /* v * c */
static inline v3 smul(double c, v3 a) { return V(c * a.x, c * a.y, c * a.z); }     /* c * v */
static inline v3 neg(v3 a) { return V(-a.x, -a.y, -a.z); }
static inline double dot(v3 u, v3 v) { return u.x * v.x + u.y * v.y + u.z * v.z; }
static inline v3 cross(v3 u, v3 v) {
  return V(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
}
static inline double norm(v3 a) { return sqrt(a.x * a.x + a.y * a.y + a.z * a.z); }
static inline double norm2(v3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline v3 divv(v3 a, double c) { const double rc = 1.0 / c; return V(rc * a.x, rc * a.y, rc * a.z); }
static inline v3 normalize(v3 a) { const double c = 1. / norm(a); return V(a.x * c, a.y * c, a.z * c); }
static inline v3 unit(v3 a) {
  const double r = 1. / sqrt(a.x * a.x + a.y * a.y + a.z * a.z);
  return V(r * a.x, r * a.y, r * a.z);
}
static inline v3 ld3(const double* p) { return V(p[0], p[1], p[2]); }

static inline sp S(float r, float g, float b) { sp s = {r, g, b}; return s; }
static inline sp sadd(sp a, sp b) { return S(a.r + b.r, a.g + b.g, a.b + b.b); }
static inline sp sprod(sp a, sp b) { return S(a.r * b.r, a.g * b.g, a.b * b.b); }
static inline sp sscale(sp a, float s) { return S(a.r * s, a.g * s, a.b * s); }
static inline sp sdiv(sp a, float s) { return S(a.r / s, a.g / s, a.b / s); }
static inline float illum(sp a) { return 0.2126f * a.r + 0.7152f * a.g + 0.0722f * a.b; }
static inline sp sp3(const double* c) { return S((float)c[0], (float)c[1], (float)c[2]); }

/* Matrix3x3 stored by columns; M * x = x0 c0 + x1 c1 + x2 c2 (matrix3x3.cpp:138-142) */
typedef struct { v3 c[3]; } m3;
static inline v3 mv(const m3* M, v3 x) {
  return add(add(smul(x.x, M->c[0]), smul(x.y, M->c[1])), smul(x.z, M->c[2]));
}
static inline m3 transpose(const m3* A) {
  m3 B;
  const double a[3][3] = {{A->c[0].x, A->c[0].y, A->c[0].z},
                          {A->c[1].x, A->c[1].y, A->c[1].z},
                          {A->c[2].x, A->c[2].y, A->c[2].z}}; /* a[col][row] */
  for (int j = 0; j < 3; j++) B.c[j] = V(a[0][j], a[1][j], a[2][j]);
  return B;
}

/* bsdf.cpp:13-32 */
static m3 make_coord_space(v3 n) {
  v3 z = n, h = z;
  if (fabs(h.x) <= fabs(h.y) && fabs(h.x) <= fabs(h.z)) h.x = 1.0;
  else if (fabs(h.y) <= fabs(h.x) && fabs(h.y) <= fabs(h.z)) h.y = 1.0;
  else h.z = 1.0;
  z = normalize(z);
  v3 y = normalize(cross(h, z));
  v3 x = normalize(cross(z, y));
  m3 M;
  M.c[0] = x;
  M.c[1] = y;
  M.c[2] = z;
  return M;
}

/* ---- random numbers ---------------------------------------------------------------- */
typedef struct {
  int mode;
  uint64_t key, k;
} rng_t;

static inline uint64_t splitmix64(uint64_t x) {
  uint64_t z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

/* key of sample s of pixel p: the GPU renderer derives it the same way */
static inline uint64_t path_key(uint64_t seed, uint64_t pixel, uint64_t sample) {
  return splitmix64(seed ^ splitmix64((pixel << 20) ^ sample));
}

static inline double uniform(rng_t* g) {
  if (g->mode == ORC_RNG_STD) return ((double)rand()) / RAND_MAX;
  const uint64_t z = splitmix64(g->key + (g->k++) * 0x9E3779B97F4A7C15ull);
  return (double)(z >> 40) * (1.0 / 16777216.0);
}

/* Vector2D(random_uniform(), random_uniform()) (sampler.cpp:7-11): the reference's
 * build evaluates the second argument first; the counter draws keep x first. */
static inline void sample2d(rng_t* g, double* x, double* y) {
  if (g->mode == ORC_RNG_STD) {
    *y = uniform(g);
    *x = uniform(g);
  } else {
    *x = uniform(g);
    *y = uniform(g);
  }
}

/* CosineWeightedHemisphereSampler3D::get_sample (sampler.cpp:35-45) */
static v3 cosine_sample(rng_t* g, float* pdf) {
  const double Xi1 = uniform(g);
  const double Xi2 = uniform(g);
  const double r = sqrt(Xi1);
  const double theta = 2. * PI_D * Xi2;
  *pdf = (float)(sqrt(1 - Xi1) / PI_D);
  return V(r * cos(theta), r * sin(theta), sqrt(1 - Xi1));
}

/* UniformHemisphereSampler3D::get_sample (sampler.cpp:15-28) */
static v3 hemisphere_sample(rng_t* g) {
  const double Xi1 = uniform(g);
  const double Xi2 = uniform(g);
  const double theta = acos(Xi1);
  const double phi = 2.0 * PI_D * Xi2;
  const double xs = sinf((float)theta) * cosf((float)phi);
  const double ys = sinf((float)theta) * sinf((float)phi);
  const double zs = cosf((float)theta);
  return V(xs, ys, zs);
}

static inline int coin_flip(rng_t* g, double p) { return uniform(g) < p; }

/* ---- scene -------------------------------------------------------------------------- */
typedef struct {
  const double* tri;
  const double* nrm;
  const int64_t* tri_mat;
  int64_t ntri;
  const orc_mat_t* mats;
  const orc_light_t* lights;
  int64_t nlights;
  int64_t ns_area_light;
} scene_t;

typedef struct {
  v3 o, d;
  double min_t, max_t;
  int64_t depth;
} ray_t;

typedef struct {
  double t;
  v3 n;
  int64_t tri;
} isect_t;

/* MarchingTriangle::intersect (marching_triangle.cpp:21-73); updates r->max_t */
static int tri_hit(const scene_t* sc, int64_t k, ray_t* r, isect_t* is) {
  const double* q = sc->tri + 9 * k;
  const v3 p1 = ld3(q), p2 = ld3(q + 3), p3 = ld3(q + 6);
  const v3 e1 = sub(p2, p1), e2 = sub(p3, p1), s = sub(r->o, p1);
  const v3 s1 = cross(r->d, e2), s2 = cross(s, e1);
  const double d = dot(s1, e1);
  if (d == 0) return 0;
  const double t = dot(s2, e2) / d;
  if ((t < r->min_t) || (t > r->max_t)) return 0;
  const double u = dot(s1, s) / d;
  const double v = dot(s2, r->d) / d;
  const double w = 1 - u - v;
  if ((u < 0) || (u > 1) || (v < 0) || (v > 1) || (w < 0) || (w > 1)) return 0;
  r->max_t = t;
  if (is) {
    const double* m = sc->nrm + 9 * k;
    is->t = t;
    is->n = add(add(smul(w, ld3(m)), smul(u, ld3(m + 3))), smul(v, ld3(m + 6)));
    is->tri = k;
  }
  return 1;
}

static int closest_hit(const scene_t* sc, ray_t r, isect_t* is) {
  int hit = 0;
  for (int64_t k = 0; k < sc->ntri; k++) hit |= tri_hit(sc, k, &r, is);
  return hit;
}

static int any_hit(const scene_t* sc, ray_t r) {
  for (int64_t k = 0; k < sc->ntri; k++)
    if (tri_hit(sc, k, &r, NULL)) return 1;
  return 0;
}

/* ---- BSDFs (bsdf.cpp) ----------------------------------------------------------------- */
static int is_delta(const orc_mat_t* m) {
  return m->kind == MAT_MIRROR || m->kind == MAT_GLASS || m->kind == MAT_REFRACTION;
}

static sp bsdf_f(const orc_mat_t* m) {
  if (m->kind == MAT_DIFFUSE) return sscale(sp3(m->c1), (float)(1.0 / PI_D));
  return S(0, 0, 0);
}

static sp emission(const orc_mat_t* m) {
  return m->kind == MAT_EMISSION ? sp3(m->c1) : S(0, 0, 0);
}

/* BSDF::refract (bsdf.cpp:118-145) */
static int refract(v3 wo, v3* wi, float ior) {
  double ni, no;
  if (wo.z > 0) {
    no = 1.0;
    ni = ior;
  } else {
    no = ior;
    ni = 1.0;
  }
  const double sint2 = (1.0 - wo.z * wo.z) * no * no / ni / ni;
  if (sint2 >= 1.0) return 0;
  double cost = sqrt(1.0 - sint2);
  if (wo.z > 0) cost = -cost;
  *wi = normalize(V(-wo.x * no / ni, -wo.y * no / ni, cost));
  return 1;
}

/* sample_f of each BSDF; *valid = 0 where the reference leaves wi and pdf unset */
static sp bsdf_sample_f(const orc_mat_t* m, v3 wo, v3* wi, float* pdf, rng_t* g) {
  switch (m->kind) {
    case MAT_DIFFUSE:
      *wi = cosine_sample(g, pdf);
      return sscale(sp3(m->c1), (float)(1.0 / PI_D));
    case MAT_MIRROR:
      *wi = V(-wo.x, -wo.y, wo.z);
      *pdf = 1.0f;
      return sscale(sp3(m->c1), (float)(1 / fabs(wi->z)));
    case MAT_GLASS: {
      const float ior = (float)m->ior;
      if (!refract(wo, wi, ior)) {
        *wi = V(-wo.x, -wo.y, wo.z);
        *pdf = 1.0f;
        return sscale(sp3(m->c2), (float)(1.0 / fabs(wi->z)));
      }
      double R = (ior - 1.0) * (ior - 1.0) / (ior + 1.0) / (ior + 1.0);
      const double c = 1.0 - fabs(wi->z);
      R = R + (1.0 - R) * c * c * c * c * c;
      if (coin_flip(g, R)) {
        *wi = V(-wo.x, -wo.y, wo.z);
        *pdf = (float)R;
        return sscale(sp3(m->c2), (float)(R / fabs(wi->z)));
      }
      *pdf = (float)(1.0 - R);
      const double nr = wi->z > 0 ? ior : 1.0 / ior;
      return sscale(sp3(m->c1), (float)((1.0 - R) * nr * nr / fabs(wi->z)));
    }
    case MAT_EMISSION:
      *pdf = (float)(1.0 / PI_D);
      *wi = cosine_sample(g, pdf);
      return S(0, 0, 0);
    default: /* RefractionBSDF::sample_f returns black and sets nothing */
      *wi = V(0, 0, 1);
      *pdf = 1.0f;
      return S(0, 0, 0);
  }
}

/* ---- lights (light.cpp) ------------------------------------------------------------------ */
static int light_is_delta(const orc_light_t* l) {
  return l->kind == LIGHT_DIRECTIONAL || l->kind == LIGHT_POINT;
}

static sp sample_L(const orc_light_t* l, v3 p, v3* wi, float* dist, float* pdf, rng_t* g) {
  switch (l->kind) {
    case LIGHT_DIRECTIONAL:
      *wi = neg(unit(ld3(l->direction)));
      *dist = INFINITY;
      *pdf = 1.0f;
      return sp3(l->radiance);
    case LIGHT_HEMISPHERE: {
      const v3 dir = hemisphere_sample(g);
      m3 M;
      M.c[0] = V(1, 0, 0);
      M.c[1] = V(0, 0, -1);
      M.c[2] = V(0, 1, 0);
      *wi = mv(&M, dir);
      *dist = INFINITY;
      *pdf = (float)(1.0 / (2.0 * PI_D));
      return sp3(l->radiance);
    }
    case LIGHT_POINT: {
      const v3 d = sub(ld3(l->position), p);
      *wi = unit(d);
      *dist = (float)norm(d);
      *pdf = 1.0f;
      return sp3(l->radiance);
    }
    default: { /* area */
      double sx, sy;
      sample2d(g, &sx, &sy);
      sx = sx - 0.5f;
      sy = sy - 0.5f;
      const v3 dx = ld3(l->dim_x), dy = ld3(l->dim_y), dir = ld3(l->direction);
      const v3 d = sub(add(add(ld3(l->position), smul(sx, dx)), smul(sy, dy)), p);
      const float cosTheta = (float)dot(d, dir);
      const float sqDist = (float)norm2(d);
      const float dist_ = sqrtf(sqDist);
      const float area = (float)(norm(dx) * norm(dy));
      *wi = divv(d, dist_);
      *dist = dist_;
      *pdf = sqDist / (area * fabsf(cosTheta));
      return cosTheta < 0 ? sp3(l->radiance) : S(0, 0, 0);
    }
  }
}

/* ---- the path tracer (pathtracer.cpp:483-582) ------------------------------------------- */
static sp trace_ray(const scene_t* sc, ray_t r, int includeLe, rng_t* g);

static sp direct_lighting(const scene_t* sc, ray_t r, const isect_t* is, rng_t* g) {
  const m3 o2w = make_coord_space(is->n);
  const m3 w2o = transpose(&o2w);
  const v3 hit_p = add(r.o, mul(r.d, is->t));
  const orc_mat_t* m = &sc->mats[sc->tri_mat[is->tri]];  /* f(wo, wi) of these BSDFs ignores both */
  sp L_out = S(0, 0, 0);
  for (int64_t li = 0; li < sc->nlights; li++) {
    const orc_light_t* l = &sc->lights[li];
    const int64_t num_samples = light_is_delta(l) ? 1 : sc->ns_area_light;
    sp L_light = S(0, 0, 0);
    for (int64_t i = 0; i < num_samples; i++) {
      v3 w_i;
      float dist, pdf;
      const sp Ls = sample_L(l, hit_p, &w_i, &dist, &pdf, g);
      const v3 w_in = mv(&w2o, w_i);
      if (w_in.z < 0.0) continue;
      const ray_t shadow = {hit_p, w_i, EPS_D, (double)dist, 0};
      if (any_hit(sc, shadow)) continue;
      L_light = sadd(L_light, sdiv(sscale(sprod(Ls, bsdf_f(m)), (float)fabs(w_in.z)), pdf));
    }
    L_out = sadd(L_out, sdiv(L_light, (float)((double)num_samples)));
  }
  return L_out;
}

static sp indirect_lighting(const scene_t* sc, ray_t r, const isect_t* is, rng_t* g) {
  const m3 o2w = make_coord_space(is->n);
  const m3 w2o = transpose(&o2w);
  const v3 hit_p = add(r.o, mul(r.d, is->t));
  const v3 w_out = mv(&w2o, neg(r.d));
  const orc_mat_t* m = &sc->mats[sc->tri_mat[is->tri]];
  v3 w_in;
  float pdf;
  const sp f = bsdf_sample_f(m, w_out, &w_in, &pdf, g);
  const double p_cont = fmin(illum(f) * 15.0, 1.0);
  if (coin_flip(g, p_cont)) {
    const ray_t next = {hit_p, mv(&o2w, w_in), EPS_D, INFINITY, r.depth - 1};
    const sp Li = trace_ray(sc, next, is_delta(m), g);
    return sdiv(sdiv(sscale(sprod(f, Li), (float)fabs(w_in.z)), (float)p_cont), pdf);
  }
  return S(0, 0, 0);
}

static sp trace_ray(const scene_t* sc, ray_t r, int includeLe, rng_t* g) {
  isect_t is;
  sp L = S(0, 0, 0);
  if (!closest_hit(sc, r, &is)) return L;
  const orc_mat_t* m = &sc->mats[sc->tri_mat[is.tri]];
  if (includeLe) L = sadd(L, emission(m));
  if (!is_delta(m)) L = sadd(L, direct_lighting(sc, r, &is, g));
  if (r.depth > 0) L = sadd(L, indirect_lighting(sc, r, &is, g));
  return L;
}

/* Camera::generate_ray (camera.cpp:117-126) */
static ray_t camera_ray(const orc_cam_t* c, double x, double y) {
  const double hFovTan = tan(c->hfov / 180.0 * PI_D * 0.5) * 2;
  const double vFovTan = tan(c->vfov / 180.0 * PI_D * 0.5) * 2;
  m3 M;
  M.c[0] = ld3(c->c2w);
  M.c[1] = ld3(c->c2w + 3);
  M.c[2] = ld3(c->c2w + 6);
  const v3 d = mv(&M, V((x - 0.5) * hFovTan, (y - 0.5) * vFovTan, -1));
  ray_t r = {ld3(c->pos), unit(d), c->nclip, c->fclip, 0};
  return r;
}

/* PathTracer::raytrace_pixel (pathtracer.cpp:584-604) */
static sp render_pixel(const scene_t* sc, const orc_cam_t* cam, int64_t x, int64_t y, int64_t W, int64_t H,
                       int64_t ns_aa, int64_t max_depth, rng_t* g, uint64_t seed) {
  const double w = (double)W, h = (double)H;
  if (ns_aa == 1) {
    if (g->mode == ORC_RNG_COUNTER) {
      g->key = path_key(seed, (uint64_t)(x + y * W), 0);
      g->k = 0;
    }
    ray_t r = camera_ray(cam, (x + 0.5) / w, (y + 0.5) / h);
    r.depth = max_depth;
    return trace_ray(sc, r, 1, g);
  }
  sp s = S(0, 0, 0);
  for (int64_t i = 0; i < ns_aa; i++) {
    if (g->mode == ORC_RNG_COUNTER) {
      g->key = path_key(seed, (uint64_t)(x + y * W), (uint64_t)i);
      g->k = 0;
    }
    double dx, dy;
    sample2d(g, &dx, &dy);
    ray_t r = camera_ray(cam, (x + dx) / w, (y + dy) / h);
    r.depth = max_depth;
    s = sadd(s, trace_ray(sc, r, 1, g));
  }
  return sdiv(s, (float)((double)ns_aa));
}

/* HDRImageBuffer::toColor + ImageBuffer::update_pixel (image.h:49-58, 174-189); the
 * reference's clamp(0.f, 1.f, c) is min(1, c) (misc.h:69) */
static uint8_t to_byte(float c) {
  const float v = (c < 1.f) ? c : 1.f;
  return (uint8_t)(uint32_t)(v * 255);
}

/* Camera::configure + Camera::place + compute_position (camera.cpp:15-31, 33-46, 92-111);
 * fov in degrees as in the reference's CameraInfo (float fields). */
void orc_camera_frame(double hfov_deg, double vfov_deg, double nclip, double fclip, const double* target,
                      double phi, double theta, double r, double min_r, double max_r, int64_t W, int64_t H,
                      orc_cam_t* out) {
  const double EPS_F = 0.00001f;
  double hFov = (float)hfov_deg, vFov = (float)vfov_deg;
  const double rad = PI_D / 180.0;
  const double ar1 = tan(hFov * rad / 2) / tan(vFov * rad / 2);
  const double ar = (double)W / H;
  if (ar1 < ar) {
    hFov = 2 * (atan(tan(vFov * rad / 2) * ar) * (180.0 / PI_D));
  } else if (ar1 > ar) {
    vFov = 2 * (atan(tan(hFov * rad / 2) / ar) * (180.0 / PI_D));
  }
  double r_ = fmin(fmax(r, min_r), max_r);
  double phi_ = (sin(phi) == 0) ? (phi + EPS_F) : phi;
  double sinPhi = sin(phi_);
  if (sinPhi == 0) {
    phi_ += EPS_F;
    sinPhi = sin(phi_);
  }
  const v3 dirToCamera = V(r_ * sinPhi * sin(theta), r_ * cos(phi_), r_ * sinPhi * cos(theta));
  const v3 pos = add(ld3(target), dirToCamera);
  const v3 upVec = V(0, sinPhi > 0 ? 1 : -1, 0);
  const v3 sx = normalize(cross(upVec, dirToCamera));
  const v3 sy = normalize(cross(dirToCamera, sx));
  const v3 sz = unit(dirToCamera);
  out->pos[0] = pos.x;
  out->pos[1] = pos.y;
  out->pos[2] = pos.z;
  const v3 cols[3] = {sx, sy, sz};
  for (int j = 0; j < 3; j++) {
    out->c2w[3 * j] = cols[j].x;
    out->c2w[3 * j + 1] = cols[j].y;
    out->c2w[3 * j + 2] = cols[j].z;
  }
  out->hfov = hFov;
  out->vfov = vFov;
  out->nclip = (float)nclip;
  out->fclip = (float)fclip;
}

/* One frame. hdr (3 W H floats, row y = 0 first as the reference's sample buffer) and
 * rgba (4 W H bytes, rows flipped as save_image writes the PNG, pathtracer.cpp:668-676)
 * may be NULL. Returns 0, or -1 on bad arguments. */
int orc_render(const double* tri, const double* nrm, const int64_t* tri_mat, int64_t ntri, const orc_mat_t* mats,
               const orc_light_t* lights, int64_t nlights, const orc_cam_t* cam, int64_t W, int64_t H, int64_t ns_aa,
               int64_t max_depth, int64_t ns_area_light, int rng_mode, uint64_t seed, float* hdr, uint8_t* rgba,
               int nthreads) {
  if (W <= 0 || H <= 0 || ns_aa <= 0 || max_depth < 0 || ns_area_light <= 0) return -1;
  const scene_t sc = {tri, nrm, tri_mat, ntri, mats, lights, nlights, ns_area_light};
  float* buf = (float*)malloc(sizeof(float) * 3 * (size_t)W * (size_t)H);
  if (!buf) return -1;
  if (rng_mode == ORC_RNG_STD) {
    srand((unsigned)seed);
    rng_t g = {ORC_RNG_STD, 0, 0};
    const int64_t T = 32;
    for (int64_t ty = 0; ty < H; ty += T)
      for (int64_t tx = 0; tx < W; tx += T)
        for (int64_t y = ty; y < ty + T && y < H; y++)
          for (int64_t x = tx; x < tx + T && x < W; x++) {
            const sp s = render_pixel(&sc, cam, x, y, W, H, ns_aa, max_depth, &g, seed);
            float* o = buf + 3 * (x + y * W);
            o[0] = s.r;
            o[1] = s.g;
            o[2] = s.b;
          }
  } else {
#ifdef _OPENMP
    if (nthreads > 0) omp_set_num_threads(nthreads);
#pragma omp parallel for schedule(dynamic, 4)
#endif
    for (int64_t y = 0; y < H; y++)
      for (int64_t x = 0; x < W; x++) {
        rng_t g = {ORC_RNG_COUNTER, 0, 0};
        const sp s = render_pixel(&sc, cam, x, y, W, H, ns_aa, max_depth, &g, seed);
        float* o = buf + 3 * (x + y * W);
        o[0] = s.r;
        o[1] = s.g;
        o[2] = s.b;
      }
  }
  (void)nthreads;
  const float gamma = 2.2f, level = 1.0f;
  const float one_over_gamma = 1.0f / gamma;
  const float exposure = (float)sqrt(pow(2, level));
  for (int64_t y = 0; y < H; y++)
    for (int64_t x = 0; x < W; x++) {
      const float* s = buf + 3 * (x + y * W);
      if (hdr) memcpy(hdr + 3 * (x + y * W), s, 3 * sizeof(float));
      if (rgba) {
        uint8_t* o = rgba + 4 * (x + (H - 1 - y) * W);
        o[0] = to_byte(powf(s[0] * exposure, one_over_gamma));
        o[1] = to_byte(powf(s[1] * exposure, one_over_gamma));
        o[2] = to_byte(powf(s[2] * exposure, one_over_gamma));
        o[3] = 255;
      }
    }
  free(buf);
  return 0;
}
