/*
 * pbf_oracle_adj.c — FP64 CPU reference gradient of one PBF step.
 *
 * TEST INFRASTRUCTURE (the oracle): the project-written reference the GPU adjoint
 * is checked against, itself checked against FP64 central finite differences.
 * The reference has no gradients; this differentiates the restatement in
 * pbf_oracle.c (included below, so the recomputed forward is bit-identical to
 * orc_step) with:
 *   - neighbour sets held fixed for the step (they are a step-level constant in
 *     the reference, particles.cpp:258-265);
 *   - every collision differentiated with its active set fixed: the stop axis,
 *     the slide and the second stop of clamp_response (particles.cpp:87-132) and
 *     clamp (:51-84), and the coordinates pinned by the clamp box. The EPS_D
 *     back-off (1e-11 along the ray) is treated as a constant offset;
 *   - vorticity confinement differentiated where |eta| > EPS_D.
 * The step maps (x, v; rho0) to (x', v'); orc_step_adjoint returns the adjoints
 * of x, v and rho0 for given adjoints of x' and v'.
 */
#include "pbf_oracle.c"

/* ---- collisions with their active set recorded ------------------------------ */

typedef struct {
  int kind;    /* 0 not moved (|delta| <= EPS_D), 1 free, 2 stop, 3 stop + slide, 4 stop + slide + stop */
  int axis, axis2;
  real c, c2;  /* plane coordinate of the stop and of the second stop */
  int clamped; /* bit per coordinate pinned by the clamp box */
  v3 p, delta; /* position before the move and the requested displacement */
} coll_t;

static int tri_axis(const ctx_t* c, int t) {
  v3 n = c->tn[t];
  return n.x != 0 ? 0 : (n.y != 0 ? 1 : 2);
}

/* scene_hit, also returning the index of the nearest triangle hit (or -1) */
static int scene_hit_idx(const ctx_t* c, ray_t* r, v3* nrm) {
  int hit = -1;
  for (int t = 0; t < c->ntri; t++)
    if (tri_hit(c, t, r, nrm)) hit = t;
  return hit;
}

/* clip_planes, also returning which plane set l last */
static int clip_planes_idx(const ctx_t* c, v3 p, v3 d, real* l, int* which) {
  int intersect = 0;
  for (int i = 0; i < c->n_clip; i++) {
    int a = c->clip_axis[i];
    real da = comp(d, a);
    if (da != 0.0) {
      real pt = (c->clip_value[i] - comp(p, a)) / da;
      if (pt > 0.0 && pt < *l) {
        *l = pt;
        intersect = 1;
        *which = i;
      }
    }
  }
  return intersect;
}

static void clamp_box_rec(const ctx_t* c, v3* p, int* clamped) {
  real v[3] = {p->x, p->y, p->z};
  for (int k = 0; k < 3; k++) {
    real w = smax(c->clamp_lo[k] + EPS_D, smin(c->clamp_hi[k] - EPS_D, v[k]));
    if (w != v[k]) *clamped |= 1 << k;
    v[k] = w;
  }
  p->x = v[0];
  p->y = v[1];
  p->z = v[2];
}

static void set_stop(const ctx_t* c, int tri, int intersect, int which, coll_t* rec) {
  if (tri >= 0) {
    rec->axis = tri_axis(c, tri);
    rec->c = comp(c->tp[tri][0], rec->axis);
  } else if (intersect) {
    rec->axis = c->clip_axis[which];
    rec->c = c->clip_value[which];
  }
}

/* clamp (particles.cpp:51-84) with the same arithmetic as clamp_move, recorded */
static void clamp_move_rec(const ctx_t* c, v3* p, v3 delta_p, coll_t* rec) {
  rec->p = *p;
  rec->delta = delta_p;
  rec->clamped = 0;
  rec->kind = 0;
  real l = vnorm(delta_p);
  if (l <= EPS_D) return;
  v3 d = vdiv(delta_p, l);
  int which = -1;
  int intersect = clip_planes_idx(c, *p, d, &l, &which);
  ray_t r = {*p, d, 0.0, l};
  v3 n = V(0, 0, 0);
  int tri = scene_hit_idx(c, &r, &n);
  if (tri >= 0 || intersect) {
    *p = vadd(*p, svmul(r.max_t - EPS_D, d));
    rec->kind = 2;
    set_stop(c, tri, intersect, which, rec);
  } else {
    *p = vadd(*p, delta_p);
    rec->kind = 1;
  }
  clamp_box_rec(c, p, &rec->clamped);
}

/* clamp_response (particles.cpp:87-132) with the same arithmetic, recorded */
static void clamp_response_rec(const ctx_t* c, v3* p, v3 v, real dt, coll_t* rec) {
  v3 delta_p = vscale(v, dt);
  rec->p = *p;
  rec->delta = delta_p;
  rec->clamped = 0;
  rec->kind = 0;
  real total_l = vnorm(delta_p), l = total_l;
  if (l <= EPS_D) return;
  v3 d = vdiv(delta_p, l);
  int which = -1;
  int intersect = clip_planes_idx(c, *p, d, &l, &which);
  ray_t r = {*p, d, 0.0, l};
  v3 n = V(0, 0, 0);
  int tri = scene_hit_idx(c, &r, &n);
  if (tri >= 0 || intersect) {
    *p = vadd(*p, svmul(r.max_t - EPS_D, d));
    rec->kind = 2;
    set_stop(c, tri, intersect, which, rec);
    if (dot(d, n) > -1 && !intersect) {
      d = unit(vsub(delta_p, svmul(dot(delta_p, n), n)));
      ray_t r2 = {*p, d, 0.0, (total_l - r.max_t) * 0.5};
      v3 n2 = V(0, 0, 0);
      int tri2 = scene_hit_idx(c, &r2, &n2);
      *p = vadd(*p, svmul(r2.max_t - EPS_D, d));
      rec->kind = 3;
      if (tri2 >= 0) {
        rec->kind = 4;
        rec->axis2 = tri_axis(c, tri2);
        rec->c2 = comp(c->tp[tri2][0], rec->axis2);
      }
    }
  } else {
    *p = vadd(*p, delta_p);
    rec->kind = 1;
  }
  clamp_box_rec(c, p, &rec->clamped);
}

/* Reverse of a recorded collision, exact for its active set (EPS_D terms included).
 * A stop moves p to p1 = P + (t - EPS_D) D / L with t = (c - P[a]) L / D[a], i.e.
 * p1 = P + tau D - EPS_D D / L, tau = (c - P[a]) / D[a]; the slide adds
 * kappa tan with tan = D without its a component, T = |tan| and
 * kappa = (L (1 - tau) / 2 - EPS_D) / T; a second stop on axis a2 at c2 instead adds
 * sigma tan - EPS_D tan / T with sigma = (c2 - p1[a2]) / tan[a2]. Coordinates the
 * clamp box pinned pass no adjoint. */

/* adds to db the adjoint of D for u = D / L (L = |D|) with adjoint ub */
static void unit_reverse(const real D[3], real L, const real ub[3], real db[3]) {
  const real u[3] = {D[0] / L, D[1] / L, D[2] / L};
  const real s = ub[0] * u[0] + ub[1] * u[1] + ub[2] * u[2];
  for (int k = 0; k < 3; k++) db[k] += (ub[k] - s * u[k]) / L;
}

/* p1 = P + tau D - EPS_D D / L: adjoints of P and D from the adjoint g of p1 and an
 * extra adjoint taub of tau */
static void stop_reverse(int a, real ca, const real P[3], const real D[3], real L, const real g[3], real taub,
                         real pb[3], real db[3]) {
  const real tau = (ca - P[a]) / D[a];
  real ub[3];
  for (int b = 0; b < 3; b++) {
    pb[b] += g[b];
    db[b] += tau * g[b];
    taub += g[b] * D[b];
    ub[b] = -EPS_D * g[b];
  }
  pb[a] -= taub / D[a];
  db[a] -= taub * tau / D[a];
  unit_reverse(D, L, ub, db);
}

/* g: adjoint of the position after the move; adds the adjoints of the position
 * before (pbar) and of the requested displacement (dbar) */
static void coll_reverse(const coll_t* rc, v3 gv, v3* pbar, v3* dbar) {
  real g[3] = {gv.x, gv.y, gv.z};
  for (int k = 0; k < 3; k++)
    if (rc->clamped & (1 << k)) g[k] = 0;
  const real P[3] = {rc->p.x, rc->p.y, rc->p.z}, D[3] = {rc->delta.x, rc->delta.y, rc->delta.z};
  real pb[3] = {0, 0, 0}, db[3] = {0, 0, 0};
  if (rc->kind == 0) {
    for (int k = 0; k < 3; k++) pb[k] += g[k];
  } else if (rc->kind == 1) {
    for (int k = 0; k < 3; k++) {
      pb[k] += g[k];
      db[k] += g[k];
    }
  } else {
    const int a = rc->axis;
    const real L = sqrt(D[0] * D[0] + D[1] * D[1] + D[2] * D[2]);
    real g1[3] = {g[0], g[1], g[2]}, taub = 0;
    if (rc->kind >= 3) {
      const real tau = (rc->c - P[a]) / D[a];
      real tan[3] = {D[0], D[1], D[2]}, tanb[3] = {0, 0, 0};
      tan[a] = 0;
      const real T = sqrt(tan[0] * tan[0] + tan[1] * tan[1] + tan[2] * tan[2]);
      if (rc->kind == 3) {
        const real kappa = (L * (1 - tau) / 2 - EPS_D) / T;
        real kappab = 0;
        for (int b = 0; b < 3; b++) {
          tanb[b] += kappa * g[b];
          kappab += g[b] * tan[b];
        }
        const real Lb = kappab * (1 - tau) / (2 * T);
        taub += -kappab * L / (2 * T);
        const real Tb = -kappab * kappa / T;
        for (int b = 0; b < 3; b++) {
          db[b] += Lb * D[b] / L;
          tanb[b] += Tb * tan[b] / T;
        }
      } else {
        const int a2 = rc->axis2;
        const real p1a2 = P[a2] + tau * D[a2] - EPS_D * D[a2] / L;
        const real sigma = (rc->c2 - p1a2) / tan[a2];
        real sigmab = 0, ub[3];
        for (int b = 0; b < 3; b++) {
          tanb[b] += sigma * g[b];
          sigmab += g[b] * tan[b];
          ub[b] = -EPS_D * g[b];
        }
        g1[a2] -= sigmab / tan[a2];
        tanb[a2] -= sigmab * sigma / tan[a2];
        unit_reverse(tan, T, ub, tanb);
      }
      for (int b = 0; b < 3; b++)
        if (b != a) db[b] += tanb[b];
    }
    stop_reverse(a, rc->c, P, D, L, g1, taub, pb, db);
  }
  pbar->x += pb[0];
  pbar->y += pb[1];
  pbar->z += pb[2];
  dbar->x += db[0];
  dbar->y += db[1];
  dbar->z += db[2];
}

/* ---- pair terms ------------------------------------------------------------- */

/* Adjoint of r = x_i - x_j from poly6 W(r) with adjoint wb and grad_spiky G(r) with
 * adjoint gb. W = c6 q^3, q = h2 - |r|^2: dW/dr = -6 c6 q^2 r. G = cs s(|r|) r with
 * s(p) = (h - p)^2 / p, s'(p) = -(h - p)(h + p) / p^2. */
static v3 pair_reverse(const ctx_t* c, v3 r, real wb, v3 gb) {
  v3 out = V(0, 0, 0);
  const real r2 = norm2(r);
  if (r2 < c->h2) {
    const real q = c->h2 - r2;
    out = svmul(-6.0 * 1.56668147106 / c->h9 * q * q * wb, r);
  }
  const real rl = vnorm(r);
  if (rl < c->h && rl >= EPS_D) {
    const real cs = -3 * 4.774648292756860 / c->h6;
    const real hm = c->h - rl;
    const real s = hm * hm / rl, sp = -hm * (c->h + rl) / (rl * rl);
    out = vadd(out, svmul(cs, vadd(svmul(s, gb), svmul(sp * dot(r, gb) / rl, r))));
  }
  return out;
}

/* d scorr / dW for scorr = -K (W tis)^n */
static inline real dscorr(const ctx_t* c, real w) {
  if (c->scorr_n <= 0) return 0.0;
  return -c->k * c->scorr_n * c->tis * intpow(w * c->tis, c->scorr_n - 1);
}

/* ---- recorded forward (same arithmetic as step_once) ------------------------ */

typedef struct {
  int64_t n;
  int iters;
  const int64_t *off, *idx;
  v3* x;       /* step input positions */
  v3* xs;      /* (iters + 1) n: x* before each iteration, then the final x* */
  real* lam;   /* iters n */
  real* rho;   /* iters n: constraint densities */
  real* den;   /* iters n: sum |g|^2 + |sum g|^2 + epsilon */
  v3* gsum;    /* iters n: sum over neighbours of grad W / rho0 */
  v3* dp;      /* iters n: the displacement requested by each iteration */
  coll_t* cpred;
  coll_t* citer; /* iters n */
  v3 *u, *omega, *eta, *vout;
} tape_t;

static void tape_free(tape_t* t) {
  free(t->x);
  free(t->xs);
  free(t->lam);
  free(t->rho);
  free(t->den);
  free(t->gsum);
  free(t->dp);
  free(t->cpred);
  free(t->citer);
  free(t->u);
  free(t->omega);
  free(t->eta);
  free(t->vout);
}

static int tape_forward(const ctx_t* c, int64_t n, const v3* x, const v3* v_in, real dt, const nbrs_t* nb,
                        tape_t* t) {
  const int I = c->iters;
  const size_t N = (size_t)(n ? n : 1);
  memset(t, 0, sizeof(*t));
  t->n = n;
  t->iters = I;
  t->off = nb->off;
  t->idx = nb->idx;
  t->x = (v3*)malloc(sizeof(v3) * N);
  t->xs = (v3*)malloc(sizeof(v3) * N * (size_t)(I + 1));
  t->lam = (real*)malloc(sizeof(real) * N * (size_t)(I ? I : 1));
  t->rho = (real*)malloc(sizeof(real) * N * (size_t)(I ? I : 1));
  t->den = (real*)malloc(sizeof(real) * N * (size_t)(I ? I : 1));
  t->gsum = (v3*)malloc(sizeof(v3) * N * (size_t)(I ? I : 1));
  t->dp = (v3*)malloc(sizeof(v3) * N * (size_t)(I ? I : 1));
  t->cpred = (coll_t*)malloc(sizeof(coll_t) * N);
  t->citer = (coll_t*)malloc(sizeof(coll_t) * N * (size_t)(I ? I : 1));
  t->u = (v3*)malloc(sizeof(v3) * N);
  t->omega = (v3*)malloc(sizeof(v3) * N);
  t->eta = (v3*)malloc(sizeof(v3) * N);
  t->vout = (v3*)malloc(sizeof(v3) * N);
  if (!t->x || !t->xs || !t->lam || !t->rho || !t->den || !t->gsum || !t->dp || !t->cpred || !t->citer ||
      !t->u || !t->omega || !t->eta || !t->vout)
    return -1;
  const int64_t* off = nb->off;
  const int64_t* idx = nb->idx;
  memcpy(t->x, x, sizeof(v3) * (size_t)n);

  /* applyForceVelocity + prediction, particles.cpp:175-183 */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    v3 vi = v_in[i];
    if (c->gravity.x != 0.0) vi.x -= (-c->gravity.x) * dt;
    if (c->gravity.y != 0.0) vi.y -= (-c->gravity.y) * dt;
    if (c->gravity.z != 0.0) vi.z -= (-c->gravity.z) * dt;
    t->xs[i] = x[i];
    clamp_response_rec(c, &t->xs[i], vi, dt, &t->cpred[i]);
  }

  for (int it = 0; it < I; it++) {
    const v3* xk = t->xs + (size_t)it * n;
    v3* xk1 = t->xs + (size_t)(it + 1) * n;
    real* lam = t->lam + (size_t)it * n;
    /* newtonStepCalculateLambda, particles.cpp:185-204 */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      real density = 0.0, denom = 0.0;
      v3 grad_i_c_i = V(0, 0, 0);
      for (int64_t e = off[i]; e < off[i + 1]; e++) {
        v3 r = vsub(xk[i], xk[idx[e]]);
        v3 g = spiky(c, r);
        density += poly6(c, r);
        g = svmul(1. / c->rest_density, g);
        grad_i_c_i = vadd(grad_i_c_i, g);
        denom += norm2(g);
      }
      real c_i = density / c->rest_density - 1.0;
      denom += norm2(grad_i_c_i);
      lam[i] = -c_i / (denom + c->epsilon);
      t->rho[(size_t)it * n + i] = density;
      t->den[(size_t)it * n + i] = denom + c->epsilon;
      t->gsum[(size_t)it * n + i] = grad_i_c_i;
    }
    /* newtonStepUpdatePosition, particles.cpp:206-213 */
#pragma omp parallel for schedule(static)
    for (int64_t i = 0; i < n; i++) {
      v3 delta_p = V(0, 0, 0);
      for (int64_t e = off[i]; e < off[i + 1]; e++) {
        v3 r = vsub(xk[i], xk[idx[e]]);
        real sc = -c->k * intpow(poly6(c, r) * c->tis, c->scorr_n);
        delta_p = vadd(delta_p, svmul(lam[i] + lam[idx[e]] + sc, spiky(c, r)));
      }
      delta_p = svmul(1. / c->rest_density, delta_p);
      t->dp[(size_t)it * n + i] = delta_p;
      xk1[i] = xk[i];
      clamp_move_rec(c, &xk1[i], delta_p, &t->citer[(size_t)it * n + i]);
    }
  }
  const v3* xf = t->xs + (size_t)I * n;

  /* updateVelocity, particles.cpp:215-217 */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) t->u[i] = vdiv(vsub(xf[i], x[i]), dt);

  /* calculateVorticityApplyXSPHViscosity, particles.cpp:219-234 */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    v3 w_acc = V(0, 0, 0), visc = V(0, 0, 0);
    for (int64_t e = off[i]; e < off[i + 1]; e++) {
      int64_t j = idx[e];
      v3 v_i_n = vsub(t->u[j], t->u[i]);
      v3 r = vsub(xf[i], xf[j]);
      w_acc = vadd(w_acc, cross(v_i_n, spiky(c, r)));
      visc = vadd(visc, vscale(v_i_n, poly6(c, r)));
    }
    t->omega[i] = w_acc;
    t->vout[i] = vadd(t->u[i], svmul(c->xsph_c, visc));
  }

  /* applyVorticity, particles.cpp:236-248 */
#pragma omp parallel for schedule(static)
  for (int64_t i = 0; i < n; i++) {
    v3 gv = V(0, 0, 0);
    for (int64_t e = off[i]; e < off[i + 1]; e++) {
      int64_t j = idx[e];
      gv = vadd(gv, svmul(vnorm(t->omega[j]), spiky(c, vsub(xf[i], xf[j]))));
    }
    t->eta[i] = gv;
    if (vnorm(gv) > EPS_D) t->vout[i] = vadd(t->vout[i], svmul(dt * c->vort_eps, cross(unit(gv), t->omega[i])));
  }
  return 0;
}

/* ---- reverse pass -------------------------------------------------------------- */

/* Adjoints of the step inputs (xb, vb, *rb0) from those of its outputs (gx: x', gv: v').
 * Serial: the pair terms scatter into both ends of each pair. */
static int tape_reverse(const ctx_t* c, const tape_t* t, real dt, const v3* gx, const v3* gv, v3* xb, v3* vb,
                        real* rb0) {
  const int64_t n = t->n;
  const int I = t->iters;
  const int64_t* off = t->off;
  const int64_t* idx = t->idx;
  const size_t N = (size_t)(n ? n : 1);
  const real rho0 = c->rest_density;
  v3* sb = (v3*)calloc(N, sizeof(v3));    /* adjoint of the current x* */
  v3* ub = (v3*)calloc(N, sizeof(v3));    /* adjoint of u = (x* - x) / dt */
  v3* wb = (v3*)calloc(N, sizeof(v3));    /* adjoint of omega */
  v3* etab = (v3*)calloc(N, sizeof(v3));  /* adjoint of eta */
  real* mwb = (real*)calloc(N, sizeof(real)); /* adjoint of |omega| */
  v3* dpb = (v3*)calloc(N, sizeof(v3));
  real* lamb = (real*)calloc(N, sizeof(real));
  if (!sb || !ub || !wb || !etab || !mwb || !dpb || !lamb) return -1;
  real r0b = 0.0;
  const v3* xf = t->xs + (size_t)I * n;

  for (int64_t i = 0; i < n; i++) {
    sb[i] = gx[i];
    xb[i] = V(0, 0, 0);
  }
  /* vorticity confinement: v'' = v' + a (eta / |eta|) x omega_i, a = dt eps_v */
  const real a = dt * c->vort_eps;
  for (int64_t i = 0; i < n; i++) {
    const real en = vnorm(t->eta[i]);
    if (en > EPS_D) {
      const v3 nrm = unit(t->eta[i]);
      wb[i] = vadd(wb[i], svmul(a, cross(gv[i], nrm)));
      const v3 nb = svmul(a, cross(t->omega[i], gv[i]));
      etab[i] = svmul(1.0 / en, vsub(nb, svmul(dot(nb, nrm), nrm)));
    }
  }
  /* eta_i = sum_j |omega_j| G(x*_i - x*_j) */
  for (int64_t i = 0; i < n; i++) {
    for (int64_t e = off[i]; e < off[i + 1]; e++) {
      const int64_t j = idx[e];
      const v3 r = vsub(xf[i], xf[j]);
      mwb[j] += dot(etab[i], spiky(c, r));
      const v3 rb = pair_reverse(c, r, 0.0, svmul(vnorm(t->omega[j]), etab[i]));
      sb[i] = vadd(sb[i], rb);
      sb[j] = vsub(sb[j], rb);
    }
  }
  for (int64_t j = 0; j < n; j++) {
    const real m = vnorm(t->omega[j]);
    if (m > 0) wb[j] = vadd(wb[j], svmul(mwb[j] / m, t->omega[j]));
  }
  /* XSPH and vorticity: v' = u + c_xsph sum_j (u_j - u_i) W, omega_i = sum_j (u_j - u_i) x G */
  for (int64_t i = 0; i < n; i++) ub[i] = vadd(ub[i], gv[i]);
  for (int64_t i = 0; i < n; i++) {
    const v3 viscb = svmul(c->xsph_c, gv[i]);
    for (int64_t e = off[i]; e < off[i + 1]; e++) {
      const int64_t j = idx[e];
      const v3 r = vsub(xf[i], xf[j]);
      const real w = poly6(c, r);
      const v3 g = spiky(c, r);
      const v3 du = vsub(t->u[j], t->u[i]);
      const v3 dub = vadd(svmul(w, viscb), cross(g, wb[i]));
      ub[j] = vadd(ub[j], dub);
      ub[i] = vsub(ub[i], dub);
      const v3 rb = pair_reverse(c, r, dot(viscb, du), cross(wb[i], du));
      sb[i] = vadd(sb[i], rb);
      sb[j] = vsub(sb[j], rb);
    }
  }
  /* u = (x* - x) / dt */
  for (int64_t i = 0; i < n; i++) {
    const v3 q = svmul(1.0 / dt, ub[i]);
    sb[i] = vadd(sb[i], q);
    xb[i] = vsub(xb[i], q);
  }
  /* Jacobi iterations, last first */
  for (int it = I - 1; it >= 0; it--) {
    const v3* xk = t->xs + (size_t)it * n;
    const real* lam = t->lam + (size_t)it * n;
    const real* rho = t->rho + (size_t)it * n;
    const real* den = t->den + (size_t)it * n;
    const v3* gsum = t->gsum + (size_t)it * n;
    const v3* dp = t->dp + (size_t)it * n;
    for (int64_t i = 0; i < n; i++) {
      v3 pb = V(0, 0, 0), db = V(0, 0, 0);
      coll_reverse(&t->citer[(size_t)it * n + i], sb[i], &pb, &db);
      sb[i] = pb;
      r0b -= dot(db, dp[i]) / rho0;
      dpb[i] = svmul(1.0 / rho0, db); /* adjoint of the unscaled sum */
      lamb[i] = 0;
    }
    /* delta_p_i = (1/rho0) sum_j (lam_i + lam_j + scorr_ij) G_ij */
    for (int64_t i = 0; i < n; i++) {
      for (int64_t e = off[i]; e < off[i + 1]; e++) {
        const real q = dot(dpb[i], spiky(c, vsub(xk[i], xk[idx[e]])));
        lamb[i] += q;
        lamb[idx[e]] += q;
      }
    }
    /* lam_i = -C_i / D_i, C_i = rho_i / rho0 - 1, D_i = sum |g|^2 + |sum g|^2 + eps, g = G / rho0 */
    for (int64_t i = 0; i < n; i++) {
      const real cb = -lamb[i] / den[i];
      const real dbar = -lamb[i] * lam[i] / den[i];
      const real rhob = cb / rho0;
      r0b -= cb * rho[i] / (rho0 * rho0);
      for (int64_t e = off[i]; e < off[i + 1]; e++) {
        const int64_t j = idx[e];
        const v3 r = vsub(xk[i], xk[j]);
        const real w = poly6(c, r);
        const v3 G = spiky(c, r);
        const real sc = -c->k * intpow(w * c->tis, c->scorr_n);
        const v3 g = svmul(1. / rho0, G);
        const v3 gbar = svmul(2 * dbar, vadd(g, gsum[i]));
        r0b -= dot(gbar, g) / rho0;
        const real wbar = dot(dpb[i], G) * dscorr(c, w) + rhob;
        const v3 Gbar = vadd(svmul(lam[i] + lam[j] + sc, dpb[i]), svmul(1.0 / rho0, gbar));
        const v3 rb = pair_reverse(c, r, wbar, Gbar);
        sb[i] = vadd(sb[i], rb);
        sb[j] = vsub(sb[j], rb);
      }
    }
  }
  /* prediction x*0 = clamp_response(x, v + g dt, dt) */
  for (int64_t i = 0; i < n; i++) {
    v3 pb = V(0, 0, 0), db = V(0, 0, 0);
    coll_reverse(&t->cpred[i], sb[i], &pb, &db);
    xb[i] = vadd(xb[i], pb);
    vb[i] = svmul(dt, db);
  }
  *rb0 = r0b;
  free(sb);
  free(ub);
  free(wb);
  free(etab);
  free(mwb);
  free(dpb);
  free(lamb);
  return 0;
}

/* ---- exported ------------------------------------------------------------------ */

/*
 * One step from (pos, vel) (float64 (n,3)) and its reverse mode. gx_out / gv_out are
 * the adjoints of the step's output positions and velocities; gx_in / gv_in receive
 * those of the input positions and velocities, *g_rho0 that of the rest density.
 * pos_out / vel_out (or NULL) receive the step's outputs (bit-identical to orc_step
 * on the same neighbour sets). in_off / in_idx (ascending lists, or NULL to search)
 * fix the neighbour sets. kinds (10 entries, or NULL) receives the census of
 * collision kinds (not moved, free, stop, stop + slide, stop + slide + stop) of the
 * prediction (0-4) and of the Jacobi iterations (5-9). Returns 0, or -1 when out of
 * memory.
 */
int orc_step_adjoint(const pbf_params* prm, int64_t n, const double* pos, const double* vel, double dt,
                     const int64_t* in_off, const int64_t* in_idx, const double* gx_out, const double* gv_out,
                     double* gx_in, double* gv_in, double* g_rho0, double* pos_out, double* vel_out,
                     int64_t* kinds, int nthreads) {
  set_threads(nthreads);
  ctx_t* c = (ctx_t*)malloc(sizeof(ctx_t));
  if (!c) return -1;
  make_ctx(c, prm);
  v3* x = to_v3(pos, n);
  v3* v = to_v3(vel, n);
  v3* gx = to_v3(gx_out, n);
  v3* gv = to_v3(gv_out, n);
  v3* xb = to_v3(NULL, n);
  v3* vb = to_v3(NULL, n);
  if (!x || !v || !gx || !gv || !xb || !vb) return -1;
  nbrs_t nb = {NULL, NULL};
  int rc = 0;
  if (in_off) {
    nb.off = (int64_t*)in_off;
    nb.idx = (int64_t*)in_idx;
  } else {
    /* the search runs on the predicted positions, as in step_once */
    v3* xp = to_v3(pos, n);
    if (!xp) return -1;
    for (int64_t i = 0; i < n; i++) {
      v3 vi = v[i];
      if (c->gravity.x != 0.0) vi.x -= (-c->gravity.x) * (real)dt;
      if (c->gravity.y != 0.0) vi.y -= (-c->gravity.y) * (real)dt;
      if (c->gravity.z != 0.0) vi.z -= (-c->gravity.z) * (real)dt;
      clamp_response(c, &xp[i], vi, (real)dt);
    }
    rc = find_neighbors(c, n, xp, &nb);
    free(xp);
  }
  tape_t t;
  memset(&t, 0, sizeof(t));
  real rb0 = 0;
  if (rc == 0) rc = tape_forward(c, n, x, v, (real)dt, &nb, &t);
  if (rc == 0) rc = tape_reverse(c, &t, (real)dt, gx, gv, xb, vb, &rb0);
  if (rc == 0) {
    from_v3(gx_in, xb, n);
    from_v3(gv_in, vb, n);
    if (g_rho0) *g_rho0 = rb0;
    if (pos_out) from_v3(pos_out, t.xs + (size_t)t.iters * n, n);
    if (vel_out) from_v3(vel_out, t.vout, n);
    if (kinds) {
      for (int k = 0; k < 10; k++) kinds[k] = 0;
      for (int64_t i = 0; i < n; i++) kinds[t.cpred[i].kind]++;
      for (int64_t i = 0; i < n * (int64_t)t.iters; i++) kinds[5 + t.citer[i].kind]++;
    }
  }
  tape_free(&t);
  if (!in_off) {
    free(nb.off);
    free(nb.idx);
  }
  free(x);
  free(v);
  free(gx);
  free(gv);
  free(xb);
  free(vb);
  free(c);
  return rc;
}
