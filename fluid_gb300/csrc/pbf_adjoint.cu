// Reverse mode of one PBF step for sm_103a (FP32, no atomics, deterministic).
//
// The step (particles.cpp:250-297, in the form of pbf_kernels.cu) is differentiated
// with its neighbour sets held fixed and every collision with its active set fixed
// (the record collide<true> wrote during the recording forward). Every pair term is
// evaluated in gather form: the neighbour relation is symmetric, so particle i sums
// the contributions of the pairs (i, j) and (j, i) itself and writes only its own
// adjoints. Launch chain after the recording forward (I iterations):
//   k_adj_in        adjoints of the outputs into cell order; the adjoints of omega_i
//                   (direct part) and of eta_i from the recorded eta
//   k_adj_vort_b    |omega| adjoint, pair terms of eta
//   k_adj_xsph      XSPH + vorticity pair terms, u = (x* - x) / dt, then the reverse of
//                   the last iteration's collision
//   per iteration k = I-1 .. 0:
//     k_adj_lambda  adjoint of lambda, density, the denominator
//     k_adj_pos     pair terms of density / lambda / delta p, then the reverse of the
//                   collision of iteration k-1, or of the prediction (k = 0) with the
//                   write-out in original order
//   k_adj_r0_*      deterministic sum of the rest-density adjoint
//
// Pair derivatives, r = x_i - x_j, q = h2 - |r|^2, rho = |r|:
//   W = poly6_c q^3                 dW/dr = -6 poly6_c q^2 r
//   G = spiky_c s r, s = (h - rho)^2 / rho
//   adjoint of r from G-bar: spiky_c (s G-bar - t (r . G-bar) r), t = (h - rho)(h + rho) / rho^3
#include <cstdint>

#include "pbf_device.cuh"

namespace pbf {
namespace {

// Pair geometry plus the spiky second-derivative factor t (0 outside [EPS_D, h)).
struct PairD {
  float3 r;
  float q, s, t;
};
__device__ __forceinline__ PairD pair_d(const float4& xi, const float4& xj, float h, float h2) {
  PairD p;
  p.r = make_float3(xi.x - xj.x, xi.y - xj.y, xi.z - xj.z);
  const float r2 = dot3(p.r, p.r);
  p.q = fmaxf(h2 - r2, 0.0f);
  const float rinv = rsqrtf(r2);
  const float rl = r2 * rinv;
  const float hr = fmaxf(h - rl, 0.0f);
  const bool ok = r2 >= kEps * kEps;
  p.s = ok ? hr * hr * rinv : 0.0f;
  p.t = ok ? hr * (h + rl) * rinv * rinv * rinv : 0.0f;
  return p;
}

// Adjoint of r_ij given the summed adjoint of W over both pair orders (wsum) and the
// difference of the adjoints of G(r_ij) and G(r_ji) (gdiff).
__device__ __forceinline__ float3 pair_rev(const PairD& p, float wsum, const float3 gdiff, const DevParams& P) {
  const float cw = -6.0f * P.poly6_c * p.q * p.q * wsum;
  const float ct = -P.spiky_c * p.t * dot3(p.r, gdiff);
  return p.r * (cw + ct) + gdiff * (P.spiky_c * p.s);
}

__device__ __forceinline__ float4 f4(const float3 a, float w) { return make_float4(a.x, a.y, a.z, w); }

// what one neighbour contributes to a reverse pass, gathered ahead of its use
struct F2 {
  float4 a, b;
};
struct F3 {
  float4 a, b, c;
};
struct F4 {
  float4 a, b, c, d;
};
__device__ __forceinline__ int scene_of(const float4& x) { return __float_as_int(x.w); }

// ---------------------------------------------------------------------------
// adjoints of the outputs into cell order
// ---------------------------------------------------------------------------
__global__ void k_adj_in(const uint32_t* __restrict__ id, const float* __restrict__ gx_out,
                         const float* __restrict__ gv_out, const float4* __restrict__ eta_rec,
                         const float4* __restrict__ omega, float4* __restrict__ gxs, float4* __restrict__ gvo,
                         float4* __restrict__ eb, float4* __restrict__ wb, float* __restrict__ r0, DevParams P,
                         float dt, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t o = id[s];
  gxs[s] = gx_out ? make_float4(gx_out[3 * o], gx_out[3 * o + 1], gx_out[3 * o + 2], 0.f)
                  : make_float4(0.f, 0.f, 0.f, 0.f);
  const float3 vb = gv_out ? make_float3(gv_out[3 * o], gv_out[3 * o + 1], gv_out[3 * o + 2])
                           : make_float3(0.f, 0.f, 0.f);
  gvo[s] = f4(vb, 0.f);
  r0[s] = 0.f;
  // vorticity confinement v'' = v' + a (eta / |eta|) x omega, a = dt eps_v (particles.cpp:236-248):
  // adjoints of omega (direct part) and of eta, from the eta the recording forward kept
  const float3 eta = f3(eta_rec[s]);
  const float en = sqrtf(dot3(eta, eta));
  float3 wbar = make_float3(0.f, 0.f, 0.f), ebar = make_float3(0.f, 0.f, 0.f);
  if (en > kEps) {
    const float3 nh = eta * (1.0f / en);
    const float a = dt * P.vort_eps;
    const float3 w = f3(omega[s]);
    wbar = cross3(vb, nh) * a;
    const float3 nb = cross3(w, vb) * a;
    ebar = (nb - nh * dot3(nb, nh)) * (1.0f / en);
  }
  eb[s] = f4(ebar, 0.f);
  wb[s] = f4(wbar, 0.f);
}

// ---------------------------------------------------------------------------
// eta_i = sum_j |omega_j| G(r_ij)   (particles.cpp:236-248)
// ---------------------------------------------------------------------------
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_adj_vort_b(const float4* __restrict__ xs, const float4* __restrict__ omega,
                                                      const uint4* __restrict__ hdr,
                                                      const uint32_t* __restrict__ words,
                                                      const float4* __restrict__ eb, float4* __restrict__ wb,
                                                      float4* __restrict__ gxs, DevParams P, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = xs[i];  // w: |omega_i|
  const float3 ebi = f3(eb[i]);
  float mwb = 0.f;
  float3 acc = make_float3(0.f, 0.f, 0.f);
  for_each_neighbor_pf<8>(
      i, n, hdr[i], words, [&](uint32_t j) { return F2{__ldg(&xs[j]), __ldg(&eb[j])}; },
      [&](uint32_t, const F2& a) {
    const float4 xj = a.a;
    const float3 ebj = f3(a.b);
    const PairD p = pair_d(xi, xj, P.h, P.h2);
    mwb -= P.spiky_c * p.s * dot3(ebj, p.r);
    acc = acc + pair_rev(p, 0.f, ebi * xj.w - ebj * xi.w, P);
  });
  float3 wbar = f3(wb[i]);
  if (xi.w > 0.f) wbar = wbar + f3(omega[i]) * (mwb / xi.w);
  wb[i] = f4(wbar, 0.f);
  const float4 g = gxs[i];
  gxs[i] = make_float4(g.x + acc.x, g.y + acc.y, g.z + acc.z, 0.f);
}

// ---------------------------------------------------------------------------
// end of a pass: gs is the complete adjoint of x* after iteration k (k = -1: after
// the prediction). Applies the reverse of that collision and hands on to the next
// pass, or writes the step's input adjoints (original order) after the prediction.
// ---------------------------------------------------------------------------
struct Finish {
  const float4* x;     // tape: step input x
  const float4* v;     // tape: step input v (w: prediction record)
  const float4* xs;    // tape: x* per iteration (w: lambda)
  const float4* dp;    // tape: requested displacement per iteration (w: record)
  const SceneDesc* scenes;
  const uint32_t* id;
  float4* gxs;
  float4* pl0;
  float4* pl1;
  float4* gx;
  float* r0;
  float* gx_in;
  float* gv_in;
  size_t n;
};

__device__ __forceinline__ void finish(int i, const float3 gs, int k, const Finish& F, const DevParams& P,
                                       float dt) {
  const float4 x4 = F.x[i];
  const SceneDesc& sc = F.scenes[scene_of(x4)];
  float3 pb, db;
  if (k >= 0) {
    const size_t e = static_cast<size_t>(k) * F.n + i;
    const float4 xk = F.xs[e];
    const float4 d4 = F.dp[e];
    const float3 D = f3(d4);
    collide_reverse(__float_as_uint(d4.w), f3(xk), D, gs, sc, P, &pb, &db);
    F.gxs[i] = f4(pb, 0.f);
    float4* pl = (k & 1) ? F.pl1 : F.pl0;
    pl[i] = f4(db * P.inv_rho0, xk.w);
    F.r0[i] -= dot3(db, D) * P.inv_rho0;
  } else {
    const float4 v4 = F.v[i];
    collide_reverse(__float_as_uint(v4.w), f3(x4), predict_delta(v4, P, dt), gs, sc, P, &pb, &db);
    const float3 gxi = f3(F.gx[i]) + pb;
    const float3 gvi = db * dt;
    const uint32_t o = F.id[i];
    F.gx_in[3 * o] = gxi.x;
    F.gx_in[3 * o + 1] = gxi.y;
    F.gx_in[3 * o + 2] = gxi.z;
    F.gv_in[3 * o] = gvi.x;
    F.gv_in[3 * o + 1] = gvi.y;
    F.gv_in[3 * o + 2] = gvi.z;
  }
}

// ---------------------------------------------------------------------------
// XSPH and vorticity (particles.cpp:215-234): u = (x* - x) / dt,
// v' = u_i + c sum_j (u_j - u_i) W_ij, omega_i = sum_j (u_j - u_i) x G_ij
// ---------------------------------------------------------------------------
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_adj_xsph(const float4* __restrict__ xs, const float4* __restrict__ disp,
                                                    const uint4* __restrict__ hdr,
                                                    const uint32_t* __restrict__ words,
                                                    const float4* __restrict__ gvo, const float4* __restrict__ wb,
                                                    Finish F, DevParams P, float dt, float inv_dt, int last,
                                                    int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = xs[i];
  const float3 ui = f3(disp[i]) * inv_dt;
  const float3 vbi = f3(gvo[i]);
  const float3 cbi = vbi * P.xsph_c;
  const float3 wbi = f3(wb[i]);
  float3 ub = vbi, acc = make_float3(0.f, 0.f, 0.f);
  for_each_neighbor_pf<4>(
      i, n, hdr[i], words,
      [&](uint32_t j) { return F4{__ldg(&xs[j]), __ldg(&disp[j]), __ldg(&gvo[j]), __ldg(&wb[j])}; },
      [&](uint32_t, const F4& a) {
    const float4 xj = a.a;
    const float3 du = f3(a.b) * inv_dt - ui;
    const float3 cbj = f3(a.c) * P.xsph_c;
    const float3 ws = wbi + f3(a.d);
    const PairD p = pair_d(xi, xj, P.h, P.h2);
    const float W = P.poly6_c * (p.q * p.q * p.q);
    const float3 G = p.r * (P.spiky_c * p.s);
    ub = ub + (cbj - cbi) * W - cross3(G, ws);
    acc = acc + pair_rev(p, dot3(cbi - cbj, du), cross3(ws, du), P);
  });
  const float3 q = ub * inv_dt;
  F.gx[i] = f4(q * -1.0f, 0.f);
  finish(i, f3(F.gxs[i]) + acc + q, last, F, P, dt);
}

// ---------------------------------------------------------------------------
// one Jacobi iteration (particles.cpp:185-213), reverse:
// lambda_i = -C_i / D_i, C_i = rho_i / rho0 - 1, D_i = sum |g|^2 + |sum g|^2 + eps, g = G / rho0,
// S_i = sum_j (lambda_i + lambda_j + s_corr(W_ij)) G_ij, delta p_i = S_i / rho0
// pl = (adjoint of S, lambda); gr = (sum g, adjoint of rho); D-bar = lambda rho-bar rho0
// ---------------------------------------------------------------------------
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_adj_lambda(const float4* __restrict__ xs, const uint4* __restrict__ hdr,
                                                      const uint32_t* __restrict__ words,
                                                      const float4* __restrict__ pl, float4* __restrict__ gr,
                                                      float* __restrict__ r0, DevParams P, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = xs[i];
  const float4 ai = pl[i];
  const float3 sbi = f3(ai);
  float qsum = 0.f, g2 = 0.f, lb = 0.f;
  float3 gs = make_float3(0.f, 0.f, 0.f);
  for_each_neighbor_pf<8>(
      i, n, hdr[i], words, [&](uint32_t j) { return F2{__ldg(&xs[j]), __ldg(&pl[j])}; },
      [&](uint32_t, const F2& a) {
    const float4 xj = a.a;
    const float3 sbj = f3(a.b);
    const Pair p = pair_of(xi, xj, P.h, P.h2);
    const float3 rs = p.r * p.s;
    qsum += p.q * p.q * p.q;
    gs = gs + rs;
    g2 += p.s * p.s * p.r2;
    lb += dot3(rs, sbi - sbj);
  });
  lb *= P.spiky_c;
  const float rho = P.poly6_c * qsum;
  const float kg = P.spiky_c * P.inv_rho0;
  const float dg = kg * kg * (g2 + dot3(gs, gs));
  const float D = dg + P.epsilon;
  const float cb = -lb / D;
  const float rhob = cb * P.inv_rho0;
  const float dbar = -lb * ai.w / D;
  r0[i] += -cb * rho * P.inv_rho0 * P.inv_rho0 - 2.0f * dbar * dg * P.inv_rho0;
  gr[i] = f4(gs * kg, rhob);
}

template <int BLOCK, bool N4>
__global__ void __launch_bounds__(BLOCK) k_adj_pos(const float4* __restrict__ xs, const uint4* __restrict__ hdr,
                                                   const uint32_t* __restrict__ words,
                                                   const float4* __restrict__ pl, const float4* __restrict__ gr,
                                                   Finish F, DevParams P, float dt, int next, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = xs[i];
  const float4 ai = pl[i];
  const float4 gi = gr[i];
  const float3 sbi = f3(ai), gsi = f3(gi);
  const float li = ai.w, rbi = gi.w;
  const float dbi2 = 2.0f * li * rbi;  // 2 D-bar_i / rho0
  const float wt = P.poly6_c * P.tis;
  const float ks = -P.scorr_k * P.tis;  // d s_corr / dW = ks * n (W tis)^(n-1)
  float3 acc = make_float3(0.f, 0.f, 0.f);
  for_each_neighbor_pf<4>(
      i, n, hdr[i], words, [&](uint32_t j) { return F3{__ldg(&xs[j]), __ldg(&pl[j]), __ldg(&gr[j])}; },
      [&](uint32_t, const F3& nb) {
    const float4 xj = nb.a;
    const float4 aj = nb.b;
    const float4 gj = nb.c;
    const PairD p = pair_d(xi, xj, P.h, P.h2);
    const float q3 = p.q * p.q * p.q;
    const float a = wt * q3;  // W tis
    float an, dan;
    if (N4) {
      const float a2 = a * a;
      an = a2 * a2;
      dan = 4.0f * a2 * a;
    } else {
      an = 1.0f;
      dan = 0.0f;
      for (int e = 0; e < P.scorr_n; ++e) {
        dan = dan * a + an;
        an *= a;
      }
    }
    const float coef = (li + aj.w) - P.scorr_k * an;
    const float3 G = p.r * (P.spiky_c * p.s);
    const float3 g = G * P.inv_rho0;
    const float3 dS = sbi - f3(aj);
    const float dbj2 = 2.0f * aj.w * gj.w;
    const float wsum = ks * dan * dot3(dS, G) + rbi + gj.w;
    const float3 gd = dS * coef + (gsi + g) * dbi2 - (f3(gj) - g) * dbj2;
    acc = acc + pair_rev(p, wsum, gd, P);
  });
  finish(i, f3(F.gxs[i]) + acc, next, F, P, dt);
}

// ---------------------------------------------------------------------------
// rest-density adjoint: fixed-shape two-level sum (deterministic)
// ---------------------------------------------------------------------------
__global__ void __launch_bounds__(256) k_adj_r0_part(const float* __restrict__ r0, double* __restrict__ part, int n) {
  double acc = 0.0;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) acc += r0[i];
  __shared__ double sh[256];
  sh[threadIdx.x] = acc;
  __syncthreads();
  for (int o = 128; o > 0; o >>= 1) {
    if (threadIdx.x < static_cast<unsigned>(o)) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(kAdjReduceBlocks) k_adj_r0_final(const double* __restrict__ part,
                                                                   double* __restrict__ out) {
  __shared__ double sh[kAdjReduceBlocks];
  sh[threadIdx.x] = part[threadIdx.x];
  __syncthreads();
  for (int o = kAdjReduceBlocks / 2; o > 0; o >>= 1) {
    if (threadIdx.x < static_cast<unsigned>(o)) sh[threadIdx.x] += sh[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = sh[0];
}

inline unsigned blocks_for(size_t n, int block) { return static_cast<unsigned>((n + block - 1) / block); }

}  // namespace

cudaError_t launch_adjoint(const Buffers& b, const DevParams& P, const Tuning& t, int cur, float dt,
                           const Tape& tp, const float* gx_out, const float* gv_out, float* gx_in,
                           float* gv_in, double* g_rho0, cudaStream_t s) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaMemsetAsync(g_rho0, 0, sizeof(double), s);
  const int B = 1 - cur;  // buffers holding the step's output (and its cell order)
  const int I = tp.iters;
  const float inv_dt = 1.0f / dt;
  const float4* fin = tp.xs + static_cast<size_t>(I) * b.n;
  Finish F;
  F.x = tp.x;
  F.v = tp.v;
  F.xs = tp.xs;
  F.dp = tp.dp;
  F.scenes = b.scenes;
  F.id = b.id[B];
  F.gxs = tp.gxs;
  F.pl0 = tp.pl[0];
  F.pl1 = tp.pl[1];
  F.gx = tp.gx;
  F.r0 = tp.r0;
  F.gx_in = gx_in;
  F.gv_in = gv_in;
  F.n = b.n;
  k_adj_in<<<blocks_for(n, 256), 256, 0, s>>>(b.id[B], gx_out, gv_out, tp.eta, b.omega, tp.gxs, tp.gvo, tp.eb,
                                              tp.wb, tp.r0, P, dt, n);
  PBF_BLOCK_SWITCH(t.block_solve,
                   k_adj_vort_b<BLOCK><<<blocks_for(n, BLOCK), BLOCK, 0, s>>>(
                       fin, b.omega, b.nbr_hdr, b.nbr_w, tp.eb, tp.wb, tp.gxs, P, n));
  PBF_BLOCK_SWITCH(t.block_solve,
                   k_adj_xsph<BLOCK><<<blocks_for(n, BLOCK), BLOCK, 0, s>>>(
                       fin, b.disp[1], b.nbr_hdr, b.nbr_w, tp.gvo, tp.wb, F, P, dt, inv_dt, I - 1, n));
  for (int k = I - 1; k >= 0; --k) {
    const float4* xk = tp.xs + static_cast<size_t>(k) * b.n;
    const float4* plk = tp.pl[k & 1];
    PBF_BLOCK_SWITCH(t.block_solve,
                     k_adj_lambda<BLOCK><<<blocks_for(n, BLOCK), BLOCK, 0, s>>>(
                         xk, b.nbr_hdr, b.nbr_w, plk, tp.gr, tp.r0, P, n));
    if (P.scorr_n == 4) {
      PBF_BLOCK_SWITCH(t.block_solve,
                       (k_adj_pos<BLOCK, true><<<blocks_for(n, BLOCK), BLOCK, 0, s>>>(
                           xk, b.nbr_hdr, b.nbr_w, plk, tp.gr, F, P, dt, k - 1, n)));
    } else {
      PBF_BLOCK_SWITCH(t.block_solve,
                       (k_adj_pos<BLOCK, false><<<blocks_for(n, BLOCK), BLOCK, 0, s>>>(
                           xk, b.nbr_hdr, b.nbr_w, plk, tp.gr, F, P, dt, k - 1, n)));
    }
  }
  k_adj_r0_part<<<kAdjReduceBlocks, 256, 0, s>>>(tp.r0, tp.r0_part, n);
  k_adj_r0_final<<<1, kAdjReduceBlocks, 0, s>>>(tp.r0_part, g_rho0);
  return cudaGetLastError();
}

}  // namespace pbf
