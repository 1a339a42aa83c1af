// PBF step kernels for sm_103a (FP32 on CUDA cores; the step is a sparse
// stencil with no dense contraction, so no tensor cores).
//
// One step (Particles::timeStep, particles.cpp:250-297) is this launch chain
// on one stream; every phase covers all scenes of a batch in one launch:
//   k_predict     gravity + predicted move + collision, cell key, per-cell
//                 count and rank (particles.cpp:175-183, 87-132)
//   k_scan_*      exclusive prefix sum of the cell counts
//   k_scatter     slot = cell start + rank
//   k_cellsort    order each cell's slots by original index (determinism)
//   k_gather      reorder x, delta, id, cell key into cell order; x* = x + delta
//   k_cells_build neighbour sets |x*_i - x*_j|^2 <= H2 over the 27 cells
//                 (particles.cpp:258-265) + lambda of iteration 0
//   k_cells_lambda  density + lambda      (particles.cpp:185-204)   x (iters - 1)
//   k_cells_deltap  delta p + collision   (particles.cpp:206-213)   x iters
//   k_cells_xsph    velocity, vorticity, XSPH, reported density
//                   (particles.cpp:215-234, order-independent form)
//   k_cells_vort    vorticity confinement, x <- x* (particles.cpp:236-248)
// The k_cells_* kernels are cell-cooperative (pbf_cells.cuh).
#include <cfloat>
#include <climits>
#include <cstdint>

#include "pbf_cells.cuh"

namespace pbf {
namespace {

constexpr int kScanItems = 4;
constexpr int kScanThreads = 256;
constexpr int kScanTile = kScanItems * kScanThreads;
constexpr uint32_t kMaxSortedCell = 256;

__device__ __forceinline__ unsigned lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

__device__ __forceinline__ int scene_of_slot(const float4& p) { return __float_as_int(p.w); }

// ---------------------------------------------------------------------------
// prediction + cell count
// ---------------------------------------------------------------------------
__global__ void k_predict(const float4* __restrict__ pos, const float4* __restrict__ vel,
                          float4* __restrict__ disp_out, uint32_t* __restrict__ key_out,
                          uint32_t* __restrict__ rank_out, uint32_t* __restrict__ cell_count,
                          const SceneDesc* __restrict__ scenes, DevParams P, float dt, int move,
                          int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < n;
  uint32_t key = 0xffffffffu;
  if (live) {
    const float4 x4 = pos[i];
    const SceneDesc& sc = scenes[scene_of_slot(x4)];
    const float3 x = f3(x4);
    float3 d = make_float3(0.f, 0.f, 0.f);
    if (move) {
      const float4 v4 = vel[i];
      // applyForceVelocity, particles.cpp:180: v += g dt
      const float3 v = make_float3(v4.x + P.g[0] * dt, v4.y + P.g[1] * dt, v4.z + P.g[2] * dt);
      collide(x, d, v * dt, true, sc, P);
      disp_out[i] = make_float4(d.x, d.y, d.z, 0.f);
    }
    key = cell_key(cell_of(x + d, sc, P.inv_cell), sc);
    key_out[i] = key;
  }
  // warp-aggregated per-cell rank
  const unsigned active = __ballot_sync(0xffffffffu, live);
  if (!live) return;
  const unsigned peers = __match_any_sync(active, key);
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (static_cast<int>(lane_id()) == leader) base = atomicAdd(&cell_count[key], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  rank_out[i] = base + __popc(peers & lanemask_lt());
}

// ---------------------------------------------------------------------------
// exclusive scan of cell counts (three phases)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* total) {
  __shared__ uint32_t warp_sums[32];
  const unsigned lane = lane_id(), warp = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= static_cast<unsigned>(o)) x += y;
  }
  if (lane == 31) warp_sums[warp] = x;
  __syncthreads();
  if (warp == 0) {
    const int nw = blockDim.x >> 5;
    uint32_t w = lane < static_cast<unsigned>(nw) ? warp_sums[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= static_cast<unsigned>(o)) w += y;
    }
    if (lane < static_cast<unsigned>(nw)) warp_sums[lane] = w;
  }
  __syncthreads();
  const uint32_t warp_off = warp ? warp_sums[warp - 1] : 0u;
  *total = warp_sums[(blockDim.x >> 5) - 1];
  __syncthreads();
  return warp_off + x - v;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t* __restrict__ count,
                                                              uint32_t* __restrict__ start,
                                                              uint32_t* __restrict__ tile_sum,
                                                              uint32_t m) {
  const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  uint32_t v[kScanItems];
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < m) ? count[base + k] : 0u;
    s += v[k];
  }
  uint32_t total;
  uint32_t off = block_exclusive_scan(s, &total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < m) start[base + k] = off;
    off += v[k];
  }
  if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t* __restrict__ tile_sum, uint32_t tiles,
                                                     uint32_t* __restrict__ start, uint32_t m) {
  uint32_t carry = 0;
  for (uint32_t b = 0; b < tiles; b += blockDim.x) {
    const uint32_t idx = b + threadIdx.x;
    const uint32_t v = idx < tiles ? tile_sum[idx] : 0u;
    uint32_t total;
    const uint32_t ex = block_exclusive_scan(v, &total);
    if (idx < tiles) tile_sum[idx] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) start[m] = carry;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_add(uint32_t* __restrict__ start,
                                                            const uint32_t* __restrict__ tile_sum,
                                                            uint32_t m) {
  const uint32_t add = tile_sum[blockIdx.x];
  const uint32_t base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k)
    if (base + k < m) start[base + k] += add;
}

// ---------------------------------------------------------------------------
// reorder
// ---------------------------------------------------------------------------
__global__ void k_scatter(const uint32_t* __restrict__ key, const uint32_t* __restrict__ rank,
                          const uint32_t* __restrict__ cell_start, uint32_t* __restrict__ perm, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) perm[cell_start[key[i]] + rank[i]] = static_cast<uint32_t>(i);
}

// Insertion sort of each cell's slots by original particle index, so the
// cell order (hence every neighbour sum) is independent of atomic timing.
// Cells above kMaxSortedCell particles keep the atomic order (bounded time).
__global__ void k_cellsort(const uint32_t* __restrict__ cell_start, uint32_t* __restrict__ perm,
                           const uint32_t* __restrict__ id, uint32_t m) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m) return;
  const uint32_t b = cell_start[c], e = cell_start[c + 1];
  if (e - b < 2 || e - b > kMaxSortedCell) return;
  for (uint32_t x = b + 1; x < e; ++x) {
    const uint32_t v = perm[x];
    const uint32_t kv = id[v];
    uint32_t y = x;
    while (y > b && id[perm[y - 1]] > kv) {
      perm[y] = perm[y - 1];
      --y;
    }
    perm[y] = v;
  }
}

__global__ void k_gather(const uint32_t* __restrict__ perm, const float4* __restrict__ pos_a,
                         const float4* __restrict__ disp_a, const float4* __restrict__ vel_a,
                         const uint32_t* __restrict__ id_a, const uint32_t* __restrict__ key_a,
                         float4* __restrict__ pos_b, float4* __restrict__ disp_b, float4* __restrict__ xs_b,
                         float4* __restrict__ vel_b, uint32_t* __restrict__ id_b, uint32_t* __restrict__ key_b,
                         int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t i = perm[s];
  key_b[s] = key_a[i];
  const float4 x = pos_a[i];
  pos_b[s] = x;
  id_b[s] = id_a[i];
  if (disp_a) {
    const float4 d = disp_a[i];
    disp_b[s] = d;
    xs_b[s] = make_float4(x.x + d.x, x.y + d.y, x.z + d.z, 0.f);
  }
  if (vel_a) vel_b[s] = vel_a[i];
}

// ---------------------------------------------------------------------------
// neighbour sets + first-iteration lambda; lambda / delta-p / XSPH / vorticity
// passes (cell-cooperative, see pbf_cells.cuh)
// ---------------------------------------------------------------------------
struct LambdaAcc {
  float qsum, g2;
  float3 gs;
};
__device__ __forceinline__ void lambda_add(LambdaAcc& a, const Pair& p) {
  a.qsum += p.q * p.q * p.q;
  a.gs = a.gs + p.r * p.s;
  a.g2 += p.s * p.s * p.r2;
}
__device__ __forceinline__ void lambda_reduce(LambdaAcc& a, int L) {
  a.qsum = group_sum(a.qsum, L);
  a.g2 = group_sum(a.g2, L);
  a.gs.x = group_sum(a.gs.x, L);
  a.gs.y = group_sum(a.gs.y, L);
  a.gs.z = group_sum(a.gs.z, L);
}
// newtonStepCalculateLambda, particles.cpp:185-204
__device__ __forceinline__ float lambda_of(const LambdaAcc& a, const DevParams& P, float* rho) {
  *rho = P.poly6_c * a.qsum;
  const float kg = P.spiky_c * P.inv_rho0;
  const float denom = kg * kg * (a.g2 + dot3(a.gs, a.gs)) + P.epsilon;
  return -(*rho * P.inv_rho0 - 1.0f) / denom;
}

__device__ __forceinline__ uint32_t entry_of(uint32_t w, int half) { return half ? (w >> 16) : (w & 0xffffu); }

// The build: neighbour sets N(i) = {j != i : fl(|x*_i - x*_j|^2) <= H2}
// (particles.cpp:258-265) as candidate indices, and lambda of iteration 0.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_cells_build(float4* xs, const float4* __restrict__ pos,
                                                            const uint32_t* __restrict__ skey,
                                                            const uint32_t* __restrict__ cell_start,
                                                            const SceneDesc* __restrict__ scenes,
                                                            uint32_t* __restrict__ nbr_cnt,
                                                            uint32_t* __restrict__ words, float* __restrict__ lam,
                                                            float* __restrict__ rho_iter0,
                                                            unsigned* __restrict__ err, DevParams P, int n) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = static_cast<int>(threadIdx.x >> 5);
  unsigned char* my = smem + warp * kBuildWarpBytes;
  float4* cand = reinterpret_cast<float4*>(my);
  uint16_t* list = reinterpret_cast<uint16_t*>(my + kCandMax * 16);
  int* cnt_s = reinterpret_cast<int*>(my + kCandMax * 16 + kBuildM * kBuildCap * 2);
  CellRows* rows = reinterpret_cast<CellRows*>(my + kCandMax * 16 + kBuildM * kBuildCap * 2 + 128);
  const unsigned lane = lane_id();
  const unsigned lt = lanemask_lt_();
  const int cap = P.max_words * 2;
  const int fast_cap = cap < kBuildCap ? cap : kBuildCap;
  unsigned flags = 0;
  for_each_owned_cell(skey, cell_start, pos, n, static_cast<int>(blockIdx.x) * WARPS + warp,
                      [&](const CellInfo& c, uint32_t key) {
    const SceneDesc& sc = scenes[c.sid];
    cell_rows(key, sc, cell_start, rows, &flags);
    const uint32_t total = rows->pref[9];
    const uint32_t self0 = rows->pref[4] + (c.cs - rows->start[4]);
    // fast: the cell fits the buffers and lies inside its own (uncapped) staged row
    bool fast = c.m <= static_cast<uint32_t>(kBuildM) && total <= static_cast<uint32_t>(kCandMax) &&
                (c.cs - rows->start[4]) + c.m <= rows->pref[5] - rows->pref[4];
    if (fast) {
      stage_rows(rows, xs, cand);
      __syncwarp();
      int cnt = 0;
      for (uint32_t t0 = 0; t0 < total; t0 += 32) {
        const uint32_t t = t0 + lane;
        const bool has = t < total;
        const float4 xj = has ? cand[t] : make_float4(0.f, 0.f, 0.f, 0.f);
        for (uint32_t q = 0; q < c.m; ++q) {
          const float4 xq = cand[self0 + q];
          const bool hit = has && t != self0 + q && dist2_rn(xq, xj) <= P.h2;
          const unsigned b = __ballot_sync(0xffffffffu, hit);
          if (b) {
            const int cq = __shfl_sync(0xffffffffu, cnt, static_cast<int>(q));
            if (hit) {
              const int rank = cq + __popc(b & lt);
              if (rank < fast_cap) list[q * kBuildCap + rank] = static_cast<uint16_t>(t);
            }
            if (lane == q) cnt += __popc(b);
          }
        }
      }
      if (__any_sync(0xffffffffu, lane < c.m && cnt > fast_cap)) {
        fast = false;  // a list overflows the buffer: redo the cell per particle
      } else {
        if (lane < c.m) {
          cnt_s[lane] = cnt;
          nbr_cnt[c.cs + lane] = static_cast<uint32_t>(cnt);
        }
        __syncwarp();
        const unsigned mw = __reduce_max_sync(0xffffffffu, lane < c.m ? static_cast<unsigned>((cnt + 1) >> 1) : 0u);
        for (uint32_t idx = lane; idx < c.m * mw; idx += 32) {
          const uint32_t q = idx % c.m, w = idx / c.m;
          const int cq = cnt_s[q];
          if (static_cast<int>(2 * w) < cq) {
            const uint32_t e0 = list[q * kBuildCap + 2 * w];
            const uint32_t e1 = static_cast<int>(2 * w + 1) < cq ? list[q * kBuildCap + 2 * w + 1] : 0u;
            words[static_cast<size_t>(w) * n + c.cs + q] = e0 | (e1 << 16);
          }
        }
        const int L = lanes_per_particle(c.m), per = 32 / L;
        for (uint32_t q0 = 0; q0 < c.m; q0 += per) {
          const uint32_t q = q0 + lane / L;
          const int sub = static_cast<int>(lane) % L;
          const bool act = q < c.m;
          LambdaAcc a{0.f, 0.f, make_float3(0.f, 0.f, 0.f)};
          if (act) {
            const float4 xi = cand[self0 + q];
            const int cq = cnt_s[q];
            for (int k = sub; k < cq; k += L) lambda_add(a, pair_of(xi, cand[list[q * kBuildCap + k]], P.h, P.h2));
          }
          lambda_reduce(a, L);
          if (act && sub == 0) {
            float rho;
            const float l = lambda_of(a, P, &rho);
            const uint32_t i = c.cs + q;
            lam[i] = l;
            reinterpret_cast<float*>(xs)[4 * i + 3] = l;
            if (rho_iter0) rho_iter0[i] = rho;
          }
        }
      }
    }
    if (!fast) {
      for (uint32_t q = lane; q < c.m; q += 32) {
        const uint32_t i = c.cs + q;
        const float4 xi = xs[i];
        int cnt = 0;
        uint32_t word = 0;
        for (int r = 0; r < 9; ++r) {
          const uint32_t p0 = rows->pref[r], len = rows->pref[r + 1] - p0, s0 = rows->start[r];
          for (uint32_t u = 0; u < len; ++u) {
            const uint32_t j = s0 + u;
            if (j == i) continue;
            if (dist2_rn(xi, __ldg(&xs[j])) <= P.h2) {
              if (cnt < cap) {
                const uint32_t e = p0 + u;
                if ((cnt & 1) == 0) {
                  word = e;
                } else {
                  word |= e << 16;
                  words[static_cast<size_t>(cnt >> 1) * n + i] = word;
                }
                ++cnt;
              } else {
                flags |= PBF_ERRBIT_NEIGHBOR_CAPACITY;
              }
            }
          }
        }
        if (cnt & 1) words[static_cast<size_t>(cnt >> 1) * n + i] = word;
        nbr_cnt[i] = static_cast<uint32_t>(cnt);
        LambdaAcc a{0.f, 0.f, make_float3(0.f, 0.f, 0.f)};
        for (int k = 0; k < cnt; ++k) {
          const uint32_t e = entry_of(words[static_cast<size_t>(k >> 1) * n + i], k & 1);
          lambda_add(a, pair_of(xi, __ldg(&xs[cand_slot(rows, e)]), P.h, P.h2));
        }
        float rho;
        const float l = lambda_of(a, P, &rho);
        lam[i] = l;
        reinterpret_cast<float*>(xs)[4 * i + 3] = l;
        if (rho_iter0) rho_iter0[i] = rho;
      }
    }
    __syncwarp();
  });
  if (flags) atomicOr(err, flags);
}

// Passes. Per owned cell: rows, staging (when the candidates fit), then L lanes
// per particle walk the particle's list words (lane sub takes words sub, sub+L,
// ...), each word holding two candidate indices; partial sums are reduced over
// the L lanes and lane sub = 0 finishes the particle.
#define PBF_PASS_PROLOGUE(STAGE)                                                   \
  cell_rows(key, sc, cell_start, rows, &flags);                                    \
  const uint32_t total = rows->pref[9];                                            \
  const uint32_t self0 = rows->pref[4] + (c.cs - rows->start[4]);                  \
  const bool fast = total <= static_cast<uint32_t>(kCandMax) &&                   \
                    (c.cs - rows->start[4]) + c.m <= rows->pref[5] - rows->pref[4];  \
  if (fast) {                                                                      \
    STAGE;                                                                         \
    __syncwarp();                                                                  \
  }                                                                                \
  const int L = lanes_per_particle(c.m), per = 32 / L;

#define PBF_FOR_NEIGHBORS(BODY)                                                    \
  for (int wk_ = sub; 2 * wk_ < cq; wk_ += L) {                                    \
    const uint32_t wd = __ldg(&words[static_cast<size_t>(wk_) * n + i]);           \
    _Pragma("unroll") for (int hh = 0; hh < 2; ++hh) {                             \
      if (2 * wk_ + hh < cq) {                                                     \
        const uint32_t t = entry_of(wd, hh);                                       \
        const uint32_t jj = fast ? t : cand_slot(rows, t);                         \
        BODY;                                                                      \
      }                                                                            \
    }                                                                              \
  }

template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_cells_lambda(float4* xs, const float4* __restrict__ pos,
                                                             const uint32_t* __restrict__ skey,
                                                             const uint32_t* __restrict__ cell_start,
                                                             const SceneDesc* __restrict__ scenes,
                                                             const uint32_t* __restrict__ nbr_cnt,
                                                             const uint32_t* __restrict__ words,
                                                             float* __restrict__ lam, unsigned* __restrict__ err,
                                                             DevParams P, int n) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = static_cast<int>(threadIdx.x >> 5);
  unsigned char* my = smem + warp * kPassWarpBytes;
  float4* cand = reinterpret_cast<float4*>(my);
  CellRows* rows = reinterpret_cast<CellRows*>(my + kCandMax * 16);
  const unsigned lane = lane_id();
  unsigned flags = 0;
  for_each_owned_cell(skey, cell_start, pos, n, static_cast<int>(blockIdx.x) * WARPS + warp,
                      [&](const CellInfo& c, uint32_t key) {
    const SceneDesc& sc = scenes[c.sid];
    PBF_PASS_PROLOGUE(stage_rows(rows, xs, cand))
    for (uint32_t q0 = 0; q0 < c.m; q0 += per) {
      const uint32_t q = q0 + lane / L;
      const int sub = static_cast<int>(lane) % L;
      const bool act = q < c.m;
      const uint32_t i = c.cs + q;
      const int cq = act ? static_cast<int>(__ldg(&nbr_cnt[i])) : 0;
      const float4 xi = act ? (fast ? cand[self0 + q] : xs[i]) : make_float4(0.f, 0.f, 0.f, 0.f);
      LambdaAcc a{0.f, 0.f, make_float3(0.f, 0.f, 0.f)};
      PBF_FOR_NEIGHBORS(lambda_add(a, pair_of(xi, fast ? cand[jj] : __ldg(&xs[jj]), P.h, P.h2)))
      lambda_reduce(a, L);
      if (act && sub == 0) {
        float rho;
        const float l = lambda_of(a, P, &rho);
        lam[i] = l;
        reinterpret_cast<float*>(xs)[4 * i + 3] = l;
      }
    }
    __syncwarp();
  });
  if (flags) atomicOr(err, flags);
}

// newtonStepUpdatePosition (particles.cpp:206-213) + clamp (:51-84). lambda_j
// arrives in x*_j.w; N4 specialises the tensile exponent N = 4 (particles.cpp:40).
template <int WARPS, bool N4>
__global__ void __launch_bounds__(WARPS * 32) k_cells_deltap(const float4* __restrict__ xs,
                                                             const float4* __restrict__ pos,
                                                             const uint32_t* __restrict__ skey,
                                                             const uint32_t* __restrict__ cell_start,
                                                             const SceneDesc* __restrict__ scenes,
                                                             const uint32_t* __restrict__ nbr_cnt,
                                                             const uint32_t* __restrict__ words,
                                                             float4* __restrict__ disp, float4* __restrict__ xs_next,
                                                             unsigned* __restrict__ err, DevParams P, int n) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = static_cast<int>(threadIdx.x >> 5);
  unsigned char* my = smem + warp * kPassWarpBytes;
  float4* cand = reinterpret_cast<float4*>(my);
  CellRows* rows = reinterpret_cast<CellRows*>(my + kCandMax * 16);
  const unsigned lane = lane_id();
  const float wt = P.poly6_c * P.tis;
  unsigned flags = 0;
  for_each_owned_cell(skey, cell_start, pos, n, static_cast<int>(blockIdx.x) * WARPS + warp,
                      [&](const CellInfo& c, uint32_t key) {
    const SceneDesc& sc = scenes[c.sid];
    PBF_PASS_PROLOGUE(stage_rows(rows, xs, cand))
    for (uint32_t q0 = 0; q0 < c.m; q0 += per) {
      const uint32_t q = q0 + lane / L;
      const int sub = static_cast<int>(lane) % L;
      const bool act = q < c.m;
      const uint32_t i = c.cs + q;
      const int cq = act ? static_cast<int>(__ldg(&nbr_cnt[i])) : 0;
      const float4 xi = act ? (fast ? cand[self0 + q] : __ldg(&xs[i])) : make_float4(0.f, 0.f, 0.f, 0.f);
      float3 dp = make_float3(0.f, 0.f, 0.f);
      PBF_FOR_NEIGHBORS({
        const float4 xj = fast ? cand[jj] : __ldg(&xs[jj]);
        const Pair p = pair_of(xi, xj, P.h, P.h2);
        const float a = wt * (p.q * p.q * p.q);  // W / W(dq)
        float an;
        if (N4) {
          const float a2 = a * a;
          an = a2 * a2;
        } else {
          an = a;
          for (int e = 1; e < P.scorr_n; ++e) an *= a;
        }
        const float coef = (xi.w + xj.w) - P.scorr_k * an;  // lambda_i + lambda_j + s_corr
        dp = dp + p.r * (coef * p.s);
      })
      dp.x = group_sum(dp.x, L);
      dp.y = group_sum(dp.y, L);
      dp.z = group_sum(dp.z, L);
      if (act && sub == 0) {
        dp = dp * (P.spiky_c * P.inv_rho0);
        const float4 x4 = __ldg(&pos[i]);
        float3 d = f3(disp[i]);
        const float3 x = f3(x4);
        collide(x, d, dp, false, sc, P);
        disp[i] = make_float4(d.x, d.y, d.z, 0.f);
        xs_next[i] = make_float4(x.x + d.x, x.y + d.y, x.z + d.z, 0.f);
      }
    }
    __syncwarp();
  });
  if (flags) atomicOr(err, flags);
}

// updateVelocity + calculateVorticityApplyXSPHViscosity (particles.cpp:215-234) in
// the order-independent form; |omega_i| goes to x*_i.w for the vorticity pass.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_cells_xsph(float4* xs, const float4* __restrict__ pos,
                                                           const uint32_t* __restrict__ skey,
                                                           const uint32_t* __restrict__ cell_start,
                                                           const SceneDesc* __restrict__ scenes,
                                                           const uint32_t* __restrict__ nbr_cnt,
                                                           const uint32_t* __restrict__ words,
                                                           const float4* __restrict__ disp,
                                                           float4* __restrict__ vel_out, float4* __restrict__ omega,
                                                           float* __restrict__ rho_out, unsigned* __restrict__ err,
                                                           DevParams P, float inv_dt, int n) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = static_cast<int>(threadIdx.x >> 5);
  unsigned char* my = smem + warp * kPass2WarpBytes;
  float4* cand = reinterpret_cast<float4*>(my);
  float4* cand_d = cand + kCandMax;
  CellRows* rows = reinterpret_cast<CellRows*>(my + 2 * kCandMax * 16);
  const unsigned lane = lane_id();
  unsigned flags = 0;
  for_each_owned_cell(skey, cell_start, pos, n, static_cast<int>(blockIdx.x) * WARPS + warp,
                      [&](const CellInfo& c, uint32_t key) {
    const SceneDesc& sc = scenes[c.sid];
    PBF_PASS_PROLOGUE({
      stage_rows(rows, xs, cand);
      stage_rows(rows, disp, cand_d);
    })
    for (uint32_t q0 = 0; q0 < c.m; q0 += per) {
      const uint32_t q = q0 + lane / L;
      const int sub = static_cast<int>(lane) % L;
      const bool act = q < c.m;
      const uint32_t i = c.cs + q;
      const int cq = act ? static_cast<int>(__ldg(&nbr_cnt[i])) : 0;
      const float4 xi = act ? (fast ? cand[self0 + q] : xs[i]) : make_float4(0.f, 0.f, 0.f, 0.f);
      const float3 vi = act ? f3(fast ? cand_d[self0 + q] : __ldg(&disp[i])) * inv_dt : make_float3(0.f, 0.f, 0.f);
      float qsum = 0.f;
      float3 visc = make_float3(0.f, 0.f, 0.f), w = make_float3(0.f, 0.f, 0.f);
      PBF_FOR_NEIGHBORS({
        const Pair p = pair_of(xi, fast ? cand[jj] : xs[jj], P.h, P.h2);
        const float3 vij = f3(fast ? cand_d[jj] : __ldg(&disp[jj])) * inv_dt - vi;
        const float q3 = p.q * p.q * p.q;
        visc = visc + vij * q3;
        qsum += q3;
        w = w + cross3(vij, p.r * p.s);
      })
      qsum = group_sum(qsum, L);
      visc.x = group_sum(visc.x, L);
      visc.y = group_sum(visc.y, L);
      visc.z = group_sum(visc.z, L);
      w.x = group_sum(w.x, L);
      w.y = group_sum(w.y, L);
      w.z = group_sum(w.z, L);
      if (act && sub == 0) {
        const float rho = P.poly6_c * qsum;
        w = w * P.spiky_c;
        const float3 v = vi + visc * (P.xsph_c * P.poly6_c);
        vel_out[i] = make_float4(v.x, v.y, v.z, 0.f);
        const float wn = sqrtf(dot3(w, w));
        omega[i] = make_float4(w.x, w.y, w.z, wn);
        reinterpret_cast<float*>(xs)[4 * i + 3] = wn;
        rho_out[i] = rho;
      }
    }
    __syncwarp();
  });
  if (flags) atomicOr(err, flags);
}

// applyVorticity + updatePosition (particles.cpp:236-248); |omega_j| in x*_j.w.
template <int WARPS>
__global__ void __launch_bounds__(WARPS * 32) k_cells_vort(const float4* __restrict__ xs, float4* __restrict__ pos,
                                                           const uint32_t* __restrict__ skey,
                                                           const uint32_t* __restrict__ cell_start,
                                                           const SceneDesc* __restrict__ scenes,
                                                           const uint32_t* __restrict__ nbr_cnt,
                                                           const uint32_t* __restrict__ words,
                                                           const float4* __restrict__ omega, float4* __restrict__ vel,
                                                           unsigned* __restrict__ err, DevParams P, float dt, int n) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int warp = static_cast<int>(threadIdx.x >> 5);
  unsigned char* my = smem + warp * kPassWarpBytes;
  float4* cand = reinterpret_cast<float4*>(my);
  CellRows* rows = reinterpret_cast<CellRows*>(my + kCandMax * 16);
  const unsigned lane = lane_id();
  unsigned flags = 0;
  for_each_owned_cell(skey, cell_start, pos, n, static_cast<int>(blockIdx.x) * WARPS + warp,
                      [&](const CellInfo& c, uint32_t key) {
    const SceneDesc& sc = scenes[c.sid];
    PBF_PASS_PROLOGUE(stage_rows(rows, xs, cand))
    for (uint32_t q0 = 0; q0 < c.m; q0 += per) {
      const uint32_t q = q0 + lane / L;
      const int sub = static_cast<int>(lane) % L;
      const bool act = q < c.m;
      const uint32_t i = c.cs + q;
      const int cq = act ? static_cast<int>(__ldg(&nbr_cnt[i])) : 0;
      const float4 xi = act ? (fast ? cand[self0 + q] : __ldg(&xs[i])) : make_float4(0.f, 0.f, 0.f, 0.f);
      float3 eta = make_float3(0.f, 0.f, 0.f);
      PBF_FOR_NEIGHBORS({
        const float4 xj = fast ? cand[jj] : __ldg(&xs[jj]);
        const Pair p = pair_of(xi, xj, P.h, P.h2);
        eta = eta + p.r * (xj.w * p.s);
      })
      eta.x = group_sum(eta.x, L);
      eta.y = group_sum(eta.y, L);
      eta.z = group_sum(eta.z, L);
      if (act && sub == 0) {
        eta = eta * P.spiky_c;
        float3 v = f3(vel[i]);
        const float en = sqrtf(dot3(eta, eta));
        if (en > kEps) v = v + cross3(eta * (1.0f / en), f3(__ldg(&omega[i]))) * (dt * P.vort_eps);
        vel[i] = make_float4(v.x, v.y, v.z, 0.f);
        pos[i] = make_float4(xi.x, xi.y, xi.z, pos[i].w);  // updatePosition, particles.cpp:246-248
        if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(xi.x) && isfinite(xi.y) &&
              isfinite(xi.z)))
          flags |= PBF_ERRBIT_NONFINITE;
      }
    }
    __syncwarp();
  });
  if (flags) atomicOr(err, flags);
}

// Step statistics (the prints of particles.cpp:267-295 and the neighbour
// alert of :168-172, as numbers): one pass over densities and list headers.
__global__ void __launch_bounds__(256) k_stats(const float* __restrict__ rho, const float* __restrict__ rho0,
                                               const uint32_t* __restrict__ nbr_cnt, DevStats* __restrict__ st,
                                               float inv_rho0, int n) {
  double r = 0.0, r0 = 0.0, es = 0.0;
  float em = 0.f;
  unsigned cmin = 0xffffffffu, cmax = 0u;
  unsigned long long csum = 0ull, low = 0ull;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float x = rho[i];
    r += x;
    r0 += rho0[i];
    const float e = fabsf(x * inv_rho0 - 1.0f);
    es += e;
    em = fmaxf(em, e);
    const unsigned c = nbr_cnt[i];
    cmin = min(cmin, c);
    cmax = max(cmax, c);
    csum += c;
    low += c < static_cast<unsigned>(kNeighborAlert) ? 1ull : 0ull;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    r += __shfl_down_sync(0xffffffffu, r, o);
    r0 += __shfl_down_sync(0xffffffffu, r0, o);
    es += __shfl_down_sync(0xffffffffu, es, o);
    em = fmaxf(em, __shfl_down_sync(0xffffffffu, em, o));
    cmin = min(cmin, __shfl_down_sync(0xffffffffu, cmin, o));
    cmax = max(cmax, __shfl_down_sync(0xffffffffu, cmax, o));
    csum += __shfl_down_sync(0xffffffffu, csum, o);
    low += __shfl_down_sync(0xffffffffu, low, o);
  }
  __shared__ double sd[3][8];
  __shared__ float sem[8];
  __shared__ unsigned smin[8], smax[8];
  __shared__ unsigned long long ssum[8], slow[8];
  const unsigned w = threadIdx.x >> 5;
  if (lane_id() == 0) {
    sd[0][w] = r;
    sd[1][w] = r0;
    sd[2][w] = es;
    sem[w] = em;
    smin[w] = cmin;
    smax[w] = cmax;
    ssum[w] = csum;
    slow[w] = low;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (unsigned k = 1; k < (blockDim.x >> 5); ++k) {
      r += sd[0][k];
      r0 += sd[1][k];
      es += sd[2][k];
      em = fmaxf(em, sem[k]);
      cmin = min(cmin, smin[k]);
      cmax = max(cmax, smax[k]);
      csum += ssum[k];
      low += slow[k];
    }
    atomicAdd(&st->rho_sum, r);
    atomicAdd(&st->rho_iter0_sum, r0);
    atomicAdd(&st->err_sum, es);
    atomicMax(&st->err_max_bits, __float_as_uint(em));
    atomicMin(&st->nbr_min, cmin);
    atomicMax(&st->nbr_max, cmax);
    atomicAdd(&st->nbr_sum, csum);
    atomicAdd(&st->low_cnt, low);
  }
}

__global__ void k_stats_init(DevStats* st) {
  st->rho_iter0_sum = 0.0;
  st->rho_sum = 0.0;
  st->err_sum = 0.0;
  st->err_max_bits = 0u;
  st->nbr_min = 0xffffffffu;
  st->nbr_max = 0u;
  st->nbr_sum = 0ull;
  st->low_cnt = 0ull;
}

// ---------------------------------------------------------------------------
// transfers between original order and cell order
// ---------------------------------------------------------------------------
__global__ void k_upload(const float* __restrict__ xyz, const float* __restrict__ v,
                         const SceneDesc* __restrict__ scenes, int n_scenes, float4* __restrict__ pos,
                         float4* __restrict__ vel, uint32_t* __restrict__ id, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  int lo = 0, hi = n_scenes - 1;  // scene whose particle range holds s
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (scenes[mid].p_off <= static_cast<uint32_t>(s)) lo = mid; else hi = mid - 1;
  }
  pos[s] = make_float4(xyz[3 * s], xyz[3 * s + 1], xyz[3 * s + 2], __int_as_float(lo));
  vel[s] = v ? make_float4(v[3 * s], v[3 * s + 1], v[3 * s + 2], 0.f) : make_float4(0.f, 0.f, 0.f, 0.f);
  id[s] = static_cast<uint32_t>(s);
}

__global__ void k_download(const float4* __restrict__ pos, const float4* __restrict__ vel,
                           const float* __restrict__ rho, const uint32_t* __restrict__ id,
                           float* __restrict__ xyz, float* __restrict__ v, float* __restrict__ r, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t o = id[s];
  if (xyz) {
    const float4 p = pos[s];
    xyz[3 * o] = p.x;
    xyz[3 * o + 1] = p.y;
    xyz[3 * o + 2] = p.z;
  }
  if (v) {
    const float4 q = vel[s];
    v[3 * o] = q.x;
    v[3 * o + 1] = q.y;
    v[3 * o + 2] = q.z;
  }
  if (r) r[o] = rho[s];
}

__global__ void k_unsort_u32(const uint32_t* __restrict__ src, const uint32_t* __restrict__ id,
                             uint32_t* __restrict__ dst, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) dst[id[s]] = src[s];
}

__global__ void k_unsort_f4(const float4* __restrict__ src, const uint32_t* __restrict__ id,
                            float* __restrict__ dst, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const float4 p = src[s];
  const uint32_t o = id[s];
  dst[3 * o] = p.x;
  dst[3 * o + 1] = p.y;
  dst[3 * o + 2] = p.z;
}

__global__ void k_cells_of(const float4* __restrict__ xs, const float4* __restrict__ pos,
                           const SceneDesc* __restrict__ scenes, const uint32_t* __restrict__ id,
                           uint32_t* __restrict__ cells, DevParams P, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const SceneDesc& sc = scenes[scene_of_slot(pos[s])];
  cells[id[s]] = cell_key(cell_of(f3(xs[s]), sc, P.inv_cell), sc);
}

__global__ void k_nbr_counts(const uint32_t* __restrict__ nbr_cnt, const uint32_t* __restrict__ id,
                             uint32_t* __restrict__ counts, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) counts[id[s]] = nbr_cnt[s];
}

// Candidate rows of a cell computed by one thread (introspection paths).
__device__ void cell_rows_thread(uint32_t key, const SceneDesc& sc, const uint32_t* __restrict__ cell_start,
                                 CellRows* rows) {
  const uint32_t local = key - sc.cell_off;
  const int nx = sc.dim[0], ny = sc.dim[1], nz = sc.dim[2];
  const int cx = static_cast<int>(local % nx), cy = static_cast<int>((local / nx) % ny);
  const int cz = static_cast<int>(local / (nx * ny));
  uint32_t acc = 0;
  for (int r = 0; r < 9; ++r) {
    const int z = cz + r / 3 - 1, y = cy + r % 3 - 1;
    uint32_t start = 0, len = 0;
    if (z >= 0 && z < nz && y >= 0 && y < ny) {
      const int x0 = cx > 0 ? cx - 1 : 0, x1 = cx + 1 < nx ? cx + 1 : nx - 1;
      const uint32_t row = sc.cell_off + static_cast<uint32_t>((z * ny + y) * nx);
      start = cell_start[row + x0];
      len = cell_start[row + x1 + 1] - start;
      if (len > static_cast<uint32_t>(kMaxRowCandidates)) len = kMaxRowCandidates;
    }
    rows->start[r] = start;
    rows->pref[r] = acc;
    acc += len;
  }
  rows->pref[9] = acc;
}

// ids[offsets[id[i]] ...] = original ids of i's neighbours (cell order).
__global__ void k_nbr_ids(const float4* __restrict__ pos, const uint32_t* __restrict__ skey,
                          const uint32_t* __restrict__ cell_start, const SceneDesc* __restrict__ scenes,
                          const uint32_t* __restrict__ nbr_cnt, const uint32_t* __restrict__ words,
                          const uint32_t* __restrict__ id, const uint32_t* __restrict__ offsets,
                          uint32_t* __restrict__ ids, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  CellRows rows;
  cell_rows_thread(skey[i], scenes[__float_as_int(pos[i].w)], cell_start, &rows);
  uint32_t o = offsets[id[i]];
  const int cnt = static_cast<int>(nbr_cnt[i]);
  for (int k = 0; k < cnt; ++k) {
    const uint32_t t = entry_of(words[static_cast<size_t>(k >> 1) * n + i], k & 1);
    ids[o++] = id[cand_slot(&rows, t)];
  }
}

// Particles::estimateDensities (particles.cpp:440-444) on cell-sorted x: self included.
__global__ void k_density_self(const float4* __restrict__ pos, const uint32_t* __restrict__ cell_start,
                               const SceneDesc* __restrict__ scenes, float* __restrict__ rho,
                               DevParams P, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = pos[i];
  const SceneDesc& sc = scenes[scene_of_slot(xi)];
  const CellCoord cc = cell_of(f3(xi), sc, P.inv_cell);
  float qsum = 0.f;
  for (int r = 0; r < 9; ++r) {
    const int z = cc.z + r / 3 - 1, y = cc.y + r % 3 - 1;
    if (z < 0 || z >= sc.dim[2] || y < 0 || y >= sc.dim[1]) continue;
    const uint32_t row = sc.cell_off + static_cast<uint32_t>((z * sc.dim[1] + y) * sc.dim[0]);
    const int x0 = cc.x > 0 ? cc.x - 1 : 0;
    const int x1 = cc.x + 1 < sc.dim[0] ? cc.x + 1 : sc.dim[0] - 1;
    for (uint32_t j = cell_start[row + x0]; j < cell_start[row + x1 + 1]; ++j) {
      const float4 xj = __ldg(&pos[j]);
      const float3 d = make_float3(xj.x - xi.x, xj.y - xi.y, xj.z - xi.z);
      const float r2 = dot3(d, d);
      if (r2 < P.h2) {
        const float q = P.h2 - r2;
        qsum += q * q * q;
      }
    }
  }
  rho[i] = P.poly6_c * qsum;
}

// Particles::estimateDensityAt (particles.cpp:446-453) at query points, scene 0.
__global__ void k_density_at(const float4* __restrict__ pos, const uint32_t* __restrict__ cell_start,
                             const SceneDesc* __restrict__ scenes, const float* __restrict__ pts,
                             float* __restrict__ out, DevParams P, int m) {
  const int q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q >= m) return;
  const SceneDesc& sc = scenes[0];
  const float3 p = make_float3(pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]);
  const CellCoord cc = cell_of(p, sc, P.inv_cell);
  float qsum = 0.f;
  for (int r = 0; r < 9; ++r) {
    const int z = cc.z + r / 3 - 1, y = cc.y + r % 3 - 1;
    if (z < 0 || z >= sc.dim[2] || y < 0 || y >= sc.dim[1]) continue;
    const uint32_t row = sc.cell_off + static_cast<uint32_t>((z * sc.dim[1] + y) * sc.dim[0]);
    const int x0 = cc.x > 0 ? cc.x - 1 : 0;
    const int x1 = cc.x + 1 < sc.dim[0] ? cc.x + 1 : sc.dim[0] - 1;
    for (uint32_t j = cell_start[row + x0]; j < cell_start[row + x1 + 1]; ++j) {
      const float4 xj = __ldg(&pos[j]);
      const float3 d = make_float3(xj.x - p.x, xj.y - p.y, xj.z - p.z);
      const float r2 = dot3(d, d);
      if (r2 < P.h2) {
        const float qq = P.h2 - r2;
        qsum += qq * qq * qq;
      }
    }
  }
  out[q] = P.poly6_c * qsum;
}

inline unsigned blocks_for(size_t n, int block) { return static_cast<unsigned>((n + block - 1) / block); }

// Shared front half of a step and of a resort: keys, counts, scan, slots.
cudaError_t sort_into_cells(const Buffers& b, const DevParams& P, const Tuning& t, int cur, float dt,
                            bool move, cudaStream_t s, PhaseMarks* mk = nullptr) {
  const int n = static_cast<int>(b.n);
  const uint32_t m = b.n_cells;
  cudaError_t e = cudaMemsetAsync(b.cell_count, 0, sizeof(uint32_t) * m, s);
  if (e != cudaSuccess) return e;
  k_predict<<<blocks_for(n, t.block_predict), t.block_predict, 0, s>>>(
      b.pos[cur], b.vel[cur], b.disp[0], b.key, b.rank, b.cell_count, b.scenes, P, dt, move ? 1 : 0, n);
  if (mk) mk->mark(kPhasePredict, s);
  const uint32_t tiles = (m + kScanTile - 1) / kScanTile;
  k_scan_tiles<<<tiles, kScanThreads, 0, s>>>(b.cell_count, b.cell_start, b.scan_tmp, m);
  k_scan_sums<<<1, 1024, 0, s>>>(b.scan_tmp, tiles, b.cell_start, m);
  k_scan_add<<<tiles, kScanThreads, 0, s>>>(b.cell_start, b.scan_tmp, m);
  if (mk) mk->mark(kPhaseScan, s);
  k_scatter<<<blocks_for(n, t.block_misc), t.block_misc, 0, s>>>(b.key, b.rank, b.cell_start, b.perm, n);
  k_cellsort<<<blocks_for(m, t.block_misc), t.block_misc, 0, s>>>(b.cell_start, b.perm, b.id[cur], m);
  if (mk) mk->mark(kPhaseSort, s);
  return cudaGetLastError();
}

}  // namespace

// Threads per block -> warps per block for the cell-cooperative kernels.
#define PBF_WARPS_SWITCH(block, ...)                                    \
  switch (block) {                                                      \
    case 64: { constexpr int WARPS = 2; __VA_ARGS__; } break;           \
    case 256: { constexpr int WARPS = 8; __VA_ARGS__; } break;          \
    case 512: { constexpr int WARPS = 16; __VA_ARGS__; } break;         \
    default: { constexpr int WARPS = 4; __VA_ARGS__; } break;           \
  }

// One warp per 32 slots.
inline unsigned cell_grid(int n, int warps) { return static_cast<unsigned>((n + 32 * warps - 1) / (32 * warps)); }

// Dynamic shared memory above 48 KB needs an opt-in per kernel; granted once
// per process for every instantiation at its largest launch shape.
template <typename K>
cudaError_t optin(K* k, int bytes) {
  return cudaFuncSetAttribute(reinterpret_cast<const void*>(k), cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
}

template <int W>
cudaError_t optin_all() {
  cudaError_t e = optin(k_cells_build<W>, W * kBuildWarpBytes);
  if (e == cudaSuccess) e = optin(k_cells_lambda<W>, W * kPassWarpBytes);
  if (e == cudaSuccess) e = optin(k_cells_deltap<W, true>, W * kPassWarpBytes);
  if (e == cudaSuccess) e = optin(k_cells_deltap<W, false>, W * kPassWarpBytes);
  if (e == cudaSuccess) e = optin(k_cells_xsph<W>, W * kPass2WarpBytes);
  if (e == cudaSuccess) e = optin(k_cells_vort<W>, W * kPassWarpBytes);
  return e;
}

#define PBF_BLOCK_SWITCH(block, ...)                          \
  switch (block) {                                            \
    case 64: { constexpr int BLOCK = 64; __VA_ARGS__; } break;   \
    case 128: { constexpr int BLOCK = 128; __VA_ARGS__; } break; \
    case 512: { constexpr int BLOCK = 512; __VA_ARGS__; } break; \
    default: { constexpr int BLOCK = 256; __VA_ARGS__; } break;  \
  }

cudaError_t configure_kernels() {
  cudaError_t e = optin_all<2>();
  if (e == cudaSuccess) e = optin_all<4>();
  if (e == cudaSuccess) e = optin_all<8>();
  if (e == cudaSuccess) e = optin_all<16>();
  return e;
}

cudaError_t launch_step(const Buffers& b, const DevParams& P, const Tuning& t, int cur, float dt,
                        int iters, bool keep_pred, cudaStream_t s, PhaseMarks* mk) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  const int A = cur, B = 1 - cur;
  if (mk) mk->mark(-1, s);
  if (P.stats) k_stats_init<<<1, 1, 0, s>>>(b.stats);
  if (mk) mk->mark(kPhaseStats, s);
  cudaError_t e = sort_into_cells(b, P, t, A, dt, true, s, mk);
  if (e != cudaSuccess) return e;
  k_gather<<<blocks_for(n, t.block_misc), t.block_misc, 0, s>>>(
      b.perm, b.pos[A], b.disp[0], nullptr, b.id[A], b.key, b.pos[B], b.disp[1], b.xs[0], nullptr, b.id[B],
      b.skey, n);
  if (keep_pred && b.pred) {
    e = cudaMemcpyAsync(b.pred, b.xs[0], sizeof(float4) * b.n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  if (mk) mk->mark(kPhaseGather, s);
  {
    PBF_WARPS_SWITCH(t.block_nbr, {
      const int bytes = WARPS * kBuildWarpBytes;
      k_cells_build<WARPS><<<cell_grid(n, WARPS), WARPS * 32, bytes, s>>>(
          b.xs[0], b.pos[B], b.skey, b.cell_start, b.scenes, b.nbr_cnt, b.nbr_w, b.lam,
          P.stats ? b.rho_iter0 : nullptr, b.err, P, n);
    });
  }
  if (mk) mk->mark(kPhaseNeighbors, s);
  for (int it = 0; it < iters; ++it) {
    float4* xcur = b.xs[it & 1];
    float4* xnext = b.xs[(it + 1) & 1];
    if (it > 0) {  // iteration 0's lambda comes with the neighbour build
      PBF_WARPS_SWITCH(t.block_solve, {
        const int bytes = WARPS * kPassWarpBytes;
        k_cells_lambda<WARPS><<<cell_grid(n, WARPS), WARPS * 32, bytes, s>>>(
            xcur, b.pos[B], b.skey, b.cell_start, b.scenes, b.nbr_cnt, b.nbr_w, b.lam, b.err, P, n);
      });
    }
    if (mk) mk->mark(kPhaseLambda, s);
    if (P.scorr_n == 4) {
      PBF_WARPS_SWITCH(t.block_solve, {
        const int bytes = WARPS * kPassWarpBytes;
        k_cells_deltap<WARPS, true><<<cell_grid(n, WARPS), WARPS * 32, bytes, s>>>(
            xcur, b.pos[B], b.skey, b.cell_start, b.scenes, b.nbr_cnt, b.nbr_w, b.disp[1], xnext, b.err, P, n);
      });
    } else {
      PBF_WARPS_SWITCH(t.block_solve, {
        const int bytes = WARPS * kPassWarpBytes;
        k_cells_deltap<WARPS, false><<<cell_grid(n, WARPS), WARPS * 32, bytes, s>>>(
            xcur, b.pos[B], b.skey, b.cell_start, b.scenes, b.nbr_cnt, b.nbr_w, b.disp[1], xnext, b.err, P, n);
      });
    }
    if (mk) mk->mark(kPhaseDeltaP, s);
  }
  float4* fin = b.xs[iters & 1];
  PBF_WARPS_SWITCH(t.block_solve, {
    const int bytes = WARPS * kPass2WarpBytes;
    k_cells_xsph<WARPS><<<cell_grid(n, WARPS), WARPS * 32, bytes, s>>>(
        fin, b.pos[B], b.skey, b.cell_start, b.scenes, b.nbr_cnt, b.nbr_w, b.disp[1], b.vel[B], b.omega, b.rho,
        b.err, P, 1.0f / dt, n);
  });
  if (mk) mk->mark(kPhaseXsph, s);
  PBF_WARPS_SWITCH(t.block_solve, {
    const int bytes = WARPS * kPassWarpBytes;
    k_cells_vort<WARPS><<<cell_grid(n, WARPS), WARPS * 32, bytes, s>>>(
        fin, b.pos[B], b.skey, b.cell_start, b.scenes, b.nbr_cnt, b.nbr_w, b.omega, b.vel[B], b.err, P, dt, n);
  });
  if (mk) mk->mark(kPhaseVorticity, s);
  if (P.stats)
    k_stats<<<min(blocks_for(n, 256), 1216u), 256, 0, s>>>(b.rho, b.rho_iter0, b.nbr_cnt, b.stats, P.inv_rho0, n);
  if (mk) mk->mark(kPhaseStats, s);
  return cudaGetLastError();
}

// Reorder the state into cells of the current positions (no motion); the
// result lands in buffers 1 - cur.
cudaError_t launch_resort(const Buffers& b, const DevParams& P, const Tuning& t, int cur, cudaStream_t s) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  cudaError_t e = sort_into_cells(b, P, t, cur, 0.f, false, s);
  if (e != cudaSuccess) return e;
  k_gather<<<blocks_for(n, t.block_misc), t.block_misc, 0, s>>>(
      b.perm, b.pos[cur], nullptr, b.vel[cur], b.id[cur], b.key, b.pos[1 - cur], nullptr, nullptr,
      b.vel[1 - cur], b.id[1 - cur], b.skey, n);
  return cudaGetLastError();
}

cudaError_t launch_upload(const Buffers& b, int cur, const float* xyz, const float* vel,
                          const uint32_t* /*scene_of*/, cudaStream_t s) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  k_upload<<<blocks_for(n, 256), 256, 0, s>>>(xyz, vel, b.scenes, b.n_scenes, b.pos[cur], b.vel[cur],
                                              b.id[cur], n);
  return cudaGetLastError();
}

cudaError_t launch_download(const Buffers& b, int cur, float* xyz, float* vel, float* rho, cudaStream_t s) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  k_download<<<blocks_for(n, 256), 256, 0, s>>>(b.pos[cur], b.vel[cur], b.rho, b.id[cur], xyz, vel, rho, n);
  return cudaGetLastError();
}

cudaError_t launch_unsort_u32(const Buffers& b, int cur, const uint32_t* src, uint32_t* dst, cudaStream_t s) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  k_unsort_u32<<<blocks_for(n, 256), 256, 0, s>>>(src, b.id[cur], dst, n);
  return cudaGetLastError();
}

cudaError_t launch_unsort_f4(const Buffers& b, int cur, const float4* src, float* dst_xyz, cudaStream_t s) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  k_unsort_f4<<<blocks_for(n, 256), 256, 0, s>>>(src, b.id[cur], dst_xyz, n);
  return cudaGetLastError();
}

cudaError_t launch_cells_of(const Buffers& b, const DevParams& P, int cur, uint32_t* cells, cudaStream_t s) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  k_cells_of<<<blocks_for(n, 256), 256, 0, s>>>(b.pred, b.pos[cur], b.scenes, b.id[cur], cells, P, n);
  return cudaGetLastError();
}

cudaError_t launch_neighbor_counts(const Buffers& b, int cur, uint32_t* counts, cudaStream_t s) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  k_nbr_counts<<<blocks_for(n, 256), 256, 0, s>>>(b.nbr_cnt, b.id[cur], counts, n);
  return cudaGetLastError();
}

cudaError_t launch_neighbor_ids(const Buffers& b, int cur, const uint32_t* offsets, uint32_t* ids,
                                cudaStream_t s) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  k_nbr_ids<<<blocks_for(n, 256), 256, 0, s>>>(b.pos[cur], b.skey, b.cell_start, b.scenes, b.nbr_cnt, b.nbr_w,
                                               b.id[cur], offsets, ids, n);
  return cudaGetLastError();
}

cudaError_t launch_density_self(const Buffers& b, const DevParams& P, const Tuning& t, int cur,
                                float* rho_sorted, cudaStream_t s) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  k_density_self<<<blocks_for(n, t.block_misc), t.block_misc, 0, s>>>(b.pos[cur], b.cell_start, b.scenes,
                                                                       rho_sorted, P, n);
  return cudaGetLastError();
}

cudaError_t launch_density_at(const Buffers& b, const DevParams& P, int cur, size_t m, const float* pts,
                              float* out, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  k_density_at<<<blocks_for(m, 256), 256, 0, s>>>(b.pos[cur], b.cell_start, b.scenes, pts, out, P,
                                                  static_cast<int>(m));
  return cudaGetLastError();
}

}  // namespace pbf
