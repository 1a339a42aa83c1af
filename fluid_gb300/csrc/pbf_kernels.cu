// PBF step kernels for sm_103a (FP32 on CUDA cores; the step is a sparse
// stencil with no dense contraction, so no tensor cores).
//
// One step (Particles::timeStep, particles.cpp:250-297) is this launch chain
// on one stream; every phase covers all scenes of a batch in one launch:
//   k_predict     gravity + predicted move + collision, cell key, per-cell
//                 count and rank (particles.cpp:175-183, 87-132)
//   k_scan_*      exclusive prefix sum of the cell counts
//   k_scatter     slot = cell start + rank (atomic order within a cell)
//   k_cellrank    order each cell's slots by x, then original index (determinism)
//   k_gather      reorder x, delta, id into cell order; x* = x + delta
//   k_nbr_build   neighbour sets |x*_i - x*_j|^2 <= H2 over the 27 cells,
//                 stored row-compressed (particles.cpp:258-265)
//   k_lambda      density + lambda            (particles.cpp:185-204)   x iters
//   k_deltap      delta p + collision         (particles.cpp:206-213)   x iters
//   k_xsph        velocity, vorticity, XSPH, reported density
//                 (particles.cpp:215-234, order-independent form)
//   k_vort        vorticity confinement, x <- x* (particles.cpp:236-248)
#include <cfloat>
#include <climits>
#include <cstdint>

#include "pbf_device.cuh"

namespace pbf {
namespace {

constexpr int kScanItems = 4;
constexpr int kScanThreads = 256;
constexpr int kScanTile = kScanItems * kScanThreads;
constexpr uint32_t kSmallCell = 32;       // cells up to this size: ranked slot by slot (k_cellrank)
constexpr uint32_t kMaxSortedCell = 4096;  // larger cells: rank sort by one block (in shared memory)
constexpr int kBigSortThreads = 256;
constexpr int kBigSortBlocks = 64;

__device__ __forceinline__ int scene_of_slot(const float4& p) { return __float_as_int(p.w); }

// Order-preserving unsigned image of a float (a total order, NaN included).
__device__ __forceinline__ uint32_t order_bits(float x) {
  const uint32_t u = __float_as_uint(x);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

// ---------------------------------------------------------------------------
// prediction + cell count
// ---------------------------------------------------------------------------
// REC (recording forward of the adjoint) also stores the collision record in disp.w.
template <bool REC>
__global__ void k_predict(const float4* __restrict__ pos, const float4* __restrict__ vel,
                          float4* __restrict__ disp_out, uint32_t* __restrict__ key_out,
                          uint32_t* __restrict__ xkey_out, uint32_t* __restrict__ rank_out,
                          uint32_t* __restrict__ cell_count,
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
      uint32_t code = 0u;
      collide<REC>(x, d, predict_delta(v4, P, dt), true, sc, P, &code);
      disp_out[i] = make_float4(d.x, d.y, d.z, REC ? __uint_as_float(code) : 0.f);
    }
    const float3 xp = x + d;  // x*, as k_gather forms it
    key = cell_key(cell_of(xp, sc, P.inv_cell), sc);
    key_out[i] = key;
    xkey_out[i] = order_bits(xp.x);
  }
  // per-cell rank, one atomic per run of equal keys among consecutive lanes (the slots are
  // still mostly in the cell order of the last step; measured 38 against 42 us a step for
  // one atomic per distinct key of the warp by __match_any_sync on scrambled cells). Dead
  // lanes carry the key 0xffffffff, a run of their own.
  const unsigned lane = lane_id();
  const uint32_t prev = __shfl_up_sync(0xffffffffu, key, 1);
  const bool head = lane == 0 || prev != key;
  const unsigned heads = __ballot_sync(0xffffffffu, head);
  const unsigned upto = lane == 31 ? 0xffffffffu : ((2u << lane) - 1u);  // lanes 0..lane
  const int start = 31 - __clz(heads & upto);                            // this lane's run head
  const unsigned above = heads & ~upto;
  const int next = above ? __ffs(above) - 1 : 32;                        // the next run's head
  uint32_t base = 0;
  if (head && live) base = atomicAdd(&cell_count[key], static_cast<uint32_t>(next - static_cast<int>(lane)));
  base = __shfl_sync(0xffffffffu, base, start);
  if (live) rank_out[i] = base + (lane - static_cast<unsigned>(start));
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

// Exclusive scan of the tile sums in place (carry over rounds of blockDim.x); start[m] =
// the total. zero_word (or null): a counter the following phases need at zero (the cell
// sort's worklist). The sums are read through L2: they may come from other blocks.
__device__ __forceinline__ void scan_tile_sums(uint32_t* __restrict__ tile_sum, uint32_t tiles,
                                               uint32_t* __restrict__ start, uint32_t m,
                                               uint32_t* __restrict__ zero_word) {
  if (zero_word && threadIdx.x == 0) *zero_word = 0u;
  uint32_t carry = 0;
  for (uint32_t b = 0; b < tiles; b += blockDim.x) {
    const uint32_t idx = b + threadIdx.x;
    const uint32_t v = idx < tiles ? __ldcg(&tile_sum[idx]) : 0u;
    uint32_t total;
    const uint32_t ex = block_exclusive_scan(v, &total);
    if (idx < tiles) tile_sum[idx] = carry + ex;
    carry += total;
  }
  if (threadIdx.x == 0) start[m] = carry;
}

// Scan of each tile of kScanTile counts. With a ticket (a zeroed word), the last block to
// finish also scans the tile sums (no block waits: each block counts itself in after its
// sum is visible, and the one that counts last does the work, then clears the ticket).
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const uint32_t* __restrict__ count,
                                                              uint32_t* __restrict__ start,
                                                              uint32_t* __restrict__ tile_sum,
                                                              uint32_t m, uint32_t* __restrict__ ticket,
                                                              uint32_t* __restrict__ zero_word) {
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
  if (!ticket) {
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
    return;
  }
  __shared__ bool last;
  if (threadIdx.x == 0) {
    tile_sum[blockIdx.x] = total;
    __threadfence();
    last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __threadfence();
  }
  __syncthreads();
  if (last) {
    scan_tile_sums(tile_sum, gridDim.x, start, m, zero_word);
    if (threadIdx.x == 0) *ticket = 0u;
  }
}

__global__ void __launch_bounds__(1024) k_scan_sums(uint32_t* __restrict__ tile_sum, uint32_t tiles,
                                                     uint32_t* __restrict__ start, uint32_t m,
                                                     uint32_t* __restrict__ zero_word) {
  scan_tile_sums(tile_sum, tiles, start, m, zero_word);
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

// Order each cell's slots by the x coordinate of x* (pos + disp, as k_gather forms it;
// pos for a resort), ties by original particle index: the cell order (hence every
// neighbour sum) is independent of atomic timing, and since cells along x are adjacent
// slot ranges, every row of cells is sorted by x, which lets the neighbour build stop a
// row at the first candidate beyond the reach. Cells up to kSmallCell particles are
// ranked by k_cellrank; larger ones go to a worklist for k_cellsort_big.
// The x keys (order_bits of x*.x) are written by k_predict, indexed by the pre-sort slot.
__device__ __forceinline__ uint64_t slot_order_key(const uint32_t* __restrict__ xkey, const uint32_t* __restrict__ id,
                                                   uint32_t v) {
  return (static_cast<uint64_t>(xkey[v]) << 32) | id[v];
}

// One thread per slot s of the scatter's (atomic) order: the entry moves to its cell's
// start plus its rank, the number of the cell's entries with a smaller key (keys are
// distinct). A cell's threads are neighbours, so its keys are read from L1. Cells over
// kSmallCell particles are copied in atomic order and listed for k_cellsort_big (their
// first slot's thread adds them).
__global__ void k_cellrank(const uint32_t* __restrict__ cell_start, const uint32_t* __restrict__ atomic_order,
                           const uint32_t* __restrict__ key, const uint32_t* __restrict__ xkey,
                           const uint32_t* __restrict__ id, uint32_t* __restrict__ perm,
                           uint32_t* __restrict__ big_cells, uint32_t* __restrict__ big_count, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t v = atomic_order[s];
  const uint32_t c = key[v];
  const uint32_t b = cell_start[c], e = cell_start[c + 1];
  if (e - b > kSmallCell) {
    perm[s] = v;
    if (static_cast<uint32_t>(s) == b) big_cells[atomicAdd(big_count, 1u)] = c;
    return;
  }
  const uint64_t kv = slot_order_key(xkey, id, v);
  uint32_t r = 0;
  for (uint32_t u = b; u < e; ++u) r += slot_order_key(xkey, id, atomic_order[u]) < kv ? 1u : 0u;
  perm[b + r] = v;
}

// Rank sort of the worklist's cells, one block per cell: the rank of an element is the
// number of the cell's elements with a smaller key (keys are distinct). Cells over
// kMaxSortedCell particles keep the atomic order (bounded time); such a cell makes its
// rows exceed kMaxRowCandidates, which the neighbour build reports as an error.
__global__ void __launch_bounds__(kBigSortThreads) k_cellsort_big(const uint32_t* __restrict__ cell_start,
                                                                 uint32_t* __restrict__ perm,
                                                                 const uint32_t* __restrict__ xkey,
                                                                 const uint32_t* __restrict__ id,
                                                                 const uint32_t* __restrict__ big_cells,
                                                                 const uint32_t* __restrict__ big_count) {
  __shared__ uint32_t slot[kMaxSortedCell];
  __shared__ uint32_t khi[kMaxSortedCell];
  __shared__ uint32_t klo[kMaxSortedCell];
  const uint32_t cnt = *big_count;
  for (uint32_t w = blockIdx.x; w < cnt; w += gridDim.x) {
    const uint32_t c = big_cells[w];
    const uint32_t b = cell_start[c], e = cell_start[c + 1];
    const uint32_t m = e - b;
    if (m > kMaxSortedCell) continue;  // uniform across the block
    for (uint32_t t = threadIdx.x; t < m; t += blockDim.x) {
      const uint32_t v = perm[b + t];
      const uint64_t k = slot_order_key(xkey, id, v);
      slot[t] = v;
      khi[t] = static_cast<uint32_t>(k >> 32);
      klo[t] = static_cast<uint32_t>(k);
    }
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < m; t += blockDim.x) {
      const uint32_t kh = khi[t], kl = klo[t];
      uint32_t r = 0;
      for (uint32_t u = 0; u < m; ++u) r += (khi[u] < kh || (khi[u] == kh && klo[u] < kl)) ? 1u : 0u;
      perm[b + r] = slot[t];
    }
    __syncthreads();
  }
}

__global__ void k_gather(const uint32_t* __restrict__ perm, const float4* __restrict__ pos_a,
                         const float4* __restrict__ disp_a, const float4* __restrict__ vel_a,
                         const uint32_t* __restrict__ id_a, float4* __restrict__ pos_b,
                         float4* __restrict__ disp_b, float4* __restrict__ xs_b,
                         float4* __restrict__ vel_b, uint32_t* __restrict__ id_b, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t i = perm[s];
  const float4 x = pos_a[i];
  pos_b[s] = x;
  id_b[s] = id_a[i];
  float rec = 0.f;
  if (disp_a) {
    const float4 d = disp_a[i];
    disp_b[s] = d;
    xs_b[s] = make_float4(x.x + d.x, x.y + d.y, x.z + d.z, 0.f);
    rec = d.w;
  }
  if (vel_a) {  // with disp_a (recording forward): w carries the prediction's collision record
    float4 v = vel_a[i];
    v.w = rec;
    vel_b[s] = v;
  }
}

// ---------------------------------------------------------------------------
// neighbour sets
// ---------------------------------------------------------------------------
// Each of the 9 candidate rows (3 z-slabs x 3 y-rows) is skipped when its cells lie
// beyond h in y/z, and otherwise trimmed in x to the cells that reach [x - w, x + w],
// w = sqrt(h^2 - d_yz^2): about 20 of the 27 cells on average. Within the trimmed row
// (sorted by x, see k_cellrank) only candidates with |dx| <= w are tested. All tests keep
// a margin of 1e-3 cell, far above the FP32 rounding of the cell binning and of the
// predicate, so no pair within h is dropped.
template <int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_nbr_build(const float4* __restrict__ xs,
                                                     const float4* __restrict__ pos,
                                                     const uint32_t* __restrict__ cell_start,
                                                     const SceneDesc* __restrict__ scenes,
                                                     uint4* __restrict__ hdr, uint32_t* __restrict__ words,
                                                     unsigned* __restrict__ err, DevParams P, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = xs[i];
  const SceneDesc& sc = scenes[scene_of_slot(pos[i])];
  const CellCoord cc = cell_of(f3(xi), sc, P.inv_cell);
  const int cap = P.max_words * 2;
  uint32_t gbase[3] = {0u, 0u, 0u};
  int total = 0;
  // List entries are stored one 16-bit half-word at a time: entry k of the slot is
  // half-word k % 8 of its group k / 8 (list_word's word k / 2, low half first), so an
  // append is one straight path with no word to assemble. (Pairing entries into words before
  // storing: 0.232 against 0.210 ms; collecting a group in registers or in shared memory and
  // storing it as one 16-byte write measured slower still: the appends run divergently, and
  // extra instructions and a smaller L1 cost more than coalesced stores save.)
  uint16_t* eptr = reinterpret_cast<uint16_t*>(words) + 8 * static_cast<size_t>(i);
  const size_t estep = 8 * static_cast<size_t>(n) - 7;
  unsigned flags = 0;
  // position inside the own cell, in cells, and the reach in cells with its margin
  const float fy = (xi.y - sc.origin[1]) * P.inv_cell - static_cast<float>(cc.y);
  const float fz = (xi.z - sc.origin[2]) * P.inv_cell - static_cast<float>(cc.z);
  const float m = 1e-3f;
  const float reach = sqrtf(P.h2) * P.inv_cell + m;
  const float reach2 = reach * reach;
  const float ux = (xi.x - sc.origin[0]) * P.inv_cell;
  const float cell_w = 1.0f / P.inv_cell;
  const int y0 = cc.y > 0 ? cc.y - 1 : 0;
  const float2 nxy = make_float2(-xi.x, -xi.y);
  const float nz = -xi.z;
#pragma unroll
  for (int g = 0; g < 3; ++g) {
    const int z = cc.z + g - 1;
    if (z < 0 || z >= sc.dim[2]) continue;
    const uint32_t slab = sc.cell_off + static_cast<uint32_t>(z * sc.dim[1] * sc.dim[0]);
    const int x0 = cc.x > 0 ? cc.x - 1 : 0;
    gbase[g] = __ldg(&cell_start[slab + static_cast<uint32_t>(y0 * sc.dim[0] + x0)]);
    const float dz = g == 0 ? fmaxf(fz - m, 0.f) : (g == 2 ? fmaxf(1.f - fz - m, 0.f) : 0.f);
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      const int y = cc.y + r - 1;
      if (y < 0 || y >= sc.dim[1]) continue;
      const float dy = r == 0 ? fmaxf(fy - m, 0.f) : (r == 2 ? fmaxf(1.f - fy - m, 0.f) : 0.f);
      const float w2 = reach2 - (dy * dy + dz * dz);
      if (w2 < 0.f) continue;
      const float w = sqrtf(w2);
      const int xa = max(max(static_cast<int>(floorf(ux - w)), cc.x - 1), 0);
      const int xb = min(min(static_cast<int>(floorf(ux + w)), cc.x + 1), sc.dim[0] - 1);
      if (xa > xb) continue;
      const uint32_t row = slab + static_cast<uint32_t>(y * sc.dim[0]);
      const uint32_t start = __ldg(&cell_start[row + xa]);
      uint32_t end = __ldg(&cell_start[row + xb + 1]);
      if (end - start > static_cast<uint32_t>(kMaxRowCandidates)) {
        flags |= PBF_ERRBIT_ROW_CAPACITY;
        end = start + kMaxRowCandidates;
      }
      const uint32_t gb = gbase[g];
      const uint32_t gbits = static_cast<uint32_t>(g) << kOffsetBits;
      // the row is sorted by x: a binary search over the window's first cell (the only
      // one reaching below x - W) finds the first candidate at or above x - W, and the
      // first one above x + W ends the row (W = w cells, margin included; with NaN
      // coordinates in the cell the search may start early, never late). The predicate
      // reuses the x difference: the same roundings as dist2_rn. The own slot is a hit at
      // distance 0 and is dropped there, which keeps one loop per row (two half-row loops
      // around it: 0.209 against 0.206 ms; one loop over a slab's three rows, lanes moving
      // on to the next row when theirs ends: 0.243 against 0.234 ms, 48 registers).
      const uint32_t ui = static_cast<uint32_t>(i);
      const float W = w * cell_w;
      const uint32_t first_end = __ldg(&cell_start[row + xa + 1]);
      uint32_t a = start, hi = min(end, first_end);
      while (a < hi) {
        const uint32_t md = (a + hi) >> 1;
        if (__ldg(&xs[md].x) - xi.x < -W) a = md + 1; else hi = md;
      }
      for (uint32_t j = a; j < end; ++j) {
        const float4 xj = __ldg(&xs[j]);
        // x and y of x*_j - x*_i as one packed FP32x2 add against -x*_i (negation is
        // exact: the same roundings as x*_i - x*_j up to sign) and one packed square
        const float2 dxy = __fadd2_rn(make_float2(xj.x, xj.y), nxy);
        if (dxy.x > W) break;
        const float2 sq = __fmul2_rn(dxy, dxy);
        const float dz = __fadd_rn(xj.z, nz);
        if (__fadd_rn(__fadd_rn(sq.x, sq.y), __fmul_rn(dz, dz)) <= P.h2 && j != ui) {
          const uint32_t off = j - gb;
          if (off <= kOffsetMask && total < cap) {
            *eptr = static_cast<uint16_t>(gbits | off);
            eptr += ((total & 7) == 7) ? estep : 1;
            ++total;
          } else {
            flags |= off > kOffsetMask ? PBF_ERRBIT_ROW_CAPACITY : PBF_ERRBIT_NEIGHBOR_CAPACITY;
          }
        }
      }
    }
  }
  // the slab bases relative to slab 0's, less the tag bits (nbr_decode)
  hdr[i] = make_uint4(gbase[0], gbase[1] - gbase[0] - (1u << kOffsetBits),
                      gbase[2] - gbase[0] - (2u << kOffsetBits), static_cast<uint32_t>(total));
  if (flags) atomicOr(err, flags);
}

// ---------------------------------------------------------------------------
// Jacobi density-constraint iterations
// ---------------------------------------------------------------------------
// lambda_i is stored in x*_i.w of the same buffer: within this pass every
// thread reads only .xyz of its neighbours' x*, which no thread writes.
template <int BLOCK, int D, bool ST>
__global__ void __launch_bounds__(BLOCK) k_lambda(float4* xs, const uint4* __restrict__ hdr,
                                                  const uint32_t* __restrict__ words,
                                                  float* __restrict__ rho_iter0,
                                                  DevParams P, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = xs[i];
  float qsum = 0.f, g2 = 0.f;
  float3 gs = make_float3(0.f, 0.f, 0.f);
  // D gathers in flight: this pass is bound by the latency of the neighbour loads
  for_each_neighbor_pf<D, Decode::kBits, ST>(i, n, ld_hdr<ST>(&hdr[i]), words,
                                              [&](uint32_t j) -> float4 { return xs[j]; },
                                              [&](uint32_t, const float4& xj) {
    const Pair p = pair_of(xi, xj, P.h, P.h2);
    qsum = __fmaf_rn(__fmul_rn(p.q, p.q), p.q, qsum);
    gs = fma3(p.r, p.s, gs);
    g2 = __fmaf_rn(__fmul_rn(p.s, p.s), p.r2, g2);
  });
  const float rho = __fmul_rn(P.poly6_c, qsum);
  const float kg = __fmul_rn(P.spiky_c, P.inv_rho0);
  const float denom = __fmaf_rn(__fmul_rn(kg, kg), __fadd_rn(g2, dot3_rn(gs, gs)), P.epsilon);
  const float l = -__fdiv_rn(__fmaf_rn(rho, P.inv_rho0, -1.0f), denom);
  reinterpret_cast<float*>(xs)[4 * i + 3] = l;
  if (rho_iter0) rho_iter0[i] = rho;
}

// (lambda_i + lambda_j + s_corr) grad W summed over neighbours; N4 specialises the
// tensile exponent N = 4 of particles.cpp:40. REC (recording forward of the adjoint)
// also stores the requested displacement and the collision record in dp_rec. MESH =
// false (no collider triangles) leaves the triangle tests out of the collision: 40
// registers a thread instead of 55.
template <int BLOCK, bool N4, bool REC, bool MESH, int D, bool ST>
__global__ void __launch_bounds__(BLOCK) k_deltap(const float4* __restrict__ xs,
                                                  const float4* __restrict__ pos,
                                                  const uint4* __restrict__ hdr,
                                                  const uint32_t* __restrict__ words,
                                                  const SceneDesc* __restrict__ scenes,
                                                  float4* __restrict__ disp, float4* __restrict__ xs_next,
                                                  float4* __restrict__ dp_rec, DevParams P, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = xs[i];
  const float li = xi.w;  // lambda_i (k_lambda stores it in x*.w)
  const float wt = P.poly6_c * P.tis;
  float3 dp = make_float3(0.f, 0.f, 0.f);
  for_each_neighbor_pf<D, Decode::kBits, ST>(i, n, ld_hdr<ST>(&hdr[i]), words,
                                              [&](uint32_t j) -> float4 { return __ldg(&xs[j]); },
                                              [&](uint32_t, const float4& xj) {
    const Pair p = pair_of(xi, xj, P.h, P.h2);
    const float a = __fmul_rn(wt, __fmul_rn(__fmul_rn(p.q, p.q), p.q));  // W / W(dq)
    float an;
    if (N4) {
      const float a2 = __fmul_rn(a, a);
      an = __fmul_rn(a2, a2);
    } else {
      an = a;
      for (int e = 1; e < P.scorr_n; ++e) an = __fmul_rn(an, a);
    }
    const float coef = __fmaf_rn(-P.scorr_k, an, __fadd_rn(li, xj.w));  // lambda_i + lambda_j + s_corr
    dp = fma3(p.r, __fmul_rn(coef, p.s), dp);
  });
  const float sc_dp = __fmul_rn(P.spiky_c, P.inv_rho0);
  dp = make_float3(__fmul_rn(dp.x, sc_dp), __fmul_rn(dp.y, sc_dp), __fmul_rn(dp.z, sc_dp));
  const float4 x4 = pos[i];
  const SceneDesc& sc = scenes[scene_of_slot(x4)];
  const float4 d4 = disp[i];
  float3 d = f3(d4);
  const float3 x = f3(x4);
  uint32_t code = 0u;
  collide<REC, MESH>(x, d, dp, false, sc, P, &code);
  if (REC) dp_rec[i] = make_float4(dp.x, dp.y, dp.z, __uint_as_float(code));
  disp[i] = make_float4(d.x, d.y, d.z, 0.f);
  xs_next[i] = make_float4(x.x + d.x, x.y + d.y, x.z + d.z, 0.f);
}

// ---------------------------------------------------------------------------
// velocity, vorticity, XSPH, reported density; then vorticity confinement
// ---------------------------------------------------------------------------
// |omega_i| is stored in x*_i.w of the same buffer (neighbours read only .xyz here).
template <int BLOCK, int D, bool ST>
__global__ void __launch_bounds__(BLOCK) k_xsph(float4* xs, const float4* __restrict__ disp,
                                                const uint4* __restrict__ hdr,
                                                const uint32_t* __restrict__ words,
                                                float4* __restrict__ vel_out, float4* __restrict__ omega,
                                                float* __restrict__ rho_out, DevParams P, float inv_dt,
                                                int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = xs[i];
  const float3 vi = f3(disp[i]) * inv_dt;  // updateVelocity, particles.cpp:215-217
  float qsum = 0.f;
  float3 visc = make_float3(0.f, 0.f, 0.f), w = make_float3(0.f, 0.f, 0.f);
  struct XD {
    float4 x, d;
  };
  for_each_neighbor_pf<D, Decode::kBits, ST>(
      i, n, ld_hdr<ST>(&hdr[i]), words, [&](uint32_t j) { return XD{xs[j], __ldg(&disp[j])}; },
      [&](uint32_t, const XD& a) {
    const Pair p = pair_of(xi, a.x, P.h, P.h2);
    const float3 vij = make_float3(__fmaf_rn(a.d.x, inv_dt, -vi.x), __fmaf_rn(a.d.y, inv_dt, -vi.y),
                                   __fmaf_rn(a.d.z, inv_dt, -vi.z));
    const float q3 = __fmul_rn(__fmul_rn(p.q, p.q), p.q);
    visc = fma3(vij, q3, visc);
    qsum = __fadd_rn(qsum, q3);
    const float3 rs = make_float3(__fmul_rn(p.r.x, p.s), __fmul_rn(p.r.y, p.s), __fmul_rn(p.r.z, p.s));
    w = make_float3(__fadd_rn(w.x, __fmaf_rn(vij.y, rs.z, -__fmul_rn(vij.z, rs.y))),
                    __fadd_rn(w.y, __fmaf_rn(vij.z, rs.x, -__fmul_rn(vij.x, rs.z))),
                    __fadd_rn(w.z, __fmaf_rn(vij.x, rs.y, -__fmul_rn(vij.y, rs.x))));
  });
  const float rho = __fmul_rn(P.poly6_c, qsum);
  w = make_float3(__fmul_rn(w.x, P.spiky_c), __fmul_rn(w.y, P.spiky_c), __fmul_rn(w.z, P.spiky_c));
  const float3 v = fma3(visc, __fmul_rn(P.xsph_c, P.poly6_c), vi);
  vel_out[i] = make_float4(v.x, v.y, v.z, 0.f);
  const float wn = __fsqrt_rn(dot3_rn(w, w));
  omega[i] = make_float4(w.x, w.y, w.z, wn);
  reinterpret_cast<float*>(xs)[4 * i + 3] = wn;
  rho_out[i] = rho;
}

template <int BLOCK, int D, bool ST>
__global__ void __launch_bounds__(BLOCK) k_vort(const float4* __restrict__ xs,
                                                float4* __restrict__ pos,
                                                const float4* __restrict__ omega,
                                                const uint4* __restrict__ hdr,
                                                const uint32_t* __restrict__ words,
                                                float4* __restrict__ vel, unsigned* __restrict__ err,
                                                float4* __restrict__ eta_rec, DevParams P, float dt, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float4 xi = xs[i];
  float3 eta = make_float3(0.f, 0.f, 0.f);
  for_each_neighbor_pf<D, Decode::kBits, ST>(i, n, ld_hdr<ST>(&hdr[i]), words,
                                              [&](uint32_t j) -> float4 { return __ldg(&xs[j]); },
                                              [&](uint32_t, const float4& xj) {
    const Pair p = pair_of<true>(xi, xj, P.h, P.h2);
    eta = fma3(p.r, __fmul_rn(xj.w, p.s), eta);  // |omega_j| (k_xsph stores it in x*.w)
  });
  eta = make_float3(__fmul_rn(eta.x, P.spiky_c), __fmul_rn(eta.y, P.spiky_c), __fmul_rn(eta.z, P.spiky_c));
  if (eta_rec) eta_rec[i] = make_float4(eta.x, eta.y, eta.z, 0.f);  // recording forward of the adjoint
  float3 v = f3(vel[i]);
  const float en = __fsqrt_rn(dot3_rn(eta, eta));
  if (en > kEps) {
    const float4 wi = omega[i];
    const float ie = __fdiv_rn(1.0f, en);
    const float3 nh = make_float3(__fmul_rn(eta.x, ie), __fmul_rn(eta.y, ie), __fmul_rn(eta.z, ie));
    const float3 c = make_float3(__fmaf_rn(nh.y, wi.z, -__fmul_rn(nh.z, wi.y)),
                                 __fmaf_rn(nh.z, wi.x, -__fmul_rn(nh.x, wi.z)),
                                 __fmaf_rn(nh.x, wi.y, -__fmul_rn(nh.y, wi.x)));
    v = fma3(c, __fmul_rn(dt, P.vort_eps), v);
  }
  const float4 p4 = pos[i];
  vel[i] = make_float4(v.x, v.y, v.z, 0.f);
  pos[i] = make_float4(xi.x, xi.y, xi.z, p4.w);  // updatePosition, particles.cpp:246-248
  if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(xi.x) && isfinite(xi.y) &&
        isfinite(xi.z)))
    atomicOr(err, PBF_ERRBIT_NONFINITE);
}

// Step statistics (the prints of particles.cpp:267-295 and the neighbour
// alert of :168-172, as numbers): one pass over densities and list headers, reduced in
// a fixed shape (kStatsBlocks partial records, then one block), so the sums are
// deterministic and no block contends on an atomic.

__device__ __forceinline__ void stats_merge(DevStats& a, const DevStats& b) {
  a.rho_sum += b.rho_sum;
  a.rho_iter0_sum += b.rho_iter0_sum;
  a.err_sum += b.err_sum;
  a.err_max_bits = max(a.err_max_bits, b.err_max_bits);  // non-negative floats order as their bits
  a.nbr_min = min(a.nbr_min, b.nbr_min);
  a.nbr_max = max(a.nbr_max, b.nbr_max);
  a.nbr_sum += b.nbr_sum;
  a.low_cnt += b.low_cnt;
}

__device__ __forceinline__ DevStats stats_shfl_down(const DevStats& a, int o) {
  DevStats b;
  b.rho_sum = __shfl_down_sync(0xffffffffu, a.rho_sum, o);
  b.rho_iter0_sum = __shfl_down_sync(0xffffffffu, a.rho_iter0_sum, o);
  b.err_sum = __shfl_down_sync(0xffffffffu, a.err_sum, o);
  b.err_max_bits = __shfl_down_sync(0xffffffffu, a.err_max_bits, o);
  b.nbr_min = __shfl_down_sync(0xffffffffu, a.nbr_min, o);
  b.nbr_max = __shfl_down_sync(0xffffffffu, a.nbr_max, o);
  b.nbr_sum = __shfl_down_sync(0xffffffffu, a.nbr_sum, o);
  b.low_cnt = __shfl_down_sync(0xffffffffu, a.low_cnt, o);
  return b;
}

// Reduces the block's records into thread 0 (blockDim.x a multiple of 32, at most 1024).
__device__ __forceinline__ DevStats stats_block_reduce(DevStats a) {
  __shared__ DevStats sw[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) stats_merge(a, stats_shfl_down(a, o));
  const unsigned w = threadIdx.x >> 5;
  if (lane_id() == 0) sw[w] = a;
  __syncthreads();
  if (threadIdx.x == 0)
    for (unsigned k = 1; k < (blockDim.x >> 5); ++k) stats_merge(a, sw[k]);
  return a;
}

__device__ __forceinline__ DevStats stats_zero() {
  DevStats a;
  a.rho_sum = a.rho_iter0_sum = a.err_sum = 0.0;
  a.err_max_bits = 0u;
  a.nbr_min = 0xffffffffu;
  a.nbr_max = 0u;
  a.pad = 0u;
  a.nbr_sum = a.low_cnt = 0ull;
  return a;
}

// Each thread takes 4 consecutive particles per turn (vector loads of the densities, the
// 4 list headers issued together) and sums its share (about 16 particles at 1M) in FP32;
// the partial sums join in FP64 from the warp level up. FP64 adds per particle would
// bound the kernel: FP64 throughput on this part is a small fraction of FP32's.
struct StatsAcc {
  float rho, rho0, err, err_max;
  unsigned nmin, nmax, nsum, low;
};

__device__ __forceinline__ void stats_add(StatsAcc& a, float x, float x0, unsigned c, float inv_rho0) {
  a.rho += x;
  a.rho0 += x0;
  const float e = fabsf(x * inv_rho0 - 1.0f);
  a.err += e;
  a.err_max = fmaxf(a.err_max, e);
  a.nmin = min(a.nmin, c);
  a.nmax = max(a.nmax, c);
  a.nsum += c;
  a.low += c < static_cast<unsigned>(kNeighborAlert) ? 1u : 0u;
}

__global__ void __launch_bounds__(256) k_stats(const float* __restrict__ rho, const float* __restrict__ rho0,
                                               const uint4* __restrict__ hdr, DevStats* __restrict__ part,
                                               float inv_rho0, int n) {
  StatsAcc s{0.f, 0.f, 0.f, 0.f, 0xffffffffu, 0u, 0u, 0u};
  const int n4 = n / 4;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n4; k += gridDim.x * blockDim.x) {
    const float4 x = reinterpret_cast<const float4*>(rho)[k];
    const float4 x0 = reinterpret_cast<const float4*>(rho0)[k];
    const uint4 h0 = hdr[4 * k], h1 = hdr[4 * k + 1], h2 = hdr[4 * k + 2], h3 = hdr[4 * k + 3];
    stats_add(s, x.x, x0.x, h0.w, inv_rho0);
    stats_add(s, x.y, x0.y, h1.w, inv_rho0);
    stats_add(s, x.z, x0.z, h2.w, inv_rho0);
    stats_add(s, x.w, x0.w, h3.w, inv_rho0);
  }
  const int t = 4 * n4 + blockIdx.x * blockDim.x + threadIdx.x;  // the last n % 4 particles
  if (t < n) stats_add(s, rho[t], rho0[t], static_cast<unsigned>(nbr_total(hdr[t])), inv_rho0);
  DevStats a = stats_zero();
  a.rho_sum = s.rho;
  a.rho_iter0_sum = s.rho0;
  a.err_sum = s.err;
  a.err_max_bits = __float_as_uint(s.err_max);
  a.nbr_min = s.nmin;
  a.nbr_max = s.nmax;
  a.nbr_sum = s.nsum;
  a.low_cnt = s.low;
  a = stats_block_reduce(a);
  if (threadIdx.x == 0) part[blockIdx.x] = a;
}

__global__ void __launch_bounds__(kStatsBlocks) k_stats_final(const DevStats* __restrict__ part,
                                                              DevStats* __restrict__ st) {
  DevStats a = part[threadIdx.x];
  a = stats_block_reduce(a);
  if (threadIdx.x == 0) *st = a;
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

__global__ void k_nbr_counts(const uint4* __restrict__ hdr, const uint32_t* __restrict__ id,
                             uint32_t* __restrict__ counts, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s < n) counts[id[s]] = static_cast<uint32_t>(nbr_total(hdr[s]));
}

// ids[offsets[id[i]] ...] = original ids of i's neighbours (cell order).
__global__ void k_nbr_ids(const uint4* __restrict__ hdr, const uint32_t* __restrict__ words,
                          const uint32_t* __restrict__ id, const uint32_t* __restrict__ offsets,
                          uint32_t* __restrict__ ids, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint32_t o = offsets[id[i]];
  for_each_neighbor(i, n, hdr[i], words, [&](uint32_t j) { ids[o++] = id[j]; });
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
  out[q] = density_at_point(make_float3(pts[3 * q], pts[3 * q + 1], pts[3 * q + 2]), pos, cell_start, scenes[0], P);
}

inline unsigned blocks_for(size_t n, int block) { return static_cast<unsigned>((n + block - 1) / block); }

// Launches neighbour kernel KERN (a template-id, parenthesised) over n particles, BLOCK threads a block.
#define PBF_PASS_LAUNCH(KERN, ...) KERN<<<blocks_for(n, BLOCK), BLOCK, 0, s>>>(__VA_ARGS__)

// Instantiates a neighbour pass for the tuned gather depth (D = 4 or 8 neighbour loads in
// flight per thread) and list-load policy (ST: streaming). Neither changes the order in
// which a particle's neighbours are summed, so every form gives the same bits.
#define PBF_FORM_SWITCH(depth, stream, ...)                                          \
  if ((depth) == 4) {                                                                \
    if (stream) { constexpr int D = 4; constexpr bool ST = true; __VA_ARGS__; }      \
    else { constexpr int D = 4; constexpr bool ST = false; __VA_ARGS__; }            \
  } else {                                                                           \
    if (stream) { constexpr int D = 8; constexpr bool ST = true; __VA_ARGS__; }      \
    else { constexpr int D = 8; constexpr bool ST = false; __VA_ARGS__; }            \
  }

// One delta-p pass (B = the buffer index holding this step's cell-ordered x and delta).
// The recording forward of the adjoint keeps the default form (8 deep, cached lists).
template <bool N4, bool REC, bool MESH>
void launch_deltap(const Tuning& t, const Buffers& b, int B, float4* xcur, float4* xnext, float4* dprec,
                   const DevParams& P, int n, cudaStream_t s) {
  if (REC) {
    PBF_BLOCK_SWITCH(t.block_solve,
                     PBF_PASS_LAUNCH((k_deltap<BLOCK, N4, REC, MESH, 8, false>), xcur, b.pos[B], b.nbr_hdr,
                                     b.nbr_w, b.scenes, b.disp[1], xnext, dprec, P, n));
    return;
  }
  PBF_FORM_SWITCH(t.gather_depth, t.list_stream,
                  PBF_BLOCK_SWITCH(t.block_solve,
                                   PBF_PASS_LAUNCH((k_deltap<BLOCK, N4, REC, MESH, D, ST>), xcur, b.pos[B],
                                                   b.nbr_hdr, b.nbr_w, b.scenes, b.disp[1], xnext, dprec, P, n)));
}

// Shared front half of a step and of a resort: keys, counts, scan, slots.
cudaError_t sort_into_cells(const Buffers& b, const DevParams& P, const Tuning& t, int cur, float dt,
                            bool move, cudaStream_t s, PhaseMarks* mk = nullptr, bool rec = false) {
  const int n = static_cast<int>(b.n);
  const uint32_t m = b.n_cells;
  cudaError_t e = cudaMemsetAsync(b.cell_count, 0, sizeof(uint32_t) * m, s);
  if (e != cudaSuccess) return e;
  if (rec)
    k_predict<true><<<blocks_for(n, t.block_predict), t.block_predict, 0, s>>>(
        b.pos[cur], b.vel[cur], b.disp[0], b.key, b.xkey, b.rank, b.cell_count, b.scenes, P, dt, move ? 1 : 0, n);
  else
    k_predict<false><<<blocks_for(n, t.block_predict), t.block_predict, 0, s>>>(
        b.pos[cur], b.vel[cur], b.disp[0], b.key, b.xkey, b.rank, b.cell_count, b.scenes, P, dt, move ? 1 : 0, n);
  if (mk) mk->mark(kPhasePredict, s);
  const uint32_t tiles = (m + kScanTile - 1) / kScanTile;
  // scan_tmp holds the tile sums and, after them, the ticket of k_scan_tiles' last block
  k_scan_tiles<<<tiles, kScanThreads, 0, s>>>(b.cell_count, b.cell_start, b.scan_tmp, m, b.scan_tmp + tiles,
                                               b.big_count);
  k_scan_add<<<tiles, kScanThreads, 0, s>>>(b.cell_start, b.scan_tmp, m);
  if (mk) mk->mark(kPhaseScan, s);
  k_scatter<<<blocks_for(n, t.block_misc), t.block_misc, 0, s>>>(b.key, b.rank, b.cell_start, b.perm_atomic, n);
  k_cellrank<<<blocks_for(n, t.block_misc), t.block_misc, 0, s>>>(b.cell_start, b.perm_atomic, b.key, b.xkey,
                                                                   b.id[cur], b.perm, b.big_cells, b.big_count, n);
  k_cellsort_big<<<kBigSortBlocks, kBigSortThreads, 0, s>>>(b.cell_start, b.perm, b.xkey, b.id[cur], b.big_cells,
                                                             b.big_count);
  if (mk) mk->mark(kPhaseSort, s);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_step(const Buffers& b, const DevParams& P, const Tuning& t, int cur, float dt,
                        int iters, bool keep_pred, cudaStream_t s, PhaseMarks* mk, const Tape* tape) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  const int A = cur, B = 1 - cur;
  const bool rec = tape != nullptr;
  if (mk) mk->mark(-1, s);
  cudaError_t e = sort_into_cells(b, P, t, A, dt, true, s, mk, rec);
  if (e != cudaSuccess) return e;
  float4* xs0 = rec ? tape->xs : b.xs[0];
  k_gather<<<blocks_for(n, t.block_misc), t.block_misc, 0, s>>>(
      b.perm, b.pos[A], b.disp[0], rec ? b.vel[A] : nullptr, b.id[A], b.pos[B], b.disp[1], xs0,
      rec ? tape->v : nullptr, b.id[B], n);
  if (rec) {
    e = cudaMemcpyAsync(tape->x, b.pos[B], sizeof(float4) * b.n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  if (keep_pred && b.pred) {
    e = cudaMemcpyAsync(b.pred, xs0, sizeof(float4) * b.n, cudaMemcpyDeviceToDevice, s);
    if (e != cudaSuccess) return e;
  }
  if (mk) mk->mark(kPhaseGather, s);
  PBF_BLOCK_SWITCH(t.block_nbr, PBF_PASS_LAUNCH(k_nbr_build<BLOCK>, xs0, b.pos[B], b.cell_start, b.scenes,
                                                b.nbr_hdr, b.nbr_w, b.err, P, n));
  if (mk) mk->mark(kPhaseNeighbors, s);
  for (int it = 0; it < iters; ++it) {
    float4* xcur = rec ? tape->xs + static_cast<size_t>(it) * b.n : b.xs[it & 1];
    float4* xnext = rec ? tape->xs + static_cast<size_t>(it + 1) * b.n : b.xs[(it + 1) & 1];
    float4* dprec = rec ? tape->dp + static_cast<size_t>(it) * b.n : nullptr;
    PBF_FORM_SWITCH(t.gather_depth, t.list_stream,
                    PBF_BLOCK_SWITCH(t.block_solve,
                                     PBF_PASS_LAUNCH((k_lambda<BLOCK, D, ST>), xcur, b.nbr_hdr,
                                                     b.nbr_w, (it == 0 && P.stats) ? b.rho_iter0 : nullptr, P,
                                                     n)));
    if (mk) mk->mark(kPhaseLambda, s);
    const bool n4 = P.scorr_n == 4, mesh = P.n_mesh > 0 || P.n_sph > 0;
    if (rec) {  // the adjoint takes box colliders only; the recording keeps the general form
      if (n4) launch_deltap<true, true, true>(t, b, B, xcur, xnext, dprec, P, n, s);
      else launch_deltap<false, true, true>(t, b, B, xcur, xnext, dprec, P, n, s);
    } else if (n4) {
      if (mesh) launch_deltap<true, false, true>(t, b, B, xcur, xnext, nullptr, P, n, s);
      else launch_deltap<true, false, false>(t, b, B, xcur, xnext, nullptr, P, n, s);
    } else {
      if (mesh) launch_deltap<false, false, true>(t, b, B, xcur, xnext, nullptr, P, n, s);
      else launch_deltap<false, false, false>(t, b, B, xcur, xnext, nullptr, P, n, s);
    }
    if (mk) mk->mark(kPhaseDeltaP, s);
  }
  float4* fin = rec ? tape->xs + static_cast<size_t>(iters) * b.n : b.xs[iters & 1];
  PBF_FORM_SWITCH(t.gather_depth, t.list_stream,
                  PBF_BLOCK_SWITCH(t.block_solve,
                                   PBF_PASS_LAUNCH((k_xsph<BLOCK, D, ST>), fin, b.disp[1],
                                                   b.nbr_hdr, b.nbr_w, b.vel[B], b.omega, b.rho, P, 1.0f / dt, n)));
  if (mk) mk->mark(kPhaseXsph, s);
  PBF_FORM_SWITCH(t.gather_depth, t.list_stream,
                  PBF_BLOCK_SWITCH(t.block_solve,
                                   PBF_PASS_LAUNCH((k_vort<BLOCK, D, ST>), fin, b.pos[B], b.omega,
                                                   b.nbr_hdr, b.nbr_w, b.vel[B], b.err, rec ? tape->eta : nullptr,
                                                   P, dt, n)));
  if (mk) mk->mark(kPhaseVorticity, s);
  if (P.stats) {
    k_stats<<<kStatsBlocks, 256, 0, s>>>(b.rho, b.rho_iter0, b.nbr_hdr, b.stats_part, P.inv_rho0, n);
    k_stats_final<<<1, kStatsBlocks, 0, s>>>(b.stats_part, b.stats);
  }
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
      b.perm, b.pos[cur], nullptr, b.vel[cur], b.id[cur], b.pos[1 - cur], nullptr, nullptr, b.vel[1 - cur],
      b.id[1 - cur], n);
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
  k_nbr_counts<<<blocks_for(n, 256), 256, 0, s>>>(b.nbr_hdr, b.id[cur], counts, n);
  return cudaGetLastError();
}

cudaError_t launch_neighbor_ids(const Buffers& b, int cur, const uint32_t* offsets, uint32_t* ids,
                                cudaStream_t s) {
  const int n = static_cast<int>(b.n);
  if (n == 0) return cudaSuccess;
  k_nbr_ids<<<blocks_for(n, 256), 256, 0, s>>>(b.nbr_hdr, b.nbr_w, b.id[cur], offsets, ids, n);
  return cudaGetLastError();
}

cudaError_t launch_exclusive_scan(const uint32_t* count, uint32_t* start, uint32_t* tile_sums, uint32_t m,
                                  cudaStream_t s) {
  const uint32_t tiles = (m + kScanTile - 1) / kScanTile;
  k_scan_tiles<<<tiles, kScanThreads, 0, s>>>(count, start, tile_sums, m, nullptr, nullptr);
  k_scan_sums<<<1, 1024, 0, s>>>(tile_sums, tiles, start, m, nullptr);
  k_scan_add<<<tiles, kScanThreads, 0, s>>>(start, tile_sums, m);
  return cudaGetLastError();
}

uint32_t exclusive_scan_tiles(uint32_t m) { return (m + kScanTile - 1) / kScanTile; }

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
