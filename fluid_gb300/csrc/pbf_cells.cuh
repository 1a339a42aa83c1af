// Cell-cooperative neighbour build and neighbour passes.
//
// Work decomposition: warp w owns the cells whose first slot lies in slots
// [32w, 32w+32) of the cell-sorted arrays and processes them one at a time.
// For a cell the warp enumerates its candidate rows -- the 9 (dz, dy) rows of
// cells cx-1..cx+1 around it, each a contiguous slot range -- and stages the
// candidates' data into the warp's shared memory with coalesced loads. A
// neighbour is stored as the u16 index of the candidate in that enumeration,
// so every pass re-stages the same enumeration and reads neighbours from
// shared memory instead of gathering them from global memory.
//
//   build:  lanes = candidates, a warp-uniform loop over the cell's particles,
//           ballot/popc compaction of each particle's hits (ascending order),
//           then lambda of the first Jacobi iteration from the staged data.
//   passes: L lanes per particle (L = 4, 2, 1 for cells of <= 8, <= 16, more
//           particles), each lane a strided share of the particle's list, then
//           a shuffle reduction.
// Cells with more candidates than fit (kCandMax) or, for the build, more
// particles than kBuildM, take a per-particle path with global loads.
#pragma once

#include "pbf_device.cuh"

namespace pbf {

constexpr int kCandMax = 384;    // staged candidates per cell (27 cells x ~14)
constexpr int kBuildM = 16;      // particles per cell on the build's fast path
constexpr int kBuildCap = 96;    // neighbours per particle buffered by the build's fast path

struct CellRows {
  uint32_t start[9];  // first slot of each candidate row
  uint32_t pref[10];  // exclusive prefix of the row lengths; pref[9] = candidates
};

// Per-warp shared-memory footprint of the kernels (bytes, 16-byte multiples).
constexpr int kRowsBytes = 80;
constexpr int kBuildWarpBytes = kCandMax * 16 + kBuildM * kBuildCap * 2 + 32 * 4 + kRowsBytes;
constexpr int kPassWarpBytes = kCandMax * 16 + kRowsBytes;
constexpr int kPass2WarpBytes = 2 * kCandMax * 16 + kRowsBytes;

__device__ __forceinline__ unsigned lanemask_lt_() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

struct CellInfo {
  uint32_t cs, m;   // first slot, particle count
  uint32_t self0;   // candidate index of the cell's first particle
  int sid;
};

// Candidate rows of cell `key` into rows (warp-cooperative; lanes 0..8 compute,
// all lanes see the result after the internal __syncwarp). Row lengths above
// kMaxRowCandidates are capped and flagged.
__device__ __forceinline__ void cell_rows(uint32_t key, const SceneDesc& sc,
                                          const uint32_t* __restrict__ cell_start, CellRows* rows,
                                          unsigned* flags) {
  const unsigned lane = lane_id();
  const uint32_t local = key - sc.cell_off;
  const int nx = sc.dim[0], ny = sc.dim[1], nz = sc.dim[2];
  const int cx = static_cast<int>(local % nx);
  const int cy = static_cast<int>((local / nx) % ny);
  const int cz = static_cast<int>(local / (nx * ny));
  uint32_t start = 0, len = 0;
  if (lane < 9) {
    const int z = cz + static_cast<int>(lane) / 3 - 1, y = cy + static_cast<int>(lane) % 3 - 1;
    if (z >= 0 && z < nz && y >= 0 && y < ny) {
      const int x0 = cx > 0 ? cx - 1 : 0;
      const int x1 = cx + 1 < nx ? cx + 1 : nx - 1;
      const uint32_t row = sc.cell_off + static_cast<uint32_t>((z * ny + y) * nx);
      start = __ldg(&cell_start[row + x0]);
      len = __ldg(&cell_start[row + x1 + 1]) - start;
      if (len > static_cast<uint32_t>(kMaxRowCandidates)) {
        len = kMaxRowCandidates;
        *flags |= PBF_ERRBIT_ROW_CAPACITY;
      }
    }
  }
  // exclusive scan of len over lanes 0..8
  uint32_t x = len;
#pragma unroll
  for (int o = 1; o < 16; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= static_cast<unsigned>(o)) x += y;
  }
  if (lane < 9) {
    rows->start[lane] = start;
    rows->pref[lane] = x - len;
  }
  if (lane == 8) rows->pref[9] = x;
  __syncwarp();
}

// Slot of candidate t (per-particle paths; rows in shared memory).
__device__ __forceinline__ uint32_t cand_slot(const CellRows* rows, uint32_t t) {
  int r = 0;
#pragma unroll
  for (int k = 1; k < 9; ++k) r += (t >= rows->pref[k]) ? 1 : 0;
  return rows->start[r] + (t - rows->pref[r]);
}

// Stage src[row slots] into dst[candidate index] for all candidates.
__device__ __forceinline__ void stage_rows(const CellRows* rows, const float4* __restrict__ src, float4* dst) {
  const unsigned lane = lane_id();
#pragma unroll
  for (int r = 0; r < 9; ++r) {
    const uint32_t p0 = rows->pref[r], len = rows->pref[r + 1] - p0, s0 = rows->start[r];
    for (uint32_t t = lane; t < len; t += 32) dst[p0 + t] = __ldg(&src[s0 + t]);
  }
}

// Iterate the cells owned by this warp: calls body(CellInfo, key).
template <typename Body>
__device__ __forceinline__ void for_each_owned_cell(const uint32_t* __restrict__ skey,
                                                    const uint32_t* __restrict__ cell_start,
                                                    const float4* __restrict__ pos, int n, int warp_global,
                                                    Body&& body) {
  const unsigned lane = lane_id();
  const int base = warp_global * 32;
  if (base >= n) return;
  const int s = base + static_cast<int>(lane);
  const bool live = s < n;
  const uint32_t k = live ? __ldg(&skey[s]) : 0xffffffffu;
  const uint32_t prev = (live && s > 0) ? __ldg(&skey[s - 1]) : 0xfffffffeu;
  unsigned starters = __ballot_sync(0xffffffffu, live && k != prev);
  while (starters) {
    const int sl = __ffs(starters) - 1;
    starters &= starters - 1;
    const uint32_t key = __shfl_sync(0xffffffffu, k, sl);
    CellInfo c;
    c.cs = static_cast<uint32_t>(base + sl);
    c.m = __ldg(&cell_start[key + 1]) - c.cs;
    c.sid = __float_as_int(__ldg(&pos[c.cs]).w);
    c.self0 = 0;
    body(c, key);
  }
}

// Sum over the L lanes of a particle group (L = 1, 2, 4; lanes of a group adjacent).
__device__ __forceinline__ float group_sum(float v, int L) {
  if (L >= 4) v += __shfl_xor_sync(0xffffffffu, v, 2);
  if (L >= 2) v += __shfl_xor_sync(0xffffffffu, v, 1);
  return v;
}

__device__ __forceinline__ int lanes_per_particle(uint32_t m) { return m <= 8 ? 4 : (m <= 16 ? 2 : 1); }

}  // namespace pbf
