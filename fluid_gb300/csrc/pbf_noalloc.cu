// pbf_density_noalloc: the load-time density estimate of Particles::estimateDensities
// (particles.cpp:440-444) for callers that cannot allocate device memory.
//
// Why it exists. pbf_estimate_densities runs on a pbf_handle, and creating a
// handle allocates its buffers with cudaMalloc. Some callers cannot do that: an
// application whose device memory is entirely owned by another framework's
// caching allocator (so a foreign cudaMalloc can fail or fragment its pool), or
// a latency-critical loop where cudaMalloc/cudaFree would implicitly
// synchronize the device. This entry point takes device inputs and outputs from
// the caller and does its cell sort in one fixed scratch array compiled into the
// library instead of allocating.
//
// The scratch array. `g_noalloc_scratch` below is a file-scope __device__ array
// of kScratchBytes (about 3.9 MB). Every GPU that loads this library holds it
// until the process exits, whether or not the function is called. In host code
// the array's name is only a host-side stand-in; the device address is obtained
// with cudaGetSymbolAddress once per device, with that device current, on the
// first call made while it is current (so make that first call outside any
// stream capture). Every call shares the one array and leaves its contents
// behind; the call clears the per-cell counters it needs before use. Two calls
// whose work overlaps on the GPU (different streams, or different host threads
// on the same device) race on the array and must be serialized by the caller.
#include <cmath>
#include <cstdint>
#include <mutex>
#include <string>

#include "pbf_device.cuh"
#include "pbf_handle.h"

namespace pbf {
namespace {

constexpr size_t kNaMaxParticles = PBF_NOALLOC_MAX_PARTICLES;
constexpr size_t kNaMaxCells = PBF_NOALLOC_MAX_CELLS;
constexpr size_t kNaTiles = (kNaMaxCells + 1023) / 1024 + 1;

// Layout of the scratch array (byte offsets, each 256-aligned).
constexpr size_t align256(size_t x) { return (x + 255) / 256 * 256; }
constexpr size_t kOffCount = 0;
constexpr size_t kOffStart = align256(kOffCount + 4 * kNaMaxCells);
constexpr size_t kOffTiles = align256(kOffStart + 4 * (kNaMaxCells + 1));
constexpr size_t kOffKey = align256(kOffTiles + 4 * kNaTiles);
constexpr size_t kOffRank = align256(kOffKey + 4 * kNaMaxParticles);
constexpr size_t kOffPerm = align256(kOffRank + 4 * kNaMaxParticles);
constexpr size_t kOffSorted = align256(kOffPerm + 4 * kNaMaxParticles);
constexpr size_t kScratchBytes = align256(kOffSorted + 16 * kNaMaxParticles);

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

// Device address of g_noalloc_scratch, resolved once per device.
constexpr int kMaxDevices = 64;
std::mutex g_na_mutex;
void* g_na_ptr[kMaxDevices] = {};

cudaError_t scratch_for_current_device(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_na_mutex);
  if (!g_na_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_na_ptr[dev] = p;
  }
  *out = static_cast<unsigned char*>(g_na_ptr[dev]);
  return cudaSuccess;
}

__device__ __forceinline__ unsigned na_lanemask_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Cell key and rank of each particle (warp-aggregated per-cell counting).
__global__ void k_na_count(const float* __restrict__ xyz, SceneDesc sc, DevParams P, uint32_t* __restrict__ count,
                           uint32_t* __restrict__ key, uint32_t* __restrict__ rank, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool live = i < n;
  uint32_t k = 0;
  if (live) {
    const float3 p = make_float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
    k = cell_key(cell_of(p, sc, P.inv_cell), sc);
    key[i] = k;
  }
  const unsigned active = __ballot_sync(0xffffffffu, live);
  if (!live) return;
  const unsigned peers = __match_any_sync(active, k);
  const int leader = __ffs(peers) - 1;
  uint32_t base = 0;
  if (static_cast<int>(threadIdx.x & 31u) == leader) base = atomicAdd(&count[k], __popc(peers));
  base = __shfl_sync(peers, base, leader);
  rank[i] = base + __popc(peers & na_lanemask_lt());
}

__global__ void k_na_scatter(const uint32_t* __restrict__ key, const uint32_t* __restrict__ rank,
                             const uint32_t* __restrict__ start, uint32_t* __restrict__ perm, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) perm[start[key[i]] + rank[i]] = static_cast<uint32_t>(i);
}

// Order each cell's slots by particle index (bounded: larger cells keep the atomic order).
__global__ void k_na_cellsort(const uint32_t* __restrict__ start, uint32_t* __restrict__ perm, uint32_t m) {
  const uint32_t c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= m) return;
  const uint32_t b = start[c], e = start[c + 1];
  if (e - b < 2 || e - b > 256) return;
  for (uint32_t x = b + 1; x < e; ++x) {
    const uint32_t v = perm[x];
    uint32_t y = x;
    while (y > b && perm[y - 1] > v) {
      perm[y] = perm[y - 1];
      --y;
    }
    perm[y] = v;
  }
}

__global__ void k_na_gather(const float* __restrict__ xyz, const uint32_t* __restrict__ perm,
                            float4* __restrict__ sorted, int n) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  const uint32_t i = perm[s];
  sorted[s] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], 0.f);
}

// rho_i = sum_j W(x_j - x_i) over the 27 cells around x_i, self included, in the
// caller's particle order.
__global__ void k_na_density(const float* __restrict__ xyz, const float4* __restrict__ sorted,
                             const uint32_t* __restrict__ start, SceneDesc sc, DevParams P,
                             float* __restrict__ rho, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float3 xi = make_float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
  const CellCoord cc = cell_of(xi, sc, P.inv_cell);
  float qsum = 0.f;
  for (int r = 0; r < 9; ++r) {
    const int z = cc.z + r / 3 - 1, y = cc.y + r % 3 - 1;
    if (z < 0 || z >= sc.dim[2] || y < 0 || y >= sc.dim[1]) continue;
    const uint32_t row = sc.cell_off + static_cast<uint32_t>((z * sc.dim[1] + y) * sc.dim[0]);
    const int x0 = cc.x > 0 ? cc.x - 1 : 0;
    const int x1 = cc.x + 1 < sc.dim[0] ? cc.x + 1 : sc.dim[0] - 1;
    for (uint32_t j = start[row + x0]; j < start[row + x1 + 1]; ++j) {
      const float4 xj = sorted[j];
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

// The message is readable through pbf_last_error(NULL).
pbf_status na_fail(pbf_status st, const std::string& msg) {
  set_global_error(msg);
  return st;
}

}  // namespace
}  // namespace pbf

extern "C" pbf_status pbf_density_noalloc(const pbf_params* params, size_t n, const float* xyz, float* rho,
                                          void* stream) {
  using namespace pbf;
  if (!params || (n > 0 && (!xyz || !rho))) return na_fail(PBF_ERR_INVALID, "params, xyz and rho are required");
  if (n > kNaMaxParticles)
    return na_fail(PBF_ERR_INVALID, "pbf_density_noalloc: n exceeds PBF_NOALLOC_MAX_PARTICLES (" +
                                        std::to_string(kNaMaxParticles) + ")");
  DevParams dp;
  double cell;
  std::string why;
  if (!make_dev_params(*params, &dp, &cell, &why)) return na_fail(PBF_ERR_INVALID, why);
  float lo[3], hi[3];
  for (int a = 0; a < 3; ++a) {
    lo[a] = static_cast<float>(params->box_lo[a]);
    hi[a] = static_cast<float>(params->box_hi[a]);
  }
  SceneDesc sc;
  if (!make_scene(*params, cell, lo, hi, &sc, &why)) return na_fail(PBF_ERR_INVALID, why);
  const uint64_t cells = static_cast<uint64_t>(sc.dim[0]) * sc.dim[1] * sc.dim[2];
  if (cells > kNaMaxCells)
    return na_fail(PBF_ERR_INVALID, "pbf_density_noalloc: the box needs " + std::to_string(cells) +
                                        " cells of size h, more than PBF_NOALLOC_MAX_CELLS (" +
                                        std::to_string(kNaMaxCells) + ")");
  if (n == 0) return PBF_OK;
  // xyz and rho must be memory of the current device (a host pointer here would make the
  // kernels fault or, where the GPU can reach host memory, read and write the wrong memory)
  int cur_dev = 0;
  cudaError_t e0 = cudaGetDevice(&cur_dev);
  if (e0 != cudaSuccess) return na_fail(PBF_ERR_CUDA, std::string("cudaGetDevice: ") + cudaGetErrorString(e0));
  const void* ptrs[2] = {xyz, rho};
  for (const void* q : ptrs) {
    cudaPointerAttributes at;
    e0 = cudaPointerGetAttributes(&at, q);
    if (e0 != cudaSuccess) {
      cudaGetLastError();
      return na_fail(PBF_ERR_INVALID, "pbf_density_noalloc: xyz and rho must be device memory");
    }
    const bool ok = (at.type == cudaMemoryTypeDevice && at.device == cur_dev) || at.type == cudaMemoryTypeManaged;
    if (!ok)
      return na_fail(PBF_ERR_INVALID, "pbf_density_noalloc: xyz and rho must be device (or managed) memory of "
                                      "the current device");
  }
  unsigned char* base = nullptr;
  cudaError_t e = scratch_for_current_device(&base);
  if (e != cudaSuccess) return na_fail(PBF_ERR_CUDA, std::string("cudaGetSymbolAddress: ") + cudaGetErrorString(e));
  uint32_t* count = reinterpret_cast<uint32_t*>(base + kOffCount);
  uint32_t* start = reinterpret_cast<uint32_t*>(base + kOffStart);
  uint32_t* tiles = reinterpret_cast<uint32_t*>(base + kOffTiles);
  uint32_t* key = reinterpret_cast<uint32_t*>(base + kOffKey);
  uint32_t* rank = reinterpret_cast<uint32_t*>(base + kOffRank);
  uint32_t* perm = reinterpret_cast<uint32_t*>(base + kOffPerm);
  float4* sorted = reinterpret_cast<float4*>(base + kOffSorted);
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const int ni = static_cast<int>(n);
  const uint32_t m = static_cast<uint32_t>(cells);
  const unsigned gb = static_cast<unsigned>((n + 255) / 256);
  e = cudaMemsetAsync(count, 0, sizeof(uint32_t) * m, s);  // the array keeps the previous call's counts
  if (e == cudaSuccess) {
    k_na_count<<<gb, 256, 0, s>>>(xyz, sc, dp, count, key, rank, ni);
    e = launch_exclusive_scan(count, start, tiles, m, s);
  }
  if (e == cudaSuccess) {
    k_na_scatter<<<gb, 256, 0, s>>>(key, rank, start, perm, ni);
    k_na_cellsort<<<(m + 255) / 256, 256, 0, s>>>(start, perm, m);
    k_na_gather<<<gb, 256, 0, s>>>(xyz, perm, sorted, ni);
    k_na_density<<<gb, 256, 0, s>>>(xyz, sorted, start, sc, dp, rho, ni);
    e = cudaGetLastError();
  }
  if (e != cudaSuccess) return na_fail(PBF_ERR_CUDA, std::string("pbf_density_noalloc: ") + cudaGetErrorString(e));
  return PBF_OK;
}
