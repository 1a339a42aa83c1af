// Marching-cubes surface of the density field: Particles::getSurfacePrims
// (particles.cpp:352-385) with generateGridCell (:309-323), getVertexNormal (:399-412),
// estimateDensityAt (:446-453) and polygonise / vertexInterp (marching.cpp).
//
//   k_surf_density  the field at every grid corner (one evaluation per corner; the
//                   reference evaluates each cube's 8 corners separately, at the same
//                   points up to the last bit of x1 + step)
//   k_surf_count    cube index (bit k set when corner k is below the iso level) and its
//                   triangle count
//   exclusive scan  first triangle of every cube
//   k_surf_emit     edge vertices (vertexInterp), triangles in cube order, vertex
//                   normals from central differences of the field at +-0.001
//
// Cubes are visited in the reference's loop order (x outer, then y, then z) and
// corners and edges are numbered as in generateGridCell and polygonise, so the
// vertices and their order follow the reference. The triangulation of each cube
// configuration is this library's own table (built by build_table below): on a
// face with four crossing edges the segments cut off the corners below the iso
// level, the segments of the six faces close into loops, and each loop is a fan
// from the first of its vertices that shares no face with a non-adjacent vertex of
// the loop. The surface is closed across cubes.
#include <cstdint>
#include <cstring>
#include <mutex>
#include <vector>

#include "pbf_device.cuh"

namespace pbf {

namespace {

// corner k of a cube, as generateGridCell lays it out: (x, y, z) in {0, 1}
constexpr int kCorner[8][3] = {{0, 0, 0}, {0, 1, 0}, {1, 1, 0}, {1, 0, 0},
                               {0, 0, 1}, {0, 1, 1}, {1, 1, 1}, {1, 0, 1}};
// edge e joins corners kEdge[e][0] and kEdge[e][1], as polygonise numbers them
constexpr int kEdge[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                              {6, 7}, {7, 4}, {0, 4}, {1, 5}, {2, 6}, {3, 7}};

int edge_between(int a, int b) {
  for (int e = 0; e < 12; ++e)
    if ((kEdge[e][0] == a && kEdge[e][1] == b) || (kEdge[e][0] == b && kEdge[e][1] == a)) return e;
  return -1;
}

}  // namespace

void build_table(SurfTable* t) {
  std::memset(t, 0, sizeof(*t));
  // the six faces as corner cycles (corners of a face in order around it)
  int face[6][4];
  int nf = 0;
  for (int axis = 0; axis < 3; ++axis) {
    for (int side = 0; side < 2; ++side) {
      const int u = (axis + 1) % 3, v = (axis + 2) % 3;
      // corners of this face in the cycle (0,0) (1,0) (1,1) (0,1) of (u, v)
      const int cyc[4][2] = {{0, 0}, {1, 0}, {1, 1}, {0, 1}};
      for (int k = 0; k < 4; ++k) {
        for (int c = 0; c < 8; ++c) {
          if (kCorner[c][axis] == side && kCorner[c][u] == cyc[k][0] && kCorner[c][v] == cyc[k][1]) face[nf][k] = c;
        }
      }
      ++nf;
    }
  }
  auto same_face = [&](int ea, int eb) {
    for (int f = 0; f < 6; ++f) {
      bool a = false, b = false;
      for (int k = 0; k < 4; ++k) {
        const int e = edge_between(face[f][k], face[f][(k + 1) % 4]);
        a |= e == ea;
        b |= e == eb;
      }
      if (a && b) return true;
    }
    return false;
  };
  for (int ci = 0; ci < 256; ++ci) {
    bool in[8];
    for (int c = 0; c < 8; ++c) in[c] = (ci >> c) & 1;
    uint16_t mask = 0;
    for (int e = 0; e < 12; ++e)
      if (in[kEdge[e][0]] != in[kEdge[e][1]]) mask |= static_cast<uint16_t>(1u << e);
    t->edges[ci] = mask;
    // face segments: partner[e][0..1] = the edges joined to e on its two faces
    int partner[12][2], np[12] = {};
    for (int f = 0; f < 6; ++f) {
      int es[4], cross[4], nc = 0;
      for (int k = 0; k < 4; ++k) {
        es[k] = edge_between(face[f][k], face[f][(k + 1) % 4]);
        if (in[face[f][k]] != in[face[f][(k + 1) % 4]]) cross[nc++] = k;
      }
      auto join = [&](int a, int b) {
        partner[a][np[a]++] = b;
        partner[b][np[b]++] = a;
      };
      if (nc == 2) {
        join(es[cross[0]], es[cross[1]]);
      } else if (nc == 4) {  // cut off the corners below the iso level
        for (int k = 0; k < 4; ++k)
          if (in[face[f][k]]) join(es[(k + 3) % 4], es[k]);
      }
    }
    // loops, from the lowest unused edge, and their fans
    bool used[12] = {};
    int ntri = 0;
    for (int start = 0; start < 12; ++start) {
      if (!(mask & (1u << start)) || used[start]) continue;
      int loop[12], k = 0, prev = -1, cur = start;
      for (;;) {
        loop[k++] = cur;
        used[cur] = true;
        const int next = (prev < 0 || partner[cur][0] != prev) ? partner[cur][0] : partner[cur][1];
        prev = cur;
        cur = next;
        if (cur == start) break;
      }
      int apex = 0;
      for (int a = 0; a < k; ++a) {
        bool ok = true;
        for (int i = 2; i < k - 1 && ok; ++i) ok = !same_face(loop[a], loop[(a + i) % k]);
        if (ok) {
          apex = a;
          break;
        }
      }
      for (int i = 1; i < k - 1; ++i) {
        t->tri[ci][3 * ntri] = static_cast<int8_t>(loop[apex]);
        t->tri[ci][3 * ntri + 1] = static_cast<int8_t>(loop[(apex + i) % k]);
        t->tri[ci][3 * ntri + 2] = static_cast<int8_t>(loop[(apex + i + 1) % k]);
        ++ntri;
      }
    }
    t->ntri[ci] = static_cast<uint8_t>(ntri);
  }
}

const SurfTable& surf_table() {
  static SurfTable table;
  static std::once_flag once;
  std::call_once(once, [] { build_table(&table); });
  return table;
}

namespace {

// kCorner / kEdge for device code: corner k has x = 1 for k in {2, 3, 6, 7}, y = 1 for
// k in {1, 2, 5, 6}, z = k / 4; edge e < 8 joins e and (e & 4) | ((e + 1) & 3), edge e >= 8
// joins e - 8 and e - 4
__device__ __forceinline__ int corner_x(int k) { return (0xCC >> k) & 1; }
__device__ __forceinline__ int corner_y(int k) { return (0x66 >> k) & 1; }
__device__ __forceinline__ int corner_z(int k) { return k >> 2; }
__device__ __forceinline__ int edge_a(int e) { return e < 8 ? e : e - 8; }
__device__ __forceinline__ int edge_b(int e) { return e < 8 ? ((e & 4) | ((e + 1) & 3)) : e - 4; }

// x1 = min(lo + i step, hi) per axis, computed in FP64 as the reference computes it (on
// the host, SurfGrid::axis)
__device__ __forceinline__ float3 corner_point(const SurfGrid& g, int i, int j, int k) {
  return make_float3(__ldg(&g.axis[i]), __ldg(&g.axis[g.nc[0] + 1 + j]), __ldg(&g.axis[g.nc[0] + g.nc[1] + 2 + k]));
}

__global__ void k_surf_density(const float4* __restrict__ pos, const uint32_t* __restrict__ cell_start,
                               const SceneDesc* __restrict__ scenes, SurfGrid g, float* __restrict__ field,
                               DevParams P) {
  const int nx = g.nc[0] + 1, ny = g.nc[1] + 1, nz = g.nc[2] + 1;
  const int64_t q = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (q >= static_cast<int64_t>(nx) * ny * nz) return;
  const int i = static_cast<int>(q % nx), j = static_cast<int>((q / nx) % ny), k = static_cast<int>(q / (nx * ny));
  field[q] = density_at_point(corner_point(g, i, j, k), pos, cell_start, scenes[0], P);
}

// cube c in the reference's loop order: c = (ix * nc_y + iy) * nc_z + iz
__device__ __forceinline__ void cube_of(const SurfGrid& g, int64_t c, int* ix, int* iy, int* iz) {
  *iz = static_cast<int>(c % g.nc[2]);
  *iy = static_cast<int>((c / g.nc[2]) % g.nc[1]);
  *ix = static_cast<int>(c / (static_cast<int64_t>(g.nc[2]) * g.nc[1]));
}

__device__ __forceinline__ float corner_value(const float* __restrict__ field, const SurfGrid& g, int i, int j,
                                              int k) {
  return field[(static_cast<int64_t>(k) * (g.nc[1] + 1) + j) * (g.nc[0] + 1) + i];
}

__global__ void k_surf_count(const float* __restrict__ field, const SurfTable* __restrict__ tab, SurfGrid g,
                             float iso, uint32_t* __restrict__ count, int64_t ncubes) {
  const int64_t c = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (c >= ncubes) return;
  int ix, iy, iz;
  cube_of(g, c, &ix, &iy, &iz);
  int ci = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if (corner_value(field, g, ix + corner_x(k), iy + corner_y(k), iz + corner_z(k)) < iso) ci |= 1 << k;
  count[c] = tab->ntri[ci];
}

// vertexInterp (marching.cpp): the iso crossing on the edge p1 -> p2
__device__ __forceinline__ float3 vertex_interp(float iso, float3 p1, float3 p2, float v1, float v2) {
  if (fabsf(iso - v1) < 0.00001f) return p1;
  if (fabsf(iso - v2) < 0.00001f) return p2;
  if (fabsf(v1 - v2) < 0.00001f) return p1;
  const float mu = (iso - v1) / (v2 - v1);
  return make_float3(p1.x + mu * (p2.x - p1.x), p1.y + mu * (p2.y - p1.y), p1.z + mu * (p2.z - p1.z));
}

// Triangle t lies in the cube c with first[c] <= t < first[c + 1] (binary search; empty
// cubes have first[c] == first[c + 1]), as the q-th of its cube's triangles; its vertex v
// sits on cube edge e between corners a and b (the cube's own corner order).
struct TriVertex {
  int ix, iy, iz, a, b;
};
__device__ __forceinline__ TriVertex tri_vertex(const float* __restrict__ field, const SurfTable* __restrict__ tab,
                                                const SurfGrid& g, float iso, const uint32_t* __restrict__ first,
                                                int64_t ncubes, uint32_t t, int v) {
  int64_t lo = 0, hi = ncubes;  // first[lo] <= t < first[hi] (first[ncubes] = total > t)
  while (hi - lo > 1) {
    const int64_t mid = (lo + hi) >> 1;
    if (first[mid] <= t) lo = mid;
    else hi = mid;
  }
  TriVertex r;
  cube_of(g, lo, &r.ix, &r.iy, &r.iz);
  int ci = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k)
    if (corner_value(field, g, r.ix + corner_x(k), r.iy + corner_y(k), r.iz + corner_z(k)) < iso) ci |= 1 << k;
  const int e = tab->tri[ci][3 * static_cast<int>(t - first[lo]) + v];
  r.a = edge_a(e);
  r.b = edge_b(e);
  return r;
}

// The grid edge of a cube edge, independent of the cube: 3 * (index of its lower corner)
// + its axis.
__device__ __forceinline__ unsigned long long edge_key(const SurfGrid& g, const TriVertex& r) {
  const int i = r.ix + min(corner_x(r.a), corner_x(r.b)), j = r.iy + min(corner_y(r.a), corner_y(r.b)),
            k = r.iz + min(corner_z(r.a), corner_z(r.b));
  const int axis = corner_x(r.a) != corner_x(r.b) ? 0 : (corner_y(r.a) != corner_y(r.b) ? 1 : 2);
  const unsigned long long corner =
      (static_cast<unsigned long long>(k) * (g.nc[1] + 1) + j) * static_cast<unsigned long long>(g.nc[0] + 1) + i;
  return 3ull * corner + static_cast<unsigned long long>(axis);
}

constexpr unsigned long long kNoKey = ~0ull;

__device__ __forceinline__ uint32_t key_hash(unsigned long long k) {
  k ^= k >> 33;
  k *= 0xff51afd7ed558ccdull;
  k ^= k >> 33;
  return static_cast<uint32_t>(k);
}

// One thread per triangle vertex: the vertex's grid edge goes into an open-addressing table
// (linear probing, compare-and-swap; the table holds at least twice the vertices, so a probe
// ends) and the vertex keeps its slot. Vertices shared by the triangles around an edge get
// one slot, so each normal is evaluated once; the thread that filled a slot lists it in
// ulist (warp-aggregated count in *ucount), so that the normals are computed by a dense grid.
__global__ void k_surf_vkeys(const float* __restrict__ field, const SurfTable* __restrict__ tab, SurfGrid g,
                             float iso, const uint32_t* __restrict__ first, uint32_t count, int64_t ncubes,
                             unsigned long long* keys, uint32_t cap_mask, uint32_t* __restrict__ vslot,
                             uint32_t* __restrict__ ulist, uint32_t* ucount) {
  const int64_t tid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (tid >= 3 * static_cast<int64_t>(count)) return;
  const TriVertex r = tri_vertex(field, tab, g, iso, first, ncubes, static_cast<uint32_t>(tid / 3),
                                 static_cast<int>(tid % 3));
  const unsigned long long key = edge_key(g, r);
  uint32_t h = key_hash(key) & cap_mask;
  bool fresh = false;
  for (uint32_t probe = 0; probe <= cap_mask; ++probe) {
    const unsigned long long prev = atomicCAS(&keys[h], kNoKey, key);
    if (prev == kNoKey || prev == key) {
      fresh = prev == kNoKey;
      break;
    }
    h = (h + 1) & cap_mask;
  }
  vslot[tid] = h;
  const unsigned act = __activemask();
  const unsigned m = __ballot_sync(act, fresh);
  if (m) {
    const int leader = __ffs(m) - 1;
    uint32_t base = 0;
    if (static_cast<int>(threadIdx.x & 31u) == leader) base = atomicAdd(ucount, static_cast<uint32_t>(__popc(m)));
    base = __shfl_sync(act, base, leader);
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    if (fresh) ulist[base + __popc(m & lt)] = h;
  }
}

// One thread per filled table slot (ulist[0, *ucount)): the normal of the slot's edge
// vertex (getVertexNormal: normalized central differences of estimateDensityAt at
// +-GRADIENT_EPS), the vertex taken by vertexInterp from the edge's lower corner to its
// upper corner.
__global__ void k_surf_vnormals(const float* __restrict__ field, SurfGrid g, float iso,
                                const unsigned long long* __restrict__ keys, const uint32_t* __restrict__ ulist,
                                const uint32_t* __restrict__ ucount, float4* __restrict__ nslot,
                                const float4* __restrict__ pos, const uint32_t* __restrict__ cell_start,
                                const SceneDesc* __restrict__ scenes, DevParams P) {
  const uint32_t u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= *ucount) return;
  const uint32_t sidx = ulist[u];
  const unsigned long long key = keys[sidx];
  const int axis = static_cast<int>(key % 3ull);
  unsigned long long c = key / 3ull;
  const int nx = g.nc[0] + 1, ny = g.nc[1] + 1;
  const int i = static_cast<int>(c % nx);
  c /= nx;
  const int j = static_cast<int>(c % ny), k = static_cast<int>(c / ny);
  const int i2 = i + (axis == 0), j2 = j + (axis == 1), k2 = k + (axis == 2);
  const float3 x = vertex_interp(iso, corner_point(g, i, j, k), corner_point(g, i2, j2, k2),
                                 corner_value(field, g, i, j, k), corner_value(field, g, i2, j2, k2));
  const SceneDesc& sc = scenes[0];
  const float eps = 0.001f;  // GRADIENT_EPS, particles.cpp:16
  float3 n;
  n.x = density_at_point(make_float3(x.x - eps, x.y, x.z), pos, cell_start, sc, P) -
        density_at_point(make_float3(x.x + eps, x.y, x.z), pos, cell_start, sc, P);
  n.y = density_at_point(make_float3(x.x, x.y - eps, x.z), pos, cell_start, sc, P) -
        density_at_point(make_float3(x.x, x.y + eps, x.z), pos, cell_start, sc, P);
  n.z = density_at_point(make_float3(x.x, x.y, x.z - eps), pos, cell_start, sc, P) -
        density_at_point(make_float3(x.x, x.y, x.z + eps), pos, cell_start, sc, P);
  const float nn = sqrtf(dot3(n, n));
  if (nn > 0.f) n = n * (1.0f / nn);
  nslot[sidx] = make_float4(n.x, n.y, n.z, 0.f);
}

// One thread per triangle vertex: the vertex by vertexInterp on its cube's edge in the
// cube's own corner order (as the reference computes it per cube), the normal of its
// grid edge from the table. A thread per cube instead would leave most lanes of a warp on
// empty cubes while one lane did up to 5 triangles.
__global__ void k_surf_emit(const float* __restrict__ field, const SurfTable* __restrict__ tab, SurfGrid g,
                            float iso, const uint32_t* __restrict__ first, const uint32_t* __restrict__ vslot,
                            const float4* __restrict__ nslot, float* __restrict__ xyz, float* __restrict__ nrm,
                            uint32_t count, int64_t ncubes) {
  const int64_t tid = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x;
  if (tid >= 3 * static_cast<int64_t>(count)) return;
  const uint32_t t = static_cast<uint32_t>(tid / 3);
  const int v = static_cast<int>(tid % 3);
  const TriVertex r = tri_vertex(field, tab, g, iso, first, ncubes, t, v);
  const int ia = r.ix + corner_x(r.a), ja = r.iy + corner_y(r.a), ka = r.iz + corner_z(r.a);
  const int ib = r.ix + corner_x(r.b), jb = r.iy + corner_y(r.b), kb = r.iz + corner_z(r.b);
  const float3 x = vertex_interp(iso, corner_point(g, ia, ja, ka), corner_point(g, ib, jb, kb),
                                 corner_value(field, g, ia, ja, ka), corner_value(field, g, ib, jb, kb));
  const float4 n = nslot[vslot[tid]];
  float* o = xyz + 9 * static_cast<size_t>(t) + 3 * v;
  float* m = nrm + 9 * static_cast<size_t>(t) + 3 * v;
  o[0] = x.x;
  o[1] = x.y;
  o[2] = x.z;
  m[0] = n.x;
  m[1] = n.y;
  m[2] = n.z;
}

inline unsigned blocks_for(int64_t n, int block) { return static_cast<unsigned>((n + block - 1) / block); }

}  // namespace

cudaError_t launch_surface_count(const Buffers& b, const DevParams& P, int cur, const SurfGrid& g, float iso,
                                 const SurfTable* tab, float* field, uint32_t* count, uint32_t* first,
                                 uint32_t* tile_sums, cudaStream_t s) {
  const int64_t corners = static_cast<int64_t>(g.nc[0] + 1) * (g.nc[1] + 1) * (g.nc[2] + 1);
  const int64_t cubes = static_cast<int64_t>(g.nc[0]) * g.nc[1] * g.nc[2];
  k_surf_density<<<blocks_for(corners, 128), 128, 0, s>>>(b.pos[cur], b.cell_start, b.scenes, g, field, P);
  k_surf_count<<<blocks_for(cubes, 256), 256, 0, s>>>(field, tab, g, iso, count, cubes);
  return launch_exclusive_scan(count, first, tile_sums, static_cast<uint32_t>(cubes), s);
}

uint32_t surface_hash_slots(uint32_t triangles) {
  uint32_t c = 1024;
  while (c < 6ull * triangles && c < (1u << 31)) c <<= 1;
  return c;
}

cudaError_t launch_surface_emit(const Buffers& b, const DevParams& P, int cur, const SurfGrid& g, float iso,
                                const SurfTable* tab, const float* field, const uint32_t* first, float* xyz,
                                float* nrm, uint32_t cap, const SurfHash& hs, cudaStream_t s) {
  const int64_t cubes = static_cast<int64_t>(g.nc[0]) * g.nc[1] * g.nc[2];
  if (cap == 0) return cudaSuccess;
  const uint32_t slots = surface_hash_slots(cap);
  cudaError_t e = cudaMemsetAsync(hs.keys, 0xff, sizeof(unsigned long long) * slots, s);
  if (e == cudaSuccess) e = cudaMemsetAsync(hs.ucount, 0, sizeof(uint32_t), s);
  if (e != cudaSuccess) return e;
  const int64_t verts = 3 * static_cast<int64_t>(cap);
  k_surf_vkeys<<<blocks_for(verts, 128), 128, 0, s>>>(field, tab, g, iso, first, cap, cubes, hs.keys, slots - 1,
                                                      hs.vslot, hs.ulist, hs.ucount);
  k_surf_vnormals<<<blocks_for(verts, 128), 128, 0, s>>>(field, g, iso, hs.keys, hs.ulist, hs.ucount, hs.nslot,
                                                          b.pos[cur], b.cell_start, b.scenes, P);
  k_surf_emit<<<blocks_for(verts, 128), 128, 0, s>>>(field, tab, g, iso, first, hs.vslot, hs.nslot, xyz, nrm, cap,
                                                      cubes);
  return cudaGetLastError();
}

}  // namespace pbf
