// Path tracer of the fluid surface and its scene for sm_103a: the reference's
// PathTracer (src/pathtracer.cpp:483-632) on the GPU, one thread per pixel.
//
//   k_surf_tris        marching-cubes output -> ray-test triangles (fluid material)
//   k_bounds_*         bounds of the triangle centroids
//   k_morton           30-bit Morton code of each centroid
//   k_sort_*           stable LSD radix sort of the codes (4 passes of 8 bits)
//   k_tree             binary radix tree over the sorted codes (Karras 2012,
//                      "Maximizing parallelism in the construction of BVHs, octrees
//                      and k-d trees"), ties broken by sorted position
//   k_refit            bottom-up boxes: the second child to finish fills its parent
//   k_wf_camera        a batch of paths (whole samples of every pixel): camera rays
//   per bounce level, over the queue of live paths (wavefront):
//     k_wf_trace<false>  closest hits, persistent threads fetching rays as they finish
//     k_wf_shade         emission, light samples as shadow-ray slots, BSDF sample and
//                        Russian roulette; continuing paths to the next queue
//     k_wf_trace<true>   visibility of the shadow-ray slots
//     k_wf_resolve       visible light samples added to the paths' radiance
//   k_accumulate       per-pixel sums of the paths' radiance in sample order
//   k_tonemap          HDRImageBuffer::toColor + ImageBuffer::update_pixel
//
// Every random number is a pure function of (seed, pixel, sample, draw index), so a
// frame does not depend on scheduling: draw k of sample s of pixel p is the top 24 bits
// of splitmix64(key(p, s) + k * 0x9E3779B97F4A7C15) times 2^-24 (splitmix64: Steele,
// Lea and Flood, "Fast splittable pseudorandom number generators", 2014). The draws
// are consumed in the reference's order: camera jitter (x, y) when ns_aa > 1; at each
// hit, per light and sample the light's draws, then the BSDF's, then the roulette coin.
#include <algorithm>
#include <cfloat>
#include <cstdint>

#include "pbf_internal.h"
#include "pbf_render.h"

namespace pbf {
namespace {

constexpr int kSortThreads = 256;
constexpr int kSortItems = 8;
constexpr uint32_t kSortTile = kSortThreads * kSortItems;
constexpr float kPi = 3.14159265358979323846f;

// ---- small vector helpers --------------------------------------------------------------
struct V3 {
  float x, y, z;
};
__device__ __forceinline__ V3 mk(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 v3(const float4& a) { return V3{a.x, a.y, a.z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
__device__ __forceinline__ V3 operator*(V3 a, float c) { return mk(a.x * c, a.y * c, a.z * c); }
__device__ __forceinline__ V3 operator*(float c, V3 a) { return mk(a.x * c, a.y * c, a.z * c); }
__device__ __forceinline__ V3 mulv(V3 a, V3 b) { return mk(a.x * b.x, a.y * b.y, a.z * b.z); }
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ V3 cross(V3 u, V3 v) {
  return mk(u.y * v.z - u.z * v.y, u.z * v.x - u.x * v.z, u.x * v.y - u.y * v.x);
}
__device__ __forceinline__ V3 unit(V3 a) { return a * rsqrtf(dot(a, a)); }
__device__ __forceinline__ V3 ld3(const float* p) { return mk(p[0], p[1], p[2]); }
__device__ __forceinline__ float illum(V3 s) { return 0.2126f * s.x + 0.7152f * s.y + 0.0722f * s.z; }

// ---- random numbers --------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long splitmix64(unsigned long long x) {
  unsigned long long z = x + 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}
struct Rng {
  unsigned long long key;
  unsigned long long k;
  __device__ __forceinline__ float next() {
    const unsigned long long z = splitmix64(key + (k++) * 0x9E3779B97F4A7C15ull);
    return static_cast<float>(z >> 40) * (1.0f / 16777216.0f);
  }
};
__device__ __forceinline__ unsigned long long path_key(unsigned long long seed, unsigned long long pixel,
                                                       unsigned long long sample) {
  return splitmix64(seed ^ splitmix64((pixel << 20) ^ sample));
}

// ---- surface triangles -----------------------------------------------------------------------
__global__ void k_surf_tris(const float* __restrict__ xyz, const float* __restrict__ nrm, uint32_t m, int material,
                            RTri* __restrict__ tri, RNrm* __restrict__ nn) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= m) return;
  const float* p = xyz + 9 * static_cast<size_t>(i);
  const float* q = nrm + 9 * static_cast<size_t>(i);
  tri[i] = RTri{make_float4(p[0], p[1], p[2], __int_as_float(material)), make_float4(p[3], p[4], p[5], 0.f),
                make_float4(p[6], p[7], p[8], 0.f)};
  nn[i] = RNrm{make_float4(q[0], q[1], q[2], 0.f), make_float4(q[3], q[4], q[5], 0.f),
               make_float4(q[6], q[7], q[8], 0.f)};
}

// ---- BVH build -------------------------------------------------------------------------------
__device__ __forceinline__ V3 centroid(const RTri& t) {
  return mk((t.p1.x + t.p2.x + t.p3.x) * (1.f / 3.f), (t.p1.y + t.p2.y + t.p3.y) * (1.f / 3.f),
            (t.p1.z + t.p2.z + t.p3.z) * (1.f / 3.f));
}

__device__ __forceinline__ void block_minmax(V3& lo, V3& hi) {
  __shared__ float s[6][32];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  float v[6] = {lo.x, lo.y, lo.z, hi.x, hi.y, hi.z};
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int c = 0; c < 6; ++c) {
      const float u = __shfl_xor_sync(0xffffffffu, v[c], o);
      v[c] = c < 3 ? fminf(v[c], u) : fmaxf(v[c], u);
    }
  if (lane == 0)
    for (int c = 0; c < 6; ++c) s[c][warp] = v[c];
  __syncthreads();
  if (warp == 0) {
    const unsigned nw = blockDim.x >> 5;
    for (int c = 0; c < 6; ++c) v[c] = lane < nw ? s[c][lane] : (c < 3 ? FLT_MAX : -FLT_MAX);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int c = 0; c < 6; ++c) {
        const float u = __shfl_xor_sync(0xffffffffu, v[c], o);
        v[c] = c < 3 ? fminf(v[c], u) : fmaxf(v[c], u);
      }
  }
  lo = mk(v[0], v[1], v[2]);
  hi = mk(v[3], v[4], v[5]);
}

// bounds[2 + 2 b], bounds[3 + 2 b]: the centroid box of block b's share
__global__ void __launch_bounds__(256) k_bounds_part(const RTri* __restrict__ tri, uint32_t n, float4* bounds) {
  V3 lo = mk(FLT_MAX, FLT_MAX, FLT_MAX), hi = mk(-FLT_MAX, -FLT_MAX, -FLT_MAX);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const V3 c = centroid(tri[i]);
    lo = mk(fminf(lo.x, c.x), fminf(lo.y, c.y), fminf(lo.z, c.z));
    hi = mk(fmaxf(hi.x, c.x), fmaxf(hi.y, c.y), fmaxf(hi.z, c.z));
  }
  block_minmax(lo, hi);
  if (threadIdx.x == 0) {
    bounds[2 + 2 * blockIdx.x] = make_float4(lo.x, lo.y, lo.z, 0.f);
    bounds[3 + 2 * blockIdx.x] = make_float4(hi.x, hi.y, hi.z, 0.f);
  }
}

__global__ void __launch_bounds__(kBoundsBlocks) k_bounds_final(float4* bounds) {
  const float4 a = bounds[2 + 2 * threadIdx.x], b = bounds[3 + 2 * threadIdx.x];
  V3 lo = v3(a), hi = v3(b);
  block_minmax(lo, hi);
  if (threadIdx.x == 0) {
    bounds[0] = make_float4(lo.x, lo.y, lo.z, 0.f);
    bounds[1] = make_float4(hi.x, hi.y, hi.z, 0.f);
  }
}

__device__ __forceinline__ uint32_t spread10(uint32_t v) {  // 10 bits -> every third bit
  v = (v * 0x00010001u) & 0xFF0000FFu;
  v = (v * 0x00000101u) & 0x0F00F00Fu;
  v = (v * 0x00000011u) & 0xC30C30C3u;
  v = (v * 0x00000005u) & 0x49249249u;
  return v;
}

__global__ void k_morton(const RTri* __restrict__ tri, uint32_t n, const float4* __restrict__ bounds,
                         uint32_t* __restrict__ keys, uint32_t* __restrict__ vals) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const V3 lo = v3(bounds[0]), hi = v3(bounds[1]);
  const V3 c = centroid(tri[i]);
  const float e[3] = {hi.x - lo.x, hi.y - lo.y, hi.z - lo.z};
  const float r[3] = {c.x - lo.x, c.y - lo.y, c.z - lo.z};
  uint32_t q[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float f = e[a] > 0.f ? r[a] / e[a] : 0.f;
    q[a] = static_cast<uint32_t>(fminf(fmaxf(f * 1024.f, 0.f), 1023.f));
  }
  keys[i] = (spread10(q[0]) << 2) | (spread10(q[1]) << 1) | spread10(q[2]);
  vals[i] = i;
}

// hist[d * nb + b]: count of digit d in tile b
__global__ void __launch_bounds__(kSortThreads) k_sort_hist(const uint32_t* __restrict__ keys, uint32_t n, int shift,
                                                             uint32_t* __restrict__ hist) {
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t base = blockIdx.x * kSortTile;
  for (int k = 0; k < kSortItems; ++k) {
    const uint32_t i = base + k * kSortThreads + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[threadIdx.x * gridDim.x + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: the tile's items go in order, 256 at a time; an item's place is its
// digit's running start + the same-digit items before it in earlier warps of the chunk
// + those before it in its own warp.
__global__ void __launch_bounds__(kSortThreads) k_sort_scatter(const uint32_t* __restrict__ keys,
                                                                const uint32_t* __restrict__ vals, uint32_t n,
                                                                int shift, const uint32_t* __restrict__ start,
                                                                uint32_t* __restrict__ keys_out,
                                                                uint32_t* __restrict__ vals_out) {
  constexpr int W = kSortThreads / 32;
  __shared__ uint32_t run[256];
  __shared__ uint32_t cnt[W][256];
  const unsigned lane = threadIdx.x & 31u, warp = threadIdx.x >> 5;
  run[threadIdx.x] = start[threadIdx.x * gridDim.x + blockIdx.x];
  const uint32_t base = blockIdx.x * kSortTile;
  for (int k = 0; k < kSortItems; ++k) {
    for (int w = 0; w < W; ++w) cnt[w][threadIdx.x] = 0;
    __syncthreads();
    const uint32_t i = base + k * kSortThreads + threadIdx.x;
    const bool live = i < n;
    const uint32_t key = live ? keys[i] : 0u;
    const uint32_t d = live ? ((key >> shift) & 255u) : 256u;
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    unsigned lt;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(lt));
    if (live && lane == static_cast<unsigned>(__ffs(peers) - 1)) cnt[warp][d] = __popc(peers);
    __syncthreads();
    if (live) {
      uint32_t pre = 0;
      for (unsigned w = 0; w < warp; ++w) pre += cnt[w][d];
      const uint32_t pos = run[d] + pre + __popc(peers & lt);
      keys_out[pos] = key;
      vals_out[pos] = vals[i];
    }
    __syncthreads();
    uint32_t add = 0;
    for (int w = 0; w < W; ++w) add += cnt[w][threadIdx.x];
    run[threadIdx.x] += add;
    __syncthreads();
  }
}

// Common-prefix length of the augmented keys (code, sorted position) of a and b.
__device__ __forceinline__ int prefix(const uint32_t* __restrict__ keys, int n, int a, int b) {
  if (b < 0 || b >= n) return -1;
  const unsigned long long ka = (static_cast<unsigned long long>(keys[a]) << 32) | static_cast<uint32_t>(a);
  const unsigned long long kb = (static_cast<unsigned long long>(keys[b]) << 32) | static_cast<uint32_t>(b);
  return __clzll(ka ^ kb);
}

// Internal node i of n - 1 (node 0 is the root); children: internal index, or kLeafBit |
// sorted position. parent[] over internal nodes [0, n-1) then leaves [n-1, 2n-1).
__global__ void k_tree(const uint32_t* __restrict__ keys, int n, BvhNode* __restrict__ nodes,
                       uint32_t* __restrict__ parent) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n - 1) return;
  const int d = (prefix(keys, n, i, i + 1) - prefix(keys, n, i, i - 1)) >= 0 ? 1 : -1;
  const int dmin = prefix(keys, n, i, i - d);
  int lmax = 2;
  while (prefix(keys, n, i, i + lmax * d) > dmin) lmax *= 2;
  int l = 0;
  for (int t = lmax / 2; t >= 1; t /= 2)
    if (prefix(keys, n, i, i + (l + t) * d) > dmin) l += t;
  const int j = i + l * d;
  const int dnode = prefix(keys, n, i, j);
  int s = 0;
  for (int t = (l + 1) / 2;; t = (t + 1) / 2) {
    if (prefix(keys, n, i, i + (s + t) * d) > dnode) s += t;
    if (t == 1) break;
  }
  const int gamma = i + s * d + min(d, 0);
  const uint32_t left = (min(i, j) == gamma) ? (kLeafBit | static_cast<uint32_t>(gamma)) : static_cast<uint32_t>(gamma);
  const uint32_t right = (max(i, j) == gamma + 1) ? (kLeafBit | static_cast<uint32_t>(gamma + 1))
                                                  : static_cast<uint32_t>(gamma + 1);
  nodes[i].lo_l.w = __uint_as_float(left);
  nodes[i].lo_r.w = __uint_as_float(right);
  parent[(left & kLeafBit) ? (n - 1 + (left & ~kLeafBit)) : left] = static_cast<uint32_t>(i);
  parent[(right & kLeafBit) ? (n - 1 + (right & ~kLeafBit)) : right] = static_cast<uint32_t>(i);
  if (i == 0) parent[0] = 0xffffffffu;
}

__device__ __forceinline__ float pad(float v, float s) { return v + s * (1e-6f * fabsf(v) + 1e-7f); }

// One thread per leaf: its triangle's box (padded by a few ulps), then up the tree; the
// second thread to reach a node writes its children's boxes and its own.
__global__ void k_refit(const RTri* __restrict__ tri, const uint32_t* __restrict__ vals, int n,
                        BvhNode* __restrict__ nodes, const uint32_t* __restrict__ parent, uint32_t* flags,
                        float4* box_lo, float4* box_hi) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const RTri t = tri[vals[k]];
  const uint32_t self = static_cast<uint32_t>(n - 1 + k);
  box_lo[self] = make_float4(pad(fminf(fminf(t.p1.x, t.p2.x), t.p3.x), -1.f),
                             pad(fminf(fminf(t.p1.y, t.p2.y), t.p3.y), -1.f),
                             pad(fminf(fminf(t.p1.z, t.p2.z), t.p3.z), -1.f), 0.f);
  box_hi[self] = make_float4(pad(fmaxf(fmaxf(t.p1.x, t.p2.x), t.p3.x), 1.f),
                             pad(fmaxf(fmaxf(t.p1.y, t.p2.y), t.p3.y), 1.f),
                             pad(fmaxf(fmaxf(t.p1.z, t.p2.z), t.p3.z), 1.f), 0.f);
  uint32_t p = parent[self];
  while (p != 0xffffffffu) {
    __threadfence();
    if (atomicAdd(&flags[p], 1u) == 0u) return;  // the sibling finishes this node
    __threadfence();
    const uint32_t cl = __float_as_uint(__ldcg(&nodes[p].lo_l.w)), cr = __float_as_uint(__ldcg(&nodes[p].lo_r.w));
    const uint32_t bl = (cl & kLeafBit) ? static_cast<uint32_t>(n - 1) + (cl & ~kLeafBit) : cl;
    const uint32_t br = (cr & kLeafBit) ? static_cast<uint32_t>(n - 1) + (cr & ~kLeafBit) : cr;
    const float4 ll = __ldcg(&box_lo[bl]), lh = __ldcg(&box_hi[bl]);
    const float4 rl = __ldcg(&box_lo[br]), rh = __ldcg(&box_hi[br]);
    nodes[p].lo_l = make_float4(ll.x, ll.y, ll.z, __uint_as_float(cl));
    nodes[p].hi_l = lh;
    nodes[p].lo_r = make_float4(rl.x, rl.y, rl.z, __uint_as_float(cr));
    nodes[p].hi_r = rh;
    box_lo[p] = make_float4(fminf(ll.x, rl.x), fminf(ll.y, rl.y), fminf(ll.z, rl.z), 0.f);
    box_hi[p] = make_float4(fmaxf(lh.x, rh.x), fmaxf(lh.y, rh.y), fmaxf(lh.z, rh.z), 0.f);
    p = parent[p];
  }
}

// ---- ray queries -------------------------------------------------------------------------------
struct Ray {
  V3 o, d, inv;
  float tmin, tmax;
};
__device__ __forceinline__ Ray make_ray(V3 o, V3 d, float tmin, float tmax) {
  return Ray{o, d, mk(1.f / d.x, 1.f / d.y, 1.f / d.z), tmin, tmax};
}

// MarchingTriangle::intersect (marching_triangle.cpp:46-73) in FP32
__device__ __forceinline__ bool tri_test(const RTri& t, const Ray& r, float tmax, float* tt, float* uu, float* vv) {
  const V3 p1 = v3(t.p1);
  const V3 e1 = v3(t.p2) - p1, e2 = v3(t.p3) - p1, s = r.o - p1;
  const V3 s1 = cross(r.d, e2), s2 = cross(s, e1);
  const float d = dot(s1, e1);
  if (d == 0.f) return false;
  const float tv = dot(s2, e2) / d;
  if (tv < r.tmin || tv > tmax) return false;
  const float u = dot(s1, s) / d, v = dot(s2, r.d) / d, w = 1.f - u - v;
  if (u < 0.f || u > 1.f || v < 0.f || v > 1.f || w < 0.f || w > 1.f) return false;
  *tt = tv;
  *uu = u;
  *vv = v;
  return true;
}

__device__ __forceinline__ bool box_test(const float4& lo, const float4& hi, const Ray& r, float tmax, float* tn) {
  const float tx0 = (lo.x - r.o.x) * r.inv.x, tx1 = (hi.x - r.o.x) * r.inv.x;
  const float ty0 = (lo.y - r.o.y) * r.inv.y, ty1 = (hi.y - r.o.y) * r.inv.y;
  const float tz0 = (lo.z - r.o.z) * r.inv.z, tz1 = (hi.z - r.o.z) * r.inv.z;
  const float t0 = fmaxf(fmaxf(fminf(tx0, tx1), fminf(ty0, ty1)), fmaxf(fminf(tz0, tz1), r.tmin));
  const float t1 = fminf(fminf(fmaxf(tx0, tx1), fmaxf(ty0, ty1)), fminf(fmaxf(tz0, tz1), tmax));
  *tn = t0;
  return t0 <= t1;
}

// Every triangle of tris[0, n) in index order.
template <bool ANY>
__device__ bool brute(const RTri* __restrict__ tris, uint32_t n, const Ray& r, float& tmax, int& best, float& bu,
                      float& bv) {
  for (uint32_t k = 0; k < n; ++k) {
    float t, u, v;
    if (tri_test(tris[k], r, tmax, &t, &u, &v)) {
      best = static_cast<int>(k);
      tmax = t;
      bu = u;
      bv = v;
      if (ANY) return true;
    }
  }
  return false;
}

// ---- BSDFs and lights (bsdf.cpp, light.cpp) --------------------------------------------------------
struct Frame {
  V3 x, y, z;
  __device__ __forceinline__ V3 to_local(V3 w) const { return mk(dot(x, w), dot(y, w), dot(z, w)); }
  __device__ __forceinline__ V3 to_world(V3 w) const { return x * w.x + y * w.y + z * w.z; }
};

// make_coord_space (bsdf.cpp:13-32)
__device__ __forceinline__ Frame coord_space(V3 n) {
  V3 h = n;
  if (fabsf(h.x) <= fabsf(h.y) && fabsf(h.x) <= fabsf(h.z)) h.x = 1.f;
  else if (fabsf(h.y) <= fabsf(h.x) && fabsf(h.y) <= fabsf(h.z)) h.y = 1.f;
  else h.z = 1.f;
  const V3 z = unit(n);
  const V3 y = unit(cross(h, z));
  const V3 x = unit(cross(z, y));
  return Frame{x, y, z};
}

__device__ __forceinline__ bool mat_delta(int kind) {
  return kind == kMatMirror || kind == kMatGlass || kind == kMatRefraction;
}

__device__ __forceinline__ V3 cosine_sample(Rng& g, float* pdf) {
  const float xi1 = g.next(), xi2 = g.next();
  const float r = sqrtf(xi1), th = 2.f * kPi * xi2;
  const float c = sqrtf(1.f - xi1);
  *pdf = c / kPi;
  float sn, cs;
  sincosf(th, &sn, &cs);
  return mk(r * cs, r * sn, c);
}

// sample_f of each BSDF (bsdf.cpp); wo, wi in the local frame
__device__ V3 sample_f(const RMat& m, V3 wo, V3* wi, float* pdf, Rng& g) {
  const V3 c1 = ld3(m.c1), c2 = ld3(m.c2);
  switch (m.kind) {
    case kMatDiffuse:
      *wi = cosine_sample(g, pdf);
      return c1 * (1.f / kPi);
    case kMatMirror:
      *wi = mk(-wo.x, -wo.y, wo.z);
      *pdf = 1.f;
      return c1 * (1.f / fabsf(wi->z));
    case kMatGlass: {
      const float ior = m.ior;
      const float no = wo.z > 0.f ? 1.f : ior, ni = wo.z > 0.f ? ior : 1.f;
      const float sint2 = (1.f - wo.z * wo.z) * no * no / ni / ni;
      if (sint2 >= 1.f) {  // total internal reflection
        *wi = mk(-wo.x, -wo.y, wo.z);
        *pdf = 1.f;
        return c2 * (1.f / fabsf(wi->z));
      }
      const float cost = wo.z > 0.f ? -sqrtf(1.f - sint2) : sqrtf(1.f - sint2);
      *wi = unit(mk(-wo.x * no / ni, -wo.y * no / ni, cost));
      float R = (ior - 1.f) * (ior - 1.f) / (ior + 1.f) / (ior + 1.f);
      const float c = 1.f - fabsf(wi->z);
      R = R + (1.f - R) * c * c * c * c * c;
      if (g.next() < R) {
        *wi = mk(-wo.x, -wo.y, wo.z);
        *pdf = R;
        return c2 * (R / fabsf(wi->z));
      }
      *pdf = 1.f - R;
      const float nr = wi->z > 0.f ? ior : 1.f / ior;
      return c1 * ((1.f - R) * nr * nr / fabsf(wi->z));
    }
    case kMatEmission:
      *wi = cosine_sample(g, pdf);
      return mk(0.f, 0.f, 0.f);
    default:  // the reference's RefractionBSDF returns black
      *wi = mk(0.f, 0.f, 1.f);
      *pdf = 1.f;
      return mk(0.f, 0.f, 0.f);
  }
}

__device__ V3 sample_L(const RLight& l, V3 p, V3* wi, float* dist, float* pdf, Rng& g) {
  switch (l.kind) {
    case kLightDirectional:
      *wi = ld3(l.dir);
      *dist = FLT_MAX;
      *pdf = 1.f;
      return ld3(l.rad);
    case kLightHemisphere: {
      const float xi1 = g.next(), xi2 = g.next();
      const float th = acosf(xi1), ph = 2.f * kPi * xi2;
      const float xs = sinf(th) * cosf(ph), ys = sinf(th) * sinf(ph), zs = cosf(th);
      *wi = mk(xs, zs, -ys);  // sampleToWorld columns (1,0,0), (0,0,-1), (0,1,0)
      *dist = FLT_MAX;
      *pdf = 1.f / (2.f * kPi);
      return ld3(l.rad);
    }
    case kLightPoint: {
      const V3 d = ld3(l.pos) - p;
      const float len = sqrtf(dot(d, d));
      *wi = d * (1.f / len);
      *dist = len;
      *pdf = 1.f;
      return ld3(l.rad);
    }
    default: {  // area (light.cpp:79-93)
      const float sx = g.next() - 0.5f, sy = g.next() - 0.5f;
      const V3 d = ld3(l.pos) + sx * ld3(l.dx) + sy * ld3(l.dy) - p;
      const float cosTheta = dot(d, ld3(l.dir));
      const float sq = dot(d, d);
      const float dd = sqrtf(sq);
      *wi = d * (1.f / dd);
      *dist = dd;
      *pdf = sq / (l.area * fabsf(cosTheta));
      return cosTheta < 0.f ? ld3(l.rad) : mk(0.f, 0.f, 0.f);
    }
  }
}

// ---- the path tracer ---------------------------------------------------------------------------
// The scene's triangles (few and large: walls, meshes) and the fluid surface's (many and
// small) sit in two hierarchies, so that the scene's large boxes do not widen the
// surface tree's nodes; a scene of at most kBruteScene triangles is tested triangle by
// triangle. tri holds the scene's n_scene triangles, then the surface's.
struct Scene {
  const RTri* tri;
  const RNrm* nrm;
  const RMat* mats;
  const RLight* lights;
  uint32_t n_scene, n_surf;
  const BvhNode* scene_nodes;  // null: brute force
  const RTri* scene_ltri;      // leaf-ordered triangles of each tree
  const BvhNode* surf_nodes;
  const RTri* surf_ltri;
};

constexpr uint32_t kNoItem = 0xffffffffu;

__device__ __forceinline__ unsigned lane_lt() {
  unsigned m;
  asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
  return m;
}

// Warp-aggregated append: every lane of the warp calls it (converged); lanes with want
// get consecutive indices of *counter.
__device__ __forceinline__ uint32_t warp_append(uint32_t* counter, bool want) {
  const unsigned full = 0xffffffffu;
  const unsigned m = __ballot_sync(full, want);
  if (m == 0) return 0;
  const int leader = __ffs(m) - 1;
  uint32_t base = 0;
  if (static_cast<int>(threadIdx.x & 31u) == leader) base = atomicAdd(counter, static_cast<uint32_t>(__popc(m)));
  base = __shfl_sync(full, base, leader);
  return base + static_cast<uint32_t>(__popc(m & lane_lt()));
}

// A ray walk that advances one node at a time, so that a lane whose ray is done can take
// the next ray while the warp's other lanes keep walking theirs (persistent traversal
// with dynamic ray fetch, Aila and Laine, "Understanding the efficiency of ray traversal
// on GPUs", 2009). Phase 0 walks the scene's tree (when the scene has one), phase 1 the
// surface's; phase 2 is done.
struct Walk {
  uint32_t node;
  int sp;
  int phase;
  int best;
  float tmax, bu, bv;
  uint32_t stack[kBvhStack];
};

// Enters the first tree from s.phase on with more than one triangle (a tree of one is
// tested at once).
template <bool ANY>
__device__ __forceinline__ void walk_enter(const Scene& sc, const Ray& r, Walk& s) {
  while (s.phase < 2) {
    const uint32_t n = s.phase == 0 ? (sc.scene_nodes ? sc.n_scene : 0u) : sc.n_surf;
    const uint32_t base = s.phase == 0 ? 0u : sc.n_scene;
    if (n >= 2) {
      s.node = 0;
      s.sp = 0;
      return;
    }
    if (n == 1) {
      float t, u, v;
      if (tri_test(sc.tri[base], r, s.tmax, &t, &u, &v)) {
        s.best = static_cast<int>(base);
        s.tmax = t;
        s.bu = u;
        s.bv = v;
        if (ANY) {
          s.phase = 2;
          return;
        }
      }
    }
    ++s.phase;
  }
}

template <bool ANY>
__device__ __forceinline__ void walk_begin(const Scene& sc, const Ray& r, Walk& s) {
  s.tmax = r.tmax;
  s.best = -1;
  s.bu = s.bv = 0.f;
  s.phase = 0;
  if (!sc.scene_nodes && brute<ANY>(sc.tri, sc.n_scene, r, s.tmax, s.best, s.bu, s.bv)) {
    s.phase = 2;  // any hit found among the scene's triangles
    return;
  }
  walk_enter<ANY>(sc, r, s);
}

// One node of the current tree: both children's boxes, leaves tested at once, the nearer
// hit child next and the farther one pushed.
template <bool ANY>
__device__ __forceinline__ void walk_step(const Scene& sc, const Ray& r, Walk& s, unsigned* err) {
  const bool scene = s.phase == 0;
  const BvhNode* __restrict__ nodes = scene ? sc.scene_nodes : sc.surf_nodes;
  const RTri* __restrict__ ltri = scene ? sc.scene_ltri : sc.surf_ltri;
  const uint32_t base = scene ? 0u : sc.n_scene;
  const BvhNode nd = nodes[s.node];
  float tl, tr;
  bool hl = box_test(nd.lo_l, nd.hi_l, r, s.tmax, &tl);
  bool hr = box_test(nd.lo_r, nd.hi_r, r, s.tmax, &tr);
  const uint32_t cl = __float_as_uint(nd.lo_l.w), cr = __float_as_uint(nd.lo_r.w);
#pragma unroll
  for (int side = 0; side < 2; ++side) {
    const uint32_t c = side ? cr : cl;
    bool& h = side ? hr : hl;
    if (h && (c & kLeafBit)) {
      h = false;
      const RTri tv = ltri[c & ~kLeafBit];
      const uint32_t ti = base + __float_as_uint(tv.p1.w);
      float t, u, v;
      if (tri_test(tv, r, s.tmax, &t, &u, &v)) {
        s.best = static_cast<int>(ti);
        s.tmax = t;
        s.bu = u;
        s.bv = v;
        if (ANY) {
          s.phase = 2;
          return;
        }
      }
    }
  }
  if (hl && hr) {
    const bool lfirst = tl <= tr;
    if (s.sp < kBvhStack) {
      s.stack[s.sp++] = lfirst ? cr : cl;
    } else {
      atomicOr(err, 1u);
    }
    s.node = lfirst ? cl : cr;
  } else if (hl) {
    s.node = cl;
  } else if (hr) {
    s.node = cr;
  } else if (s.sp > 0) {
    s.node = s.stack[--s.sp];
  } else {
    ++s.phase;
    walk_enter<ANY>(sc, r, s);
  }
}

using WfArgs = WfBuffers;

// Closest hits (ANY = false) of the paths in queue[0, *count), or visibility (ANY = true)
// of the shadow slots in queue[0, *count); persistent threads with dynamic fetch.
template <bool ANY>
__global__ void __launch_bounds__(128) k_wf_trace(Scene sc, WfArgs w, const uint32_t* __restrict__ queue,
                                                  const uint32_t* __restrict__ count, uint32_t* fetch, float ray_eps,
                                                  unsigned* err) {
  const unsigned full = 0xffffffffu, lane = threadIdx.x & 31u;
  const uint32_t total = *count;
  uint32_t item = kNoItem;
  bool drained = false;
  Ray r = make_ray(mk(0.f, 0.f, 0.f), mk(0.f, 0.f, 1.f), 0.f, 0.f);
  Walk s;
  s.phase = 2;
  while (true) {
    if (!drained) {
      const unsigned need = __ballot_sync(full, item == kNoItem);
      if (need) {
        const int leader = __ffs(need) - 1;
        uint32_t base = 0;
        if (static_cast<int>(lane) == leader) base = atomicAdd(fetch, static_cast<uint32_t>(__popc(need)));
        base = __shfl_sync(full, base, leader);
        if (base + static_cast<uint32_t>(__popc(need)) >= total) drained = true;
        if (item == kNoItem) {
          const uint32_t idx = base + static_cast<uint32_t>(__popc(need & lane_lt()));
          if (idx < total) {
            item = queue[idx];
            if (ANY) {
              const uint32_t q = item / static_cast<uint32_t>(w.slots);
              const float4 o = w.o[q], sd = w.sdir[item];
              r = make_ray(mk(o.x, o.y, o.z), mk(sd.x, sd.y, sd.z), ray_eps, sd.w);
            } else {
              const float4 o = w.o[item], d = w.d[item];
              r = make_ray(mk(o.x, o.y, o.z), mk(d.x, d.y, d.z), o.w, d.w);
            }
            walk_begin<ANY>(sc, r, s);
          }
        }
      }
    }
    if (__ballot_sync(full, item != kNoItem) == 0) break;
    if (item == kNoItem) continue;
    for (int k = 0; k < 4 && s.phase < 2; ++k) walk_step<ANY>(sc, r, s, err);
    if (s.phase >= 2) {
      if (ANY) {
        w.scon[item].w = s.best >= 0 ? 0.f : 1.f;
      } else {
        w.hit[item] = make_float4(__int_as_float(s.best), s.tmax, s.bu, s.bv);
      }
      item = kNoItem;
    }
  }
}

// Camera rays of the batch's paths (PathTracer::raytrace_pixel, pathtracer.cpp:584-604):
// path q is sample s0 + q / npix of pixel q % npix; all paths join queue a.
__global__ void k_wf_camera(WfArgs w, RCam cam, RArgs a, int s0, uint32_t paths) {
  const uint32_t q = blockIdx.x * blockDim.x + threadIdx.x;
  if (q == 0) {
    w.cnt[0] = paths;
    w.cnt[1] = w.cnt[2] = w.cnt[3] = w.cnt[4] = 0;
  }
  if (q >= paths) return;
  const uint32_t npix = static_cast<uint32_t>(a.width) * static_cast<uint32_t>(a.height);
  const uint32_t pix = q % npix;
  const int s = s0 + static_cast<int>(q / npix);
  Rng g{path_key(a.seed, pix, static_cast<unsigned long long>(s)), 0ull};
  float jx = 0.5f, jy = 0.5f;
  if (a.ns_aa > 1) {
    jx = g.next();
    jy = g.next();
  }
  const int px = static_cast<int>(pix % static_cast<uint32_t>(a.width));
  const int py = static_cast<int>(pix / static_cast<uint32_t>(a.width));
  const float xn = (px + jx) / a.width, yn = (py + jy) / a.height;
  const V3 cx = ld3(cam.c2w), cy = ld3(cam.c2w + 3), cz = ld3(cam.c2w + 6);
  const V3 dir = unit(cx * ((xn - 0.5f) * cam.htan) + cy * ((yn - 0.5f) * cam.vtan) - cz);
  w.o[q] = make_float4(cam.pos[0], cam.pos[1], cam.pos[2], cam.nclip);
  w.d[q] = make_float4(dir.x, dir.y, dir.z, cam.fclip);
  w.beta[q] = make_float4(1.f, 1.f, 1.f, 1.f);
  w.L[q] = make_float4(0.f, 0.f, 0.f, 0.f);
  w.st[q] = make_uint2(static_cast<uint32_t>(a.max_depth), static_cast<uint32_t>(g.k));
  w.qa[q] = q;
}

// Clears the next queue's length, the shadow slot count and the fetch counters.
__global__ void k_wf_reset(uint32_t* cnt, int next) {
  cnt[next] = 0;
  cnt[2] = cnt[3] = cnt[4] = 0;
}

// One bounce of trace_ray (pathtracer.cpp:553-582) at the closest hit of every queued
// path: emission, the light samples of estimate_direct_lighting (:483-524) as shadow ray
// slots (their contribution, throughput included, added by k_wf_resolve when the light is
// visible), then estimate_indirect_lighting's BSDF sample and roulette (:526-551): the
// continuing paths join queue_out. Random numbers are drawn in the reference's order.
// Every lane of a warp runs the loops to the same trip counts so that the appends meet.
__global__ void __launch_bounds__(128) k_wf_shade(Scene sc, WfArgs w, RArgs a, int s0,
                                                  const uint32_t* __restrict__ queue,
                                                  const uint32_t* __restrict__ count, uint32_t* queue_out,
                                                  uint32_t* count_out) {
  const uint32_t total = *count;
  const uint32_t stride = gridDim.x * blockDim.x;  // a multiple of 32: each warp keeps one base
  const uint32_t S = static_cast<uint32_t>(w.slots);
  const uint32_t npix = static_cast<uint32_t>(a.width) * static_cast<uint32_t>(a.height);
  for (uint32_t wbase = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; wbase < total; wbase += stride) {
    const uint32_t idx = wbase + (threadIdx.x & 31u);
    const bool live = idx < total;
    const uint32_t q = live ? queue[idx] : 0u;
    float4 h = live ? w.hit[q] : make_float4(__int_as_float(-1), 0.f, 0.f, 0.f);
    const int ti = __float_as_int(h.x);
    const bool hit = live && ti >= 0;
    // shading state (only meaningful where hit)
    RMat m{};
    V3 n = mk(0.f, 0.f, 1.f), P = mk(0.f, 0.f, 0.f), rd = mk(0.f, 0.f, 1.f), beta = mk(0.f, 0.f, 0.f);
    V3 L = mk(0.f, 0.f, 0.f);
    bool includeLe = false;
    uint2 st = make_uint2(0u, 0u);
    if (hit) {
      const RTri tr = sc.tri[ti];
      m = sc.mats[__float_as_int(tr.p1.w)];
      const RNrm nn = sc.nrm[ti];
      const float u = h.z, v = h.w, ww = 1.f - u - v;
      n = ww * v3(nn.n1) + u * v3(nn.n2) + v * v3(nn.n3);
      const float4 o = w.o[q], d = w.d[q];
      rd = mk(d.x, d.y, d.z);
      P = mk(o.x, o.y, o.z) + rd * h.y;
      const float4 b = w.beta[q], l = w.L[q];
      beta = mk(b.x, b.y, b.z);
      includeLe = b.w != 0.f;
      L = mk(l.x, l.y, l.z);
      st = w.st[q];
      if (includeLe && m.kind == kMatEmission) L = L + mulv(beta, ld3(m.c1));
    }
    Rng g{hit ? path_key(a.seed, q % npix, static_cast<unsigned long long>(s0) + q / npix) : 0ull, st.y};
    const Frame f = coord_space(n);
    const bool direct = hit && !mat_delta(m.kind);
    const V3 fval = m.kind == kMatDiffuse ? ld3(m.c1) * (1.f / kPi) : mk(0.f, 0.f, 0.f);
    uint32_t j = 0;
    for (int li = 0; li < a.n_light; ++li) {
      const RLight& l = sc.lights[li];
      const int ns = (l.kind == kLightDirectional || l.kind == kLightPoint) ? 1 : a.ns_area;
      for (int i = 0; i < ns; ++i, ++j) {
        bool want = false;
        float4 dir4 = make_float4(0.f, 0.f, 0.f, 0.f), con = make_float4(0.f, 0.f, 0.f, 0.f);
        if (direct) {
          V3 wi;
          float dist, pdf;
          const V3 Ls = sample_L(l, P, &wi, &dist, &pdf, g);
          const float cz_in = dot(f.z, wi);
          if (cz_in >= 0.f) {
            const V3 c = mulv(beta, mulv(Ls, fval) * (fabsf(cz_in) / pdf));
            con = make_float4(c.x / ns, c.y / ns, c.z / ns, 0.f);
            dir4 = make_float4(wi.x, wi.y, wi.z, dist);
            want = true;
          }
        }
        if (hit) {
          w.scon[static_cast<size_t>(q) * S + j] = con;
          if (want) w.sdir[static_cast<size_t>(q) * S + j] = dir4;
        }
        const uint32_t at = warp_append(&w.cnt[2], want);
        if (want) w.sq[at] = q * S + j;
      }
    }
    if (hit) {
      for (uint32_t k = j; k < S; ++k) w.scon[static_cast<size_t>(q) * S + k] = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    bool cont = false;
    if (hit) {
      w.L[q] = make_float4(L.x, L.y, L.z, 0.f);
      w.o[q] = make_float4(P.x, P.y, P.z, a.ray_eps);  // the shadow rays' origin, and the next ray's
      uint32_t depth = st.x;
      if (depth > 0) {
        const V3 wo = f.to_local(mk(-rd.x, -rd.y, -rd.z));
        V3 wi;
        float pdf;
        const V3 fs = sample_f(m, wo, &wi, &pdf, g);
        const float p_cont = fminf(illum(fs) * 15.f, 1.f);
        if (g.next() < p_cont) {
          beta = mulv(beta, fs) * (fabsf(wi.z) / p_cont / pdf);
          const V3 nd = f.to_world(wi);
          w.d[q] = make_float4(nd.x, nd.y, nd.z, FLT_MAX);
          w.beta[q] = make_float4(beta.x, beta.y, beta.z, mat_delta(m.kind) ? 1.f : 0.f);
          --depth;
          cont = true;
        }
      }
      w.st[q] = make_uint2(depth, static_cast<uint32_t>(g.k));
    }
    const uint32_t at = warp_append(count_out, cont);
    if (cont) queue_out[at] = q;
  }
}

// Adds each shaded path's visible light samples, in slot order (light by light, sample by
// sample, as estimate_direct_lighting sums them).
__global__ void k_wf_resolve(WfArgs w, const uint32_t* __restrict__ queue, const uint32_t* __restrict__ count) {
  const uint32_t total = *count;
  const uint32_t S = static_cast<uint32_t>(w.slots);
  for (uint32_t idx = blockIdx.x * blockDim.x + threadIdx.x; idx < total; idx += gridDim.x * blockDim.x) {
    const uint32_t q = queue[idx];
    if (__float_as_int(w.hit[q].x) < 0) continue;
    const float4 l = w.L[q];
    V3 L = mk(l.x, l.y, l.z);
    for (uint32_t j = 0; j < S; ++j) {
      const float4 c = w.scon[static_cast<size_t>(q) * S + j];
      if (c.w > 0.5f) L = L + mk(c.x, c.y, c.z);
    }
    w.L[q] = make_float4(L.x, L.y, L.z, 0.f);
  }
}

// Sums a batch of nb samples per pixel (path radiance rad[s * npix + pixel]) into acc in
// sample order (the reference adds trace_ray's results in sample order,
// pathtracer.cpp:597-602); the last batch divides by ns_aa.
__global__ void k_accumulate(const float4* __restrict__ rad, uint32_t npix, int nb, int first, int last, int ns_aa,
                             float* __restrict__ acc) {
  const uint32_t pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= npix) return;
  float* o = acc + 3 * static_cast<size_t>(pix);
  V3 v = first ? mk(0.f, 0.f, 0.f) : mk(o[0], o[1], o[2]);
  for (int s = 0; s < nb; ++s) {
    const float4 x = rad[static_cast<size_t>(s) * npix + pix];
    v = v + mk(x.x, x.y, x.z);
  }
  if (last) {
    const float ns = static_cast<float>(ns_aa);
    v = mk(v.x / ns, v.y / ns, v.z / ns);
  }
  o[0] = v.x;
  o[1] = v.y;
  o[2] = v.z;
}

// HDRImageBuffer::toColor (image.h:174-189) with ImageBuffer::update_pixel (image.h:49-58):
// gamma 2.2, exposure sqrt(2), min(1, c) * 255 truncated (the reference's clamp call
// reduces to min(1, c)), rows flipped as PathTracer::save_image writes the PNG.
__device__ __forceinline__ uint8_t to_byte(float c) {
  const float v = c < 1.f ? c : 1.f;
  return static_cast<uint8_t>(static_cast<uint32_t>(v * 255.f));
}
__global__ void k_tonemap(const float* __restrict__ hdr, int W, int H, uint8_t* __restrict__ rgba) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= W * H) return;
  const int x = pix % W, y = pix / W;
  const float exposure = 1.41421356237309515f, g = 1.f / 2.2f;
  const float* s = hdr + 3 * static_cast<size_t>(pix);
  uint8_t* o = rgba + 4 * (static_cast<size_t>(H - 1 - y) * W + x);
  o[0] = to_byte(powf(s[0] * exposure, g));
  o[1] = to_byte(powf(s[1] * exposure, g));
  o[2] = to_byte(powf(s[2] * exposure, g));
  o[3] = 255;
}

inline unsigned blocks(size_t n, int b) { return static_cast<unsigned>((n + b - 1) / b); }

}  // namespace

uint32_t sort_blocks(uint32_t n) { return (n + kSortTile - 1) / kSortTile; }

cudaError_t launch_surface_to_tris(const float* xyz, const float* nrm, uint32_t m, int material, RTri* tri,
                                   RNrm* nn, cudaStream_t s) {
  if (m == 0) return cudaSuccess;
  k_surf_tris<<<blocks(m, 256), 256, 0, s>>>(xyz, nrm, m, material, tri, nn);
  return cudaGetLastError();
}

// Triangles in leaf order with their index in p1.w (walk_step reads them directly).
__global__ void k_leaf_tris(const RTri* __restrict__ tri, const uint32_t* __restrict__ vals, uint32_t n,
                            RTri* __restrict__ ltri) {
  const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  const uint32_t i = vals[k];
  RTri t = tri[i];
  t.p1.w = __uint_as_float(i);
  ltri[k] = t;
}

cudaError_t launch_bvh_build(const RTri* tri, uint32_t n, const BvhScratch& w, BvhNode* nodes, cudaStream_t s) {
  if (n < 2) return cudaSuccess;
  k_bounds_part<<<kBoundsBlocks, 256, 0, s>>>(tri, n, w.bounds);
  k_bounds_final<<<1, kBoundsBlocks, 0, s>>>(w.bounds);
  k_morton<<<blocks(n, 256), 256, 0, s>>>(tri, n, w.bounds, w.keys, w.vals);
  const uint32_t nb = sort_blocks(n);
  uint32_t *ka = w.keys, *va = w.vals, *kb = w.keys2, *vb = w.vals2;
  for (int shift = 0; shift < 32; shift += 8) {
    k_sort_hist<<<nb, kSortThreads, 0, s>>>(ka, n, shift, w.hist);
    cudaError_t e = launch_exclusive_scan(w.hist, w.start, w.tile_sums, 256u * nb, s);
    if (e != cudaSuccess) return e;
    k_sort_scatter<<<nb, kSortThreads, 0, s>>>(ka, va, n, shift, w.start, kb, vb);
    uint32_t* t = ka;
    ka = kb;
    kb = t;
    t = va;
    va = vb;
    vb = t;
  }
  // four passes: the sorted codes and triangle indices are back in keys / vals
  k_tree<<<blocks(n - 1, 256), 256, 0, s>>>(w.keys, static_cast<int>(n), nodes, w.parent);
  cudaError_t e = cudaMemsetAsync(w.flags, 0, sizeof(uint32_t) * (n - 1), s);
  if (e != cudaSuccess) return e;
  k_refit<<<blocks(n, 256), 256, 0, s>>>(tri, w.vals, static_cast<int>(n), nodes, w.parent, w.flags, w.box_lo,
                                         w.box_hi);
  k_leaf_tris<<<blocks(n, 256), 256, 0, s>>>(tri, w.vals, n, w.ltri);
  return cudaGetLastError();
}

int render_slots(const RLight* lights, int n_light, int ns_area) {
  int S = 0;
  for (int l = 0; l < n_light; ++l)
    S += (lights[l].kind == kLightDirectional || lights[l].kind == kLightPoint) ? 1 : ns_area;
  return S;
}

size_t render_path_bytes(int slots) {
  return 5 * sizeof(float4) + sizeof(uint2) + 2 * sizeof(uint32_t) +
         static_cast<size_t>(slots) * (2 * sizeof(float4) + sizeof(uint32_t));
}

uint32_t render_batch_samples(int width, int height, int ns_aa, int slots, uint32_t budget_mib) {
  const size_t px = static_cast<size_t>(width) * height;
  const size_t budget = static_cast<size_t>(budget_mib ? budget_mib : 2048) << 20;
  const size_t per = std::max<size_t>(1, budget / (render_path_bytes(slots) * std::max<size_t>(px, 1)));
  return static_cast<uint32_t>(std::min<size_t>(per, static_cast<size_t>(ns_aa)));
}

cudaError_t launch_render(const RTri* tri, const RNrm* nrm, uint32_t n_scene, uint32_t n_surf,
                          const BvhNode* scene_nodes, const RTri* scene_ltri, const BvhNode* surf_nodes,
                          const RTri* surf_ltri, const RMat* mats, const RLight* lights, const RCam& cam,
                          const RArgs& a, const WfBuffers& wb, float* hdr, unsigned* err, cudaStream_t s) {
  const size_t px = static_cast<size_t>(a.width) * a.height;
  if (px == 0) return cudaSuccess;
  const Scene sc{tri, nrm, mats, lights, n_scene, n_surf, scene_nodes, scene_ltri, surf_nodes, surf_ltri};
  int dev = 0, sms = 0, per_trace = 0, per_shade = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_trace, k_wf_trace<false>, 128, 0);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_shade, k_wf_shade, 128, 0);
  if (e != cudaSuccess) return e;
  const unsigned g_trace = static_cast<unsigned>(std::max(1, sms * std::max(per_trace, 1)));
  const unsigned g_shade = static_cast<unsigned>(std::max(1, sms * std::max(per_shade, 1)));
  const unsigned g_res = static_cast<unsigned>(std::max(1, sms * 8));
  const uint32_t nb = static_cast<uint32_t>(std::max(a.batch, 1));
  for (int s0 = 0; s0 < a.ns_aa; s0 += static_cast<int>(nb)) {
    const int cnt = std::min(static_cast<int>(nb), a.ns_aa - s0);
    const uint32_t paths = static_cast<uint32_t>(px * static_cast<size_t>(cnt));
    k_wf_camera<<<blocks(paths, 128), 128, 0, s>>>(wb, cam, a, s0, paths);
    for (int level = 0; level <= a.max_depth; ++level) {
      const int cur = level & 1;
      const uint32_t* qin = cur ? wb.qb : wb.qa;
      uint32_t* qout = cur ? wb.qa : wb.qb;
      k_wf_reset<<<1, 1, 0, s>>>(wb.cnt, 1 - cur);
      k_wf_trace<false><<<g_trace, 128, 0, s>>>(sc, wb, qin, wb.cnt + cur, wb.cnt + 3, a.ray_eps, err);
      k_wf_shade<<<g_shade, 128, 0, s>>>(sc, wb, a, s0, qin, wb.cnt + cur, qout, wb.cnt + 1 - cur);
      k_wf_trace<true><<<g_trace, 128, 0, s>>>(sc, wb, wb.sq, wb.cnt + 2, wb.cnt + 4, a.ray_eps, err);
      k_wf_resolve<<<g_res, 256, 0, s>>>(wb, qin, wb.cnt + cur);
    }
    k_accumulate<<<blocks(px, 256), 256, 0, s>>>(wb.L, static_cast<uint32_t>(px), cnt, s0 == 0, s0 + cnt >= a.ns_aa,
                                                 a.ns_aa, hdr);
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_tonemap(const float* hdr, int width, int height, uint8_t* rgba, cudaStream_t s) {
  const size_t px = static_cast<size_t>(width) * height;
  if (px == 0) return cudaSuccess;
  k_tonemap<<<blocks(px, 256), 256, 0, s>>>(hdr, width, height, rgba);
  return cudaGetLastError();
}

}  // namespace pbf
