// Path tracer of the fluid and its scene (PathTracer, src/pathtracer.cpp): device
// layouts and launchers shared by pbf_render.cu and the C ABI (pbf_api.cu).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>

namespace pbf {

// BSDF and light kinds as the C ABI numbers them (src/bsdf.h, src/static_scene/light.h)
enum { kMatDiffuse = 0, kMatMirror = 1, kMatGlass = 2, kMatRefraction = 3, kMatEmission = 4 };
enum { kLightDirectional = 0, kLightHemisphere = 1, kLightPoint = 2, kLightArea = 3 };

// A triangle for the ray test: its vertices, the material index in p1.w (int bits).
struct RTri {
  float4 p1, p2, p3;
};
// Its vertex normals, read only at the closest hit.
struct RNrm {
  float4 n1, n2, n3;
};
// Internal node of the BVH: the boxes of both children; lo_l.w / lo_r.w hold the child
// index (int bits), leaves (triangles) tagged with kLeafBit.
struct BvhNode {
  float4 lo_l, hi_l, lo_r, hi_r;
};
constexpr uint32_t kLeafBit = 0x80000000u;
constexpr int kBvhStack = 64;

struct RMat {
  int kind;
  float c1[3], c2[3];
  float ior;
};

struct RLight {
  int kind;
  float rad[3];
  float pos[3];
  float dir[3];  // area: direction; directional: unit vector towards the light
  float dx[3], dy[3];
  float area;
};

struct RCam {
  float pos[3];
  float c2w[9];  // columns: screen x, screen y, view direction reversed
  float htan, vtan, nclip, fclip;
};

struct RArgs {
  int width, height, ns_aa, max_depth, ns_area;
  int n_mat, n_light;
  unsigned long long seed;
  int batch;      // samples per pixel per batch (render_batch_samples)
  float ray_eps;  // start of secondary rays (the reference's EPS_D is below FP32 resolution)
};

// Scratch of one BVH build over n triangles (device pointers, sized by the caller):
// keys / vals / keys2 / vals2 n each (after the build vals maps a leaf's sorted position
// to its triangle), hist 256 * sort_blocks(n), start 256 * sort_blocks(n) + 1,
// tile_sums exclusive_scan_tiles(256 * sort_blocks(n)), parent 2n - 1, flags n - 1,
// box_lo / box_hi 2n - 1, bounds 2 + 2 * kBoundsBlocks float4; ltri n: the triangles in
// leaf order, p1.w holding each one's index in the build's range (int bits), so a leaf
// visit reads its triangle without a dependent index load.
struct BvhScratch {
  uint32_t *keys, *vals, *keys2, *vals2, *hist, *start, *tile_sums, *parent, *flags;
  float4 *box_lo, *box_hi, *bounds;
  RTri* ltri;
};
uint32_t sort_blocks(uint32_t n);
constexpr int kBoundsBlocks = 128;

// The handle's renderer: the scene (device copies) and grow-only buffers of the last frame.
struct RenderState {
  RTri* scene_tri = nullptr;
  RNrm* scene_nrm = nullptr;
  uint32_t n_scene = 0;
  RMat* mats_host = nullptr;  // n_mat scene materials (host), the fluid's appended per frame
  RLight* lights_host = nullptr;
  int n_mat = 0, n_light = 0;
  void* buf = nullptr;  // per frame: triangles, hierarchy, build scratch, image
  size_t buf_bytes = 0;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  void release();
};

cudaError_t launch_surface_to_tris(const float* xyz, const float* nrm, uint32_t m, int material, RTri* tri,
                                   RNrm* nn, cudaStream_t s);
cudaError_t launch_bvh_build(const RTri* tri, uint32_t n, const BvhScratch& w, BvhNode* nodes, cudaStream_t s);
// Path state of one batch (wavefront), device arrays: per path o (next ray origin, w
// tmin), d (direction, w tmax), beta (throughput, w 1 when the next hit adds emission), L
// (radiance), hit (x triangle as int bits or -1, y t, z u, w v), st (x depth left, y draws
// used), queues qa / qb; per path and bounce `slots` shadow-ray slots sdir (direction, w
// distance) and scon (contribution, w 1 when visible) with their queue sq; cnt[8] counters.
struct WfBuffers {
  float4 *o, *d, *beta, *L, *hit, *sdir, *scon;
  uint2* st;
  uint32_t *qa, *qb, *sq, *cnt;
  int slots;
};
// Shadow-ray slots per path and bounce: one per delta light, ns_area per other light.
int render_slots(const RLight* lights, int n_light, int ns_area);
size_t render_path_bytes(int slots);
// Samples per pixel traced in one batch, the batch's path state within budget_mib MiB
// (0: 2048).
uint32_t render_batch_samples(int width, int height, int ns_aa, int slots, uint32_t budget_mib);
// hdr: W * H * 3 floats, row y = 0 first (the bottom row, as the reference's sample buffer).
// tri / nrm: the scene's n_scene triangles, then the surface's n_surf. scene_nodes null:
// the scene's triangles are tested one by one (at most kBruteScene of them). *_ltri: a
// build's leaf-ordered triangles; err bit 0: a traversal stack overflowed (deeper than
// kBvhStack levels).
constexpr uint32_t kBruteScene = 32;
cudaError_t launch_render(const RTri* tri, const RNrm* nrm, uint32_t n_scene, uint32_t n_surf,
                          const BvhNode* scene_nodes, const RTri* scene_ltri, const BvhNode* surf_nodes,
                          const RTri* surf_ltri, const RMat* mats, const RLight* lights, const RCam& cam,
                          const RArgs& a, const WfBuffers& wb, float* hdr, unsigned* err, cudaStream_t s);
// rgba: W * H * 4 bytes, rows flipped (top first) as PathTracer::save_image writes them.
cudaError_t launch_tonemap(const float* hdr, int width, int height, uint8_t* rgba, cudaStream_t s);

}  // namespace pbf
