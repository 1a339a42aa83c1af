// Internal types shared by the PBF CUDA translation units.
//
// Data layout in HBM (N particles, C cells over all scenes), all arrays in the
// cell-sorted order of the current step unless noted:
//   pos    float4  x (w: scene id as int bits)             16 B
//   disp   float4  delta = x* - x (displacement form)       16 B
//   xs[2]  float4  x* ping-pong over the Jacobi iterations  16 B each
//   vel    float4  v                                        16 B
//   omega  float4  vorticity (w: |omega|)                   16 B
//   lam    float   lambda                                    4 B
//   rho    float   reported density                          4 B
//   id     u32     original particle index                   4 B
//   nbr_hdr uint4  first candidate slot of z-slab 0, the other two slabs' first slots
//                  relative to it (less the entries' tag bits), neighbour count
//   nbr_w   u32    [words/4][N][4] neighbour entries, 2 x u16 per word, in groups of 4 words
//   cell_count / cell_start u32 [C] / [C+1]
#pragma once

#include <cstddef>
#include <cstdint>

#include <cuda_runtime.h>

#include "../../include/pbf.h"

namespace pbf {

constexpr int kMaxRowCandidates = 4096;  // bound on the candidates scanned in one 3-cell row
constexpr int kNeighborAlert = 18;      // NUM_NEIGHBOR_ALERT_THRESHOLD, particles.cpp:32
constexpr float kEps = 1e-11f;          // EPS_D, CGL/include/CGL/misc.h:11
// Margin of the collider's interior box and clip planes, relative to the largest coordinate
// of the walls, the clamp box or the planes (at least 1): about 1,000 FP32 ulps of it.
constexpr double kInteriorMargin = 1e-4;

// Per-scene collider and grid (device table, one entry per scene).
struct SceneDesc {
  float lo[3], hi[3];       // collider walls
  float origin[3];          // grid origin
  int dim[3];               // grid cells per axis
  uint32_t cell_off;        // first global cell id
  uint32_t p_off, p_cnt;    // particle range in original order
  float in_lo[3], in_hi[3];  // interior box: the closed walls and the clamp box, shrunk by a
                             // margin (a move that stays inside it touches neither)
};

// Uniform physics parameters in FP32, derived on the host from pbf_params.
struct DevParams {
  float h, h2, inv_cell, cell;
  float poly6_c;     // 1.56668147106 / h^9            (particles.cpp:140)
  float spiky_c;     // -3 * 4.774648292756860 / h^6  (particles.cpp:148)
  float tis;         // 1 / W(scorr_dq * h)           (particles.cpp:151)
  float scorr_k, epsilon, rest_density, inv_rho0;
  float xsph_c, vort_eps;
  float g[3];
  float clip_value[2];
  float clamp_lo[3], clamp_hi[3];
  float clip_margin;  // a move that keeps this far from every clip plane crosses none
  int scorr_n, n_clip, clip_axis[2], open_mask, max_words;
  int stats;
  int n_mesh;                // collider triangles besides the box walls (pbf_set_collider_mesh)
  const float4* mesh;        // 4 float4 per triangle, in hierarchy leaf order: p1, p2 - p1,
                             // p3 - p1, normal (w: the triangle's index as given, int bits)
  const float4* mesh_nodes;  // bounding-volume hierarchy over the triangles, 2 float4 per node:
                             // lo (w: a), hi (w: b) as int bits; b < 0: leaf of triangles
                             // [a, a - b), else children a and b; node 0 is the root
  int n_sph;                 // collider spheres (pbf_set_collider_spheres)
  const float4* sph;         // centre xyz, radius w
};
constexpr int kMaxMeshTriangles = 1 << 22;
constexpr int kMaxSpheres = 1024;
constexpr int kMeshLeafSize = 4;     // triangles per hierarchy leaf (at most)
constexpr int kMeshMaxDepth = 40;    // hierarchy depth bound (the walk's stack holds one entry per level)

// Step statistics accumulated on the device (reset every step).
struct DevStats {
  double rho_iter0_sum;
  double rho_sum;
  double err_sum;
  unsigned int err_max_bits;   // float bits of max |rho/rho0 - 1| (non-negative)
  unsigned int nbr_min;
  unsigned int nbr_max;
  unsigned int pad;
  unsigned long long nbr_sum;
  unsigned long long low_cnt;
};

struct Buffers {
  size_t n = 0;
  int n_scenes = 0;
  uint32_t n_cells = 0;
  int max_words = 0;
  float4* pos[2] = {nullptr, nullptr};
  float4* disp[2] = {nullptr, nullptr};
  float4* xs[2] = {nullptr, nullptr};
  float4* vel[2] = {nullptr, nullptr};
  float4* omega = nullptr;
  float4* pred = nullptr;  // optional copy of x* after prediction (sorted order)
  uint32_t* xkey = nullptr;  // order_bits(x*.x) per pre-sort slot (cell sort key)
  float* rho = nullptr;
  float* rho_iter0 = nullptr;  // density after the first lambda pass (stats)
  uint32_t* id[2] = {nullptr, nullptr};
  uint32_t* key = nullptr;
  uint32_t* rank = nullptr;
  uint32_t* perm = nullptr;         // slot -> pre-sort slot, cells ordered by x
  uint32_t* perm_atomic = nullptr;  // the same in the per-cell atomic order of the counts
  uint4* nbr_hdr = nullptr;
  uint32_t* nbr_w = nullptr;
  uint32_t* cell_count = nullptr;
  uint32_t* cell_start = nullptr;  // n_cells + 1
  uint32_t* scan_tmp = nullptr;    // block sums
  uint32_t* big_cells = nullptr;   // cells over kSmallCell particles this step (worklist)
  uint32_t* big_count = nullptr;   // entries in big_cells
  SceneDesc* scenes = nullptr;
  DevStats* stats = nullptr;
  DevStats* stats_part = nullptr;  // per-block partial records of the stats pass
  unsigned int* err = nullptr;     // sticky PBF_ERRBIT_* word
  float* io = nullptr;             // (n, 3) staging for host/device packed transfers
  float* io2 = nullptr;
};

// Recording of one step for its reverse mode, plus the adjoint work arrays (cell
// order of that step; allocated on the first adjoint call).
struct Tape {
  size_t n = 0;
  int iters = 0;
  float4* x = nullptr;    // step input x (w: scene id bits)
  float4* v = nullptr;    // step input v (w: the prediction's collision record)
  float4* xs = nullptr;   // (iters + 1) n: x* before each iteration (w: lambda),
                          // then the final x* (w: |omega|)
  float4* dp = nullptr;   // iters n: requested displacement (w: collision record)
  float4* eta = nullptr;  // vorticity location vector eta of the step
  float4* gxs = nullptr;  // adjoint of the current x*
  float4* pl[2] = {nullptr, nullptr};  // (adjoint of the unscaled delta-p sum, lambda), ping-pong
  float4* gr = nullptr;   // (sum of grad W / rho0, adjoint of rho)
  float4* gvo = nullptr;  // adjoint of the output velocity
  float4* gx = nullptr;   // adjoint of the input x
  float4* wb = nullptr;   // adjoint of omega
  float4* eb = nullptr;   // adjoint of eta (vorticity location vector)
  float* r0 = nullptr;    // per-particle parts of the rest-density adjoint
  double* r0_part = nullptr;  // block sums of r0
};
constexpr int kAdjReduceBlocks = 256;
constexpr int kStatsBlocks = 256;  // partial records of the step statistics pass

// Marching-cubes triangulation table (pbf_surface.cu): for every cube configuration
// (bit k set when corner k is below the iso level) the crossing edges, the triangle
// count and the triangles as edge triples.
struct SurfTable {
  uint16_t edges[256];
  uint8_t ntri[256];
  int8_t tri[256][15];
};
// The surface grid of Particles::getSurfacePrims: cubes [x1, min(hi, x1 + step)] with
// x1 = lo + i step, i = 0 .. nc - 1 per axis (nc = (int)((hi - lo) / step) + 1).
struct SurfGrid {
  double lo[3], hi[3], step;
  int nc[3];
  // device: the corner coordinates per axis, float(min(lo + i step, hi)) computed in FP64
  // on the host (x: nc[0] + 1 values, then y, then z), so no kernel needs FP64
  const float* axis = nullptr;
};
void build_table(SurfTable* t);
const SurfTable& surf_table();

// Launch shapes and kernel forms picked by the autotuner (threads per block per kernel
// family; the neighbour passes' gather depth and list-load policy).
struct Tuning {
  int block_predict = 256;
  int block_nbr = 128;
  int block_solve = 128;
  int block_misc = 256;
  int gather_depth = 8;  // neighbour loads in flight per thread in the neighbour passes (4 or 8)
  int list_stream = 0;   // 1: neighbour-list words loaded with the streaming cache policy
};

// Phases of a step for CUDA-event timing (pbf_get_phase_times).
enum Phase {
  kPhasePredict = 0,
  kPhaseScan,
  kPhaseSort,
  kPhaseGather,
  kPhaseNeighbors,
  kPhaseLambda,
  kPhaseDeltaP,
  kPhaseXsph,
  kPhaseVorticity,
  kPhaseStats,
  kNumPhases
};

// Events recorded between phases of one step (optional).
struct PhaseMarks {
  cudaEvent_t* ev = nullptr;
  int* phase = nullptr;
  int count = 0;
  int cap = 0;
  bool in_graph = false;  // recorded while capturing a graph: event-record nodes
  void mark(int ph, cudaStream_t s) {
    if (ev && count < cap) {
      if (in_graph)
        cudaEventRecordWithFlags(ev[count], s, cudaEventRecordExternal);
      else
        cudaEventRecord(ev[count], s);
      phase[count] = ph;
      ++count;
    }
  }
};

// ---- launchers (pbf_kernels.cu) ----
// cur: index of the buffers holding the current (sorted) state; the step
// writes the next state into 1 - cur.
// With a tape, the step is the recording forward of the adjoint (same arithmetic).
cudaError_t launch_step(const Buffers& b, const DevParams& p, const Tuning& t, int cur,
                        float dt, int iters, bool keep_pred, cudaStream_t s,
                        PhaseMarks* marks = nullptr, const Tape* tape = nullptr);
// ---- reverse mode (pbf_adjoint.cu) ----
// After launch_step(..., tape) from buffers cur (the step's output now in 1 - cur):
// adjoints of the step's inputs from those of its outputs, all original order
// (n, 3) device arrays; gx_out / gv_out may be null (zero); *g_rho0 (device) receives
// the rest-density adjoint.
cudaError_t launch_adjoint(const Buffers& b, const DevParams& p, const Tuning& t, int cur, float dt,
                           const Tape& tape, const float* gx_out, const float* gv_out, float* gx_in,
                           float* gv_in, double* g_rho0, cudaStream_t s);
cudaError_t launch_resort(const Buffers& b, const DevParams& p, const Tuning& t, int cur,
                          cudaStream_t s);
cudaError_t launch_upload(const Buffers& b, int cur, const float* xyz, const float* vel,
                          const uint32_t* scene_of, cudaStream_t s);
cudaError_t launch_download(const Buffers& b, int cur, float* xyz, float* vel, float* rho,
                            cudaStream_t s);
cudaError_t launch_unsort_u32(const Buffers& b, int cur, const uint32_t* src, uint32_t* dst,
                              cudaStream_t s);
cudaError_t launch_unsort_f4(const Buffers& b, int cur, const float4* src, float* dst_xyz,
                             cudaStream_t s);
cudaError_t launch_cells_of(const Buffers& b, const DevParams& p, int cur, uint32_t* cells,
                            cudaStream_t s);
cudaError_t launch_neighbor_ids(const Buffers& b, int cur, const uint32_t* offsets,
                                uint32_t* ids, cudaStream_t s);
cudaError_t launch_neighbor_counts(const Buffers& b, int cur, uint32_t* counts, cudaStream_t s);
cudaError_t launch_density_self(const Buffers& b, const DevParams& p, const Tuning& t, int cur,
                                float* rho_sorted, cudaStream_t s);
// Exclusive prefix sum of count[0, m) into start[0, m] (start[m] = total);
// tile_sums holds exclusive_scan_tiles(m) entries of scratch.
cudaError_t launch_exclusive_scan(const uint32_t* count, uint32_t* start, uint32_t* tile_sums, uint32_t m,
                                  cudaStream_t s);
uint32_t exclusive_scan_tiles(uint32_t m);
cudaError_t launch_density_at(const Buffers& b, const DevParams& p, int cur, size_t m,
                              const float* pts, float* out, cudaStream_t s);
// ---- surface (pbf_surface.cu), on the cell-sorted state in buffers cur ----
// field: (nc+1)^3 corner values; count: per-cube triangle counts; first: their exclusive
// scan (first[cubes] = total); tile_sums: exclusive_scan_tiles(cubes) entries.
cudaError_t launch_surface_count(const Buffers& b, const DevParams& p, int cur, const SurfGrid& g, float iso,
                                 const SurfTable* tab, float* field, uint32_t* count, uint32_t* first,
                                 uint32_t* tile_sums, cudaStream_t s);
// Scratch of launch_surface_emit for cap triangles: keys and nslot hold
// surface_hash_slots(cap) entries, vslot and ulist 3 * cap, ucount one.
struct SurfHash {
  unsigned long long* keys;
  float4* nslot;
  uint32_t *vslot, *ulist, *ucount;
};
uint32_t surface_hash_slots(uint32_t triangles);
// Triangles with index < cap (cap at most the total of the counts): 9 floats of vertices
// and 9 of vertex normals each. Each vertex normal is evaluated once per grid edge.
cudaError_t launch_surface_emit(const Buffers& b, const DevParams& p, int cur, const SurfGrid& g, float iso,
                                const SurfTable* tab, const float* field, const uint32_t* first, float* xyz,
                                float* nrm, uint32_t cap, const SurfHash& hs, cudaStream_t s);

}  // namespace pbf
