// The object behind a pbf_handle*: parameters, device buffers, stream, graphs.
#pragma once

#include <string>
#include <vector>

#include "pbf_internal.h"
#include "pbf_render.h"

namespace pbf {

struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(int dev);
  ~DeviceGuard();
};

// Message returned by pbf_last_error(NULL) on this thread.
void set_global_error(const std::string& msg);

bool make_dev_params(const pbf_params& p, DevParams* d, double* cell_out, std::string* why);
bool make_scene(const pbf_params& p, double cell, const float* lo, const float* hi, SceneDesc* sc,
                std::string* why);

struct Handle {
  int device = 0;
  cudaStream_t stream = nullptr;
  pbf_params params{};
  DevParams dp{};
  Buffers b;
  Tuning tune;
  std::vector<SceneDesc> scenes_host;
  int cur = 0;               // buffers holding the current state
  uint64_t steps = 0;
  double simulate_time = 0;  // Particles::simulate_time
  bool nbr_valid = false;    // neighbour lists / x* copy describe the current order
  std::string err;
  unsigned host_err_word = 0;
  cudaGraphExec_t graph[2] = {nullptr, nullptr};  // one step starting from buffers 0 / 1
  float graph_dt = -1.f;
  void* scratch = nullptr;   // grow-only scratch for introspection and queries
  size_t scratch_bytes = 0;
  // per-phase CUDA-event timing (pbf_set_profiling)
  bool profiling = false;
  std::vector<std::vector<cudaEvent_t>> prof_events;  // one set per step in flight
  std::vector<std::vector<int>> prof_phase;
  std::vector<int> prof_count;
  size_t prof_used = 0;
  // with PBF_FLAG_GRAPH and profiling: one graph per event set and buffer parity, the
  // phase events being event-record nodes of that graph
  std::vector<cudaGraphExec_t> prof_graph[2];
  std::vector<int> prof_graph_count[2];
  // device-side snapshot (pbf_snapshot / pbf_restore)
  float4* snap_pos = nullptr;
  float4* snap_vel = nullptr;
  uint32_t* snap_id = nullptr;
  bool snap_valid = false;
  uint64_t snap_steps = 0;
  double snap_time = 0;
  Tape tape;                 // recording + work arrays of the adjoint (first use)
  SurfTable* surf_table_dev = nullptr;  // marching-cubes table (first pbf_surface)
  void* surf_hash = nullptr;            // grow-only scratch of the surface's vertex-normal table
  size_t surf_hash_bytes = 0;
  float4* mesh_dev = nullptr;           // collider triangles and their hierarchy (pbf_set_collider_mesh)
  float4* sph_dev = nullptr;            // collider spheres (pbf_set_collider_spheres)
  RenderState render;                   // path tracer (pbf_render_set_scene, pbf_render)
  double phase_ms[kNumPhases] = {};
  uint64_t phase_launches[kNumPhases] = {};

  pbf_status fail(pbf_status st, const std::string& msg);
  pbf_status cuda(cudaError_t e, const char* what);
  pbf_status alloc_all();
  void free_all();
  pbf_status ensure_scratch(size_t bytes);
  pbf_status ensure_tape();
  void free_tape();
  pbf_status surface_count(double isolevel, double step, const double* lo, const double* hi, SurfGrid* g,
                           uint32_t* total);
  pbf_status surface_emit(const SurfGrid& g, double isolevel, float* xyz, float* nrm, uint32_t cap);
  pbf_status enqueue_steps(float dt, int nsteps);
  pbf_status sync_and_check();
  void drop_graphs();
  PhaseMarks next_marks();
  pbf_status collect_phase_times();
  void free_profiling();

  // Order the handle's stream after `other` (or the legacy default stream
  // when other is null), and back.
  pbf_status join_from(cudaStream_t other) {
    cudaEvent_t ev;
    pbf_status st = cuda(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
    if (st != PBF_OK) return st;
    st = cuda(cudaEventRecord(ev, other), "event record");
    if (st == PBF_OK) st = cuda(cudaStreamWaitEvent(stream, ev, 0), "stream wait");
    cudaEventDestroy(ev);
    return st;
  }
  pbf_status join_to(cudaStream_t other) {
    cudaEvent_t ev;
    pbf_status st = cuda(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming), "event");
    if (st != PBF_OK) return st;
    st = cuda(cudaEventRecord(ev, stream), "event record");
    if (st == PBF_OK) st = cuda(cudaStreamWaitEvent(other, ev, 0), "stream wait");
    cudaEventDestroy(ev);
    return st;
  }
};

}  // namespace pbf
