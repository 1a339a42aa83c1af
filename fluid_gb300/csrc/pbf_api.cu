// C ABI of the PBF step (include/pbf.h): handle lifetime, device memory,
// stream and CUDA-graph management, host/device transfers, introspection.
#include <algorithm>
#include <array>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "pbf_handle.h"

namespace {

thread_local std::string g_create_error;

double ipow(double b, int e) {
  double r = 1;
  for (int i = 0; i < e; ++i) r = r * b;
  return r;
}

// poly6 of the reference (particles.cpp:134-141) in FP64, for derived constants.
double poly6_ref(double r2, double h, double h2) {
  if (r2 >= h2) return 0.0;
  const double t = h2 - r2;
  return 1.56668147106 * ipow(t, 3) / ipow(h, 9);
}

}  // namespace

namespace pbf {

void set_global_error(const std::string& msg) { g_create_error = msg; }

pbf_status Handle::fail(pbf_status st, const std::string& msg) {
  err = msg;
  return st;
}

pbf_status Handle::cuda(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return PBF_OK;
  err = std::string(what) + ": " + cudaGetErrorString(e);
  (void)cudaGetLastError();
  return e == cudaErrorMemoryAllocation ? PBF_ERR_NOMEM : PBF_ERR_CUDA;
}

DeviceGuard::DeviceGuard(int dev) {
  if (cudaGetDevice(&prev) != cudaSuccess) prev = -1;
  if (prev != dev) cudaSetDevice(dev);
}
DeviceGuard::~DeviceGuard() {
  if (prev >= 0) cudaSetDevice(prev);
}

bool make_dev_params(const pbf_params& p, DevParams* d, double* cell_out, std::string* why) {
  if (!(p.h > 0) || !(p.h2 > 0) || !std::isfinite(p.h) || !std::isfinite(p.h2)) {
    *why = "h and h2 must be positive and finite";
    return false;
  }
  if (p.iters < 0 || p.iters > 1000) {
    *why = "iters must be in [0, 1000]";
    return false;
  }
  if (p.scorr_n < 1 || p.scorr_n > 16) {
    *why = "scorr_n must be in [1, 16]";
    return false;
  }
  if (!(p.rest_density > 0) || !std::isfinite(p.rest_density)) {
    *why = "rest_density must be positive";
    return false;
  }
  if (p.n_clip < 0 || p.n_clip > 2) {
    *why = "n_clip must be 0, 1 or 2";
    return false;
  }
  for (int c = 0; c < p.n_clip; ++c)
    if (p.clip_axis[c] < 0 || p.clip_axis[c] > 2) {
      *why = "clip_axis must be 0, 1 or 2";
      return false;
    }
  const int max_nbr = p.max_neighbors == 0 ? 128 : p.max_neighbors;
  if (max_nbr < 4 || max_nbr > 1024) {
    *why = "max_neighbors must be in [4, 1024]";
    return false;
  }
  std::memset(d, 0, sizeof(*d));
  const double cell = std::sqrt(p.h2) * 1.001;
  *d = DevParams();
  d->h = static_cast<float>(p.h);
  d->h2 = static_cast<float>(p.h2);
  d->cell = static_cast<float>(cell);
  d->inv_cell = static_cast<float>(1.0 / cell);
  d->poly6_c = static_cast<float>(1.56668147106 / ipow(p.h, 9));
  d->spiky_c = static_cast<float>(-3 * 4.774648292756860 / ipow(p.h, 6));
  const double dq = p.scorr_dq * p.h;
  d->tis = static_cast<float>(1.0 / poly6_ref(dq * dq, p.h, p.h2));
  d->scorr_k = static_cast<float>(p.scorr_k);
  d->epsilon = static_cast<float>(p.epsilon);
  d->rest_density = static_cast<float>(p.rest_density);
  d->inv_rho0 = static_cast<float>(1.0 / p.rest_density);
  d->xsph_c = static_cast<float>(p.xsph_c);
  d->vort_eps = static_cast<float>(p.vort_eps);
  for (int k = 0; k < 3; ++k) {
    d->g[k] = static_cast<float>(p.gravity[k]);
    d->clamp_lo[k] = static_cast<float>(p.clamp_lo[k]);
    d->clamp_hi[k] = static_cast<float>(p.clamp_hi[k]);
  }
  d->n_clip = p.n_clip;
  double clip_scale = 1.0;
  for (int c = 0; c < p.n_clip; ++c) {
    d->clip_axis[c] = p.clip_axis[c];
    d->clip_value[c] = static_cast<float>(p.clip_value[c]);
    clip_scale = std::max(clip_scale, std::fabs(p.clip_value[c]));
  }
  d->clip_margin = static_cast<float>(kInteriorMargin * clip_scale);
  d->scorr_n = p.scorr_n;
  d->open_mask = p.box_open_mask;
  d->max_words = (max_nbr + 1) / 2;
  d->stats = (p.flags & PBF_FLAG_STATS) ? 1 : 0;
  *cell_out = cell;
  return true;
}

// Grid of one scene: the collider box (extended to the clamp box across open
// faces) plus one margin cell on each side.
bool make_scene(const pbf_params& p, double cell, const float* lo, const float* hi, SceneDesc* sc,
                std::string* why) {
  std::memset(sc, 0, sizeof(*sc));
  for (int a = 0; a < 3; ++a) {
    if (!(hi[a] > lo[a])) {
      *why = "box_hi must exceed box_lo on every axis";
      return false;
    }
    double e0 = lo[a], e1 = hi[a];
    if (p.box_open_mask & (1 << (2 * a))) e0 = std::min(e0, p.clamp_lo[a]);
    if (p.box_open_mask & (1 << (2 * a + 1))) e1 = std::max(e1, p.clamp_hi[a]);
    sc->lo[a] = lo[a];
    sc->hi[a] = hi[a];
    sc->origin[a] = static_cast<float>(e0 - cell);
    const double dim = std::ceil((e1 - e0) / cell) + 2.0;
    const double lim = a == 0 ? 1024.0 : 2048.0;
    if (!(dim <= lim)) {
      *why = "grid too fine for the box: at most 1024 x 2048 x 2048 cells of size h";
      return false;
    }
    sc->dim[a] = static_cast<int>(dim);
  }
  // Interior box (collide's shortcut): inside the closed walls and the clamp box by a margin
  // of kInteriorMargin times the largest coordinate among them (at least 1). A move whose
  // ends both lie inside it stops at no wall by more than the FP32 rounding of the stop
  // distances, and no coordinate is clamped. A box left empty (in_lo >= in_hi) takes no move.
  double scale = 1.0;
  for (int a = 0; a < 3; ++a)
    scale = std::max({scale, std::fabs(static_cast<double>(lo[a])), std::fabs(static_cast<double>(hi[a])),
                      std::fabs(p.clamp_lo[a]), std::fabs(p.clamp_hi[a])});
  const double m = kInteriorMargin * scale;
  for (int a = 0; a < 3; ++a) {
    double ilo = p.clamp_lo[a], ihi = p.clamp_hi[a];
    if (!(p.box_open_mask & (1 << (2 * a)))) ilo = std::max(ilo, static_cast<double>(lo[a]));
    if (!(p.box_open_mask & (1 << (2 * a + 1)))) ihi = std::min(ihi, static_cast<double>(hi[a]));
    sc->in_lo[a] = static_cast<float>(ilo + m);
    sc->in_hi[a] = static_cast<float>(ihi - m);
  }
  return true;
}

void Handle::free_all() {
  DeviceGuard g(device);
  for (int k = 0; k < 2; ++k) {
    if (graph[k]) cudaGraphExecDestroy(graph[k]);
    graph[k] = nullptr;
  }
  void* ptrs[] = {b.pos[0], b.pos[1], b.disp[0], b.disp[1], b.xs[0], b.xs[1], b.vel[0], b.vel[1],
                  b.omega, b.pred, b.xkey, b.rho, b.rho_iter0, b.id[0], b.id[1], b.key, b.rank,
                  b.perm, b.perm_atomic, b.nbr_hdr, b.nbr_w, b.cell_count, b.cell_start, b.scan_tmp, b.big_cells, b.big_count, b.scenes, b.stats_part,
                  b.stats, b.err, b.io, b.io2, scratch, snap_pos, snap_vel, snap_id};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  b = Buffers();
  free_tape();
  if (surf_table_dev) cudaFree(surf_table_dev);
  surf_table_dev = nullptr;
  if (surf_hash) cudaFree(surf_hash);
  surf_hash = nullptr;
  surf_hash_bytes = 0;
  if (mesh_dev) cudaFree(mesh_dev);
  mesh_dev = nullptr;
  if (sph_dev) cudaFree(sph_dev);
  sph_dev = nullptr;
  render.release();
  snap_pos = snap_vel = nullptr;
  snap_id = nullptr;
  snap_valid = false;
  free_profiling();
  scratch = nullptr;
  scratch_bytes = 0;
  if (stream) cudaStreamDestroy(stream);
  stream = nullptr;
}

pbf_status Handle::alloc_all() {
  const size_t n = b.n ? b.n : 1;
  const size_t f4 = sizeof(float4) * n, u4 = sizeof(uint32_t) * n;
  struct A {
    void** p;
    size_t bytes;
  } list[] = {
      {(void**)&b.pos[0], f4}, {(void**)&b.pos[1], f4}, {(void**)&b.disp[0], f4}, {(void**)&b.disp[1], f4},
      {(void**)&b.xs[0], f4}, {(void**)&b.xs[1], f4}, {(void**)&b.vel[0], f4}, {(void**)&b.vel[1], f4},
      {(void**)&b.omega, f4}, {(void**)&b.xkey, u4}, {(void**)&b.rho, u4}, {(void**)&b.rho_iter0, u4},
      {(void**)&b.id[0], u4}, {(void**)&b.id[1], u4}, {(void**)&b.key, u4}, {(void**)&b.rank, u4},
      {(void**)&b.perm, u4}, {(void**)&b.perm_atomic, u4}, {(void**)&b.nbr_hdr, sizeof(uint4) * n},
      {(void**)&b.nbr_w, u4 * static_cast<size_t>((b.max_words + 3) / 4 * 4)},  // groups of 4 words
      {(void**)&b.cell_count, sizeof(uint32_t) * b.n_cells},
      {(void**)&b.cell_start, sizeof(uint32_t) * (b.n_cells + 1)},
      {(void**)&b.scan_tmp, sizeof(uint32_t) * ((b.n_cells + 1023) / 1024 + 1)},
      {(void**)&b.big_cells, sizeof(uint32_t) * (b.n_cells ? b.n_cells : 1)},
      {(void**)&b.big_count, sizeof(uint32_t)},
      {(void**)&b.scenes, sizeof(SceneDesc) * b.n_scenes}, {(void**)&b.stats, sizeof(DevStats)},
      {(void**)&b.stats_part, sizeof(DevStats) * kStatsBlocks},
      {(void**)&b.err, sizeof(unsigned)}, {(void**)&b.io, 3 * sizeof(float) * n},
      {(void**)&b.io2, 3 * sizeof(float) * n},
  };
  for (auto& a : list) {
    pbf_status st = cuda(cudaMalloc(a.p, a.bytes), "cudaMalloc");
    if (st != PBF_OK) return st;
  }
  if (params.flags & PBF_FLAG_KEEP_PREDICTED) {
    pbf_status st = cuda(cudaMalloc((void**)&b.pred, f4), "cudaMalloc");
    if (st != PBF_OK) return st;
  }
  pbf_status st = cuda(cudaMemsetAsync(b.scan_tmp, 0, sizeof(uint32_t) * ((b.n_cells + 1023) / 1024 + 1), stream),
                       "cudaMemsetAsync");  // the scan's ticket word (after the tile sums) starts at zero
  if (st != PBF_OK) return st;
  return cuda(cudaMemsetAsync(b.err, 0, sizeof(unsigned), stream), "cudaMemsetAsync");
}

void Handle::free_tape() {
  void* ptrs[] = {tape.x, tape.v, tape.xs, tape.dp, tape.eta, tape.gxs, tape.pl[0], tape.pl[1], tape.gr,
                  tape.gvo, tape.gx, tape.wb, tape.eb, tape.r0, tape.r0_part};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  tape = Tape();
}

pbf_status Handle::ensure_tape() {
  if (tape.x && tape.n == b.n && tape.iters == params.iters) return PBF_OK;
  free_tape();
  const size_t n = b.n ? b.n : 1;
  const size_t f4 = sizeof(float4) * n;
  const size_t it = static_cast<size_t>(params.iters);
  struct A {
    void** p;
    size_t bytes;
  } list[] = {
      {(void**)&tape.x, f4}, {(void**)&tape.v, f4}, {(void**)&tape.xs, f4 * (it + 1)},
      {(void**)&tape.dp, f4 * (it ? it : 1)}, {(void**)&tape.eta, f4}, {(void**)&tape.gxs, f4}, {(void**)&tape.pl[0], f4},
      {(void**)&tape.pl[1], f4}, {(void**)&tape.gr, f4}, {(void**)&tape.gvo, f4}, {(void**)&tape.gx, f4},
      {(void**)&tape.wb, f4}, {(void**)&tape.eb, f4}, {(void**)&tape.r0, sizeof(float) * n},
      {(void**)&tape.r0_part, sizeof(double) * kAdjReduceBlocks},
  };
  for (auto& a : list) {
    pbf_status st = cuda(cudaMalloc(a.p, a.bytes), "cudaMalloc(adjoint)");
    if (st != PBF_OK) {
      free_tape();
      return st;
    }
  }
  tape.n = b.n;
  tape.iters = params.iters;
  return PBF_OK;
}

pbf_status Handle::ensure_scratch(size_t bytes) {
  if (bytes <= scratch_bytes) return PBF_OK;
  if (scratch) cudaFree(scratch);
  scratch = nullptr;
  scratch_bytes = 0;
  pbf_status st = cuda(cudaMalloc(&scratch, bytes), "cudaMalloc(scratch)");
  if (st == PBF_OK) scratch_bytes = bytes;
  return st;
}

pbf_status Handle::sync_and_check() {
  pbf_status st = cuda(cudaMemcpyAsync(&host_err_word, b.err, sizeof(unsigned), cudaMemcpyDeviceToHost, stream),
                       "read error word");
  if (st != PBF_OK) return st;
  st = cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
  if (st != PBF_OK) return st;
  if (host_err_word & PBF_ERRBIT_NONFINITE) return fail(PBF_ERR_NONFINITE, "a position or velocity became non-finite");
  if (host_err_word & PBF_ERRBIT_NEIGHBOR_CAPACITY)
    return fail(PBF_ERR_CAPACITY, "a particle had more neighbours than max_neighbors");
  if (host_err_word & PBF_ERRBIT_ROW_CAPACITY)
    return fail(PBF_ERR_CAPACITY,
                "more than 4096 particles in one 3-cell row, or a neighbour more than 16383 slots past its "
                "z-slab's first candidate");
  return PBF_OK;
}

PhaseMarks Handle::next_marks() {
  const int cap = 8 + 2 * params.iters + 4;
  if (prof_used == prof_events.size()) {
    std::vector<cudaEvent_t> ev(cap, nullptr);
    for (auto& e : ev) cudaEventCreate(&e);
    prof_events.push_back(ev);
    prof_phase.push_back(std::vector<int>(cap, -1));
    prof_count.push_back(0);
  }
  PhaseMarks m;
  m.ev = prof_events[prof_used].data();
  m.phase = prof_phase[prof_used].data();
  m.cap = static_cast<int>(prof_events[prof_used].size());
  return m;
}

pbf_status Handle::collect_phase_times() {
  if (prof_used == 0) return PBF_OK;
  pbf_status st = cuda(cudaStreamSynchronize(stream), "cudaStreamSynchronize");
  if (st != PBF_OK) return st;
  for (size_t k = 0; k < prof_used; ++k) {
    for (int q = 1; q < prof_count[k]; ++q) {
      float ms = 0.f;
      st = cuda(cudaEventElapsedTime(&ms, prof_events[k][q - 1], prof_events[k][q]), "cudaEventElapsedTime");
      if (st != PBF_OK) return st;
      const int ph = prof_phase[k][q];
      if (ph >= 0 && ph < kNumPhases) phase_ms[ph] += ms;
    }
  }
  prof_used = 0;
  return PBF_OK;
}

void Handle::free_profiling() {
  for (int q = 0; q < 2; ++q) {
    for (auto& g : prof_graph[q])
      if (g) cudaGraphExecDestroy(g);
    prof_graph[q].clear();
    prof_graph_count[q].clear();
  }
  for (auto& set : prof_events)
    for (auto& e : set)
      if (e) cudaEventDestroy(e);
  prof_events.clear();
  prof_phase.clear();
  prof_count.clear();
  prof_used = 0;
}

// Capture one step (launch_step with the given marks) into an executable graph.
static pbf_status capture_step(Handle* h, float dt, bool keep_pred, PhaseMarks* m, cudaGraphExec_t* out) {
  cudaGraph_t g = nullptr;
  pbf_status st = h->cuda(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture");
  if (st != PBF_OK) return st;
  cudaError_t le = launch_step(h->b, h->dp, h->tune, h->cur, dt, h->params.iters, keep_pred, h->stream, m);
  cudaError_t ee = cudaStreamEndCapture(h->stream, &g);
  if (le != cudaSuccess) {
    if (g) cudaGraphDestroy(g);
    return h->cuda(le, "capture step");
  }
  st = h->cuda(ee, "end capture");
  if (st != PBF_OK) return st;
  st = h->cuda(cudaGraphInstantiate(out, g, 0), "instantiate graph");
  cudaGraphDestroy(g);
  return st;
}

pbf_status Handle::enqueue_steps(float dt, int nsteps) {
  const bool use_graph = (params.flags & PBF_FLAG_GRAPH) != 0;
  const bool keep_pred = b.pred != nullptr;
  const int it = params.iters;
  // kernels per phase: k_predict; k_scan_tiles (with the tile sums' scan), k_scan_add; k_scatter,
  // k_cellrank, k_cellsort_big;
  // k_gather; k_nbr_build; k_lambda and k_deltap per iteration; k_xsph; k_vort; k_stats and
  // k_stats_final when statistics are on
  const uint64_t per_step[kNumPhases] = {1, 2, 3, 1, 1, static_cast<uint64_t>(it), static_cast<uint64_t>(it),
                                         1, 1, dp.stats ? 2u : 0u};
  for (int k = 0; k < nsteps; ++k) {
    if (use_graph && graph_dt != dt) {
      drop_graphs();
      graph_dt = dt;
    }
    if (use_graph && profiling) {
      PhaseMarks m = next_marks();
      m.in_graph = true;
      const size_t set = prof_used;
      if (prof_graph[cur].size() <= set) {
        prof_graph[cur].resize(set + 1, nullptr);
        prof_graph_count[cur].resize(set + 1, 0);
      }
      if (!prof_graph[cur][set]) {
        pbf_status st = capture_step(this, dt, keep_pred, &m, &prof_graph[cur][set]);
        if (st != PBF_OK) return st;
        prof_graph_count[cur][set] = m.count;
      }
      pbf_status st = cuda(cudaGraphLaunch(prof_graph[cur][set], stream), "cudaGraphLaunch");
      if (st != PBF_OK) return st;
      prof_count[prof_used++] = prof_graph_count[cur][set];
      for (int q = 0; q < kNumPhases; ++q) phase_launches[q] += per_step[q];
      if (prof_used >= 64) {
        st = collect_phase_times();
        if (st != PBF_OK) return st;
      }
    } else if (use_graph) {
      if (!graph[cur]) {
        pbf_status st = capture_step(this, dt, keep_pred, nullptr, &graph[cur]);
        if (st != PBF_OK) return st;
      }
      pbf_status st = cuda(cudaGraphLaunch(graph[cur], stream), "cudaGraphLaunch");
      if (st != PBF_OK) return st;
    } else if (profiling) {
      PhaseMarks m = next_marks();
      pbf_status st =
          cuda(launch_step(b, dp, tune, cur, dt, params.iters, keep_pred, stream, &m), "launch step");
      if (st != PBF_OK) return st;
      prof_count[prof_used++] = m.count;
      for (int q = 0; q < kNumPhases; ++q) phase_launches[q] += per_step[q];
      if (prof_used >= 256) {
        st = collect_phase_times();
        if (st != PBF_OK) return st;
      }
    } else {
      pbf_status st = cuda(launch_step(b, dp, tune, cur, dt, params.iters, keep_pred, stream), "launch step");
      if (st != PBF_OK) return st;
    }
    cur ^= 1;
    ++steps;
  }
  nbr_valid = nsteps > 0 || nbr_valid;
  return PBF_OK;
}

void Handle::drop_graphs() {
  for (int q = 0; q < 2; ++q) {
    if (graph[q]) cudaGraphExecDestroy(graph[q]);
    graph[q] = nullptr;
    for (auto& g : prof_graph[q])
      if (g) cudaGraphExecDestroy(g);
    prof_graph[q].clear();
    prof_graph_count[q].clear();
  }
  graph_dt = -1.f;
}

}  // namespace pbf

using pbf::Handle;

extern "C" {

void pbf_params_default(pbf_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->h = 0.3;
  p->h2 = 0.09;
  p->iters = 12;
  p->scorr_n = 4;
  p->epsilon = 2;
  p->scorr_k = 0.0001;
  p->scorr_dq = 0.1;
  p->vort_eps = 0.001;
  p->xsph_c = 0.001;
  p->dt = 0.016;
  p->gravity[0] = 0;
  p->gravity[1] = -10;
  p->gravity[2] = 0;
  p->rest_density = 1000.0;
  p->box_lo[0] = -1; p->box_lo[1] = 0; p->box_lo[2] = -1;
  p->box_hi[0] = 1; p->box_hi[1] = 1.5; p->box_hi[2] = 1;
  p->box_open_mask = 0;
  p->n_clip = 2;
  p->clip_axis[0] = 2; p->clip_value[0] = 1.0;
  p->clip_axis[1] = 1; p->clip_value[1] = 1.49;
  p->clamp_lo[0] = -1; p->clamp_lo[1] = 0; p->clamp_lo[2] = -1;
  p->clamp_hi[0] = 1; p->clamp_hi[1] = 1.49; p->clamp_hi[2] = 1;
  p->max_neighbors = 128;
  p->flags = PBF_FLAG_STATS;
}

int pbf_abi_version(void) { return PBF_ABI_VERSION; }

pbf_status pbf_batch_create(const pbf_params* params, int n_scenes, const size_t* counts,
                            const float* box_lo, const float* box_hi, const float* xyz, const float* vel,
                            int device, pbf_handle** out) {
  g_create_error.clear();
  if (!out) {
    g_create_error = "out is NULL";
    return PBF_ERR_INVALID;
  }
  *out = nullptr;
  if (!params || n_scenes < 1 || !counts) {
    g_create_error = "params, counts and n_scenes >= 1 are required";
    return PBF_ERR_INVALID;
  }
  size_t n = 0;
  for (int s = 0; s < n_scenes; ++s) {
    if (counts[s] >= (size_t(1) << 31)) {  // also keeps the sum below from wrapping
      g_create_error = "at most 2^31 - 1 particles";
      return PBF_ERR_INVALID;
    }
    n += counts[s];
  }
  if (n > 0 && !xyz) {
    g_create_error = "xyz is NULL";
    return PBF_ERR_INVALID;
  }
  if (n >= (size_t(1) << 31)) {
    g_create_error = "at most 2^31 - 1 particles";
    return PBF_ERR_INVALID;
  }
  pbf::DevParams dp;
  double cell;
  std::string why;
  if (!pbf::make_dev_params(*params, &dp, &cell, &why)) {
    g_create_error = why;
    return PBF_ERR_INVALID;
  }
  std::vector<pbf::SceneDesc> scenes(n_scenes);
  uint64_t cells = 0, poff = 0;
  for (int s = 0; s < n_scenes; ++s) {
    float lo[3], hi[3];
    for (int a = 0; a < 3; ++a) {
      lo[a] = box_lo ? box_lo[3 * s + a] : static_cast<float>(params->box_lo[a]);
      hi[a] = box_hi ? box_hi[3 * s + a] : static_cast<float>(params->box_hi[a]);
    }
    if (!pbf::make_scene(*params, cell, lo, hi, &scenes[s], &why)) {
      g_create_error = "scene " + std::to_string(s) + ": " + why;
      return PBF_ERR_INVALID;
    }
    scenes[s].cell_off = static_cast<uint32_t>(cells);
    scenes[s].p_off = static_cast<uint32_t>(poff);
    scenes[s].p_cnt = static_cast<uint32_t>(counts[s]);
    cells += static_cast<uint64_t>(scenes[s].dim[0]) * scenes[s].dim[1] * scenes[s].dim[2];
    poff += counts[s];
    if (cells >= (uint64_t(1) << 31)) {
      g_create_error = "too many grid cells over all scenes";
      return PBF_ERR_INVALID;
    }
  }
  Handle* h = new (std::nothrow) Handle();
  if (!h) {
    g_create_error = "out of host memory";
    return PBF_ERR_NOMEM;
  }
  h->device = device;
  h->params = *params;
  if (h->params.max_neighbors == 0) h->params.max_neighbors = 128;
  h->dp = dp;
  h->scenes_host = scenes;
  h->b.n = n;
  h->b.n_scenes = n_scenes;
  h->b.n_cells = static_cast<uint32_t>(cells);
  h->b.max_words = dp.max_words;
  pbf::DeviceGuard g(device);
  pbf_status st = h->cuda(cudaSetDevice(device), "cudaSetDevice");
  if (st == PBF_OK) st = h->cuda(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking), "stream");
  if (st == PBF_OK) st = h->alloc_all();
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(h->b.scenes, scenes.data(), sizeof(pbf::SceneDesc) * n_scenes,
                                 cudaMemcpyHostToDevice, h->stream),
                 "upload scenes");
  if (st == PBF_OK && n > 0) {
    st = h->cuda(cudaMemcpyAsync(h->b.io, xyz, 3 * sizeof(float) * n, cudaMemcpyHostToDevice, h->stream),
                 "upload positions");
    if (st == PBF_OK && vel)
      st = h->cuda(cudaMemcpyAsync(h->b.io2, vel, 3 * sizeof(float) * n, cudaMemcpyHostToDevice, h->stream),
                   "upload velocities");
    if (st == PBF_OK)
      st = h->cuda(pbf::launch_upload(h->b, 0, h->b.io, vel ? h->b.io2 : nullptr, nullptr, h->stream),
                   "upload kernel");
    if (st == PBF_OK)
      st = h->cuda(cudaMemsetAsync(h->b.rho, 0, sizeof(float) * n, h->stream), "memset");
  }
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
  if (st != PBF_OK) {
    g_create_error = h->err;
    h->free_all();
    delete h;
    return st;
  }
  *out = reinterpret_cast<pbf_handle*>(h);
  return PBF_OK;
}

pbf_status pbf_create(const pbf_params* params, size_t n, const float* xyz, const float* vel, int device,
                      pbf_handle** out) {
  return pbf_batch_create(params, 1, &n, nullptr, nullptr, xyz, vel, device, out);
}

pbf_status pbf_destroy(pbf_handle* hh) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  h->free_all();
  delete h;
  return PBF_OK;
}

pbf_status pbf_step(pbf_handle* hh, double dt, int nsteps) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (nsteps < 0) return h->fail(PBF_ERR_INVALID, "nsteps must be >= 0");
  const double d = dt > 0 ? dt : h->params.dt;
  if (!(d > 0) || !std::isfinite(d)) return h->fail(PBF_ERR_INVALID, "dt must be positive");
  pbf::DeviceGuard g(h->device);
  pbf_status st = h->enqueue_steps(static_cast<float>(d), nsteps);
  if (st != PBF_OK) return st;
  h->simulate_time += d * nsteps;
  return h->sync_and_check();
}

pbf_status pbf_step_async(pbf_handle* hh, double dt, int nsteps) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (nsteps < 0) return h->fail(PBF_ERR_INVALID, "nsteps must be >= 0");
  const double d = dt > 0 ? dt : h->params.dt;
  if (!(d > 0) || !std::isfinite(d)) return h->fail(PBF_ERR_INVALID, "dt must be positive");
  pbf::DeviceGuard g(h->device);
  pbf_status st = h->enqueue_steps(static_cast<float>(d), nsteps);
  if (st == PBF_OK) h->simulate_time += d * nsteps;
  return st;
}

pbf_status pbf_sync(pbf_handle* hh) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  pbf::DeviceGuard g(h->device);
  return h->sync_and_check();
}

void* pbf_stream(pbf_handle* hh) {
  return hh ? reinterpret_cast<void*>(reinterpret_cast<Handle*>(hh)->stream) : nullptr;
}

pbf_status pbf_adjoint_step_device(pbf_handle* hh, double dt, const float* xyz, const float* vel,
                                   const float* gx_out, const float* gv_out, float* gx_in, float* gv_in,
                                   double* g_rho0, float* xyz_out, float* vel_out, void* stream) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  const double d = dt > 0 ? dt : h->params.dt;
  if (!(d > 0) || !std::isfinite(d)) return h->fail(PBF_ERR_INVALID, "dt must be positive");
  if (!g_rho0) return h->fail(PBF_ERR_INVALID, "g_rho0 is NULL");
  if (h->dp.n_mesh > 0 || h->dp.n_sph > 0)
    return h->fail(PBF_ERR_INVALID, "the adjoint step supports the box collider only");
  if (h->b.n && (!gx_in || !gv_in)) return h->fail(PBF_ERR_INVALID, "gx_in / gv_in is NULL");
  pbf::DeviceGuard g(h->device);
  pbf_status st = h->ensure_tape();
  if (st != PBF_OK) return st;
  st = h->join_from(static_cast<cudaStream_t>(stream));
  if (st != PBF_OK) return st;
  if (xyz) {
    st = h->cuda(pbf::launch_upload(h->b, h->cur, xyz, vel, nullptr, h->stream), "upload");
    if (st != PBF_OK) return st;
  }
  const float df = static_cast<float>(d);
  st = h->cuda(pbf::launch_step(h->b, h->dp, h->tune, h->cur, df, h->params.iters, false, h->stream, nullptr,
                                &h->tape),
               "recording step");
  if (st != PBF_OK) return st;
  st = h->cuda(pbf::launch_adjoint(h->b, h->dp, h->tune, h->cur, df, h->tape, gx_out, gv_out, gx_in, gv_in,
                                   g_rho0, h->stream),
               "adjoint");
  if (st != PBF_OK) return st;
  h->cur ^= 1;
  h->nbr_valid = true;
  if (xyz_out || vel_out) {
    st = h->cuda(pbf::launch_download(h->b, h->cur, xyz_out, vel_out, nullptr, h->stream), "download");
    if (st != PBF_OK) return st;
  }
  return h->join_to(static_cast<cudaStream_t>(stream));
}

// One reordering kernel into the staging arrays, the requested copies, one wait.
static pbf_status download(Handle* h, float* xyz, float* vel, float* rho) {
  pbf::DeviceGuard g(h->device);
  const size_t n = h->b.n;
  if (n == 0 || (!xyz && !vel && !rho)) return PBF_OK;
  float* tmp = reinterpret_cast<float*>(h->b.disp[0]);  // scratch between steps
  pbf_status st = h->cuda(pbf::launch_download(h->b, h->cur, xyz ? h->b.io : nullptr, vel ? h->b.io2 : nullptr,
                                               rho ? tmp : nullptr, h->stream),
                          "download");
  if (st == PBF_OK && xyz)
    st = h->cuda(cudaMemcpyAsync(xyz, h->b.io, 3 * sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK && vel)
    st = h->cuda(cudaMemcpyAsync(vel, h->b.io2, 3 * sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK && rho)
    st = h->cuda(cudaMemcpyAsync(rho, tmp, sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
  return st;
}

pbf_status pbf_get_state(pbf_handle* hh, float* xyz, float* vel, float* rho) {
  if (!hh) return PBF_ERR_INVALID;
  return download(reinterpret_cast<Handle*>(hh), xyz, vel, rho);
}

pbf_status pbf_get_positions(pbf_handle* hh, float* xyz) {
  if (!hh || !xyz) return PBF_ERR_INVALID;
  return download(reinterpret_cast<Handle*>(hh), xyz, nullptr, nullptr);
}

pbf_status pbf_get_velocities(pbf_handle* hh, float* vel) {
  if (!hh || !vel) return PBF_ERR_INVALID;
  return download(reinterpret_cast<Handle*>(hh), nullptr, vel, nullptr);
}

pbf_status pbf_get_densities(pbf_handle* hh, float* rho) {
  if (!hh || !rho) return PBF_ERR_INVALID;
  return download(reinterpret_cast<Handle*>(hh), nullptr, nullptr, rho);
}

pbf_status pbf_set_state(pbf_handle* hh, const float* xyz, const float* vel) {
  if (!hh || (!xyz && reinterpret_cast<Handle*>(hh)->b.n)) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  pbf::DeviceGuard g(h->device);
  const size_t n = h->b.n;
  if (n == 0) return PBF_OK;
  pbf_status st = h->cuda(cudaMemcpyAsync(h->b.io, xyz, 3 * sizeof(float) * n, cudaMemcpyHostToDevice, h->stream),
                          "H2D");
  if (st == PBF_OK && vel)
    st = h->cuda(cudaMemcpyAsync(h->b.io2, vel, 3 * sizeof(float) * n, cudaMemcpyHostToDevice, h->stream), "H2D");
  if (st == PBF_OK)
    st = h->cuda(pbf::launch_upload(h->b, h->cur, h->b.io, vel ? h->b.io2 : nullptr, nullptr, h->stream), "upload");
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
  h->nbr_valid = false;
  return st;
}

pbf_status pbf_set_state_device(pbf_handle* hh, const float* xyz, const float* vel, void* stream) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!xyz && h->b.n) return h->fail(PBF_ERR_INVALID, "xyz is NULL");
  pbf::DeviceGuard g(h->device);
  pbf_status st = h->join_from(static_cast<cudaStream_t>(stream));
  if (st == PBF_OK)
    st = h->cuda(pbf::launch_upload(h->b, h->cur, xyz, vel, nullptr, h->stream), "upload");
  if (st == PBF_OK) st = h->join_to(static_cast<cudaStream_t>(stream));
  h->nbr_valid = false;
  return st;
}

pbf_status pbf_get_state_device(pbf_handle* hh, float* xyz, float* vel, float* rho, void* stream) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  pbf::DeviceGuard g(h->device);
  pbf_status st = h->join_from(static_cast<cudaStream_t>(stream));
  if (st == PBF_OK)
    st = h->cuda(pbf::launch_download(h->b, h->cur, xyz, vel, rho, h->stream), "download");
  if (st == PBF_OK) st = h->join_to(static_cast<cudaStream_t>(stream));
  return st;
}

pbf_status pbf_estimate_densities(pbf_handle* hh, float* rho) {
  if (!hh || !rho) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  pbf::DeviceGuard g(h->device);
  if (h->b.n == 0) return PBF_OK;
  pbf_status st = h->cuda(pbf::launch_resort(h->b, h->dp, h->tune, h->cur, h->stream), "resort");
  if (st != PBF_OK) return st;
  h->cur ^= 1;
  h->nbr_valid = false;
  h->drop_graphs();
  st = h->cuda(pbf::launch_density_self(h->b, h->dp, h->tune, h->cur, h->b.rho, h->stream), "density");
  if (st != PBF_OK) return st;
  return download(h, nullptr, nullptr, rho);
}

namespace {

// Bounding-volume hierarchy over the collider triangles, built once on the host: median
// splits of the centroids along their longest extent down to leaves of kMeshLeafSize
// triangles (depth under kMeshMaxDepth); every node box is widened by 1e-5 of the
// largest coordinate magnitude and rounded outward to float, so the device's slab test
// never drops a triangle its exact test would hit.
struct MeshBuilder {
  const std::vector<std::array<double, 9>>& tri;
  std::vector<uint32_t> order;
  std::vector<std::array<double, 3>> cen;
  std::vector<float4> nodes;

  explicit MeshBuilder(const std::vector<std::array<double, 9>>& t) : tri(t), order(t.size()), cen(t.size()) {
    for (size_t k = 0; k < t.size(); ++k) {
      order[k] = static_cast<uint32_t>(k);
      for (int a = 0; a < 3; ++a) cen[k][a] = (t[k][a] + t[k][3 + a] + t[k][6 + a]) / 3.0;
    }
  }

  static float down(double x) {
    const float f = static_cast<float>(x);
    return static_cast<double>(f) > x ? std::nextafter(f, -INFINITY) : f;
  }
  static float up(double x) {
    const float f = static_cast<float>(x);
    return static_cast<double>(f) < x ? std::nextafter(f, INFINITY) : f;
  }
  static float bits(int v) {
    float f;
    std::memcpy(&f, &v, sizeof f);
    return f;
  }

  int build(size_t first, size_t count, int depth) {
    const int node = static_cast<int>(nodes.size() / 2);
    nodes.resize(nodes.size() + 2);
    double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    double clo[3] = {INFINITY, INFINITY, INFINITY}, chi[3] = {-INFINITY, -INFINITY, -INFINITY};
    double mag = 1.0;
    for (size_t k = first; k < first + count; ++k) {
      const auto& q = tri[order[k]];
      for (int v = 0; v < 3; ++v)
        for (int a = 0; a < 3; ++a) {
          lo[a] = std::min(lo[a], q[3 * v + a]);
          hi[a] = std::max(hi[a], q[3 * v + a]);
          mag = std::max(mag, std::fabs(q[3 * v + a]));
        }
      for (int a = 0; a < 3; ++a) {
        clo[a] = std::min(clo[a], cen[order[k]][a]);
        chi[a] = std::max(chi[a], cen[order[k]][a]);
      }
    }
    const double margin = 1e-5 * mag;
    int a_ = static_cast<int>(first), b_ = -static_cast<int>(count);
    if (count > static_cast<size_t>(pbf::kMeshLeafSize) && depth + 1 < pbf::kMeshMaxDepth) {
      int axis = 0;
      for (int a = 1; a < 3; ++a)
        if (chi[a] - clo[a] > chi[axis] - clo[axis]) axis = a;
      const size_t mid = first + count / 2;
      std::nth_element(order.begin() + first, order.begin() + mid, order.begin() + first + count,
                       [&](uint32_t x, uint32_t y) {
                         return cen[x][axis] < cen[y][axis] || (cen[x][axis] == cen[y][axis] && x < y);
                       });
      a_ = build(first, mid - first, depth + 1);
      b_ = build(mid, first + count - mid, depth + 1);
    }
    nodes[2 * node] = make_float4(down(lo[0] - margin), down(lo[1] - margin), down(lo[2] - margin), bits(a_));
    nodes[2 * node + 1] = make_float4(up(hi[0] + margin), up(hi[1] + margin), up(hi[2] + margin), bits(b_));
    return node;
  }
};

}  // namespace

pbf_status pbf_set_collider_mesh(pbf_handle* hh, size_t n, const float* tri) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (n > static_cast<size_t>(pbf::kMaxMeshTriangles))
    return h->fail(PBF_ERR_INVALID, "at most 4,194,304 collider triangles");
  if (n && !tri) return h->fail(PBF_ERR_INVALID, "tri is NULL");
  std::vector<std::array<double, 9>> q(n);
  for (size_t t = 0; t < n; ++t) {
    for (int k = 0; k < 9; ++k) {
      q[t][k] = tri[9 * t + k];
      if (!std::isfinite(q[t][k])) return h->fail(PBF_ERR_INVALID, "collider triangles must be finite");
    }
    double e1[3], e2[3];
    for (int k = 0; k < 3; ++k) {
      e1[k] = q[t][3 + k] - q[t][k];
      e2[k] = q[t][6 + k] - q[t][k];
    }
    const double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    if (!(std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]) > 0))
      return h->fail(PBF_ERR_INVALID, "degenerate collider triangle");
  }
  MeshBuilder mb(q);
  if (n) mb.build(0, n, 0);
  std::vector<float4> packed(4 * n);
  for (size_t k = 0; k < n; ++k) {  // leaf order
    const uint32_t t = mb.order[k];
    const auto& p = q[t];
    double e1[3], e2[3];
    for (int a = 0; a < 3; ++a) {
      e1[a] = p[3 + a] - p[a];
      e2[a] = p[6 + a] - p[a];
    }
    const double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
    const double cn = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
    packed[4 * k] = make_float4(static_cast<float>(p[0]), static_cast<float>(p[1]), static_cast<float>(p[2]), 0.f);
    packed[4 * k + 1] = make_float4(static_cast<float>(e1[0]), static_cast<float>(e1[1]), static_cast<float>(e1[2]), 0.f);
    packed[4 * k + 2] = make_float4(static_cast<float>(e2[0]), static_cast<float>(e2[1]), static_cast<float>(e2[2]), 0.f);
    packed[4 * k + 3] = make_float4(static_cast<float>(c[0] / cn), static_cast<float>(c[1] / cn),
                                    static_cast<float>(c[2] / cn), MeshBuilder::bits(static_cast<int>(t)));
  }
  pbf::DeviceGuard g(h->device);
  pbf_status st = h->cuda(cudaStreamSynchronize(h->stream), "sync");
  if (st != PBF_OK) return st;
  if (h->mesh_dev) cudaFree(h->mesh_dev);
  h->mesh_dev = nullptr;
  h->dp.n_mesh = 0;
  h->dp.mesh = nullptr;
  h->dp.mesh_nodes = nullptr;
  if (n) {
    const size_t bytes = sizeof(float4) * (packed.size() + mb.nodes.size());
    st = h->cuda(cudaMalloc(reinterpret_cast<void**>(&h->mesh_dev), bytes), "cudaMalloc(mesh)");
    if (st != PBF_OK) return st;
    st = h->cuda(cudaMemcpy(h->mesh_dev, packed.data(), sizeof(float4) * packed.size(), cudaMemcpyHostToDevice),
                 "H2D mesh");
    if (st == PBF_OK)
      st = h->cuda(cudaMemcpy(h->mesh_dev + packed.size(), mb.nodes.data(), sizeof(float4) * mb.nodes.size(),
                              cudaMemcpyHostToDevice),
                   "H2D mesh hierarchy");
    if (st != PBF_OK) return st;
    h->dp.n_mesh = static_cast<int>(n);
    h->dp.mesh = h->mesh_dev;
    h->dp.mesh_nodes = h->mesh_dev + packed.size();
  }
  h->drop_graphs();  // the captured steps hold the old parameters
  return PBF_OK;
}

pbf_status pbf_set_collider_spheres(pbf_handle* hh, size_t n, const float* xyzr) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (n > static_cast<size_t>(pbf::kMaxSpheres)) return h->fail(PBF_ERR_INVALID, "at most 1024 collider spheres");
  if (n && !xyzr) return h->fail(PBF_ERR_INVALID, "xyzr is NULL");
  std::vector<float4> packed(n);
  for (size_t k = 0; k < n; ++k) {
    for (int a = 0; a < 4; ++a)
      if (!std::isfinite(xyzr[4 * k + a])) return h->fail(PBF_ERR_INVALID, "collider spheres must be finite");
    if (!(xyzr[4 * k + 3] > 0.f)) return h->fail(PBF_ERR_INVALID, "collider sphere radius must be positive");
    packed[k] = make_float4(xyzr[4 * k], xyzr[4 * k + 1], xyzr[4 * k + 2], xyzr[4 * k + 3]);
  }
  pbf::DeviceGuard g(h->device);
  pbf_status st = h->cuda(cudaStreamSynchronize(h->stream), "sync");
  if (st != PBF_OK) return st;
  if (h->sph_dev) cudaFree(h->sph_dev);
  h->sph_dev = nullptr;
  h->dp.n_sph = 0;
  h->dp.sph = nullptr;
  if (n) {
    st = h->cuda(cudaMalloc(reinterpret_cast<void**>(&h->sph_dev), sizeof(float4) * n), "cudaMalloc(spheres)");
    if (st == PBF_OK)
      st = h->cuda(cudaMemcpy(h->sph_dev, packed.data(), sizeof(float4) * n, cudaMemcpyHostToDevice), "H2D spheres");
    if (st != PBF_OK) return st;
    h->dp.n_sph = static_cast<int>(n);
    h->dp.sph = h->sph_dev;
  }
  h->drop_graphs();
  return PBF_OK;
}

void pbf_mc_table(uint16_t* edges, uint8_t* ntri, int8_t* tri) {
  const pbf::SurfTable& t = pbf::surf_table();
  if (edges) std::memcpy(edges, t.edges, sizeof(t.edges));
  if (ntri) std::memcpy(ntri, t.ntri, sizeof(t.ntri));
  if (tri) std::memcpy(tri, t.tri, sizeof(t.tri));
}

namespace pbf {

// The cube grid of Particles::getSurfacePrims over [lo, hi] (NULL: the reference's fixed
// bounds, particles.cpp:330-349), the per-cube triangle counts of the current state and
// their total; the counts stay in the handle's scratch for surface_emit.
pbf_status Handle::surface_count(double isolevel, double step, const double* lo, const double* hi, SurfGrid* g,
                                 uint32_t* total) {
  if (!(step > 0) || !std::isfinite(step) || !std::isfinite(isolevel))
    return fail(PBF_ERR_INVALID, "step must be positive and isolevel finite");
  static const double kLo[3] = {-1.0, 0.0, -1.0}, kHi[3] = {1.0, 1.5, 1.0};  // particles.cpp:330-349
  g->step = step;
  double cubes = 1.0;
  for (int a = 0; a < 3; ++a) {
    g->lo[a] = lo ? lo[a] : kLo[a];
    g->hi[a] = hi ? hi[a] : kHi[a];
    if (!std::isfinite(g->lo[a]) || !std::isfinite(g->hi[a]) || g->hi[a] < g->lo[a])
      return fail(PBF_ERR_INVALID, "surface bounds must be finite with hi >= lo");
    const double steps = std::floor((g->hi[a] - g->lo[a]) / step);
    if (steps > 4095) return fail(PBF_ERR_INVALID, "surface grid too fine: at most 4096 cubes per axis");
    g->nc[a] = static_cast<int>(steps) + 1;
    cubes *= g->nc[a];
  }
  if (cubes > 2.0e9) return fail(PBF_ERR_INVALID, "surface grid too large");
  *total = 0;
  if (b.n == 0) return PBF_OK;
  pbf_status st = cuda(launch_resort(b, dp, tune, cur, stream), "resort");
  if (st != PBF_OK) return st;
  cur ^= 1;
  nbr_valid = false;
  drop_graphs();
  if (!surf_table_dev) {
    st = cuda(cudaMalloc(&surf_table_dev, sizeof(SurfTable)), "cudaMalloc(table)");
    if (st != PBF_OK) return st;
    st = cuda(cudaMemcpy(surf_table_dev, &surf_table(), sizeof(SurfTable), cudaMemcpyHostToDevice), "H2D table");
    if (st != PBF_OK) return st;
  }
  const size_t nc = static_cast<size_t>(cubes);
  const size_t corners = static_cast<size_t>(g->nc[0] + 1) * (g->nc[1] + 1) * (g->nc[2] + 1);
  const size_t tiles = exclusive_scan_tiles(static_cast<uint32_t>(nc));
  const size_t naxis = static_cast<size_t>(g->nc[0]) + g->nc[1] + g->nc[2] + 3;
  st = ensure_scratch(4 * (corners + nc + (nc + 1) + tiles + naxis) + 256);
  if (st != PBF_OK) return st;
  float* field = static_cast<float*>(scratch);
  uint32_t* cnt = reinterpret_cast<uint32_t*>(field + corners);
  uint32_t* first = cnt + nc;
  uint32_t* tile = first + nc + 1;
  float* axis = reinterpret_cast<float*>(tile + tiles);
  std::vector<float> ax;
  ax.reserve(naxis);
  for (int a = 0; a < 3; ++a)
    for (int i = 0; i <= g->nc[a]; ++i) {
      // i * step and the sum rounded separately (no fused multiply-add), as the reference's
      // x1 = xmin + ix * fStepSize
      const volatile double t = i * g->step;
      ax.push_back(static_cast<float>(std::min(g->lo[a] + t, g->hi[a])));
    }
  st = cuda(cudaMemcpyAsync(axis, ax.data(), sizeof(float) * naxis, cudaMemcpyHostToDevice, stream), "H2D axis");
  if (st != PBF_OK) return st;
  g->axis = axis;
  st = cuda(launch_surface_count(b, dp, cur, *g, static_cast<float>(isolevel), surf_table_dev, field, cnt, first,
                                 tile, stream),
            "surface count");
  if (st != PBF_OK) return st;
  st = cuda(cudaMemcpyAsync(total, first + nc, sizeof(uint32_t), cudaMemcpyDeviceToHost, stream), "D2H");
  if (st == PBF_OK) st = cuda(cudaStreamSynchronize(stream), "sync");
  return st;
}

// The first min(cap, total) triangles of the last surface_count into DEVICE arrays.
pbf_status Handle::surface_emit(const SurfGrid& g, double isolevel, float* xyz, float* nrm, uint32_t cap) {
  if (cap == 0 || b.n == 0) return PBF_OK;
  const size_t nc = static_cast<size_t>(g.nc[0]) * g.nc[1] * g.nc[2];
  const size_t corners = static_cast<size_t>(g.nc[0] + 1) * (g.nc[1] + 1) * (g.nc[2] + 1);
  const float* field = static_cast<const float*>(scratch);
  const uint32_t* first = reinterpret_cast<const uint32_t*>(field + corners) + nc;
  if (cap > (1u << 28)) return fail(PBF_ERR_INVALID, "surface too large: more than 2^28 triangles");
  const size_t slots = surface_hash_slots(cap);
  const size_t need = slots * (sizeof(unsigned long long) + sizeof(float4)) + 6 * sizeof(uint32_t) * cap + 512;
  if (need > surf_hash_bytes) {
    if (surf_hash) cudaFree(surf_hash);
    surf_hash = nullptr;
    surf_hash_bytes = 0;
    pbf_status st = cuda(cudaMalloc(&surf_hash, need), "cudaMalloc(surface table)");
    if (st != PBF_OK) return st;
    surf_hash_bytes = need;
  }
  SurfHash hs;
  hs.keys = static_cast<unsigned long long*>(surf_hash);
  hs.nslot = reinterpret_cast<float4*>(hs.keys + slots);
  hs.vslot = reinterpret_cast<uint32_t*>(hs.nslot + slots);
  hs.ulist = hs.vslot + 3 * static_cast<size_t>(cap);
  hs.ucount = hs.ulist + 3 * static_cast<size_t>(cap);
  return cuda(launch_surface_emit(b, dp, cur, g, static_cast<float>(isolevel), surf_table_dev, field, first, xyz, nrm,
                                  cap, hs, stream),
              "surface emit");
}

}  // namespace pbf

pbf_status pbf_surface(pbf_handle* hh, double isolevel, double step, const double* lo, const double* hi,
                       float* xyz, float* nrm, size_t cap, size_t* count) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!count) return h->fail(PBF_ERR_INVALID, "count is NULL");
  if (cap && (!xyz || !nrm)) return h->fail(PBF_ERR_INVALID, "xyz / nrm is NULL");
  *count = 0;
  pbf::DeviceGuard dg(h->device);
  pbf::SurfGrid g;
  uint32_t total = 0;
  pbf_status st = h->surface_count(isolevel, step, lo, hi, &g, &total);
  if (st != PBF_OK) return st;
  *count = total;
  const size_t m = std::min(static_cast<size_t>(total), cap);
  if (m == 0) return PBF_OK;
  float* dev = nullptr;
  st = h->cuda(cudaMalloc(&dev, sizeof(float) * 18 * m), "cudaMalloc(surface)");
  if (st != PBF_OK) return st;
  st = h->surface_emit(g, isolevel, dev, dev + 9 * m, static_cast<uint32_t>(m));
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(xyz, dev, sizeof(float) * 9 * m, cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(nrm, dev + 9 * m, sizeof(float) * 9 * m, cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "sync");
  cudaFree(dev);
  return st;
}

pbf_status pbf_estimate_density_at(pbf_handle* hh, size_t m, const float* pts, float* out) {
  if (!hh || (m && (!pts || !out))) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (h->b.n_scenes != 1) return h->fail(PBF_ERR_INVALID, "density queries need a single-scene handle");
  if (m == 0) return PBF_OK;
  pbf::DeviceGuard g(h->device);
  pbf_status st = h->ensure_scratch(2 * 3 * sizeof(float) * m);
  if (st != PBF_OK) return st;
  float* dpts = static_cast<float*>(h->scratch);
  float* dout = dpts + 3 * m;
  if (h->b.n) {
    st = h->cuda(pbf::launch_resort(h->b, h->dp, h->tune, h->cur, h->stream), "resort");
    if (st != PBF_OK) return st;
    h->cur ^= 1;
    h->nbr_valid = false;
    h->drop_graphs();
  }
  st = h->cuda(cudaMemcpyAsync(dpts, pts, 3 * sizeof(float) * m, cudaMemcpyHostToDevice, h->stream), "H2D");
  if (st != PBF_OK) return st;
  if (h->b.n) {
    st = h->cuda(pbf::launch_density_at(h->b, h->dp, h->cur, m, dpts, dout, h->stream), "density_at");
  } else {
    st = h->cuda(cudaMemsetAsync(dout, 0, sizeof(float) * m, h->stream), "memset");
  }
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(out, dout, sizeof(float) * m, cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
  return st;
}

pbf_status pbf_get_stats(pbf_handle* hh, pbf_stats* out) {
  if (!hh || !out) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  pbf::DeviceGuard g(h->device);
  std::memset(out, 0, sizeof(*out));
  out->steps = h->steps;
  pbf::DevStats ds;
  std::memset(&ds, 0, sizeof(ds));
  unsigned errw = 0;
  pbf_status st = h->cuda(cudaMemcpyAsync(&ds, h->b.stats, sizeof(ds), cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(&errw, h->b.err, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
  if (st != PBF_OK) return st;
  out->error_flags = errw;
  if (!h->dp.stats || h->steps == 0 || h->b.n == 0) return PBF_OK;
  const double n = static_cast<double>(h->b.n);
  out->mean_density_iter0 = ds.rho_iter0_sum / n;
  out->mean_density = ds.rho_sum / n;
  out->mean_density_error = ds.err_sum / n;
  float em;
  std::memcpy(&em, &ds.err_max_bits, sizeof(em));
  out->max_density_error = em;
  out->min_neighbors = ds.nbr_min;
  out->max_neighbors = ds.nbr_max;
  out->mean_neighbors = static_cast<double>(ds.nbr_sum) / n;
  out->low_neighbor_count = ds.low_cnt;
  return PBF_OK;
}

pbf_status pbf_get_neighbors(pbf_handle* hh, uint32_t* counts, uint32_t* ids, size_t cap, size_t* total) {
  if (!hh || !counts) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h->nbr_valid) return h->fail(PBF_ERR_INVALID, "no neighbour lists: step first");
  pbf::DeviceGuard g(h->device);
  const size_t n = h->b.n;
  if (n == 0) {
    if (total) *total = 0;
    return PBF_OK;
  }
  pbf_status st = h->ensure_scratch(sizeof(uint32_t) * (2 * n + 1));
  if (st != PBF_OK) return st;
  uint32_t* dcounts = static_cast<uint32_t*>(h->scratch);
  st = h->cuda(pbf::launch_neighbor_counts(h->b, h->cur, dcounts, h->stream), "counts");
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(counts, dcounts, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "sync");
  if (st != PBF_OK) return st;
  std::vector<uint32_t> off(n + 1, 0);
  for (size_t i = 0; i < n; ++i) off[i + 1] = off[i] + counts[i];
  if (total) *total = off[n];
  if (!ids) return PBF_OK;
  if (off[n] > cap) return h->fail(PBF_ERR_INVALID, "ids capacity too small");
  st = h->ensure_scratch(sizeof(uint32_t) * (n + 1 + static_cast<size_t>(off[n])));
  if (st != PBF_OK) return st;
  uint32_t* doff = static_cast<uint32_t*>(h->scratch);
  uint32_t* dids = doff + n + 1;
  st = h->cuda(cudaMemcpyAsync(doff, off.data(), sizeof(uint32_t) * (n + 1), cudaMemcpyHostToDevice, h->stream), "H2D");
  if (st == PBF_OK) st = h->cuda(pbf::launch_neighbor_ids(h->b, h->cur, doff, dids, h->stream), "ids");
  if (st == PBF_OK && off[n])
    st = h->cuda(cudaMemcpyAsync(ids, dids, sizeof(uint32_t) * off[n], cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "sync");
  if (st != PBF_OK) return st;
  for (size_t i = 0; i < n; ++i) std::sort(ids + off[i], ids + off[i + 1]);
  return PBF_OK;
}

pbf_status pbf_get_cells(pbf_handle* hh, uint32_t* cells) {
  if (!hh || !cells) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h->nbr_valid || !h->b.pred) return h->fail(PBF_ERR_INVALID, "needs a step taken with PBF_FLAG_KEEP_PREDICTED");
  pbf::DeviceGuard g(h->device);
  const size_t n = h->b.n;
  if (n == 0) return PBF_OK;
  pbf_status st = h->ensure_scratch(sizeof(uint32_t) * n);
  if (st != PBF_OK) return st;
  uint32_t* d = static_cast<uint32_t*>(h->scratch);
  st = h->cuda(pbf::launch_cells_of(h->b, h->dp, h->cur, d, h->stream), "cells");
  if (st == PBF_OK) st = h->cuda(cudaMemcpyAsync(cells, d, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "sync");
  return st;
}

pbf_status pbf_get_predicted(pbf_handle* hh, float* xyz) {
  if (!hh || !xyz) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h->nbr_valid || !h->b.pred) return h->fail(PBF_ERR_INVALID, "needs a step taken with PBF_FLAG_KEEP_PREDICTED");
  pbf::DeviceGuard g(h->device);
  const size_t n = h->b.n;
  if (n == 0) return PBF_OK;
  pbf_status st = h->cuda(pbf::launch_unsort_f4(h->b, h->cur, h->b.pred, h->b.io, h->stream), "unsort");
  if (st == PBF_OK) st = h->cuda(cudaMemcpyAsync(xyz, h->b.io, 3 * sizeof(float) * n, cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "sync");
  return st;
}

pbf_status pbf_sort(pbf_handle* hh) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  pbf::DeviceGuard g(h->device);
  if (h->b.n == 0) return PBF_OK;
  pbf_status st = h->cuda(pbf::launch_resort(h->b, h->dp, h->tune, h->cur, h->stream), "resort");
  if (st != PBF_OK) return st;
  h->cur ^= 1;
  h->nbr_valid = false;
  return h->cuda(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
}

pbf_status pbf_snapshot(pbf_handle* hh) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  pbf::DeviceGuard g(h->device);
  const size_t n = h->b.n ? h->b.n : 1;
  pbf_status st = PBF_OK;
  if (!h->snap_pos) st = h->cuda(cudaMalloc((void**)&h->snap_pos, sizeof(float4) * n), "cudaMalloc");
  if (st == PBF_OK && !h->snap_vel) st = h->cuda(cudaMalloc((void**)&h->snap_vel, sizeof(float4) * n), "cudaMalloc");
  if (st == PBF_OK && !h->snap_id) st = h->cuda(cudaMalloc((void**)&h->snap_id, sizeof(uint32_t) * n), "cudaMalloc");
  if (st != PBF_OK) return st;
  const size_t m = h->b.n;
  st = h->cuda(cudaMemcpyAsync(h->snap_pos, h->b.pos[h->cur], sizeof(float4) * m, cudaMemcpyDeviceToDevice, h->stream), "copy");
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(h->snap_vel, h->b.vel[h->cur], sizeof(float4) * m, cudaMemcpyDeviceToDevice, h->stream), "copy");
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(h->snap_id, h->b.id[h->cur], sizeof(uint32_t) * m, cudaMemcpyDeviceToDevice, h->stream), "copy");
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "cudaStreamSynchronize");
  if (st == PBF_OK) {
    h->snap_valid = true;
    h->snap_steps = h->steps;
    h->snap_time = h->simulate_time;
  }
  return st;
}

pbf_status pbf_restore(pbf_handle* hh) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!h->snap_valid) return h->fail(PBF_ERR_INVALID, "no snapshot taken");
  pbf::DeviceGuard g(h->device);
  const size_t m = h->b.n;
  pbf_status st =
      h->cuda(cudaMemcpyAsync(h->b.pos[h->cur], h->snap_pos, sizeof(float4) * m, cudaMemcpyDeviceToDevice, h->stream), "copy");
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(h->b.vel[h->cur], h->snap_vel, sizeof(float4) * m, cudaMemcpyDeviceToDevice, h->stream), "copy");
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(h->b.id[h->cur], h->snap_id, sizeof(uint32_t) * m, cudaMemcpyDeviceToDevice, h->stream), "copy");
  h->nbr_valid = false;
  h->steps = h->snap_steps;
  h->simulate_time = h->snap_time;
  return st;
}

pbf_status pbf_get_tuning(pbf_handle* hh, pbf_tuning* out) {
  if (!hh || !out) return PBF_ERR_INVALID;
  const pbf::Tuning& t = reinterpret_cast<Handle*>(hh)->tune;
  out->block_predict = t.block_predict;
  out->block_nbr = t.block_nbr;
  out->block_solve = t.block_solve;
  out->block_misc = t.block_misc;
  out->gather_depth = t.gather_depth;
  out->list_stream = t.list_stream;
  return PBF_OK;
}

static bool valid_block(int b) { return b == 64 || b == 128 || b == 256 || b == 512; }

pbf_status pbf_set_tuning(pbf_handle* hh, const pbf_tuning* t) {
  if (!hh || !t) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!valid_block(t->block_predict) || !valid_block(t->block_nbr) || !valid_block(t->block_solve) ||
      !valid_block(t->block_misc))
    return h->fail(PBF_ERR_INVALID, "block sizes must be 64, 128, 256 or 512");
  if ((t->gather_depth != 4 && t->gather_depth != 8) || (t->list_stream != 0 && t->list_stream != 1))
    return h->fail(PBF_ERR_INVALID, "gather_depth must be 4 or 8, list_stream 0 or 1");
  h->tune.block_predict = t->block_predict;
  h->tune.block_nbr = t->block_nbr;
  h->tune.block_solve = t->block_solve;
  h->tune.block_misc = t->block_misc;
  h->tune.gather_depth = t->gather_depth;
  h->tune.list_stream = t->list_stream;
  h->drop_graphs();
  return PBF_OK;
}

namespace {
// Device ms per phase of `reps` steps from the snapshot (restored before each step).
pbf_status time_phases(Handle* h, float dt, int reps, double* ms) {
  pbf_status st = pbf_reset_phase_times(reinterpret_cast<pbf_handle*>(h));
  for (int r = 0; r < reps && st == PBF_OK; ++r) {
    st = pbf_restore(reinterpret_cast<pbf_handle*>(h));
    if (st == PBF_OK) st = h->enqueue_steps(dt, 1);
  }
  if (st == PBF_OK) st = pbf_get_phase_times(reinterpret_cast<pbf_handle*>(h), ms, nullptr, pbf::kNumPhases);
  return st;
}
}  // namespace

pbf_status pbf_autotune(pbf_handle* hh, double dt, int reps, pbf_tuning* out) {
  if (!hh || reps < 1) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  const double d = dt > 0 ? dt : h->params.dt;
  pbf::DeviceGuard g(h->device);
  if (h->b.n == 0) return out ? pbf_get_tuning(hh, out) : PBF_OK;
  // keep the caller's checkpoint, if any, and the state
  const bool had_prof = h->profiling;
  const uint64_t steps0 = h->steps;
  const double time0 = h->simulate_time;
  std::vector<float4> keep_pos, keep_vel;
  std::vector<uint32_t> keep_id;
  const bool had_snap = h->snap_valid;
  const size_t n = h->b.n;
  if (had_snap) {  // save the caller's snapshot to host
    keep_pos.resize(n);
    keep_vel.resize(n);
    keep_id.resize(n);
    pbf_status st = h->cuda(cudaMemcpy(keep_pos.data(), h->snap_pos, sizeof(float4) * n, cudaMemcpyDeviceToHost), "D2H");
    if (st == PBF_OK) st = h->cuda(cudaMemcpy(keep_vel.data(), h->snap_vel, sizeof(float4) * n, cudaMemcpyDeviceToHost), "D2H");
    if (st == PBF_OK) st = h->cuda(cudaMemcpy(keep_id.data(), h->snap_id, sizeof(uint32_t) * n, cudaMemcpyDeviceToHost), "D2H");
    if (st != PBF_OK) return st;
  }
  const uint64_t snap_steps0 = h->snap_steps;
  const double snap_time0 = h->snap_time;
  pbf_status st = pbf_snapshot(hh);
  if (st != PBF_OK) return st;
  // candidates are timed launched stream-ordered (no graph), each with its own shapes
  const int flags0 = h->params.flags;
  h->params.flags &= ~PBF_FLAG_GRAPH;
  h->drop_graphs();
  h->profiling = true;
  pbf::Tuning best = h->tune;
  // one dimension at a time, each timed over the phases it launches, the others held at
  // their best value so far
  struct Family {
    int* field;
    int phases[4];
    int cand[4];
    int ncand;
  } fams[] = {
      {&best.block_nbr, {pbf::kPhaseNeighbors, -1, -1, -1}, {64, 128, 256, 512}, 4},
      {&best.gather_depth, {pbf::kPhaseLambda, pbf::kPhaseDeltaP, pbf::kPhaseXsph, pbf::kPhaseVorticity}, {4, 8}, 2},
      {&best.list_stream, {pbf::kPhaseLambda, pbf::kPhaseDeltaP, pbf::kPhaseXsph, pbf::kPhaseVorticity}, {0, 1}, 2},
      {&best.block_solve, {pbf::kPhaseLambda, pbf::kPhaseDeltaP, pbf::kPhaseXsph, pbf::kPhaseVorticity},
       {64, 128, 256, 512}, 4},
      {&best.block_predict, {pbf::kPhasePredict, -1, -1, -1}, {64, 128, 256, 512}, 4},
      {&best.block_misc, {pbf::kPhaseSort, pbf::kPhaseGather, -1, -1}, {64, 128, 256, 512}, 4},
  };
  for (auto& f : fams) {
    double best_ms = 1e300;
    int best_b = *f.field;
    for (int ci = 0; ci < f.ncand; ++ci) {
      const int c = f.cand[ci];
      pbf::Tuning trial = best;
      *reinterpret_cast<int*>(reinterpret_cast<char*>(&trial) +
                              (reinterpret_cast<char*>(f.field) - reinterpret_cast<char*>(&best))) = c;
      h->tune = trial;
      h->drop_graphs();
      double ms[pbf::kNumPhases] = {};
      st = time_phases(h, static_cast<float>(d), 1, ms);  // warm the shape
      if (st == PBF_OK) st = time_phases(h, static_cast<float>(d), reps, ms);
      if (st != PBF_OK) break;
      double tot = 0;
      for (int q : f.phases)
        if (q >= 0) tot += ms[q];
      if (tot < best_ms) {
        best_ms = tot;
        best_b = c;
      }
    }
    if (st != PBF_OK) break;
    *f.field = best_b;
  }
  h->tune = best;
  h->profiling = had_prof;
  h->params.flags = flags0;
  pbf_status st2 = pbf_restore(hh);
  if (st == PBF_OK) st = st2;
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "sync");
  pbf_reset_phase_times(hh);
  h->steps = steps0;
  h->simulate_time = time0;
  if (had_snap && st == PBF_OK) {
    st = h->cuda(cudaMemcpy(h->snap_pos, keep_pos.data(), sizeof(float4) * n, cudaMemcpyHostToDevice), "H2D");
    if (st == PBF_OK) st = h->cuda(cudaMemcpy(h->snap_vel, keep_vel.data(), sizeof(float4) * n, cudaMemcpyHostToDevice), "H2D");
    if (st == PBF_OK) st = h->cuda(cudaMemcpy(h->snap_id, keep_id.data(), sizeof(uint32_t) * n, cudaMemcpyHostToDevice), "H2D");
    h->snap_steps = snap_steps0;
    h->snap_time = snap_time0;
  } else {
    h->snap_valid = had_snap;
  }
  h->drop_graphs();
  if (st == PBF_OK && out) st = pbf_get_tuning(hh, out);
  return st;
}

static const char* kPhaseNames[pbf::kNumPhases] = {"predict", "scan", "sort", "gather", "neighbors",
                                                    "lambda", "deltap", "xsph", "vorticity", "stats"};

const char* pbf_phase_name(int phase) {
  return (phase >= 0 && phase < pbf::kNumPhases) ? kPhaseNames[phase] : "";
}

int pbf_num_phases(void) { return pbf::kNumPhases; }

pbf_status pbf_set_profiling(pbf_handle* hh, int enable) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  pbf::DeviceGuard g(h->device);
  pbf_status st = h->collect_phase_times();
  h->profiling = enable != 0;
  return st;
}

pbf_status pbf_get_phase_times(pbf_handle* hh, double* ms, uint64_t* launches, int max_phases) {
  if (!hh || max_phases < 0) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  pbf::DeviceGuard g(h->device);
  pbf_status st = h->collect_phase_times();
  if (st != PBF_OK) return st;
  for (int q = 0; q < max_phases && q < pbf::kNumPhases; ++q) {
    if (ms) ms[q] = h->phase_ms[q];
    if (launches) launches[q] = h->phase_launches[q];
  }
  return PBF_OK;
}

pbf_status pbf_reset_phase_times(pbf_handle* hh) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  pbf::DeviceGuard g(h->device);
  pbf_status st = h->collect_phase_times();
  for (int q = 0; q < pbf::kNumPhases; ++q) {
    h->phase_ms[q] = 0;
    h->phase_launches[q] = 0;
  }
  return st;
}

size_t pbf_size(const pbf_handle* hh) { return hh ? reinterpret_cast<const Handle*>(hh)->b.n : 0; }

int pbf_num_scenes(const pbf_handle* hh) { return hh ? reinterpret_cast<const Handle*>(hh)->b.n_scenes : 0; }

const char* pbf_last_error(const pbf_handle* hh) {
  if (!hh) return g_create_error.c_str();
  return reinterpret_cast<const Handle*>(hh)->err.c_str();
}

}  // extern "C"
