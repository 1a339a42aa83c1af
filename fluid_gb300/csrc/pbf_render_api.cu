// C ABI of the path tracer (include/pbf.h: pbf_camera_frame, pbf_render_set_scene,
// pbf_render): the PathTracer side of the reference (src/pathtracer.cpp) over a handle.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "pbf.h"
#include "pbf_handle.h"

using pbf::Handle;

namespace pbf {

void RenderState::release() {
  if (scene_tri) cudaFree(scene_tri);
  if (scene_nrm) cudaFree(scene_nrm);
  if (buf) cudaFree(buf);
  for (cudaEvent_t& e : ev) {
    if (e) cudaEventDestroy(e);
    e = nullptr;
  }
  delete[] mats_host;
  delete[] lights_host;
  *this = RenderState();
}

}  // namespace pbf

namespace {

constexpr double kPiD = 3.14159265358979323;  // CGL misc.h PI

// Bump allocator over one device buffer, 256-byte aligned pieces.
struct Carve {
  char* base;
  size_t off = 0;
  template <typename T>
  T* take(size_t count) {
    off = (off + 255) & ~static_cast<size_t>(255);
    T* p = reinterpret_cast<T*>(base ? base + off : nullptr);
    off += sizeof(T) * std::max<size_t>(count, 1);
    return p;
  }
};

struct Tree {
  pbf::BvhNode* nodes;
  pbf::BvhScratch w;
};

struct Frame {
  pbf::RTri* tri;
  pbf::RNrm* nrm;
  Tree scene, surf;
  pbf::RMat* mats;
  pbf::RLight* lights;
  float *sxyz, *snrm, *hdr;
  uint8_t* rgba;
  unsigned* err;
  pbf::WfBuffers wf;
};

Tree carve_tree(Carve& c, size_t n) {
  Tree t;
  t.nodes = c.take<pbf::BvhNode>(n > 1 ? n - 1 : 1);
  const uint32_t nb = pbf::sort_blocks(static_cast<uint32_t>(n));
  t.w.keys = c.take<uint32_t>(n);
  t.w.vals = c.take<uint32_t>(n);
  t.w.keys2 = c.take<uint32_t>(n);
  t.w.vals2 = c.take<uint32_t>(n);
  t.w.hist = c.take<uint32_t>(256u * nb);
  t.w.start = c.take<uint32_t>(256u * nb + 1);
  t.w.tile_sums = c.take<uint32_t>(pbf::exclusive_scan_tiles(256u * nb) + 1);
  t.w.parent = c.take<uint32_t>(2 * n);
  t.w.flags = c.take<uint32_t>(n);
  t.w.box_lo = c.take<float4>(2 * n);
  t.w.box_hi = c.take<float4>(2 * n);
  t.w.bounds = c.take<float4>(2 + 2 * pbf::kBoundsBlocks);
  t.w.ltri = c.take<pbf::RTri>(n);
  return t;
}

// n_scene_tree: the scene's triangle count when it gets a hierarchy, else 0.
// paths: the path state of one batch (px * samples per batch), slots per path.
Frame carve(char* base, size_t n, size_t n_scene_tree, size_t m, int n_mat, int n_light, size_t px, size_t paths,
            int slots, size_t* bytes) {
  Carve c{base};
  Frame f;
  f.tri = c.take<pbf::RTri>(n);
  f.nrm = c.take<pbf::RNrm>(n);
  f.scene = carve_tree(c, n_scene_tree);
  f.surf = carve_tree(c, m);
  f.mats = c.take<pbf::RMat>(n_mat + 1);
  f.lights = c.take<pbf::RLight>(n_light);
  f.sxyz = c.take<float>(9 * m);
  f.snrm = c.take<float>(9 * m);
  f.hdr = c.take<float>(3 * px);
  f.rgba = c.take<uint8_t>(4 * px);
  f.err = c.take<unsigned>(1);
  pbf::WfBuffers& w = f.wf;
  w.o = c.take<float4>(paths);
  w.d = c.take<float4>(paths);
  w.beta = c.take<float4>(paths);
  w.L = c.take<float4>(paths);
  w.hit = c.take<float4>(paths);
  w.st = c.take<uint2>(paths);
  w.qa = c.take<uint32_t>(paths);
  w.qb = c.take<uint32_t>(paths);
  w.sdir = c.take<float4>(paths * slots);
  w.scon = c.take<float4>(paths * slots);
  w.sq = c.take<uint32_t>(paths * slots);
  w.cnt = c.take<uint32_t>(8);
  w.slots = slots;
  *bytes = c.off + 256;
  return f;
}

}  // namespace

extern "C" {

void pbf_render_params_default(pbf_render_params* p) {
  if (!p) return;
  std::memset(p, 0, sizeof(*p));
  p->width = 640;
  p->height = 480;
  p->ns_aa = 1;
  p->max_ray_depth = 1;
  p->ns_area_light = 1;
  p->fluid_surface = 1;
  p->seed = 1;
  p->fluid_albedo[0] = 0.1f;
  p->fluid_albedo[1] = 0.1f;
  p->fluid_albedo[2] = 0.8f;
}

// Camera::configure (camera.cpp:15-31) and Camera::place / compute_position (:33-46,
// :92-111), in the reference's double arithmetic (CameraInfo's fields are float).
pbf_status pbf_camera_frame(const pbf_camera_desc* d, uint32_t width, uint32_t height, pbf_camera* out) {
  if (!d || !out || width == 0 || height == 0) return PBF_ERR_INVALID;
  const double rad = kPiD / 180, deg = 180 / kPiD;
  double hFov = static_cast<float>(d->hfov), vFov = static_cast<float>(d->vfov);
  const double ar1 = std::tan(hFov * rad / 2) / std::tan(vFov * rad / 2);
  const double ar = static_cast<double>(width) / height;
  if (ar1 < ar) {
    hFov = 2 * (std::atan(std::tan(vFov * rad / 2) * ar) * deg);
  } else if (ar1 > ar) {
    vFov = 2 * (std::atan(std::tan(hFov * rad / 2) / ar) * deg);
  }
  const double EPS_F = 0.00001f;
  const double r = std::min(std::max(d->r, d->min_r), d->max_r);
  double phi = (std::sin(d->phi) == 0) ? (d->phi + EPS_F) : d->phi;
  double sinPhi = std::sin(phi);
  if (sinPhi == 0) {
    phi += EPS_F;
    sinPhi = std::sin(phi);
  }
  const double dc[3] = {r * sinPhi * std::sin(d->theta), r * std::cos(phi), r * sinPhi * std::cos(d->theta)};
  const double up[3] = {0, sinPhi > 0 ? 1.0 : -1.0, 0};
  auto cross = [](const double* u, const double* v, double* o) {
    o[0] = u[1] * v[2] - u[2] * v[1];
    o[1] = u[2] * v[0] - u[0] * v[2];
    o[2] = u[0] * v[1] - u[1] * v[0];
  };
  auto normalize = [](double* v) {  // Vector3D::normalize: *= 1 / norm
    const double c = 1. / std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
    v[0] *= c;
    v[1] *= c;
    v[2] *= c;
  };
  double sx[3], sy[3];
  cross(up, dc, sx);
  normalize(sx);
  cross(dc, sx, sy);
  normalize(sy);
  const double rn = 1. / std::sqrt(dc[0] * dc[0] + dc[1] * dc[1] + dc[2] * dc[2]);  // Vector3D::unit
  for (int k = 0; k < 3; ++k) {
    out->position[k] = d->target[k] + dc[k];
    out->c2w[k] = sx[k];
    out->c2w[3 + k] = sy[k];
    out->c2w[6 + k] = rn * dc[k];
  }
  out->hfov = hFov;
  out->vfov = vFov;
  out->nclip = static_cast<float>(d->nclip);
  out->fclip = static_cast<float>(d->fclip);
  return PBF_OK;
}

pbf_status pbf_render_set_scene(pbf_handle* hh, const float* tri_xyz, const float* tri_nrm,
                                const uint32_t* tri_material, size_t n_tri, const pbf_material* materials,
                                size_t n_materials, const pbf_light* lights, size_t n_lights) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (n_tri && (!tri_xyz || !tri_material)) return h->fail(PBF_ERR_INVALID, "tri_xyz / tri_material is NULL");
  if ((n_materials && !materials) || (n_lights && !lights)) return h->fail(PBF_ERR_INVALID, "NULL array");
  if (n_tri > (1u << 28) || n_materials > 4096 || n_lights > 4096)
    return h->fail(PBF_ERR_INVALID, "scene too large (2^28 triangles, 4096 materials, 4096 lights)");
  std::vector<pbf::RTri> tri(n_tri);
  std::vector<pbf::RNrm> nrm(n_tri);
  for (size_t t = 0; t < n_tri; ++t) {
    const float* p = tri_xyz + 9 * t;
    for (int k = 0; k < 9; ++k)
      if (!std::isfinite(p[k])) return h->fail(PBF_ERR_INVALID, "non-finite triangle vertex");
    if (tri_material[t] >= n_materials) return h->fail(PBF_ERR_INVALID, "triangle material index out of range");
    const int mid = static_cast<int>(tri_material[t]);
    float mbits;
    std::memcpy(&mbits, &mid, sizeof(mbits));  // material index in p1.w, as int bits
    tri[t] = pbf::RTri{make_float4(p[0], p[1], p[2], mbits),
                       make_float4(p[3], p[4], p[5], 0.f), make_float4(p[6], p[7], p[8], 0.f)};
    float q[9];
    if (tri_nrm) {
      std::memcpy(q, tri_nrm + 9 * t, sizeof(q));
    } else {
      const double e1[3] = {double(p[3]) - p[0], double(p[4]) - p[1], double(p[5]) - p[2]};
      const double e2[3] = {double(p[6]) - p[0], double(p[7]) - p[1], double(p[8]) - p[2]};
      double c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
      const double l = std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
      if (!(l > 0)) return h->fail(PBF_ERR_INVALID, "degenerate triangle without normals");
      for (int v = 0; v < 3; ++v)
        for (int k = 0; k < 3; ++k) q[3 * v + k] = static_cast<float>(c[k] / l);
    }
    nrm[t] = pbf::RNrm{make_float4(q[0], q[1], q[2], 0.f), make_float4(q[3], q[4], q[5], 0.f),
                       make_float4(q[6], q[7], q[8], 0.f)};
  }
  std::vector<pbf::RMat> mats(n_materials);
  for (size_t m = 0; m < n_materials; ++m) {
    const pbf_material& a = materials[m];
    if (a.kind > PBF_MAT_EMISSION) return h->fail(PBF_ERR_INVALID, "unknown material kind");
    if (a.kind == PBF_MAT_GLASS && !(a.ior > 0)) return h->fail(PBF_ERR_INVALID, "glass needs ior > 0");
    mats[m].kind = static_cast<int>(a.kind);
    for (int k = 0; k < 3; ++k) {
      mats[m].c1[k] = a.c1[k];
      mats[m].c2[k] = a.c2[k];
    }
    mats[m].ior = a.ior;
  }
  std::vector<pbf::RLight> ls(n_lights);
  for (size_t i = 0; i < n_lights; ++i) {
    const pbf_light& a = lights[i];
    if (a.kind > PBF_LIGHT_AREA) return h->fail(PBF_ERR_INVALID, "unknown light kind");
    pbf::RLight& l = ls[i];
    l.kind = static_cast<int>(a.kind);
    for (int k = 0; k < 3; ++k) {
      l.rad[k] = a.radiance[k];
      l.pos[k] = a.position[k];
      l.dir[k] = a.direction[k];
      l.dx[k] = a.dim_x[k];
      l.dy[k] = a.dim_y[k];
    }
    if (a.kind == PBF_LIGHT_DIRECTIONAL) {  // dirToLight = -lightDir.unit() (light.cpp:12-15)
      const double n2 = double(a.direction[0]) * a.direction[0] + double(a.direction[1]) * a.direction[1] +
                        double(a.direction[2]) * a.direction[2];
      if (!(n2 > 0)) return h->fail(PBF_ERR_INVALID, "directional light without a direction");
      for (int k = 0; k < 3; ++k) l.dir[k] = static_cast<float>(-a.direction[k] / std::sqrt(n2));
    }
    const double nx = std::sqrt(double(a.dim_x[0]) * a.dim_x[0] + double(a.dim_x[1]) * a.dim_x[1] +
                                double(a.dim_x[2]) * a.dim_x[2]);
    const double ny = std::sqrt(double(a.dim_y[0]) * a.dim_y[0] + double(a.dim_y[1]) * a.dim_y[1] +
                                double(a.dim_y[2]) * a.dim_y[2]);
    l.area = static_cast<float>(nx * ny);
  }
  pbf::DeviceGuard g(h->device);
  pbf::RenderState& R = h->render;
  if (R.scene_tri) cudaFree(R.scene_tri);
  if (R.scene_nrm) cudaFree(R.scene_nrm);
  R.scene_tri = nullptr;
  R.scene_nrm = nullptr;
  R.n_scene = 0;
  if (n_tri) {
    pbf_status st = h->cuda(cudaMalloc(&R.scene_tri, sizeof(pbf::RTri) * n_tri), "cudaMalloc(scene)");
    if (st == PBF_OK) st = h->cuda(cudaMalloc(&R.scene_nrm, sizeof(pbf::RNrm) * n_tri), "cudaMalloc(scene)");
    if (st == PBF_OK)
      st = h->cuda(cudaMemcpy(R.scene_tri, tri.data(), sizeof(pbf::RTri) * n_tri, cudaMemcpyHostToDevice), "H2D");
    if (st == PBF_OK)
      st = h->cuda(cudaMemcpy(R.scene_nrm, nrm.data(), sizeof(pbf::RNrm) * n_tri, cudaMemcpyHostToDevice), "H2D");
    if (st != PBF_OK) return st;
    R.n_scene = static_cast<uint32_t>(n_tri);
  }
  delete[] R.mats_host;
  delete[] R.lights_host;
  R.mats_host = new pbf::RMat[n_materials + 1];
  R.lights_host = new pbf::RLight[std::max<size_t>(n_lights, 1)];
  std::copy(mats.begin(), mats.end(), R.mats_host);
  std::copy(ls.begin(), ls.end(), R.lights_host);
  R.n_mat = static_cast<int>(n_materials);
  R.n_light = static_cast<int>(n_lights);
  return PBF_OK;
}

pbf_status pbf_render(pbf_handle* hh, const pbf_camera* cam, const pbf_render_params* p, float* hdr, uint8_t* rgba,
                      pbf_render_stats* stats) {
  if (!hh) return PBF_ERR_INVALID;
  Handle* h = reinterpret_cast<Handle*>(hh);
  if (!cam || !p) return h->fail(PBF_ERR_INVALID, "camera / params is NULL");
  if (p->width == 0 || p->height == 0 || p->width > 16384 || p->height > 16384)
    return h->fail(PBF_ERR_INVALID, "image size must be 1..16384 per side");
  if (p->ns_aa == 0 || p->ns_aa > 65536 || p->ns_area_light == 0 || p->ns_area_light > 65536 ||
      p->max_ray_depth > 1024)
    return h->fail(PBF_ERR_INVALID, "ns_aa, ns_area_light 1..65536 and max_ray_depth <= 1024");
  for (int k = 0; k < 9; ++k)
    if (!std::isfinite(cam->c2w[k])) return h->fail(PBF_ERR_INVALID, "non-finite camera");
  if (!(cam->hfov > 0 && cam->hfov < 180 && cam->vfov > 0 && cam->vfov < 180))
    return h->fail(PBF_ERR_INVALID, "fields of view must lie in (0, 180) degrees");
  pbf::DeviceGuard dg(h->device);
  pbf::RenderState& R = h->render;
  pbf_status st = PBF_OK;
  for (cudaEvent_t& e : R.ev)
    if (!e && st == PBF_OK) st = h->cuda(cudaEventCreate(&e), "event");
  if (st != PBF_OK) return st;
  st = h->cuda(cudaEventRecord(R.ev[0], h->stream), "event");
  if (st != PBF_OK) return st;
  // the fluid surface (Particles::updateSurface, particles.cpp:392-401)
  pbf::SurfGrid grid;
  uint32_t m = 0;
  const double iso = p->isolevel > 0 ? p->isolevel : 0.95 * h->params.rest_density;
  const double step = p->step > 0 ? p->step : 0.5 * h->params.h;
  if (p->fluid_surface) {
    st = h->surface_count(iso, step, p->surface_bounds ? p->surface_lo : nullptr,
                          p->surface_bounds ? p->surface_hi : nullptr, &grid, &m);
    if (st != PBF_OK) return st;
  }
  const size_t n = static_cast<size_t>(R.n_scene) + m;
  if (n >= pbf::kLeafBit) return h->fail(PBF_ERR_INVALID, "too many triangles");
  const size_t px = static_cast<size_t>(p->width) * p->height;
  const int slots = pbf::render_slots(R.lights_host, R.n_light, static_cast<int>(p->ns_area_light));
  const size_t batch = pbf::render_batch_samples(static_cast<int>(p->width), static_cast<int>(p->height),
                                                 static_cast<int>(p->ns_aa), slots, p->path_buffer_mib);
  if (px * batch >= (size_t(1) << 32) / std::max(slots, 1))
    return h->fail(PBF_ERR_INVALID, "frame too large: more than 2^32 shadow-ray slots in one batch");
  const size_t scene_tree = R.n_scene > pbf::kBruteScene ? R.n_scene : 0;
  size_t need = 0;
  carve(nullptr, n, scene_tree, m, R.n_mat, R.n_light, px, px * batch, slots, &need);
  if (need > R.buf_bytes) {
    if (R.buf) cudaFree(R.buf);
    R.buf = nullptr;
    R.buf_bytes = 0;
    st = h->cuda(cudaMalloc(&R.buf, need), "cudaMalloc(render)");
    if (st != PBF_OK) return st;
    R.buf_bytes = need;
  }
  size_t used = 0;
  const Frame f = carve(static_cast<char*>(R.buf), n, scene_tree, m, R.n_mat, R.n_light, px, px * batch, slots,
                        &used);
  std::vector<pbf::RMat> mats(R.mats_host, R.mats_host + R.n_mat);
  pbf::RMat fluid{};
  fluid.kind = pbf::kMatDiffuse;
  for (int k = 0; k < 3; ++k) fluid.c1[k] = p->fluid_albedo[k];
  mats.push_back(fluid);
  if (R.n_scene)
    st = h->cuda(cudaMemcpyAsync(f.tri, R.scene_tri, sizeof(pbf::RTri) * R.n_scene, cudaMemcpyDeviceToDevice,
                                 h->stream),
                 "D2D");
  if (st == PBF_OK && R.n_scene)
    st = h->cuda(cudaMemcpyAsync(f.nrm, R.scene_nrm, sizeof(pbf::RNrm) * R.n_scene, cudaMemcpyDeviceToDevice,
                                 h->stream),
                 "D2D");
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(f.mats, mats.data(), sizeof(pbf::RMat) * mats.size(), cudaMemcpyHostToDevice,
                                 h->stream),
                 "H2D");
  if (st == PBF_OK && R.n_light)
    st = h->cuda(cudaMemcpyAsync(f.lights, R.lights_host, sizeof(pbf::RLight) * R.n_light, cudaMemcpyHostToDevice,
                                 h->stream),
                 "H2D");
  if (st == PBF_OK) st = h->cuda(cudaMemsetAsync(f.err, 0, sizeof(unsigned), h->stream), "memset");
  if (st == PBF_OK && m) st = h->surface_emit(grid, iso, f.sxyz, f.snrm, m);
  if (st == PBF_OK && m)
    st = h->cuda(pbf::launch_surface_to_tris(f.sxyz, f.snrm, m, R.n_mat, f.tri + R.n_scene, f.nrm + R.n_scene,
                                             h->stream),
                 "surface triangles");
  if (st == PBF_OK) st = h->cuda(cudaEventRecord(R.ev[1], h->stream), "event");
  if (st == PBF_OK && scene_tree)
    st = h->cuda(pbf::launch_bvh_build(f.tri, R.n_scene, f.scene.w, f.scene.nodes, h->stream), "bvh build");
  if (st == PBF_OK)
    st = h->cuda(pbf::launch_bvh_build(f.tri + R.n_scene, m, f.surf.w, f.surf.nodes, h->stream), "bvh build");
  if (st == PBF_OK) st = h->cuda(cudaEventRecord(R.ev[2], h->stream), "event");
  pbf::RCam rc;
  for (int k = 0; k < 3; ++k) rc.pos[k] = static_cast<float>(cam->position[k]);
  for (int k = 0; k < 9; ++k) rc.c2w[k] = static_cast<float>(cam->c2w[k]);
  rc.htan = static_cast<float>(std::tan(cam->hfov / 180.0 * kPiD * 0.5) * 2);
  rc.vtan = static_cast<float>(std::tan(cam->vfov / 180.0 * kPiD * 0.5) * 2);
  rc.nclip = static_cast<float>(cam->nclip);
  rc.fclip = static_cast<float>(cam->fclip);
  pbf::RArgs a;
  a.width = static_cast<int>(p->width);
  a.height = static_cast<int>(p->height);
  a.ns_aa = static_cast<int>(p->ns_aa);
  a.max_depth = static_cast<int>(p->max_ray_depth);
  a.ns_area = static_cast<int>(p->ns_area_light);
  a.n_mat = static_cast<int>(mats.size());
  a.n_light = R.n_light;
  a.seed = p->seed;
  a.ray_eps = p->ray_eps > 0 ? p->ray_eps : 1e-4f;
  a.batch = static_cast<int>(batch);
  if (st == PBF_OK)
    st = h->cuda(pbf::launch_render(f.tri, f.nrm, R.n_scene, m, scene_tree ? f.scene.nodes : nullptr,
                                    f.scene.w.ltri, f.surf.nodes, f.surf.w.ltri, f.mats, f.lights, rc, a, f.wf, f.hdr,
                                    f.err, h->stream),
                 "render");
  if (st == PBF_OK && rgba)
    st = h->cuda(pbf::launch_tonemap(f.hdr, a.width, a.height, f.rgba, h->stream), "tonemap");
  if (st == PBF_OK) st = h->cuda(cudaEventRecord(R.ev[3], h->stream), "event");
  unsigned err = 0;
  if (st == PBF_OK)
    st = h->cuda(cudaMemcpyAsync(&err, f.err, sizeof(unsigned), cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK && hdr)
    st = h->cuda(cudaMemcpyAsync(hdr, f.hdr, sizeof(float) * 3 * px, cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK && rgba)
    st = h->cuda(cudaMemcpyAsync(rgba, f.rgba, 4 * px, cudaMemcpyDeviceToHost, h->stream), "D2H");
  if (st == PBF_OK) st = h->cuda(cudaStreamSynchronize(h->stream), "sync");
  if (st != PBF_OK) return st;
  if (err) return h->fail(PBF_ERR_CAPACITY, "a ray's hierarchy walk went deeper than 64 levels");
  if (stats) {
    float t[3] = {0, 0, 0};
    for (int k = 0; k < 3; ++k) cudaEventElapsedTime(&t[k], R.ev[k], R.ev[k + 1]);
    stats->triangles = n;
    stats->surface_triangles = m;
    stats->ms_surface = t[0];
    stats->ms_bvh = t[1];
    stats->ms_trace = t[2];
    stats->ms_total = double(t[0]) + t[1] + t[2];
  }
  return PBF_OK;
}

}  // extern "C"
