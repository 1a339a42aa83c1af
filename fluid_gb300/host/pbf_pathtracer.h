// C++ host facade with the reference's PathTracer interface (src/pathtracer.h:57-160)
// for rendering the fluid, backed by pbf_render (include/pbf.h).
//
//   PathTracer<V> pt(ns_aa, max_ray_depth, ns_area_light);  // PathTracer(ns_aa, ...)
//   pt.set_frame_size(w, h); pt.set_camera(desc); pt.set_scene(scene);
//   pt.fluid_particles = &particles;                         // the public member
//   pt.render_to_file("frame.png");                          // render_to_file
//
// The reference builds the scene from COLLADA and renders on CPU threads with a BVH it
// rebuilds per frame (build_accel(true) with the fluid surface, pathtracer.cpp:237-270);
// here the scene is arrays of triangles, materials and lights, and each frame the device
// builds the surface, the hierarchy and the image. num_threads, ns_diff, ns_glsy, ns_refr
// and the environment map are accepted and unused (the reference's EnvironmentLight is
// black). Random numbers differ from the reference's std::rand stream: frame k uses
// seed + k. Errors throw std::runtime_error with pbf_last_error().
#pragma once

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <stdexcept>
#include <string>
#include <vector>

#include "pbf.h"
#include "pbf_particles.h"
#include "pbf_png.h"

namespace pbf_host {

// The scene the fluid is rendered in: 9 floats per triangle (vertices; vertex normals in
// nrm, or nrm empty for face normals), a material index per triangle.
struct SceneArrays {
  std::vector<float> tri, nrm;
  std::vector<uint32_t> material;
  std::vector<pbf_material> materials;
  std::vector<pbf_light> lights;
};

// A Cornell box on [lo, hi] with the front face (z = hi) open, the albedos of the
// reference's dae/sky/CBempty.dae, a 0.4 x 0.3 area light of radiance 5 under the
// ceiling and a camera in front of the opening (fluid_gb300.render.cornell_box builds
// the same scene).
inline SceneArrays cornell_box(const double lo[3], const double hi[3], pbf_camera_desc* cam) {
  SceneArrays s;
  auto mat = [](float r, float g, float b) {
    pbf_material m{};
    m.kind = PBF_MAT_DIFFUSE;
    m.c1[0] = r;
    m.c1[1] = g;
    m.c1[2] = b;
    m.ior = 1.f;
    return m;
  };
  s.materials = {mat(0.6f, 0.6f, 0.6f), mat(0.6f, 0.2f, 0.2f), mat(0.2f, 0.2f, 0.6f)};
  const double x0 = lo[0], y0 = lo[1], z0 = lo[2], x1 = hi[0], y1 = hi[1], z1 = hi[2];
  auto quad = [&](const double (&a)[3], const double (&b)[3], const double (&c)[3], const double (&d)[3], double nx,
                  double ny, double nz, uint32_t m) {
    const double* tri[2][3] = {{a, b, c}, {a, c, d}};
    for (auto& t : tri) {
      for (const double* v : t)
        for (int k = 0; k < 3; ++k) s.tri.push_back(static_cast<float>(v[k]));
      for (int v = 0; v < 3; ++v) {
        s.nrm.push_back(static_cast<float>(nx));
        s.nrm.push_back(static_cast<float>(ny));
        s.nrm.push_back(static_cast<float>(nz));
      }
      s.material.push_back(m);
    }
  };
  quad({x0, y0, z0}, {x1, y0, z0}, {x1, y0, z1}, {x0, y0, z1}, 0, 1, 0, 0);   // floor
  quad({x0, y1, z0}, {x0, y1, z1}, {x1, y1, z1}, {x1, y1, z0}, 0, -1, 0, 0);  // ceiling
  quad({x0, y0, z0}, {x0, y1, z0}, {x1, y1, z0}, {x1, y0, z0}, 0, 0, 1, 0);   // back
  quad({x0, y0, z0}, {x0, y0, z1}, {x0, y1, z1}, {x0, y1, z0}, 1, 0, 0, 1);   // left, red
  quad({x1, y0, z0}, {x1, y1, z0}, {x1, y1, z1}, {x1, y0, z1}, -1, 0, 0, 2);  // right, blue
  pbf_light l{};
  l.kind = PBF_LIGHT_AREA;
  l.radiance[0] = l.radiance[1] = l.radiance[2] = 5.f;
  l.position[0] = static_cast<float>((x0 + x1) / 2);
  l.position[1] = static_cast<float>(y1 - 0.01 * (y1 - y0));
  l.position[2] = static_cast<float>((z0 + z1) / 2);
  l.direction[1] = -1.f;
  l.dim_x[0] = static_cast<float>(0.4 * (x1 - x0));
  l.dim_y[2] = static_cast<float>(0.3 * (z1 - z0));
  s.lights = {l};
  if (cam) {
    const double size = std::max(x1 - x0, y1 - y0);
    *cam = pbf_camera_desc{};
    cam->hfov = 49.13434;
    cam->vfov = 38.0;
    cam->nclip = 0.1 * size;
    cam->fclip = 100.0 * size;
    cam->target[0] = (x0 + x1) / 2 + 0.0123 * size;
    cam->target[1] = (y0 + y1) / 2 + 0.0371 * size;
    cam->target[2] = (z0 + z1) / 2;
    cam->phi = 3.14159265358979323846 / 2 - 0.013;
    cam->theta = 0.011;
    cam->r = 2.1 * size;
    cam->min_r = 0.0;
    cam->max_r = 1e9;
  }
  return s;
}

template <class V, class C = Rgba>
class PathTracer {
 public:
  // PathTracer(ns_aa, max_ray_depth, ns_area_light, ns_diff, ns_glsy, ns_refr,
  // num_threads, envmap), pathtracer.cpp:28-64
  PathTracer(size_t ns_aa, size_t max_ray_depth, size_t ns_area_light, size_t ns_diff = 1, size_t ns_glsy = 1,
             size_t ns_refr = 1, size_t num_threads = 1, const void* envmap = nullptr)
      : ns_aa(ns_aa), max_ray_depth(max_ray_depth), ns_area_light(ns_area_light) {
    (void)ns_diff;
    (void)ns_glsy;
    (void)ns_refr;
    (void)num_threads;
    (void)envmap;
  }

  Particles<V, C>* fluid_particles = nullptr;
  size_t ns_aa, max_ray_depth, ns_area_light;
  uint64_t seed = 1;
  pbf_render_stats last_stats{};

  void set_frame_size(size_t width, size_t height) {
    if (width == 0 || height == 0) throw std::runtime_error("pbf: empty frame");
    w_ = width;
    h_ = height;
  }
  void set_camera(const pbf_camera_desc& d) {
    desc_ = d;
    have_camera_ = true;
  }
  void set_scene(const SceneArrays& s) { scene_ = s; }

  // One frame of the current particle state, written as an 8-bit RGBA PNG (top row
  // first), as render_to_file + save_image (pathtracer.cpp:187-235, 660-677).
  void render_to_file(const std::string& filename) {
    render();
    if (!write_png(filename, frame_.data(), static_cast<uint32_t>(w_), static_cast<uint32_t>(h_)))
      throw std::runtime_error("pbf: cannot write " + filename);
  }

  // One frame into frame() (RGBA, top row first).
  void render() {
    if (!fluid_particles) throw std::runtime_error("pbf: fluid_particles is not set");
    if (!have_camera_) throw std::runtime_error("pbf: no camera");
    pbf_handle* h = fluid_particles->device_handle();
    const size_t n = scene_.material.size();
    check(h, pbf_render_set_scene(h, n ? scene_.tri.data() : nullptr, scene_.nrm.empty() ? nullptr : scene_.nrm.data(),
                                  n ? scene_.material.data() : nullptr, n,
                                  scene_.materials.empty() ? nullptr : scene_.materials.data(),
                                  scene_.materials.size(), scene_.lights.empty() ? nullptr : scene_.lights.data(),
                                  scene_.lights.size()));
    pbf_camera cam;
    check(h, pbf_camera_frame(&desc_, static_cast<uint32_t>(w_), static_cast<uint32_t>(h_), &cam));
    pbf_render_params p;
    pbf_render_params_default(&p);
    p.width = static_cast<uint32_t>(w_);
    p.height = static_cast<uint32_t>(h_);
    p.ns_aa = static_cast<uint32_t>(ns_aa);
    p.max_ray_depth = static_cast<uint32_t>(max_ray_depth);
    p.ns_area_light = static_cast<uint32_t>(ns_area_light);
    p.seed = seed + frames_++;
    frame_.assign(4 * w_ * h_, 0);
    check(h, pbf_render(h, &cam, &p, nullptr, frame_.data(), &last_stats));
  }

  const std::vector<uint8_t>& frame() const { return frame_; }

 private:
  size_t w_ = 640, h_ = 480;
  pbf_camera_desc desc_{};
  bool have_camera_ = false;
  SceneArrays scene_;
  std::vector<uint8_t> frame_;
  uint64_t frames_ = 0;

  static void check(pbf_handle* h, pbf_status st) {
    if (st != PBF_OK) throw std::runtime_error(std::string("pbf: ") + pbf_last_error(h));
  }
};

}  // namespace pbf_host
