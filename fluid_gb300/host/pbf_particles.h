// C++ host facade with the reference's particle interface (src/particles.h:19-140),
// backed by the GB300 step through the C ABI of include/pbf.h.
//
// Particles / Particle keep the reference's member names and meanings so the
// reference's callers -- Application::load_particles (application.cpp:302-344),
// PathTracer's m/c/g/h keys and the -d mode (pathtracer.cpp:414-479) -- drive the
// GPU path unchanged. The classes are templates over the caller's 3-vector type V
// (anything with x, y, z members and a V(x, y, z) constructor, e.g. the
// reference's CGL::Vector3D) and colour type C (constructible from r, g, b, a).
//
//   Particles<V, C> p(rho0);              // Particles(double rest_density)
//   p.addParticle(pos, v);                // addParticle(Vector3D, Vector3D)
//   p.estimateDensities();                // estimateDensities()
//   p.timeStep(dt); p.timeStep();         // timeStep(double), timeStep()
//   p.ps[i]->getPosition() / getNewPosition() / getLatestDensityEstimate()
//   p.ps[i]->velocity, getDensityBasedColor(), p.estimateDensityAt(pos)
//   p.updateSurface(); p.surface; p.getSurfacePrims(iso, step)   // marching cubes
//   p.setColliderMesh(vertices)                                   // the BVH's triangles
//   p.setColliderSpheres(centres, radii)                           // the BVH's spheres
//   p.paramsString()                                              // the constants, as printed
//
// Differences, by design: the collider is the axis-aligned box of the pbf_params plus the
// triangles and spheres given to setColliderMesh / setColliderSpheres (the reference casts
// rays against a BVH of the scene's primitives; `bvh` is kept as an opaque, unused
// pointer); the XSPH pass is order-independent; positions, velocities and densities are
// FP32 on the device and mirrored into V after every step; Particle::neighbors stays empty
// (neighbour sets live on the device, see pbf_get_neighbors). Errors throw
// std::runtime_error with pbf_last_error().
#pragma once

#include <cstdio>
#include <iostream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "pbf.h"

namespace pbf_host {

struct Rgba {
  double r, g, b, a;
  Rgba(double r_, double g_, double b_, double a_) : r(r_), g(g_), b(b_), a(a_) {}
};

template <class V, class C>
class Particles;

template <class V, class C = Rgba>
class Particle {
 public:
  V velocity;
  std::vector<Particle*> neighbors;  // kept for source compatibility; not filled

  Particle(const V& p, const V& v, double rest_density)
      : velocity(v), position_(p), new_position_(p), density_(0.0), rest_density_(rest_density) {}

  double getLatestDensityEstimate() const { return density_; }
  const V getPosition() const { return position_; }
  const V getNewPosition() const { return new_position_; }

  // particles.h:48-52: red for dense, white at 0.8 rho0 and below.
  C getDensityBasedColor() const {
    const double ratio = (density_ - 0.8 * rest_density_) / (0.4 * rest_density_);
    const double c = ratio < 0.0 ? 0.0 : (ratio > 1.0 ? 1.0 : ratio);
    return C(1.0, 1.0 - c, 1.0 - c, 1.0);
  }

 private:
  friend class Particles<V, C>;
  V position_;
  V new_position_;
  double density_;
  double rest_density_;
};

// One triangle of the density-field surface with its vertex normals (the data of the
// reference's MarchingTriangle, static_scene/marching_triangle.h).
template <class V>
struct SurfaceTriangle {
  V p[3];
  V n[3];
};

template <class V, class C = Rgba>
class Particles {
 public:
  using ParticleT = Particle<V, C>;

  std::vector<ParticleT*> ps;
  void* bvh = nullptr;  // the reference's BVHAccel*; the GPU collider is params().box_*
  double simulate_time = 0.0;
  const double rest_density;
  std::vector<SurfaceTriangle<V>> surface;  // the reference's `surface` (MarchingTriangle primitives)
  bool surfaceUpToTimestep = false;

  explicit Particles(double rest_density_ = 1000.0, const pbf_params* params = nullptr, int device = 0)
      : rest_density(rest_density_), device_(device) {
    if (params) {
      prm_ = *params;
    } else {
      pbf_params_default(&prm_);
    }
    prm_.rest_density = rest_density_;
  }
  Particles(const Particles&) = delete;
  Particles& operator=(const Particles&) = delete;
  ~Particles() {
    if (h_) pbf_destroy(h_);
    for (ParticleT* p : ps) delete p;
  }

  void addParticle(V pos, V v) {
    ps.push_back(new ParticleT(pos, v, rest_density));
    dirty_ = true;
  }

  // Particles::timeStep(double), particles.cpp:250-297.
  void timeStep(double delta_t) {
    if (verbose_) std::cerr << "Time: " << simulate_time;
    simulate_time += delta_t;
    if (verbose_) std::cerr << " => " << simulate_time << std::endl;
    ensure_handle();
    check(pbf_step(h_, delta_t, 1));
    pull(true);
    if (verbose_) {
      pbf_stats s;
      check(pbf_get_stats(h_, &s));
      std::cout << "avg rho: " << s.mean_density_iter0 << " => " << s.mean_density << std::endl;
    }
    surfaceUpToTimestep = false;
  }
  // particles.cpp:299-301
  void timeStep() { timeStep(prm_.dt); }

  // particles.cpp:440-444: every particle's density at its position, self included.
  void estimateDensities() {
    if (ps.empty()) return;
    ensure_handle();
    std::vector<float> rho(ps.size());
    check(pbf_estimate_densities(h_, rho.data()));
    for (size_t i = 0; i < ps.size(); ++i) ps[i]->density_ = rho[i];
  }

  // particles.cpp:446-453
  double estimateDensityAt(V pos) {
    if (ps.empty()) return 0.0;
    ensure_handle();
    const float q[3] = {static_cast<float>(pos.x), static_cast<float>(pos.y), static_cast<float>(pos.z)};
    float out = 0.f;
    check(pbf_estimate_density_at(h_, 1, q, &out));
    return out;
  }

  // particles.cpp:352-385: the marching-cubes surface of the density field over the
  // reference's fixed bounds [-1, 1] x [0, 1.5] x [-1, 1] (lo / hi override them).
  std::vector<SurfaceTriangle<V>> getSurfacePrims(double isolevel, double fStepSize, const double* lo = nullptr,
                                                  const double* hi = nullptr) {
    std::vector<SurfaceTriangle<V>> out;
    if (ps.empty()) return out;
    ensure_handle();
    size_t total = 0;
    check(pbf_surface(h_, isolevel, fStepSize, lo, hi, nullptr, nullptr, 0, &total));
    std::vector<float> xyz(9 * total), nrm(9 * total);
    if (total) check(pbf_surface(h_, isolevel, fStepSize, lo, hi, xyz.data(), nrm.data(), total, &total));
    out.resize(total);
    for (size_t t = 0; t < total; ++t)
      for (int v = 0; v < 3; ++v) {
        const size_t k = 9 * t + 3 * v;
        out[t].p[v] = V(xyz[k], xyz[k + 1], xyz[k + 2]);
        out[t].n[v] = V(nrm[k], nrm[k + 1], nrm[k + 2]);
      }
    return out;
  }

  // particles.cpp:387-395: isolevel 0.95 rest density, step 0.5 H, once per time step.
  // The reference's updateSurface then takes one step of DEFAULT_DELTA_T (:397); this one
  // does not (its callers step themselves); tests/dropin/particles.h keeps that step.
  void updateSurface() {
    if (surfaceUpToTimestep) return;
    surface = getSurfacePrims(0.95 * rest_density, 0.5 * prm_.h);
    surfaceUpToTimestep = true;
  }

  // The collider's triangles besides the box walls (the reference ray-casts the triangles
  // of its scene's BVH, `bvh`): three vertices per triangle, in the order p1 p2 p3.
  void setColliderMesh(const std::vector<V>& vertices) {
    mesh_.assign(vertices.size() * 3, 0.f);
    for (size_t k = 0; k < vertices.size(); ++k) {
      mesh_[3 * k] = static_cast<float>(vertices[k].x);
      mesh_[3 * k + 1] = static_cast<float>(vertices[k].y);
      mesh_[3 * k + 2] = static_cast<float>(vertices[k].z);
    }
    if (h_ && !dirty_) check(pbf_set_collider_mesh(h_, mesh_.size() / 9, mesh_.data()));
  }

  // Solid spheres the particles collide with (the reference's Sphere primitives in its
  // scene's BVH, static_scene/sphere.cpp): one centre and one radius each.
  void setColliderSpheres(const std::vector<V>& centres, const std::vector<double>& radii) {
    if (centres.size() != radii.size()) throw std::invalid_argument("one radius per sphere centre");
    spheres_.assign(4 * centres.size(), 0.f);
    for (size_t k = 0; k < centres.size(); ++k) {
      spheres_[4 * k] = static_cast<float>(centres[k].x);
      spheres_[4 * k + 1] = static_cast<float>(centres[k].y);
      spheres_[4 * k + 2] = static_cast<float>(centres[k].z);
      spheres_[4 * k + 3] = static_cast<float>(radii[k]);
    }
    if (h_ && !dirty_) check(pbf_set_collider_spheres(h_, spheres_.size() / 4, spheres_.data()));
  }

  // particles.cpp:420-438: the step's and the surface's parameters, printed as the
  // reference prints them (its labels, default stream formatting); the visualisation
  // radius, bounce factor and marching-cube ratios are the reference's constants.
  std::string paramsString() const {
    std::ostringstream ss;
    ss << "Fluid simulation parameters: " << std::endl
       << "\tTime step: " << prm_.dt << std::endl
       << "\tSPH Density estimate radius H: " << prm_.h << std::endl
       << "\tNewton steps: " << prm_.iters << std::endl
       << "\tConstraint relaxation epsilon: " << prm_.epsilon << std::endl
       << "\tTensile artificial pressure coefficient K: " << prm_.scorr_k << std::endl
       << "\tTensile artificial pressure exponent N: " << prm_.scorr_n << std::endl
       << "\tVorticity confinement coefficient epsilon: " << prm_.vort_eps << std::endl
       << "\tViscosity coefficient C: " << prm_.xsph_c << std::endl
       << "\tParticle visualization radius: " << 0.05 << std::endl
       << "\tCollision response velocity factor: " << 0.6 << std::endl
       << "Marching cube parameters: " << std::endl
       << "\tIso-level / rest density ratio: " << 0.95 << std::endl
       << "\tGradient estimateion epsilon: " << 0.001 << std::endl
       << "\tStepsize / H ratio: " << 0.5 << std::endl;
    return ss.str();
  }

  const pbf_params& params() const { return prm_; }
  pbf_stats stats() {
    pbf_stats s{};
    if (h_) check(pbf_get_stats(h_, &s));
    return s;
  }
  // print the reference's per-step progress lines (particles.cpp:251-253, 267, 279, 295)
  void set_verbose(bool v) { verbose_ = v; }
  pbf_handle* handle() { return h_; }
  // The device simulator of the current particles (created or rebuilt if needed).
  pbf_handle* device_handle() {
    ensure_handle();
    return h_;
  }

 private:
  pbf_params prm_{};
  pbf_handle* h_ = nullptr;
  bool dirty_ = true;
  bool verbose_ = false;
  int device_ = 0;
  std::vector<float> mesh_;     // collider triangles, 9 floats each
  std::vector<float> spheres_;  // collider spheres: centre, radius

  void check(pbf_status st) const {
    if (st != PBF_OK) throw std::runtime_error(std::string("pbf: ") + pbf_last_error(h_));
  }

  // (Re)create the device simulator from the mirrors when particles were added.
  void ensure_handle() {
    if (h_ && !dirty_) return;
    if (h_) {
      pbf_destroy(h_);
      h_ = nullptr;
    }
    std::vector<float> x(3 * ps.size()), v(3 * ps.size());
    for (size_t i = 0; i < ps.size(); ++i) {
      const V& p = ps[i]->position_;
      const V& u = ps[i]->velocity;
      x[3 * i] = static_cast<float>(p.x);
      x[3 * i + 1] = static_cast<float>(p.y);
      x[3 * i + 2] = static_cast<float>(p.z);
      v[3 * i] = static_cast<float>(u.x);
      v[3 * i + 1] = static_cast<float>(u.y);
      v[3 * i + 2] = static_cast<float>(u.z);
    }
    pbf_handle* h = nullptr;
    const pbf_status st = pbf_create(&prm_, ps.size(), x.data(), v.data(), device_, &h);
    if (st != PBF_OK) throw std::runtime_error(std::string("pbf_create: ") + pbf_last_error(nullptr));
    h_ = h;
    dirty_ = false;
    if (!mesh_.empty()) check(pbf_set_collider_mesh(h_, mesh_.size() / 9, mesh_.data()));
    if (!spheres_.empty()) check(pbf_set_collider_spheres(h_, spheres_.size() / 4, spheres_.data()));
  }

  // Mirror device state into the Particle objects (original order).
  void pull(bool with_density) {
    const size_t n = ps.size();
    std::vector<float> x(3 * n), v(3 * n), rho(with_density ? n : 0);
    check(pbf_get_state(h_, x.data(), v.data(), with_density ? rho.data() : nullptr));
    for (size_t i = 0; i < n; ++i) {
      ParticleT* p = ps[i];
      p->position_ = V(x[3 * i], x[3 * i + 1], x[3 * i + 2]);
      p->new_position_ = p->position_;
      p->velocity = V(v[3 * i], v[3 * i + 1], v[3 * i + 2]);
      if (with_density) p->density_ = rho[i];
    }
  }
};

}  // namespace pbf_host
