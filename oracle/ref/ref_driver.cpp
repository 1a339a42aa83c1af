// Headless driver for the reference's own PBF step (test infrastructure: the
// oracle). It links the reference's src/particles.cpp (parameter block turned
// into runtime globals by build_ref.py), src/bvh.cpp, src/bbox.cpp and
// src/static_scene/marching_triangle.cpp, builds the reference's triangle
// collider for an axis-aligned box, and runs K steps of either
//
//   mode 0 "literal": the reference's Particles::timeStep(dt)
//                     (src/particles.cpp:250-297), unchanged; or
//   mode 1 "jacobi":  the same sequence of the reference's public Particle
//                     methods, except that the XSPH/vorticity pass
//                     (src/particles.cpp:285-288, 219-234) sees the
//                     pre-XSPH velocity (x* - x)/dt of every neighbour.
//                     This is the order-independent form a parallel
//                     implementation computes.
//
// I/O is a small little-endian binary format written/read by
// oracle/ref_runner.py:
//   in : "PBFREFI1" i64 n, steps, mode, iters, flags, open_mask
//        f64 h, h2, dt, gravity, rest_density, epsilon, k, vort_eps, xsph_c
//        f64 box_lo[3], box_hi[3], pos[3n], vel[3n]
//   out: "PBFREFO1" i64 n, f64 pos[3n], vel[3n], density[n],
//        load_density[n], i64 nnz, i64 offsets[n+1], i64 idx[nnz],
//        f64 seconds
// flags: 2 = dump neighbour lists of the last step, 4 = run
// Particles::estimateDensities() (src/particles.cpp:440-444) before stepping,
// 8 = restart: every step starts again from the input state (a fresh
// Particles built untimed), so `seconds` times K steps of the same input,
// 16 = surface: after the steps, the triangles of the reference's surface
// (appended: i64 ntri, f64 xyz[9 ntri], f64 nrm[9 ntri], i64 cube[ntri]),
// 32 = collider mesh: the input continues with i64 m, f64 tri[9 m]; each
// triangle joins the box in the BVH as a MarchingTriangle with the normal
// ((p2 - p1) x (p3 - p1)).unit() at its three vertices,
// 64 = collider spheres: the input continues with i64 m, f64 xyzr[4 m]; each sphere
// joins the BVH as the reference's Sphere primitive (static_scene/sphere.cpp).
// --params-string: construct Particles with the default constants (its constructor
// prints paramsString()) and exit.
// open_mask: bit per box face to leave out (0 x-lo, 1 x-hi, 2 y-lo, 3 y-hi,
// 4 z-lo, 5 z-hi).
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <unordered_map>
#include <vector>

#include "particles.h"  // includes marching.h (polygonise), which has no include guard
#include "ref_params.h"
#include "ref_surface.h"
#include "static_scene/marching_triangle.h"
#include "static_scene/object.h"
#include "static_scene/sphere.h"

double pbf_ref_dt = 0.016;
double pbf_ref_h = 0.3;
double pbf_ref_h2 = 0.09;
int pbf_ref_iters = 12;
double pbf_ref_epsilon = 2;
double pbf_ref_k = 0.0001;
double pbf_ref_vort_eps = 0.001;
double pbf_ref_xsph_c = 0.001;
double pbf_ref_gravity = 10;

namespace CGL {
void pbf_ref_reinit_statics();
}

using namespace CGL;

// The reference defines SphereObject's members in static_scene/object.cpp, next to the
// polygon-mesh object whose code needs the half-edge mesh library; this driver links the
// reference's Sphere primitive (sphere.cpp) without object.cpp, so the three members a
// Sphere's material lookup reaches are defined here: keep the centre, radius and
// material; list the one Sphere primitive; hand out the material.
namespace CGL {
namespace StaticScene {
SphereObject::SphereObject(const Vector3D& o_, double r_, BSDF* bsdf_) : o(o_), r(r_), bsdf(bsdf_) {}
std::vector<Primitive*> SphereObject::get_primitives() const {
  return std::vector<Primitive*>(1, new Sphere(this, o, r));
}
BSDF* SphereObject::get_bsdf() const { return bsdf; }
}  // namespace StaticScene
}  // namespace CGL

namespace {

template <typename T>
void rd(std::ifstream& f, T* p, size_t count) {
  f.read(reinterpret_cast<char*>(p), sizeof(T) * count);
  if (!f) {
    std::fprintf(stderr, "ref_driver: short read\n");
    std::exit(2);
  }
}

template <typename T>
void wr(std::ofstream& f, const T* p, size_t count) {
  f.write(reinterpret_cast<const char*>(p), sizeof(T) * count);
}

// 12 (or fewer) triangles of the box [lo, hi] with inward vertex normals.
std::vector<Primitive*> box_triangles(const double lo[3], const double hi[3],
                                      int open_mask) {
  std::vector<Primitive*> prims;
  for (int axis = 0; axis < 3; ++axis) {
    for (int side = 0; side < 2; ++side) {
      if (open_mask & (1 << (2 * axis + side))) continue;
      int u = (axis + 1) % 3, v = (axis + 2) % 3;
      double c = side ? hi[axis] : lo[axis];
      Vector3D corner[4];
      double us[4] = {lo[u], hi[u], hi[u], lo[u]};
      double vs[4] = {lo[v], lo[v], hi[v], hi[v]};
      for (int k = 0; k < 4; ++k) {
        corner[k][axis] = c;
        corner[k][u] = us[k];
        corner[k][v] = vs[k];
      }
      Vector3D n;
      n[axis] = side ? -1.0 : 1.0;
      prims.push_back(new MarchingTriangle(corner[0], corner[1], corner[2], n,
                                           n, n, nullptr));
      prims.push_back(new MarchingTriangle(corner[0], corner[2], corner[3], n,
                                           n, n, nullptr));
    }
  }
  return prims;
}

// Same call sequence as Particles::timeStep (src/particles.cpp:250-297) with
// the XSPH pass made order-independent (see file comment).
void step_jacobi(Particles& P, double dt) {
  std::vector<Particle*>& ps = P.ps;
  P.simulate_time += dt;
  for (Particle* p : ps) {
    p->neighbors.clear();
    p->applyForceVelocity(P.bvh, dt);
  }
  for (size_t i = 0; i < ps.size(); i++) {
    for (size_t j = i + 1; j < ps.size(); j++) {
      if ((ps[i]->getNewPosition() - ps[j]->getNewPosition()).norm2() <=
          pbf_ref_h2) {
        ps[i]->neighbors.push_back(ps[j]);
        ps[j]->neighbors.push_back(ps[i]);
      }
    }
  }
  for (Particle* p : ps) p->initializeWithNewNeighbors();
  for (int it = 0; it < pbf_ref_iters; it++) {
    for (Particle* p : ps) p->newtonStepCalculateLambda();
    for (Particle* p : ps) p->newtonStepUpdatePosition(P.bvh);
  }
  for (Particle* p : ps) p->updateVelocity(dt);
  std::vector<Vector3D> v_pre(ps.size()), v_post(ps.size());
  for (size_t i = 0; i < ps.size(); i++) v_pre[i] = ps[i]->velocity;
  for (size_t i = 0; i < ps.size(); i++) {
    ps[i]->calculateVorticityApplyXSPHViscosity();
    v_post[i] = ps[i]->velocity;
    ps[i]->velocity = v_pre[i];
  }
  for (size_t i = 0; i < ps.size(); i++) ps[i]->velocity = v_post[i];
  for (Particle* p : ps) {
    p->applyVorticity(dt);
    p->updatePosition();
  }
  P.surfaceUpToTimestep = false;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc == 2 && std::strcmp(argv[1], "--params-string") == 0) {
    // the reference's constructor prints Particles::paramsString() (particles.h:114-116)
    // with the reference's default constants
    Particles* P = new Particles(1000.0);
    (void)P;
    return 0;
  }
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s <in.bin> <out.bin> | --params-string\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1], std::ios::binary);
  if (!in) {
    std::fprintf(stderr, "ref_driver: cannot open %s\n", argv[1]);
    return 2;
  }
  char magic[8];
  rd(in, magic, 8);
  if (std::memcmp(magic, "PBFREFI1", 8) != 0) {
    std::fprintf(stderr, "ref_driver: bad magic\n");
    return 2;
  }
  int64_t hdr[6];
  rd(in, hdr, 6);
  const int64_t n = hdr[0], steps = hdr[1], mode = hdr[2], iters = hdr[3],
                flags = hdr[4], open_mask = hdr[5];
  double prm[9];
  rd(in, prm, 9);
  double lo[3], hi[3];
  rd(in, lo, 3);
  rd(in, hi, 3);
  std::vector<double> pos(3 * n), vel(3 * n);
  rd(in, pos.data(), pos.size());
  rd(in, vel.data(), vel.size());

  pbf_ref_h = prm[0];
  pbf_ref_h2 = prm[1];
  pbf_ref_dt = prm[2];
  pbf_ref_gravity = prm[3];
  const double rest_density = prm[4];
  pbf_ref_epsilon = prm[5];
  pbf_ref_k = prm[6];
  pbf_ref_vort_eps = prm[7];
  pbf_ref_xsph_c = prm[8];
  pbf_ref_iters = static_cast<int>(iters);
  CGL::pbf_ref_reinit_statics();

  // The reference prints per-step progress and one line per particle with
  // few neighbours; silence all of it.
  std::ostringstream sink;
  std::streambuf* old_out = std::cout.rdbuf(sink.rdbuf());
  std::streambuf* old_err = std::cerr.rdbuf(sink.rdbuf());
  std::FILE* devnull = std::freopen("/dev/null", "w", stdout);
  (void)devnull;

  std::vector<Primitive*> prims = box_triangles(lo, hi, static_cast<int>(open_mask));
  if (flags & 32) {
    int64_t m = 0;
    rd(in, &m, 1);
    std::vector<double> tri(9 * m);
    rd(in, tri.data(), tri.size());
    for (int64_t t = 0; t < m; t++) {
      const double* q = tri.data() + 9 * t;
      Vector3D p1(q[0], q[1], q[2]), p2(q[3], q[4], q[5]), p3(q[6], q[7], q[8]);
      Vector3D nn = cross(p2 - p1, p3 - p1).unit();
      prims.push_back(new MarchingTriangle(p1, p2, p3, nn, nn, nn, nullptr));
    }
  }
  if (flags & 64) {  // collider spheres: the reference's Sphere primitives in the same BVH
    int64_t m = 0;
    rd(in, &m, 1);
    std::vector<double> q(4 * m);
    rd(in, q.data(), q.size());
    for (int64_t k = 0; k < m; k++) {
      const Vector3D o(q[4 * k], q[4 * k + 1], q[4 * k + 2]);
      const SphereObject* obj = new SphereObject(o, q[4 * k + 3], nullptr);
      std::vector<Primitive*> sp = obj->get_primitives();
      prims.insert(prims.end(), sp.begin(), sp.end());
    }
  }
  BVHAccel* bvh = new BVHAccel(prims);

  auto make = [&]() {
    Particles* P = new Particles(rest_density);
    P->bvh = bvh;
    for (int64_t i = 0; i < n; i++) {
      P->addParticle(Vector3D(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]),
                     Vector3D(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]));
    }
    return P;
  };
  Particles* Pp = make();
  std::vector<double> load_density(n, 0.0);
  if (flags & 4) {
    Pp->estimateDensities();
    for (int64_t i = 0; i < n; i++)
      load_density[i] = Pp->ps[i]->getLatestDensityEstimate();
  }

  double seconds = 0.0;
  for (int64_t s = 0; s < steps; s++) {
    if ((flags & 8) && s > 0) {
      for (Particle* q : Pp->ps) delete q;
      delete Pp;
      Pp = make();
    }
    auto t0 = std::chrono::steady_clock::now();
    if (mode == 0) {
      Pp->timeStep(pbf_ref_dt);
    } else {
      step_jacobi(*Pp, pbf_ref_dt);
    }
    auto t1 = std::chrono::steady_clock::now();
    seconds += std::chrono::duration<double>(t1 - t0).count();
    sink.str("");
  }
  Particles& P = *Pp;
  std::cout.rdbuf(old_out);
  std::cerr.rdbuf(old_err);

  std::vector<double> out_pos(3 * n), out_vel(3 * n), dens(n);
  std::unordered_map<const Particle*, int64_t> index;
  for (int64_t i = 0; i < n; i++) {
    Particle* p = P.ps[i];
    index[p] = i;
    Vector3D x = p->getPosition();
    for (int k = 0; k < 3; k++) {
      out_pos[3 * i + k] = x[k];
      out_vel[3 * i + k] = p->velocity[k];
    }
    dens[i] = p->getLatestDensityEstimate();
  }
  std::vector<int64_t> offsets(n + 1, 0), idx;
  if (flags & 2) {
    for (int64_t i = 0; i < n; i++) {
      for (const Particle* q : P.ps[i]->neighbors) idx.push_back(index[q]);
      offsets[i + 1] = static_cast<int64_t>(idx.size());
    }
  }
  // flag 16: the loop of Particles::getSurfacePrims (src/particles.cpp:352-385), which
  // builds MarchingTriangle primitives whose vertices are private, run over the
  // reference's own generateGridCell, polygonise (src/marching.cpp) and
  // getVertexNormal, with updateSurface's arguments (src/particles.cpp:387-395):
  // isolevel ISO_LEVEL_REST_DENSITY_RATIO (0.95, :14) x rest density, step
  // FSTEPSIZE_RATIO (0.5, :18) x H.
  std::vector<double> sxyz, snrm;
  std::vector<int64_t> scube;
  if (flags & 16) {
    std::cout.rdbuf(sink.rdbuf());
    pbf_ref::surface_triangles(P, 0.95 * rest_density, pbf_ref_h * 0.5, &sxyz, &snrm, &scube);
    std::cout.rdbuf(old_out);
  }
  std::ofstream out(argv[2], std::ios::binary);
  out.write("PBFREFO1", 8);
  wr(out, &n, 1);
  wr(out, out_pos.data(), out_pos.size());
  wr(out, out_vel.data(), out_vel.size());
  wr(out, dens.data(), dens.size());
  wr(out, load_density.data(), load_density.size());
  int64_t nnz = static_cast<int64_t>(idx.size());
  wr(out, &nnz, 1);
  wr(out, offsets.data(), offsets.size());
  wr(out, idx.data(), idx.size());
  wr(out, &seconds, 1);
  if (flags & 16) {
    const int64_t nt = static_cast<int64_t>(scube.size());
    wr(out, &nt, 1);
    wr(out, sxyz.data(), sxyz.size());
    wr(out, snrm.data(), snrm.size());
    wr(out, scube.data(), scube.size());
  }
  return out ? 0 : 3;
}
