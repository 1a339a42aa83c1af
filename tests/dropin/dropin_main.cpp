// Drives the drop-in replacement particles.h (this directory) the way the reference's
// callers drive its src/particles.h, with the reference's own CGL::Vector3D, Color,
// BVHAccel and MarchingTriangle:
//
//   load   Application::load_particles (application.cpp:325-343): new Particles(density),
//          addParticle per <particle> record, estimateDensities();
//   bvh    PathTracer::build_accel(false) (pathtracer.cpp:237-270): the scene's primitives
//          (here the collider box's 12 walls as MarchingTriangles) in a BVHAccel, then
//          fluid_particles->bvh = bvh;
//   m      fluid_simulate_time_step (pathtracer.cpp:464-469): timeStep();
//   c      fluid_simulate_time(1) (pathtracer.cpp:444-462):
//          while (simulate_time < start + 1) timeStep();
//   h      build_accel(true): updateSurface() (the surface, then one step, as the
//          reference's does) and the surface's primitives added to the BVH.
//
// usage: pbf_dropin <particles.xml> <outdir>   |   pbf_dropin --params-string
// Each stage writes <outdir>/<stage>.bin: "PBFDROP1", int64 n, int64 steps of the stage,
// int64 surface triangles, float64 simulate_time, float32 positions (n, 3), velocities
// (n, 3), densities (n).
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "particles.h"
#include "pbf_xml.h"

using namespace CGL;
using StaticScene::BVHAccel;
using StaticScene::MarchingTriangle;
using StaticScene::Primitive;

namespace {

bool dump(const std::string& path, Particles* p, int64_t steps, int64_t surf) {
  std::FILE* f = std::fopen(path.c_str(), "wb");
  if (!f) return false;
  const int64_t n = static_cast<int64_t>(p->ps.size());
  const int64_t hdr[3] = {n, steps, surf};
  std::fwrite("PBFDROP1", 1, 8, f);
  std::fwrite(hdr, sizeof(int64_t), 3, f);
  std::fwrite(&p->simulate_time, sizeof(double), 1, f);
  std::vector<float> x(3 * n), v(3 * n), rho(n);
  for (int64_t i = 0; i < n; ++i) {
    const Vector3D q = p->ps[i]->getPosition();
    const Vector3D u = p->ps[i]->velocity;
    x[3 * i] = static_cast<float>(q.x);
    x[3 * i + 1] = static_cast<float>(q.y);
    x[3 * i + 2] = static_cast<float>(q.z);
    v[3 * i] = static_cast<float>(u.x);
    v[3 * i + 1] = static_cast<float>(u.y);
    v[3 * i + 2] = static_cast<float>(u.z);
    rho[i] = static_cast<float>(p->ps[i]->getLatestDensityEstimate());
  }
  std::fwrite(x.data(), sizeof(float), x.size(), f);
  std::fwrite(v.data(), sizeof(float), v.size(), f);
  std::fwrite(rho.data(), sizeof(float), rho.size(), f);
  return std::fclose(f) == 0;
}

// The box's six walls, two triangles each, normals facing inward (the scene geometry a
// COLLADA file would give the reference's PathTracer).
std::vector<Primitive*> box_walls(const double lo[3], const double hi[3]) {
  std::vector<Primitive*> prims;
  for (int a = 0; a < 3; ++a)
    for (int side = 0; side < 2; ++side) {
      const int b = (a + 1) % 3, c = (a + 2) % 3;
      double q[4][3];
      const double coord[4][2] = {{lo[b], lo[c]}, {hi[b], lo[c]}, {hi[b], hi[c]}, {lo[b], hi[c]}};
      for (int k = 0; k < 4; ++k) {
        q[k][a] = side ? hi[a] : lo[a];
        q[k][b] = coord[k][0];
        q[k][c] = coord[k][1];
      }
      Vector3D n(0, 0, 0);
      n[a] = side ? -1.0 : 1.0;
      const Vector3D p0(q[0][0], q[0][1], q[0][2]), p1(q[1][0], q[1][1], q[1][2]), p2(q[2][0], q[2][1], q[2][2]),
          p3(q[3][0], q[3][1], q[3][2]);
      prims.push_back(new MarchingTriangle(p0, p1, p2, n, n, n, nullptr));
      prims.push_back(new MarchingTriangle(p0, p2, p3, n, n, n, nullptr));
    }
  return prims;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc == 2 && std::string(argv[1]) == "--params-string") {
    Particles* p = new Particles(1000.0);  // prints the parameters, as the reference's constructor does
    delete p;
    return 0;
  }
  if (argc != 3) {
    std::fprintf(stderr, "usage: %s <particles.xml> <outdir> | --params-string\n", argv[0]);
    return 2;
  }
  pbf_host::ParticleFile file;
  std::string msg;
  if (pbf_host::load_particle_file(argv[1], &file, &msg) != pbf_host::LoadStatus::ok) {
    std::fprintf(stderr, "pbf_dropin: %s\n", msg.c_str());
    return 1;
  }
  const std::string out = argv[2];
  Particles::default_params() = file.params;  // the scene's constants and collider box

  // Application::load_particles
  Particles* particles = new Particles(file.rest_density);
  for (size_t i = 0; i < file.size(); ++i) {
    Vector3D pos(file.pos[3 * i], file.pos[3 * i + 1], file.pos[3 * i + 2]);
    Vector3D v(file.vel[3 * i], file.vel[3 * i + 1], file.vel[3 * i + 2]);
    particles->addParticle(pos, v);
  }
  particles->estimateDensities();
  if (!dump(out + "/load.bin", particles, 0, 0)) return 1;

  // PathTracer::build_accel(false)
  std::vector<Primitive*> primitives = box_walls(file.params.box_lo, file.params.box_hi);
  BVHAccel* bvh = new BVHAccel(primitives);
  particles->bvh = bvh;

  // key m
  particles->timeStep();
  if (!dump(out + "/m.bin", particles, 1, 0)) return 1;

  // key c
  const double start_t = particles->simulate_time;
  int64_t steps = 0;
  while (particles->simulate_time < start_t + 1) {
    particles->timeStep();
    ++steps;
  }
  if (!dump(out + "/c.bin", particles, steps, 0)) return 1;

  // key h: build_accel(true)
  particles->updateSurface();
  std::vector<Primitive*> with_surface = primitives;
  with_surface.insert(with_surface.end(), particles->surface.begin(), particles->surface.end());
  delete bvh;
  bvh = new BVHAccel(with_surface);
  particles->bvh = bvh;
  if (!dump(out + "/h.bin", particles, 1, static_cast<int64_t>(particles->surface.size()))) return 1;
  std::printf("pbf_dropin: %zu particles, %lld steps in one second, %zu surface triangles\n", particles->ps.size(),
              static_cast<long long>(steps), particles->surface.size());
  return 0;
}
