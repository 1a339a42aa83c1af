// pbf_run: headless driver for the GPU PBF step with the reference's key semantics.
//
// The reference drives its simulator from GLFW key presses (PathTracer::key_press,
// src/pathtracer.cpp:414-433) and from the windowless -d mode (src/main.cpp:159-170,
// Application::fluid_simulate_render_to_file). There is no window here, so the keys
// become command-line actions on the same Particles interface:
//
//   m  one step                                  (fluid_simulate_time_step, :464-469)
//   c  steps until one second has passed          (fluid_simulate_time(1), :444-462)
//   g  as c, dumping every frame                  (the reference saves a screenshot)
//   h  as c, dumping and path-tracing every frame (fluid_simulate_render_time, :471-479)
//   -d T  simulate T seconds, dumping and path-tracing every frame (the -d windowless
//         mode, main.cpp:159-170)
//   -f file.png  path-trace the loaded state once (the -f windowless mode)
//
// A frame dump is <dir>/frame_NNNNNN.bin: "PBFFRAME", int64 n, float64 time,
// float32 positions (n, 3), float32 densities (n). Path-traced frames are
// <dir>/frame_NNNNNN.png, rendered by pbf_render with the reference's options -s (camera
// rays per pixel), -l (samples per area light), -m (maximum ray depth) and -r W H
// (default 640 x 480), in a Cornell box on the particles' collider box (the reference
// loads its scene from a COLLADA file, which is not read here). With --surface every
// frame also writes <dir>/frame_NNNNNN.obj, the surface updateSurface builds for the
// path tracer (particles.cpp:387-395; vertices with their normals).
#include <cerrno>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <iostream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "pbf.h"
#include "pbf_particles.h"
#include "pbf_pathtracer.h"
#include "pbf_xml.h"

namespace {

struct Vec3 {
  double x = 0, y = 0, z = 0;
  Vec3() = default;
  Vec3(double a, double b, double c) : x(a), y(b), z(c) {}
};

using Sim = pbf_host::Particles<Vec3>;

struct Options {
  std::string file;
  std::string keys;
  double seconds = -1.0;
  std::string out = "pbf_out";
  bool parse_only = false;
  bool quiet = false;
  bool graph = false;
  bool surface = false;
  std::string png;  // -f
  int width = 640, height = 480, ns_aa = 1, ns_area = 1, depth = 1;
};

void usage() {
  std::fprintf(stderr,
               "usage: pbf_run -p particles.xml [-k keys] [-d seconds] [-o dir] [-f file.png] [-r W H] [-s rays]\n"
               "               [-l light_samples] [-m depth] [-t threads] [--graph] [--surface] [--quiet]\n"
               "       pbf_run -p particles.xml --parse-only\n"
               "  keys: m = one step, c = one second, g = one second with a frame dump per step,\n"
               "        h = one second with a frame dump and a path-traced PNG per step\n");
}

int frame_no = 0;

bool dump_surface = false;
pbf_host::PathTracer<Vec3>* tracer = nullptr;  // set while frames are path-traced

bool write_obj(Sim& sim, const std::string& path) {
  sim.surfaceUpToTimestep = false;
  sim.updateSurface();
  std::FILE* f = std::fopen(path.c_str(), "w");
  if (!f) return false;
  for (const auto& t : sim.surface)
    for (int v = 0; v < 3; ++v) std::fprintf(f, "v %.7g %.7g %.7g\n", t.p[v].x, t.p[v].y, t.p[v].z);
  for (const auto& t : sim.surface)
    for (int v = 0; v < 3; ++v) std::fprintf(f, "vn %.7g %.7g %.7g\n", t.n[v].x, t.n[v].y, t.n[v].z);
  for (size_t t = 0; t < sim.surface.size(); ++t) {
    const size_t a = 3 * t + 1;
    std::fprintf(f, "f %zu//%zu %zu//%zu %zu//%zu\n", a, a, a + 1, a + 1, a + 2, a + 2);
  }
  return std::fclose(f) == 0;
}

bool dump(Sim& sim, const std::string& dir) {
  char name[64];
  if (dump_surface) {
    std::snprintf(name, sizeof(name), "/frame_%06d.obj", frame_no);
    if (!write_obj(sim, dir + name)) return false;
  }
  if (tracer) {
    std::snprintf(name, sizeof(name), "/frame_%06d.png", frame_no);
    tracer->render_to_file(dir + name);
  }
  std::snprintf(name, sizeof(name), "/frame_%06d.bin", frame_no++);
  std::FILE* f = std::fopen((dir + name).c_str(), "wb");
  if (!f) return false;
  const int64_t n = static_cast<int64_t>(sim.ps.size());
  std::fwrite("PBFFRAME", 1, 8, f);
  std::fwrite(&n, sizeof(n), 1, f);
  std::fwrite(&sim.simulate_time, sizeof(double), 1, f);
  std::vector<float> x(3 * n), rho(n);
  for (int64_t i = 0; i < n; ++i) {
    const Vec3 p = sim.ps[i]->getPosition();
    x[3 * i] = static_cast<float>(p.x);
    x[3 * i + 1] = static_cast<float>(p.y);
    x[3 * i + 2] = static_cast<float>(p.z);
    rho[i] = static_cast<float>(sim.ps[i]->getLatestDensityEstimate());
  }
  std::fwrite(x.data(), sizeof(float), x.size(), f);
  std::fwrite(rho.data(), sizeof(float), rho.size(), f);
  return std::fclose(f) == 0;
}

// PathTracer::fluid_simulate_time: step until `delta` seconds have passed.
bool simulate_time(Sim& sim, double delta, bool dump_frames, const std::string& dir) {
  const double start = sim.simulate_time;
  if (dump_frames && !dump(sim, dir)) return false;
  while (sim.simulate_time < start + delta) {
    sim.timeStep();
    if (dump_frames && !dump(sim, dir)) return false;
  }
  return true;
}

}  // namespace

int main(int argc, char** argv) {
  Options o;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    auto next = [&]() -> std::string {
      if (i + 1 >= argc) {
        usage();
        std::exit(2);
      }
      return argv[++i];
    };
    if (a == "-p") o.file = next();
    else if (a == "-k") o.keys += next();
    else if (a == "-d") o.seconds = std::atof(next().c_str());
    else if (a == "-o") o.out = next();
    else if (a == "--parse-only") o.parse_only = true;
    else if (a == "--quiet") o.quiet = true;
    else if (a == "--graph") o.graph = true;
    else if (a == "--surface") o.surface = true;
    else if (a == "-f") o.png = next();
    else if (a == "-s") o.ns_aa = std::atoi(next().c_str());
    else if (a == "-l") o.ns_area = std::atoi(next().c_str());
    else if (a == "-m") o.depth = std::atoi(next().c_str());
    else if (a == "-t") (void)next();  // render threads: the GPU renders
    else if (a == "-r") {
      o.width = std::atoi(next().c_str());
      o.height = std::atoi(next().c_str());
    }
    else {
      usage();
      return 2;
    }
  }
  pbf_host::ParticleFile pf;
  std::string msg;
  const pbf_host::LoadStatus st = pbf_host::load_particle_file(o.file, &pf, &msg);
  if (st == pbf_host::LoadStatus::missing) {
    // application.cpp:303-308 warns and continues with an empty Particles()
    std::cout << "[Warning] Particle file not passed in or not found\n";
  } else if (st != pbf_host::LoadStatus::ok) {
    std::cout << "[ERROR] " << msg << std::endl;  // application.cpp:311-317 exits on XML errors
    return EXIT_FAILURE;
  }
  if (o.parse_only) {
    std::printf("particles %zu rest_density %.9g h %.9g iters %d dt %.9g params %s\n", pf.size(), pf.rest_density,
                pf.params.h, pf.params.iters, pf.params.dt, pf.has_params ? "file" : "default");
    return 0;
  }
  pbf_params prm = pf.params;
  if (o.graph) prm.flags |= PBF_FLAG_GRAPH;
  dump_surface = o.surface;
  try {
    Sim sim(pf.rest_density, &prm);
    sim.set_verbose(!o.quiet);
    for (size_t i = 0; i < pf.size(); ++i) {
      sim.addParticle(Vec3(pf.pos[3 * i], pf.pos[3 * i + 1], pf.pos[3 * i + 2]),
                      Vec3(pf.vel[3 * i], pf.vel[3 * i + 1], pf.vel[3 * i + 2]));
    }
    sim.estimateDensities();  // application.cpp:342
    if (o.ns_aa < 1 || o.ns_area < 1 || o.depth < 0 || o.width < 1 || o.height < 1) {
      usage();
      return 2;
    }
    pbf_host::PathTracer<Vec3> pt(o.ns_aa, o.depth, o.ns_area);
    pbf_camera_desc cam;
    pt.set_scene(pbf_host::cornell_box(prm.box_lo, prm.box_hi, &cam));
    pt.set_camera(cam);
    pt.set_frame_size(o.width, o.height);
    pt.fluid_particles = &sim;
    if (!o.png.empty()) {
      pt.render_to_file(o.png);
      std::cout << "[PathTracer] Saved " << o.png << "\n";
    }    const bool needs_dir = o.seconds >= 0 || o.keys.find_first_of("gGhH") != std::string::npos;
    if (needs_dir && mkdir(o.out.c_str(), 0755) != 0 && errno != EEXIST) {
      std::cerr << "cannot create " << o.out << "\n";
      return EXIT_FAILURE;
    }
    for (char k : o.keys) {
      switch (k) {
        case 'm': case 'M':
          sim.timeStep();
          std::cout << "[Fluid Simulation] Fluid particles updated.\n";
          break;
        case 'c': case 'C':
          simulate_time(sim, 1.0, false, o.out);
          std::cout << "[Fluid Simulation] Fluid particles updated.\n";
          break;
        case 'g': case 'G':
          if (!simulate_time(sim, 1.0, true, o.out)) return EXIT_FAILURE;
          std::cout << "[Fluid Simulation] Fluid particles updated, frames saved.\n";
          break;
        case 'h': case 'H':
          tracer = &pt;
          if (!simulate_time(sim, 1.0, true, o.out)) return EXIT_FAILURE;
          tracer = nullptr;
          std::cout << "[Fluid Simulation] Fluid particles updated, screenshots saved.\n";
          break;
        default:
          std::cerr << "unknown key '" << k << "'\n";
          return 2;
      }
    }
    if (o.seconds >= 0) {
      tracer = &pt;
      if (!simulate_time(sim, o.seconds, true, o.out)) return EXIT_FAILURE;
      tracer = nullptr;
    }
    if (o.keys.empty() && o.seconds < 0 && o.png.empty() && !dump(sim, o.out.empty() ? "." : o.out)) {
      // nothing requested: write the loaded state for inspection
    }
  } catch (const std::exception& e) {
    std::cerr << e.what() << "\n";
    return EXIT_FAILURE;
  }
  return 0;
}
