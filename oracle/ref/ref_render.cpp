// Headless driver for the reference's own path tracer (test infrastructure: the
// oracle of the renderer). It links the reference's src/pathtracer.cpp,
// src/bsdf.cpp, src/static_scene/light.cpp, src/camera.cpp, src/bvh.cpp and the
// particle code of the step driver, and renders one frame through the
// reference's public path: PathTracer::set_frame_size / set_camera / set_scene,
// then render_to_file (src/pathtracer.cpp:187-235), which rebuilds the BVH with
// the fluid surface of Particles::updateSurface (src/particles.cpp:392-401),
// renders every tile on one worker thread (tiles in queue order, pixels row by
// row) and writes the tone-mapped frame as a PNG through lodepng. The random
// numbers come from std::rand, seeded here with srand(seed) before the render.
//
// Scene objects are MarchingTriangle primitives with the given vertex normals
// and one BSDF each; no GL is loaded: the drawing routines the linked
// translation units reference are the aborting stubs of gl_link_stubs.cpp.
//
// I/O (little-endian, written/read by oracle/ref_runner.py):
//   in : "PBFRNDI1" i64 n, width, height, ns_aa, max_depth, ns_area_light,
//        seed, n_tri, n_mat, n_light
//        f64 h, h2, rest_density, pos[3n], tri[9 n_tri], nrm[9 n_tri]
//        i64 tri_mat[n_tri]
//        per material: i64 kind, f64 c1[3], c2[3], ior
//          (0 diffuse albedo=c1, 1 mirror reflectance=c1, 2 glass
//           transmittance=c1 reflectance=c2, 3 refraction transmittance=c1,
//           4 emission radiance=c1)
//        per light: i64 kind, f64 radiance[3], position[3], direction[3],
//          dim_x[3], dim_y[3]
//          (0 directional (direction), 1 infinite hemisphere, 2 point
//           (position), 3 area)
//        f64 hfov, vfov, nclip, fclip, target[3], phi, theta, r, min_r, max_r
//   out: argv[2] the PNG; argv[3] "PBFRNDO1" f64 camera position[3],
//        up_dir[3], v_fov, i64 ntri, f64 xyz[9 ntri], nrm[9 ntri] (the fluid
//        surface, getSurfacePrims order), f64 seconds of the render.
#include <chrono>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iostream>
#include <sstream>
#include <vector>

#include "particles.h"  // includes marching.h (polygonise), which has no include guard
#include "pathtracer.h"
#include "ref_params.h"
#include "ref_surface.h"
#include "static_scene/light.h"
#include "static_scene/marching_triangle.h"
#include "static_scene/scene.h"

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
using namespace CGL::StaticScene;

namespace {

template <typename T>
void rd(std::ifstream& f, T* p, size_t count) {
  f.read(reinterpret_cast<char*>(p), sizeof(T) * count);
  if (!f) {
    std::fprintf(stderr, "ref_render: short read\n");
    std::exit(2);
  }
}

template <typename T>
void wr(std::ofstream& f, const T* p, size_t count) {
  f.write(reinterpret_cast<const char*>(p), sizeof(T) * count);
}

Vector3D v3(const double* a) { return Vector3D(a[0], a[1], a[2]); }
Spectrum sp(const double* a) { return Spectrum(a[0], a[1], a[2]); }

// A fixed set of primitives, each carrying its own BSDF.
class TriangleSoup : public SceneObject {
 public:
  explicit TriangleSoup(std::vector<Primitive*> p) : prims_(std::move(p)) {}
  std::vector<Primitive*> get_primitives() const override { return prims_; }
  BSDF* get_bsdf() const override { return nullptr; }

 private:
  std::vector<Primitive*> prims_;
};

}  // namespace

int main(int argc, char** argv) {
  if (argc != 4) {
    std::fprintf(stderr, "usage: %s <in.bin> <out.png> <out.bin>\n", argv[0]);
    return 2;
  }
  std::ifstream in(argv[1], std::ios::binary);
  if (!in) {
    std::fprintf(stderr, "ref_render: cannot open %s\n", argv[1]);
    return 2;
  }
  char magic[8];
  rd(in, magic, 8);
  if (std::memcmp(magic, "PBFRNDI1", 8) != 0) {
    std::fprintf(stderr, "ref_render: bad magic\n");
    return 2;
  }
  int64_t hdr[10];
  rd(in, hdr, 10);
  const int64_t n = hdr[0], width = hdr[1], height = hdr[2], ns_aa = hdr[3], max_depth = hdr[4],
                ns_area = hdr[5], seed = hdr[6], n_tri = hdr[7], n_mat = hdr[8], n_light = hdr[9];
  double prm[3];
  rd(in, prm, 3);
  pbf_ref_h = prm[0];
  pbf_ref_h2 = prm[1];
  const double rest_density = prm[2];
  CGL::pbf_ref_reinit_statics();
  std::vector<double> pos(3 * n), tri(9 * n_tri), nrm(9 * n_tri);
  std::vector<int64_t> tri_mat(n_tri);
  rd(in, pos.data(), pos.size());
  rd(in, tri.data(), tri.size());
  rd(in, nrm.data(), nrm.size());
  rd(in, tri_mat.data(), tri_mat.size());

  std::vector<BSDF*> mats;
  for (int64_t m = 0; m < n_mat; m++) {
    int64_t kind;
    double c1[3], c2[3], ior;
    rd(in, &kind, 1);
    rd(in, c1, 3);
    rd(in, c2, 3);
    rd(in, &ior, 1);
    switch (kind) {
      case 0: mats.push_back(new DiffuseBSDF(sp(c1))); break;
      case 1: mats.push_back(new MirrorBSDF(sp(c1))); break;
      case 2: mats.push_back(new GlassBSDF(sp(c1), sp(c2), 0.f, static_cast<float>(ior))); break;
      case 3: mats.push_back(new RefractionBSDF(sp(c1), 0.f, static_cast<float>(ior))); break;
      case 4: mats.push_back(new EmissionBSDF(sp(c1))); break;
      default: std::fprintf(stderr, "ref_render: material kind %lld\n", (long long)kind); return 2;
    }
  }
  std::vector<SceneLight*> lights;
  for (int64_t l = 0; l < n_light; l++) {
    int64_t kind;
    double rad[3], p[3], d[3], dx[3], dy[3];
    rd(in, &kind, 1);
    rd(in, rad, 3);
    rd(in, p, 3);
    rd(in, d, 3);
    rd(in, dx, 3);
    rd(in, dy, 3);
    switch (kind) {
      case 0: lights.push_back(new DirectionalLight(sp(rad), v3(d))); break;
      case 1: lights.push_back(new InfiniteHemisphereLight(sp(rad))); break;
      case 2: lights.push_back(new PointLight(sp(rad), v3(p))); break;
      case 3: lights.push_back(new AreaLight(sp(rad), v3(p), v3(d), v3(dx), v3(dy))); break;
      default: std::fprintf(stderr, "ref_render: light kind %lld\n", (long long)kind); return 2;
    }
  }
  double cam[12];
  rd(in, cam, 12);

  std::vector<Primitive*> prims;
  for (int64_t t = 0; t < n_tri; t++) {
    const double* q = tri.data() + 9 * t;
    const double* m = nrm.data() + 9 * t;
    prims.push_back(new MarchingTriangle(v3(q), v3(q + 3), v3(q + 6), v3(m), v3(m + 3), v3(m + 6),
                                         mats.at(static_cast<size_t>(tri_mat[t]))));
  }
  std::vector<SceneObject*> objects{new TriangleSoup(prims)};
  Scene* scene = new Scene(objects, lights);

  Particles* P = new Particles(rest_density);
  for (int64_t i = 0; i < n; i++)
    P->addParticle(Vector3D(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]), Vector3D(0, 0, 0));

  Collada::CameraInfo info;
  info.hFov = static_cast<float>(cam[0]);
  info.vFov = static_cast<float>(cam[1]);
  info.nClip = static_cast<float>(cam[2]);
  info.fClip = static_cast<float>(cam[3]);
  Camera* camera = new Camera();
  camera->configure(info, static_cast<size_t>(width), static_cast<size_t>(height));
  camera->place(v3(cam + 4), cam[7], cam[8], cam[9], cam[10], cam[11]);

  // The reference prints progress; keep stdout quiet.
  std::ostringstream sink;
  std::streambuf* old_out = std::cout.rdbuf(sink.rdbuf());
  std::FILE* devnull = std::freopen("/dev/null", "w", stdout);
  (void)devnull;

  PathTracer* pt = new PathTracer(static_cast<size_t>(ns_aa), static_cast<size_t>(max_depth),
                                  static_cast<size_t>(ns_area), 1, 1, 1, 1, nullptr);
  pt->set_frame_size(static_cast<size_t>(width), static_cast<size_t>(height));
  pt->set_camera(camera);
  pt->fluid_particles = P;
  pt->set_scene(scene);
  std::srand(static_cast<unsigned>(seed));
  const auto t0 = std::chrono::steady_clock::now();
  pt->render_to_file(argv[2]);
  const auto t1 = std::chrono::steady_clock::now();
  const double seconds = std::chrono::duration<double>(t1 - t0).count();

  std::vector<double> sxyz, snrm;
  pbf_ref::surface_triangles(*P, 0.95 * rest_density, pbf_ref_h * 0.5, &sxyz, &snrm, nullptr);
  std::cout.rdbuf(old_out);

  std::ofstream out(argv[3], std::ios::binary);
  out.write("PBFRNDO1", 8);
  const Vector3D cp = camera->position(), up = camera->up_dir();
  const double cpa[3] = {cp.x, cp.y, cp.z}, upa[3] = {up.x, up.y, up.z}, vf = camera->v_fov();
  wr(out, cpa, 3);
  wr(out, upa, 3);
  wr(out, &vf, 1);
  const int64_t nt = static_cast<int64_t>(sxyz.size() / 9);
  wr(out, &nt, 1);
  wr(out, sxyz.data(), sxyz.size());
  wr(out, snrm.data(), snrm.size());
  wr(out, &seconds, 1);
  return out ? 0 : 3;
}
