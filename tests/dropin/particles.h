// The drop-in replacement of the reference's src/particles.h: its `Particles` / `Particle`
// (src/particles.h:19-140) become the GB300 facade of fluid_gb300/host/pbf_particles.h over
// the reference's own CGL::Vector3D and CGL::Color, and the members whose types belong to
// the reference's renderer -- `bvh` (BVHAccel*), `surface` (Primitive* list),
// getSurfacePrims(double, double, BSDF*), updateSurface() -- keep the reference's
// signatures here, so application.cpp and pathtracer.cpp compile against it unchanged.
// tests/test_dropin.py compiles it against the reference's headers and drives it the way
// those callers do.
//
// Differences, by design: the GPU collides against the box of the step parameters (plus
// any triangles and spheres given to setColliderMesh / setColliderSpheres); `bvh` is kept
// for the callers that assign it and is not read. updateSurface keeps the reference's
// behaviour of ending with one step of DEFAULT_DELTA_T (particles.cpp:387-398).
#ifndef CGL_PARTICLES_H
#define CGL_PARTICLES_H

#include <cstdio>
#include <vector>

#include "CGL/color.h"
#include "CGL/vector3D.h"
#include "bsdf.h"
#include "bvh.h"
#include "static_scene/marching_triangle.h"
#include "pbf_particles.h"

namespace CGL {

using Particle = pbf_host::Particle<Vector3D, Color>;

struct Particles : pbf_host::Particles<Vector3D, Color> {
  using Base = pbf_host::Particles<Vector3D, Color>;

  StaticScene::BVHAccel* bvh = nullptr;          // particles.h:107
  std::vector<StaticScene::Primitive*> surface;  // particles.h:110

  // particles.h:114-116: prints the step's parameters, as the reference does.
  explicit Particles(double rest_density = 1000.0) : Base(rest_density, &default_params()) {
    std::fprintf(stdout, "%s", paramsString().c_str());
    std::fflush(stdout);
  }

  // particles.cpp:352-385: the surface as the reference's primitives, each triangle a
  // MarchingTriangle with the field's vertex normals and the given BSDF.
  std::vector<StaticScene::Primitive*> getSurfacePrims(double isolevel, double fStepSize, BSDF* bsdf) {
    std::vector<StaticScene::Primitive*> prims;
    for (const auto& t : Base::getSurfacePrims(isolevel, fStepSize))
      prims.push_back(new StaticScene::MarchingTriangle(t.p[0], t.p[1], t.p[2], t.n[0], t.n[1], t.n[2], bsdf));
    return prims;
  }

  // particles.cpp:387-398: once per time step, then one step of DEFAULT_DELTA_T.
  void updateSurface() {
    if (surfaceUpToTimestep) return;
    surface = getSurfacePrims(0.95 * rest_density, 0.5 * params().h, new DiffuseBSDF(Spectrum(0.1, 0.1, 0.8)));
    surfaceUpToTimestep = true;
    timeStep(params().dt);
  }

  // particles.cpp:303-307 (GL spheres): the reference's own drawing code, unchanged.
  void redraw(const Color& c);

  // The step's constants (the reference compiles them in as #defines, particles.cpp:20-44);
  // a host sets the scene's collider box and constants here before creating Particles.
  static pbf_params& default_params() {
    static pbf_params p = [] {
      pbf_params q;
      pbf_params_default(&q);
      return q;
    }();
    return p;
  }
};

}  // namespace CGL

#endif  // CGL_PARTICLES_H
