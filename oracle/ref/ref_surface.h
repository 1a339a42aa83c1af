// The reference's fluid surface triangles, in the order Particles::getSurfacePrims
// (src/particles.cpp:350-390) makes them: the same loop over grid cells, the
// reference's own generateGridCell / polygonise / getVertexNormal. Test
// infrastructure of the headless oracle build (oracle/ref/build_ref.py).
#pragma once

#include <algorithm>
#include <cstdint>
#include <vector>

#include "particles.h"  // includes marching.h (polygonise), which has no include guard

namespace pbf_ref {

inline void surface_triangles(CGL::Particles& P, double iso, double fstep, std::vector<double>* xyz,
                              std::vector<double>* nrm, std::vector<int64_t>* cube) {
  using namespace CGL;
  const double xmin = P.getParticlesAxisMin(0), ymin = P.getParticlesAxisMin(1), zmin = P.getParticlesAxisMin(2);
  const double xmax = P.getParticlesAxisMax(0), ymax = P.getParticlesAxisMax(1), zmax = P.getParticlesAxisMax(2);
  const int xsteps = (int)((xmax - xmin) / fstep), ysteps = (int)((ymax - ymin) / fstep),
            zsteps = (int)((zmax - zmin) / fstep);
  for (int ix = 0; ix <= xsteps; ix++)
    for (int iy = 0; iy <= ysteps; iy++)
      for (int iz = 0; iz <= zsteps; iz++) {
        const double x1 = xmin + ix * fstep, x2 = std::min(xmax, x1 + fstep);
        const double y1 = ymin + iy * fstep, y2 = std::min(ymax, y1 + fstep);
        const double z1 = zmin + iz * fstep, z2 = std::min(zmax, z1 + fstep);
        GridCell grid = P.generateGridCell(x1, x2, y1, y2, z1, z2);
        std::vector<TriangleVertices*> tris = polygonise(grid, iso);
        for (TriangleVertices* t : tris) {
          for (int v = 0; v < 3; v++) {
            Vector3D q = t->p[v];
            Vector3D nq = P.getVertexNormal(q);
            for (int k = 0; k < 3; k++) {
              xyz->push_back(q[k]);
              nrm->push_back(nq[k]);
            }
          }
          if (cube) cube->push_back((static_cast<int64_t>(ix) * (ysteps + 1) + iy) * (zsteps + 1) + iz);
          delete t;
        }
      }
}

}  // namespace pbf_ref
