// Link-time stubs for drawing routines referenced (but never called) by the
// reference translation units that the headless oracle build compiles:
// BBox::draw (src/bbox.cpp), MarchingTriangle::draw/drawOutline
// (src/static_scene/marching_triangle.cpp) and Particles::redraw
// (src/particles.cpp:303-307). The simulation step never reaches them; the
// oracle driver never draws. Each stub aborts if it is ever reached, so a
// silent no-op can never stand in for drawing.
#include <cstdio>
#include <cstdlib>

#include "CGL/CGL.h"
#include "CGL/color.h"
#include "CGL/vector3D.h"

namespace {
[[noreturn]] void unreachable(const char* what) {
  std::fprintf(stderr, "oracle build: drawing routine %s reached\n", what);
  std::abort();
}
}  // namespace

extern "C" {
void glBegin(unsigned int) { unreachable("glBegin"); }
void glEnd(void) { unreachable("glEnd"); }
void glVertex3d(double, double, double) { unreachable("glVertex3d"); }
void glColor4f(float, float, float, float) { unreachable("glColor4f"); }
}

namespace CGL {
namespace Misc {
void draw_sphere_opengl(const Vector3D&, double, const Color&) {
  unreachable("draw_sphere_opengl");
}
}  // namespace Misc
}  // namespace CGL
