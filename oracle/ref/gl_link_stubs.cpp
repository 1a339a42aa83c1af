// Link-time stubs for drawing routines referenced (but never called) by the
// reference translation units that the headless oracle build compiles:
// BBox::draw (src/bbox.cpp), MarchingTriangle::draw/drawOutline
// (src/static_scene/marching_triangle.cpp) and Particles::redraw
// (src/particles.cpp:303-307), and the visualiser and screen routines of
// src/pathtracer.cpp (visualize_accel, update_screen, save_glimage) linked by the
// renderer driver. The simulation step and render_to_file never reach them; the
// oracle drivers never draw, and no GL library is loaded. Each stub aborts if it is ever reached, so a
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
void glVertex3f(float, float, float) { unreachable("glVertex3f"); }
void glClear(unsigned int) { unreachable("glClear"); }
void glDepthMask(unsigned char) { unreachable("glDepthMask"); }
void glDisable(unsigned int) { unreachable("glDisable"); }
void glEnable(unsigned int) { unreachable("glEnable"); }
void glDrawPixels(int, int, unsigned int, unsigned int, const void*) { unreachable("glDrawPixels"); }
void glLineWidth(float) { unreachable("glLineWidth"); }
void glPolygonOffset(float, float) { unreachable("glPolygonOffset"); }
void glPopAttrib(void) { unreachable("glPopAttrib"); }
void glPushAttrib(unsigned int) { unreachable("glPushAttrib"); }
void glReadPixels(int, int, int, int, unsigned int, unsigned int, void*) { unreachable("glReadPixels"); }
}

namespace CGL {
namespace Misc {
void draw_sphere_opengl(const Vector3D&, double, const Color&) {
  unreachable("draw_sphere_opengl");
}
}  // namespace Misc
}  // namespace CGL
