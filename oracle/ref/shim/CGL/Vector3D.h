// Case shim for the reference's src/marching.h:2, which includes
// "CGL/Vector3D.h" while the header on disk is CGL/vector3D.h. Only used by
// the headless oracle build of the reference (oracle/ref/build_ref.py).
#include "CGL/vector3D.h"
