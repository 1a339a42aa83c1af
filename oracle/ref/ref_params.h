// Runtime stand-ins for the compile-time parameter block of the reference's
// src/particles.cpp:20-44 and the gravity literal at src/particles.cpp:180.
//
// Test infrastructure only (the oracle): build_ref.py rewrites those #define
// lines of a staged copy of particles.cpp into references to these globals so
// one build of the reference step serves every scene configuration. The
// globals are defined, with the reference's own default values, in
// ref_driver.cpp.
#pragma once

extern double pbf_ref_dt;        // DEFAULT_DELTA_T  0.016
extern double pbf_ref_h;         // H                0.3
extern double pbf_ref_h2;        // H2               0.09
extern int pbf_ref_iters;        // NEWTON_NUM_STEPS 12
extern double pbf_ref_epsilon;   // EPSILON          2
extern double pbf_ref_k;         // K                0.0001
extern double pbf_ref_vort_eps;  // VORTICITY_EPSILON 0.001
extern double pbf_ref_xsph_c;    // C                0.001
extern double pbf_ref_gravity;   // literal 10 in velocity.y -= 10 * delta_t
