/*
 * pbf.h — C ABI of the GB300 Position Based Fluids step.
 *
 * This is the boundary a host (the C++ Particles facade in fluid_gb300/host,
 * Python through ctypes, or any FFI) binds. It replaces the reference's
 * in-process simulator struct `Particles` (src/particles.h:105-140) and its
 * step `Particles::timeStep(double)` (src/particles.cpp:250-297). Signatures
 * carry plain pointers and sizes only. Every function returns a pbf_status;
 * no C++ exception crosses the ABI. A handle owns all of its device memory
 * and one CUDA stream; one host thread may use a handle at a time, distinct
 * handles are independent.
 *
 * Arrays named xyz / vel are row-major (n, 3) float32 in the ORIGINAL particle
 * order (the order of pbf_create's input, as the reference's `ps` vector).
 * Functions whose name ends in _device take device pointers and a cudaStream_t
 * passed as void*; the handle's stream is ordered after that stream on entry
 * and the caller's stream after the handle's on exit.
 */
#ifndef PBF_H
#define PBF_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PBF_ABI_VERSION 6

#if defined(__GNUC__)
#define PBF_API __attribute__((visibility("default")))
#else
#define PBF_API
#endif

typedef enum pbf_status {
  PBF_OK = 0,
  PBF_ERR_INVALID = 1,   /* bad argument or handle state */
  PBF_ERR_CUDA = 2,      /* a CUDA runtime call failed (see pbf_last_error) */
  PBF_ERR_TIMEOUT = 3,   /* a bounded device-side wait gave up */
  PBF_ERR_NONFINITE = 4, /* a position or velocity became NaN/Inf */
  PBF_ERR_CAPACITY = 5,  /* neighbour list or cell-row capacity exceeded */
  PBF_ERR_NOMEM = 6      /* device allocation failed */
} pbf_status;

/* flags */
#define PBF_FLAG_STATS 1          /* accumulate pbf_stats every step */
#define PBF_FLAG_GRAPH 2          /* capture the step as a CUDA graph and replay it */
#define PBF_FLAG_KEEP_PREDICTED 4 /* keep x* after prediction (for pbf_get_predicted) */

/*
 * Step parameters. pbf_params_default() fills the reference's compile-time
 * constants (src/particles.cpp:20-44, 151, 180). The reference has implicit
 * unit particle mass, so rest_density is rho0/m for a fluid of rest density
 * rho0 and particle mass m.
 */
typedef struct pbf_params {
  double h;               /* kernel radius H (particles.cpp:26) */
  double h2;              /* neighbour radius squared H2 (particles.cpp:28) */
  int32_t iters;          /* Jacobi iterations NEWTON_NUM_STEPS (particles.cpp:34) */
  int32_t scorr_n;        /* tensile exponent N (particles.cpp:40) */
  double epsilon;         /* constraint relaxation EPSILON (particles.cpp:36) */
  double scorr_k;         /* tensile coefficient K (particles.cpp:38) */
  double scorr_dq;        /* tensile reference distance / H, 0.1 (particles.cpp:151) */
  double vort_eps;        /* VORTICITY_EPSILON (particles.cpp:42) */
  double xsph_c;          /* XSPH viscosity C (particles.cpp:44) */
  double dt;              /* DEFAULT_DELTA_T (particles.cpp:24), used by pbf_step(dt <= 0) */
  double gravity[3];      /* (0, -10, 0) (particles.cpp:180) */
  double rest_density;    /* Particles(double rest_density = 1000) (particles.h:112) */
  double box_lo[3];       /* collider: axis-aligned box walls (the reference casts */
  double box_hi[3];       /*   rays against scene triangles, particles.cpp:51-132) */
  int32_t box_open_mask;  /* bit 2*axis+side: leave that wall out */
  int32_t n_clip;         /* clip planes tested before the walls (particles.cpp:57-74) */
  int32_t clip_axis[2];   /*   default z = 1.0 and y = 1.49 */
  double clip_value[2];
  double clamp_lo[3];     /* final clamp box (particles.cpp:81-83) */
  double clamp_hi[3];
  int32_t max_neighbors;  /* neighbour capacity per particle (0: 128) */
  int32_t flags;          /* PBF_FLAG_* */
} pbf_params;

typedef struct pbf_stats {
  uint64_t steps;              /* steps taken since create / reset */
  double mean_density_iter0;   /* mean density after the first lambda pass of the last step
                                  (the first number of particles.cpp:275-280's print) */
  double mean_density;         /* mean reported density after the last step (particles.cpp:295) */
  double max_density_error;    /* max |rho/rho0 - 1| after the last step */
  double mean_density_error;   /* mean |rho/rho0 - 1| after the last step */
  uint32_t min_neighbors;      /* over particles, last step */
  uint32_t max_neighbors;
  double mean_neighbors;
  uint64_t low_neighbor_count; /* particles under NUM_NEIGHBOR_ALERT_THRESHOLD=18 (particles.cpp:32) */
  uint32_t error_flags;        /* sticky device error bits (PBF_ERRBIT_*) */
} pbf_stats;

#define PBF_ERRBIT_NONFINITE 1u
#define PBF_ERRBIT_NEIGHBOR_CAPACITY 2u
#define PBF_ERRBIT_ROW_CAPACITY 4u

typedef struct pbf_handle pbf_handle;

/* Fill *p with the reference's defaults (src/particles.cpp:20-44, 57-83, 180). */
PBF_API void pbf_params_default(pbf_params* p);

/* ABI version of the loaded library. */
PBF_API int pbf_abi_version(void);

/*
 * Create a simulator over n particles (replaces `new Particles(rho0)` followed
 * by n calls of Particles::addParticle, particles.h:112-120). xyz/vel: host,
 * (n, 3) float32; vel may be NULL (zero). device: CUDA ordinal.
 */
PBF_API pbf_status pbf_create(const pbf_params* params, size_t n, const float* xyz,
                      const float* vel, int device, pbf_handle** out);

/*
 * Batched form: n_scenes independent scenes stored back to back (scene s owns
 * counts[s] particles), each with its own collider box (box_lo/box_hi: host,
 * (n_scenes, 3); NULL = params->box_lo/hi). All scenes share the remaining
 * params. One launch per phase covers every scene.
 */
PBF_API pbf_status pbf_batch_create(const pbf_params* params, int n_scenes,
                            const size_t* counts, const float* box_lo,
                            const float* box_hi, const float* xyz,
                            const float* vel, int device, pbf_handle** out);

PBF_API pbf_status pbf_destroy(pbf_handle* h);

/* Advance nsteps steps of dt each (Particles::timeStep(double),
 * particles.cpp:250-297; dt <= 0 uses params.dt like Particles::timeStep()). */
PBF_API pbf_status pbf_step(pbf_handle* h, double dt, int nsteps);

/* Enqueue nsteps steps on the handle's stream and return without waiting
 * (no error check); pbf_sync waits and reports device-side errors. */
PBF_API pbf_status pbf_step_async(pbf_handle* h, double dt, int nsteps);
PBF_API pbf_status pbf_sync(pbf_handle* h);
/* The handle's cudaStream_t (as void*), for ordering and event timing. */
PBF_API void* pbf_stream(pbf_handle* h);

/* Host accessors, original order (Particle::getPosition, ::velocity,
 * ::getLatestDensityEstimate; particles.h:36-46). */
PBF_API pbf_status pbf_get_positions(pbf_handle* h, float* xyz);
PBF_API pbf_status pbf_get_velocities(pbf_handle* h, float* vel);
PBF_API pbf_status pbf_get_densities(pbf_handle* h, float* rho);
/* The three at once (any may be NULL): one reordering pass and one wait, for a caller
 * that mirrors the whole state after every step (the facade's timeStep). */
PBF_API pbf_status pbf_get_state(pbf_handle* h, float* xyz, float* vel, float* rho);
/* Replace positions and velocities (host). */
PBF_API pbf_status pbf_set_state(pbf_handle* h, const float* xyz, const float* vel);

/* Device-pointer forms of the accessors (see file comment for stream order). */
PBF_API pbf_status pbf_set_state_device(pbf_handle* h, const float* xyz,
                                const float* vel, void* stream);
PBF_API pbf_status pbf_get_state_device(pbf_handle* h, float* xyz, float* vel,
                                float* rho, void* stream);

/* Reorder the current state into cell order without moving it (the step
 * does this every step; a fresh handle holds the input order). */
PBF_API pbf_status pbf_sort(pbf_handle* h);

/* Device-side checkpoint of the state (positions, velocities, particle order,
 * step count, simulate_time); pbf_restore rolls back to it, enqueued on the
 * handle's stream without waiting. The reference has no checkpointing. */
PBF_API pbf_status pbf_snapshot(pbf_handle* h);
PBF_API pbf_status pbf_restore(pbf_handle* h);

/* Particles::estimateDensities (particles.cpp:440-444): density of every
 * particle at its current position, self included; host out[n]. */
PBF_API pbf_status pbf_estimate_densities(pbf_handle* h, float* rho);

/* Particles::estimateDensityAt (particles.cpp:446-453) at m query points
 * (host, (m, 3)); out[m]. */
PBF_API pbf_status pbf_estimate_density_at(pbf_handle* h, size_t m, const float* pts,
                                   float* out);

PBF_API pbf_status pbf_get_stats(pbf_handle* h, pbf_stats* out);

/* Introspection of the last step, original order. Neighbour sets are those
 * of the reference's all-pairs search (particles.cpp:258-265) on x*:
 * counts[n], then ids in ascending original index (capacity cap entries;
 * *total receives the number needed). cells[n]: linear cell id of x*.
 * pred: x* after prediction (needs PBF_FLAG_KEEP_PREDICTED). */
PBF_API pbf_status pbf_get_neighbors(pbf_handle* h, uint32_t* counts, uint32_t* ids,
                             size_t cap, size_t* total);
PBF_API pbf_status pbf_get_cells(pbf_handle* h, uint32_t* cells);
PBF_API pbf_status pbf_get_predicted(pbf_handle* h, float* xyz);

/*
 * Per-phase CUDA-event timing (the reference times nothing on this path; it
 * prints progress, particles.cpp:251-295). While enabled, steps run without
 * graph replay and record an event after each phase on the handle's stream.
 * pbf_get_phase_times waits and returns, per phase, the accumulated device
 * milliseconds and the number of kernel launches since the last reset.
 */
PBF_API pbf_status pbf_set_profiling(pbf_handle* h, int enable);
PBF_API pbf_status pbf_get_phase_times(pbf_handle* h, double* ms,
                                       uint64_t* launches, int max_phases);
PBF_API pbf_status pbf_reset_phase_times(pbf_handle* h);
PBF_API int pbf_num_phases(void);
PBF_API const char* pbf_phase_name(int phase);

/*
 * Launch shapes (threads per block) of the kernel families of a step, and the
 * forms of the neighbour kernels. No field changes any result bit: the forms
 * visit every particle's neighbours in the same order.
 */
typedef struct pbf_tuning {
  int32_t block_predict;  /* prediction, cell count */
  int32_t block_nbr;      /* neighbour-set build */
  int32_t block_solve;    /* lambda, delta-p, XSPH/vorticity passes */
  int32_t block_misc;     /* scatter, cell sort, gather */
  int32_t gather_depth;   /* neighbour loads a thread keeps in flight in the passes: 4 or 8 */
  int32_t list_stream;    /* 1: the passes load neighbour-list words with the streaming
                             (evict-first) cache policy, 0: through the read-only cache */
} pbf_tuning;

PBF_API pbf_status pbf_get_tuning(pbf_handle* h, pbf_tuning* out);
/* Each block size must be 64, 128, 256 or 512, gather_depth 4 or 8, list_stream 0 or 1.
 * Drops captured graphs. */
PBF_API pbf_status pbf_set_tuning(pbf_handle* h, const pbf_tuning* t);
/*
 * Autotuner: times every candidate of each tuning dimension (the block size of each
 * kernel family, the passes' gather depth and list policy) with
 * CUDA events over `reps` steps of dt from the current state (checkpointed
 * and restored around every trial, so the state is unchanged on return),
 * keeps the fastest candidate per dimension and reports the result in *out (may be NULL).
 */
PBF_API pbf_status pbf_autotune(pbf_handle* h, double dt, int reps, pbf_tuning* out);

PBF_API size_t pbf_size(const pbf_handle* h);
PBF_API int pbf_num_scenes(const pbf_handle* h);

/* Human-readable description of the last error on this handle (or of the
 * last failed pbf_create when h is NULL). Never NULL. */
PBF_API const char* pbf_last_error(const pbf_handle* h);

/*
 * pbf_adjoint_step_device -- no counterpart in the reference (which has no
 * gradients); the reverse mode of one Particles::timeStep (particles.cpp:250-297).
 *
 * Runs one step from the state (xyz, vel) -- recording what its reverse needs --
 * then its reverse mode with the step's neighbour sets held fixed and every
 * collision differentiated with its active set fixed. All arrays are DEVICE
 * pointers in original particle order, (n, 3) float32:
 *   xyz, vel         the step's input state (xyz NULL: the handle's current state,
 *                    vel ignored; vel NULL with xyz given: zero velocities)
 *   gx_out, gv_out   adjoints of the step's output positions / velocities (NULL: 0)
 *   gx_in, gv_in     receive the adjoints of the input positions / velocities
 *   g_rho0           one double, receives the adjoint of params.rest_density
 *   xyz_out, vel_out receive the step's outputs (NULL: not written)
 * The handle's state becomes the step's output (simulate_time is not advanced).
 * The work is enqueued on `stream` (a cudaStream_t, NULL for the legacy default
 * stream) without waiting; pbf_sync reports capacity and non-finite errors.
 * Device memory for the recording (about (64 + 32 iters) bytes per particle plus
 * 150 bytes of work arrays) is allocated on the first call. The sums are
 * evaluated in a fixed order: repeated calls give identical results.
 */
PBF_API pbf_status pbf_adjoint_step_device(pbf_handle* h, double dt, const float* xyz, const float* vel,
                                           const float* gx_out, const float* gv_out, float* gx_in,
                                           float* gv_in, double* g_rho0, float* xyz_out, float* vel_out,
                                           void* stream);

/*
 * pbf_surface -- Particles::getSurfacePrims (particles.cpp:352-385; updateSurface,
 * :387-395, calls it with isolevel = 0.95 rest_density and step = 0.5 H) on the
 * current state: a marching-cubes surface of the density field estimateDensityAt
 * (:446-453) over the grid of cubes [x1, min(hi, x1 + step)], x1 = lo + i step,
 * i = 0 .. (int)((hi - lo) / step) per axis, visited x outer, then y, then z; corners,
 * edges and edge vertices as generateGridCell (:309-323) and vertexInterp
 * (marching.cpp); vertex normals the normalized central differences of the field at
 * +-0.001 (getVertexNormal, :399-412). The triangulation of each cube configuration is
 * this library's table (pbf_mc_table), which closes the surface across cubes.
 * lo / hi NULL: the reference's fixed bounds [-1, 1] x [0, 1.5] x [-1, 1]
 * (:330-349). Scene 0 of a batch. xyz and nrm are HOST arrays of 9 floats per
 * triangle (3 vertices); the first min(cap, total) triangles are written and *count
 * receives the total (cap = 0 to query).
 */
PBF_API pbf_status pbf_surface(pbf_handle* h, double isolevel, double step, const double* lo, const double* hi,
                               float* xyz, float* nrm, size_t cap, size_t* count);

/*
 * pbf_set_collider_mesh -- triangles the particles collide with besides the box walls,
 * as the reference's colliders are the triangles of its scene's BVH (clamp and
 * clamp_response, particles.cpp:51-132; BVHAccel::intersect, bvh.cpp:142-192). tri: n
 * triangles of 9 floats (p1, p2, p3, host memory); each triangle's normal is
 * unit((p2 - p1) x (p3 - p1)), used for the slide of the predicted move. A move stops at
 * the nearest wall, clip plane, triangle or sphere; after a triangle or sphere stop the
 * particle keeps 4 FP32 ulps from it (the reference keeps EPS_D = 1e-11, below FP32
 * resolution). The triangles go into a bounding-volume hierarchy built here, on the
 * host; a move tests the triangles of the leaves its segment meets, and of hits at the
 * same distance the triangle given last wins (as in a scan of all of them). n = 0
 * removes the mesh. At most 4,194,304 triangles. pbf_adjoint_step_device refuses a
 * handle with a mesh or spheres (its collision reverse is for axis-aligned walls).
 */
PBF_API pbf_status pbf_set_collider_mesh(pbf_handle* h, size_t n, const float* tri);

/*
 * pbf_set_collider_spheres -- solid spheres the particles collide with, the reference's
 * Sphere primitives (static_scene/sphere.cpp:10-72: the nearer intersection in range,
 * else the farther; the normal from the centre to the hit point). xyzr: n spheres of 4
 * floats (centre x, y, z, radius > 0; host memory). n = 0 removes them. At most 1024,
 * each tested by every move.
 */
PBF_API pbf_status pbf_set_collider_spheres(pbf_handle* h, size_t n, const float* xyzr);

/*
 * pbf_mc_table -- the triangulation table pbf_surface uses (no GPU needed): for each of
 * the 256 cube configurations (bit k set when corner k is below the iso level; corners
 * and edges numbered as generateGridCell and polygonise number them) the crossing-edge
 * mask (edges[256]), the triangle count (ntri[256], at most 5) and the triangles as edge
 * triples (tri[256 * 15]). Any pointer may be NULL.
 */
PBF_API void pbf_mc_table(uint16_t* edges, uint8_t* ntri, int8_t* tri);

/* ---- path tracing of the fluid in its scene (PathTracer, src/pathtracer.cpp) ---------- */

/* BSDFs (src/bsdf.h): DIFFUSE c1 = albedo; MIRROR c1 = reflectance; GLASS c1 =
 * transmittance, c2 = reflectance, ior; REFRACTION (the reference's RefractionBSDF,
 * black); EMISSION c1 = radiance. */
#define PBF_MAT_DIFFUSE 0u
#define PBF_MAT_MIRROR 1u
#define PBF_MAT_GLASS 2u
#define PBF_MAT_REFRACTION 3u
#define PBF_MAT_EMISSION 4u
typedef struct pbf_material {
  uint32_t kind;
  float c1[3];
  float c2[3];
  float ior;
} pbf_material;

/* Lights (src/static_scene/light.cpp): DIRECTIONAL (direction of travel), HEMISPHERE
 * (uniform sky over +y), POINT (position, no falloff), AREA (centre position, emission
 * direction, edges dim_x and dim_y; a point p is lit where dot(q - p, direction) < 0 for
 * the sampled light point q). Spot, sphere and mesh lights of the reference return
 * black and are not taken. */
#define PBF_LIGHT_DIRECTIONAL 0u
#define PBF_LIGHT_HEMISPHERE 1u
#define PBF_LIGHT_POINT 2u
#define PBF_LIGHT_AREA 3u
typedef struct pbf_light {
  uint32_t kind;
  float radiance[3];
  float position[3];
  float direction[3];
  float dim_x[3];
  float dim_y[3];
} pbf_light;

/* Camera::configure (fields of view in degrees, clip distances) and Camera::place
 * (target, polar angle phi from +y, azimuth theta, distance r clamped to [min_r, max_r]),
 * src/camera.cpp:15-46. */
typedef struct pbf_camera_desc {
  double hfov, vfov, nclip, fclip;
  double target[3];
  double phi, theta, r, min_r, max_r;
} pbf_camera_desc;

/* A placed camera: position, c2w columns (screen x, screen y, the view direction
 * reversed), fields of view in degrees after the aspect adjustment, clip distances. */
typedef struct pbf_camera {
  double position[3];
  double c2w[9];
  double hfov, vfov, nclip, fclip;
} pbf_camera;

typedef struct pbf_render_params {
  uint32_t width, height;
  uint32_t ns_aa;          /* camera rays per pixel (-s; 1 = through the pixel centre) */
  uint32_t max_ray_depth;  /* bounces (-m) */
  uint32_t ns_area_light;  /* samples per area or hemisphere light (-l) */
  uint32_t fluid_surface;  /* 1: add the particles' surface as Particles::updateSurface does */
  uint32_t surface_bounds; /* 1: surface grid over [surface_lo, surface_hi]; 0: the reference's
                              fixed [-1, 1] x [0, 1.5] x [-1, 1] (particles.cpp:330-349) */
  uint32_t path_buffer_mib; /* the path state of one batch of samples per pixel is kept under
                              this many MiB (0: 2048); batches are summed in sample order */
  uint64_t seed;           /* random numbers: a function of (seed, pixel, sample, draw) */
  double isolevel, step;   /* surface; <= 0: 0.95 rest_density and 0.5 H (particles.cpp:392-401) */
  double surface_lo[3], surface_hi[3];
  float fluid_albedo[3];   /* the surface's DiffuseBSDF (particles.cpp:398: 0.1 0.1 0.8) */
  float ray_eps;           /* start of shadow and bounce rays; <= 0: 1e-4 */
} pbf_render_params;

typedef struct pbf_render_stats {
  uint64_t triangles;          /* scene + surface */
  uint64_t surface_triangles;
  double ms_surface, ms_bvh, ms_trace, ms_total; /* device time of the phases */
} pbf_render_stats;

/* The reference's defaults (application.h:48-56: 1 ray per pixel, depth 1, 1 light
 * sample) at 640 x 480, with the fluid surface. */
PBF_API void pbf_render_params_default(pbf_render_params* p);

/* Camera::configure + Camera::place: the frame generate_ray uses (no GPU needed). */
PBF_API pbf_status pbf_camera_frame(const pbf_camera_desc* d, uint32_t width, uint32_t height, pbf_camera* out);

/*
 * pbf_render_set_scene -- the scene the fluid is rendered in (the reference's Scene of
 * COLLADA meshes and lights): n_tri triangles of 9 floats (tri_xyz, vertices) with
 * vertex normals (tri_nrm, 9 floats; NULL: the face normal unit((p2 - p1) x (p3 - p1)) at
 * all three vertices) and a material index each; host arrays, copied.
 */
PBF_API pbf_status pbf_render_set_scene(pbf_handle* h, const float* tri_xyz, const float* tri_nrm,
                                        const uint32_t* tri_material, size_t n_tri, const pbf_material* materials,
                                        size_t n_materials, const pbf_light* lights, size_t n_lights);

/*
 * pbf_render -- one frame of PathTracer::render_to_file (pathtracer.cpp:187-235,
 * 483-632) of the scene and, with fluid_surface, the surface of the current state: a BVH
 * over all triangles built on the device (Morton-ordered binary radix tree), one thread
 * per pixel tracing ns_aa paths of estimate_direct_lighting + estimate_indirect_lighting
 * with Russian roulette, in FP32. hdr: W * H * 3 floats (HOST or NULL), row 0 = the
 * bottom row as the reference's sample buffer; rgba: W * H * 4 bytes (HOST or NULL),
 * HDRImageBuffer::toColor's 8-bit frame with the top row first, as the reference's PNG.
 * Device memory for the frame and the hierarchy is kept for the next call.
 */
PBF_API pbf_status pbf_render(pbf_handle* h, const pbf_camera* cam, const pbf_render_params* p, float* hdr,
                              uint8_t* rgba, pbf_render_stats* stats);

/*
 * pbf_density_noalloc -- no counterpart in the reference.
 *
 * The density estimate of pbf_estimate_densities (Particles::estimateDensities,
 * self term included) for callers that cannot allocate device memory: ones whose
 * device memory belongs to another framework's allocator, or that must not let
 * cudaMalloc/cudaFree synchronize the device. It creates no handle and allocates
 * nothing: xyz ((n, 3) float32) and rho (n float32) are DEVICE pointers owned by
 * the caller (device or managed memory of the current device; anything else, a host
 * pointer included, is rejected with PBF_ERR_INVALID before any work), the collider
 * box and kernel radius come from params, and the work is enqueued on `stream` (a
 * cudaStream_t, NULL for the legacy default stream) without waiting. Its cell-sort
 * scratch is one static device array of about 3.9 MB inside the library, held by
 * every GPU that loads it until the process exits. The first call on a device looks
 * up that array's device address and keeps it for the process, so make the first call
 * on each device outside any stream capture, and do not call it again after a
 * cudaDeviceReset of that device. All calls share the array: calls whose work could
 * overlap on the GPU race and must be serialized. Limits: n <= PBF_NOALLOC_MAX_PARTICLES
 * and at most PBF_NOALLOC_MAX_CELLS grid cells of size h over the box; larger inputs
 * return PBF_ERR_INVALID with the reason in pbf_last_error(NULL). A cell holding more
 * than 256 particles keeps the order its particles were counted in, so for such dense
 * inputs the sums' order, and hence their last bits, may vary from call to call.
 */
#define PBF_NOALLOC_MAX_PARTICLES 65536
#define PBF_NOALLOC_MAX_CELLS 262144
PBF_API pbf_status pbf_density_noalloc(const pbf_params* params, size_t n,
                                       const float* xyz, float* rho, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* PBF_H */
