/*
 * mpm_gb300 — C ABI of the GB300 (sm_103a) MLS-MPM substep.
 *
 * Drop-in boundary for the substep of kekeblom/mpm.  The reference has no C ABI:
 * its host class `Simulation` (include/mpm.cuh:44-106, src/mpm.cu:180-329) owns
 * device memory, uploads an AoS particle array and launches three kernels per
 * `advance()`.  Each entry point below names the reference member it replaces.
 *
 * Conventions
 *   - Every call returns an mpm_status (0 = MPM_OK).  The message of the last
 *     failure on a context is available from mpm_last_error().
 *   - The context owns every device buffer; the caller owns host buffers.
 *   - Work is enqueued on the context's stream (mpm_set_stream, default: a
 *     stream created by mpm_create).  Calls on one context are not re-entrant;
 *     use one context per host thread.
 *   - Host particle arrays are per-particle interleaved: x[3n], v[3n],
 *     C[9n] and F[9n] row-major (C[9p + 3r + c]), Jp[n], mat[n] (material index).
 *   - Kernels never trap: a non-finite particle, a bad index or an expired wait
 *     sets a device status word that mpm_sync() returns (MPM_ERR_STATE /
 *     MPM_ERR_TIMEOUT).
 */
#ifndef MPM_GB300_H
#define MPM_GB300_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum mpm_status {
  MPM_OK = 0,
  MPM_ERR_INVALID = 1,     /* bad argument or call order */
  MPM_ERR_CUDA = 2,        /* CUDA runtime error (message in mpm_last_error) */
  MPM_ERR_STATE = 3,       /* device status word: non-finite particle / index out of range */
  MPM_ERR_TIMEOUT = 4,     /* a bounded device-side wait expired */
  MPM_ERR_NOMEM = 5,       /* device allocation failed */
  MPM_ERR_UNSUPPORTED = 6, /* configuration not supported by this build */
  MPM_ERR_IO = 7           /* a file could not be written */
} mpm_status;

/* Material kinds. MMSnow is the only model the reference instantiates
 * (include/mpm.cuh:25); "elastic" and the reference's "liquid" are MMSnow with
 * hardening 0 and clamps [0, 1e30] / [0.975, 0.975] (scenes/*.toml). */
enum {
  MPM_MAT_SNOW = 0,            /* MMSnow            include/MaterialModel.cuh:67-116 */
  MPM_MAT_FIXED_COROTATED = 1, /* MMFixedCorotated  include/MaterialModel.cuh:40-62 */
  MPM_MAT_JELLY = 2,           /* MMJelly           include/MaterialModel.cuh:119-150 */
  MPM_MAT_LIQUID = 3,          /* weakly compressible liquid, P F^T = K (J-1) J I,
                                  J <- J det(I + dt C), F = J^(1/3) I (not in the reference) */
  MPM_MAT_USER_BASE = 16,      /* kinds 16..63: material models compiled into a build of the
                                  library through include/mpm_gb300_policies.cuh (the
                                  reference's MaterialModel alias, include/mpm.cuh:25); a table
                                  holding one holds that kind only */
  MPM_MAT_USER_END = 64
};

/* Boundary rule of the grid operation. */
enum {
  MPM_BOUNDARY_REF_FRACTION = 0,  /* src/mpm.cu:92-105: idx/N < 0.05 or > 0.95 sticky on
                                     x, z and the top; separating floor (v_y >= 0) */
  MPM_BOUNDARY_STICKY_CELLS = 1,  /* all six walls sticky within boundary_cells cells */
  MPM_BOUNDARY_SEPARATE_CELLS = 2 /* reference structure with a cell-count thickness */
};

#define MPM_MAX_MATERIALS 16

/* Simulation parameters.  dt and N are the reference's CLI options
 * (include/options.h:19-21, SimulationParameters in include/TransferScheme.h:6-29). */
typedef struct mpm_params {
  float dt;               /* substep length (reference default 1e-4) */
  uint32_t N;             /* grid cells per dimension over the unit cube */
  float gravity;          /* y acceleration; the reference hard-codes -9.81 (src/mpm.cu:6) */
  int32_t boundary_mode;  /* MPM_BOUNDARY_* */
  int32_t boundary_cells; /* wall thickness for the *_CELLS modes */
  int32_t g2p_guard;      /* 1: only particles with original index <= N^3 run G2P, as
                             src/mpm.cu:114 does; 0: every particle (default) */
  int32_t sort_interval;  /* re-sort particles by cell every k substeps (0 = never) */
  int32_t check_finite;   /* 1: flag non-finite positions in the device status word */
} mpm_params;

/* Constructor arguments of MMSnow(volume, density, E, Nu, hardening, lo, hi)
 * (include/MaterialModel.cuh:74-83); particle_volume is 1/particle-count
 * (src/main.cu:36).  mu0, lambda0 and the particle mass are derived in float
 * exactly as the reference constructors do. */
typedef struct mpm_material {
  int32_t kind;            /* MPM_MAT_* */
  float particle_volume;
  float density;
  float E;
  float nu;
  float hardening;
  float clamp_lo;          /* plast_clamp_lower */
  float clamp_hi;          /* plast_clamp_higher */
  float bulk;              /* MPM_MAT_LIQUID bulk modulus K */
} mpm_material;

typedef struct mpm_ctx mpm_ctx;

/* Simulation::Simulation + Simulation::initCuda (src/mpm.cu:180-207): allocates the
 * triple-buffered grid and a stream; particles come with mpm_upload_*. */
mpm_status mpm_create(const mpm_params* params, mpm_ctx** out);
/* Simulation::~Simulation (src/mpm.cu:190-195). */
mpm_status mpm_destroy(mpm_ctx* ctx);
/* Use a caller-owned cudaStream_t for all subsequent work (NULL: the context's own). */
mpm_status mpm_set_stream(mpm_ctx* ctx, void* cuda_stream);
/* Change dt / gravity / boundary / sort interval (N must stay the same). */
mpm_status mpm_set_params(mpm_ctx* ctx, const mpm_params* params);
/* The material table the reference copies to the device in initCuda
 * (src/mpm.cu:199-201); particles index it with their material byte. */
mpm_status mpm_set_materials(mpm_ctx* ctx, const mpm_material* materials, int32_t count);
/* 1 when this build can run material kind `kind`: the built-in kinds, and kinds compiled in
 * through include/mpm_gb300_policies.cuh (no counterpart in the reference, whose model is
 * fixed by a compile-time alias, include/mpm.cuh:25); 0 otherwise.  Needs no GPU. */
int32_t mpm_material_kind_available(int32_t kind);

/* Simulation::particlesToDevice (src/mpm.cu:278-286), SoA host arrays.  mat may be
 * NULL (all particles use material 0).  Replaces all particles. */
mpm_status mpm_upload_soa(mpm_ctx* ctx, int64_t n, const float* x, const float* v, const float* C,
                          const float* F, const float* Jp, const uint8_t* mat);
/* Same, from the reference's AoS MLS_APIC_Particle records (104 bytes: u8 material,
 * Vec x, Vec v, Mat F, Mat C, real Jp; Eigen column-major matrices;
 * include/types.h:24-35, include/TransferScheme.h:46-54). */
mpm_status mpm_upload_aos(mpm_ctx* ctx, const void* particles, int64_t n);

/* Simulation::advance (src/mpm.cu:323-329) repeated nsteps times; asynchronous. */
mpm_status mpm_substep(mpm_ctx* ctx, int32_t nsteps);
/* Wait for the context's stream and return the device status word. */
mpm_status mpm_sync(mpm_ctx* ctx);

/* Simulation::particlesToHost / syncDevice (src/mpm.cu:209-211, 288-306): blocking
 * copy of all particles, in upload order.  Any pointer may be NULL to skip it. */
mpm_status mpm_download_soa(mpm_ctx* ctx, float* x, float* v, float* C, float* F, float* Jp,
                            uint8_t* mat);
mpm_status mpm_download_aos(mpm_ctx* ctx, void* particles);

/* Grid of the last completed substep (N^3 x 4 floats, index N*(N*i+j)+k):
 * which = 0: after P2G (m v, m); which = 1: after the grid operation, with the
 * reference's mass slot (1 wherever m > 0, src/mpm.cu:86-88). Blocking. */
mpm_status mpm_get_grid(mpm_ctx* ctx, int32_t which, float* out);

/* Re-sort particles by cell now (also done every sort_interval substeps). */
mpm_status mpm_sort(mpm_ctx* ctx);

/* Simulation::advance over several independent scenes: nsteps substeps of each of the
 * `count` contexts, interleaved substep by substep, from one compiled host loop (the loop a
 * C++ caller of the reference writes over its Simulation objects, src/mpm.cu:323-329).
 * Asynchronous like mpm_substep; stops at the first failing context and returns its status. */
mpm_status mpm_substep_many(mpm_ctx* const* ctxs, int32_t count, int32_t nsteps);

/* Simulation::getFullParticleCount (src/mpm.cu:253-259). */
int64_t mpm_particle_count(const mpm_ctx* ctx);
/* Number of substeps advanced since the last upload. */
int64_t mpm_substep_count(const mpm_ctx* ctx);
/* ---------------------------------------------------------------------------
 * Scene objects: Simulation::addObject (src/mpm.cu:237-251) with the particle seeding of
 * Simulation::addParticles (src/mpm.cu:346-394).  An object is a shape scaled so that the
 * longest edge of its bounding box is `size`, with the box's lowest corner at `position`
 * (Simulation::loadMesh, src/mpm.cu:330-344).  Its particles are seeded on the GPU by
 * rejection sampling: u32(density x bounding-box volume) candidates uniform in the box,
 * kept when inside the shape, density = u32(1 / particle_volume) of the object's material.
 * The reference draws candidates with rand() and tests meshes with libigl's winding
 * number; here candidate i comes from a SplitMix64 hash of (seed, i), so seeding is
 * reproducible, and closed meshes are tested by +x ray parity.  Seeded particles start
 * with the object's velocity, C = 0, F = I and Jp = 1.
 * An object is active for lifetime_begin <= t < lifetime_end (SimObject::isActive,
 * include/mpm.cuh:36-38): mpm_add_object appends it at once when active at the current
 * t, and mpm_substep appends and removes objects at substep boundaries.  Downloads list
 * uploaded particles first, then active objects in activation order.
 * ------------------------------------------------------------------------- */
enum { MPM_SHAPE_BOX = 0, MPM_SHAPE_SPHERE = 1, MPM_SHAPE_MESH = 2 };
/* Inside test of MESH objects. */
enum {
  MPM_INSIDE_RAY_PARITY = 0, /* odd number of +x ray crossings: exact for closed meshes (default) */
  MPM_INSIDE_WINDING = 1     /* generalized winding number > 1/2 (libigl's winding_number, which the
                                reference calls, src/mpm.cu:383): also open or self-overlapping
                                meshes; sums every triangle for every candidate */
};

typedef struct mpm_object {
  int32_t shape;             /* MPM_SHAPE_* */
  int32_t material;          /* index into the context's material table */
  float size;                /* longest edge of the bounding box */
  float position[3];         /* lowest corner of the bounding box */
  float velocity[3];         /* initial velocity of every particle */
  float box_extent[3];       /* BOX: edge lengths relative to each other ({1,1,1}: a cube) */
  double lifetime_begin;     /* active from this time on (0: from the start) */
  double lifetime_end;       /* inactive from this time on (e.g. 1e300: never) */
  uint64_t seed;             /* seeding stream */
  const float* vertices;     /* MESH: 3 floats per vertex, any scale (host memory) */
  int64_t n_vertices;
  const int32_t* triangles;  /* MESH: 3 vertex indices per triangle (closed for ray parity) */
  int64_t n_triangles;
  int32_t inside_test;       /* MESH: MPM_INSIDE_* */
} mpm_object;

/* Seed an object's particles on the GPU and add it to the scene; *n_particles (may be
 * NULL) receives its particle count.  Removes nothing: objects live until the context is
 * destroyed or particles are uploaded again (an upload forgets all objects). */
mpm_status mpm_add_object(mpm_ctx* ctx, const mpm_object* object, int64_t* n_particles);
/* Simulated time: dt summed over the substeps run since the last upload (or creation). */
double mpm_time(const mpm_ctx* ctx);
/* Objects added (active or not). */
int32_t mpm_object_count(const mpm_ctx* ctx);
/* Seeding alone, for tools and tests: the object's particle positions at `density`
 * candidates per unit volume, 3 floats per particle in candidate order, into host x
 * (room for `capacity` particles); *n receives the count, which may exceed capacity. */
mpm_status mpm_seed_object(const mpm_object* object, uint32_t density, float* x, int64_t capacity, int64_t* n);

/* ---------------------------------------------------------------------------
 * Surface reconstruction (MeshBuilder::computeMesh, include/mesh_builder.h:170-211).  A
 * voxel grid of side grid_side (voxel_dx = N dx / grid_side) holds the distance from each
 * node to the nearest particle within (radius + 1) voxels (fillVoxelGrid_distance,
 * include/mesh_builder.h:89-137); the surface is the zero level of radius * voxel_dx -
 * distance, extracted by libigl's marching cubes.  Here the vertices are libigl's, bit
 * for bit and in its order; each cube's faces triangulate the same edge loops as
 * libigl's (the fan inside a loop may differ).  Every call synchronises.
 * ------------------------------------------------------------------------- */
/* grid_side in [2, 512], radius in [0, 64]; particles outside [0, grid_side voxel_dx)
 * touch only the nodes inside the grid.
 * The distance field (grid_side^3 floats, index (i grid_side + j) grid_side + k). */
mpm_status mpm_surface_distance(mpm_ctx* ctx, int32_t grid_side, int32_t radius, float* field);
/* Triangles of the surface, 9 floats each (3 vertices x y z), into host tris (room for
 * `capacity` triangles); *n_tris receives the count, which may exceed capacity.  The
 * triangles are the faces of mpm_surface_mesh_indexed with their vertices rounded to
 * float, in the same order. */
mpm_status mpm_surface_mesh(mpm_ctx* ctx, int32_t grid_side, int32_t radius, float* tris, int64_t capacity,
                            int64_t* n_tris);
/* The surface as MeshBuilder::computeMesh hands it to igl::writeOBJ
 * (include/mesh_builder.h:193-210, without smoothing or decimation): vertices (3 doubles
 * each, world units) in the order libigl's marching cubes creates them, bit for bit, and
 * faces (3 zero-based vertex indices each, outward).  Copies up to the capacities;
 * *n_vertices and *n_faces receive the counts, which may exceed them. */
mpm_status mpm_surface_mesh_indexed(mpm_ctx* ctx, int32_t grid_side, int32_t radius, double* vertices,
                                    int64_t vertex_capacity, int32_t* faces, int64_t face_capacity,
                                    int64_t* n_vertices, int64_t* n_faces);
/* The marching-cubes triangle table (no context, no GPU): for each inside-corner mask m
 * (bit n: libigl's corner n has S > 0), counts[m] triangles as edge-slot triples in
 * slots[30 m ...] (-1 past them). */
mpm_status mpm_surface_table(int32_t* counts, int32_t* slots);
/* The distance field left in device memory (the context's buffer, valid until the next
 * surface call or mpm_destroy), written asynchronously on the context's stream. */
mpm_status mpm_surface_distance_device(mpm_ctx* ctx, int32_t grid_side, int32_t radius, const float** field);
/* The same triangles left in device memory: *tris receives the context's buffer (valid
 * until the next surface call or mpm_destroy), written asynchronously on the context's
 * stream after the call returns (the call itself waits once, for the count). */
mpm_status mpm_surface_mesh_device(mpm_ctx* ctx, int32_t grid_side, int32_t radius, const float** tris,
                                   int64_t* n_tris);
/* The same vertices and faces left in device memory (the context's buffers, valid until
 * the next surface call or mpm_destroy), written asynchronously on the context's stream
 * after the call returns (the call itself waits once, for the counts). */
mpm_status mpm_surface_mesh_indexed_device(mpm_ctx* ctx, int32_t grid_side, int32_t radius, const double** vertices,
                                           const int32_t** faces, int64_t* n_vertices, int64_t* n_faces);
/* Laplacian smoothing of a triangle mesh (MeshBuilder::smoothMesh,
 * include/mesh_builder.h:212-245, the --laplacian_smooth step of computeMesh): one implicit
 * step U = (M - 0.001 L)^-1 M V with libigl's cotangent Laplacian L and barycentric lumped
 * mass matrix M of the input mesh, then U divided by the square root of its area (the
 * reference's rescale to unit area).  vertices (3 doubles each) are replaced by U; faces are 3
 * zero-based vertex indices each.  Solved in double on the GPU by conjugate gradients
 * preconditioned by the diagonal, to a relative residual of 1e-12 per coordinate (the
 * reference factors M - 0.001 L by a sparse Cholesky).  A vertex that no face uses keeps
 * its position (rescaled).  MPM_ERR_INVALID for a face index outside [0, n_vertices), a face
 * of zero area (the reference's cotangent weights are not finite there) or vertices without
 * faces; MPM_ERR_STATE if the solver did not converge (vertices unchanged then).
 * *iterations (may be NULL) receives the solver's iteration count.  Synchronises. */
mpm_status mpm_surface_smooth(mpm_ctx* ctx, double* vertices, int64_t n_vertices, const int32_t* faces,
                              int64_t n_faces, int32_t* iterations);
/* The same on device arrays (e.g. those of mpm_surface_mesh_indexed_device), in place, on the
 * context's stream; synchronises. */
mpm_status mpm_surface_smooth_device(mpm_ctx* ctx, double* vertices, int64_t n_vertices, const int32_t* faces,
                                     int64_t n_faces, int32_t* iterations);

/* ---------------------------------------------------------------------------
 * Particle export (ParticleWriter::writeParticles, include/particle_writer.h:19-43).  The
 * reference writes each saved frame through Partio as a .bgeo file: per active particle
 * its index "id", "position", "velocity" and "radius" 0.1.  Here the point records of that
 * file (Houdini classic binary geometry v5 as Partio writes it: P = x y z 1, id,
 * velocity, radius; 36 bytes, big-endian) are packed on the GPU from the particle arrays,
 * in the active-list order of mpm_download_*, and copied to pinned host memory on a copy
 * stream that waits only for the packing, so substeps enqueued after the export overlap
 * the copy.  Two slots let one frame be written to disk while the next is copied.
 * ------------------------------------------------------------------------- */
#define MPM_BGEO_RECORD_BYTES 36
/* Packs the records into slot (0 or 1) and starts their copy; *n receives the count.
 * Reusing a slot first waits for its previous copy (on the GPU). */
mpm_status mpm_export_particles(mpm_ctx* ctx, int32_t slot, float radius, int64_t* n);
/* Waits for slot's copy; *records = its n records in pinned host memory, valid until the
 * slot is exported into again or the context is destroyed. */
mpm_status mpm_export_wait(mpm_ctx* ctx, int32_t slot, const void** records, int64_t* n);
/* Writes a .bgeo file: header, the n records, terminator (uncompressed; readers of the
 * format also accept the gzip-compressed form the reference writes). */
mpm_status mpm_write_bgeo(const char* path, const void* records, int64_t n);
/* The .bgeo header for n points into out (when capacity allows); returns its size. */
int64_t mpm_bgeo_header(int64_t n, uint8_t* out, int64_t capacity);

/* ---------------------------------------------------------------------------
 * Headless point rendering (Renderer::render, include/renderer.h:43-63, and its shaders).
 * The reference uploads (x - 0.5) * 1.8 per particle as clip-space positions and draws
 * 2-pixel points of colour (0.59, 0.54, 0.2) on an 800 x 600 frame cleared to 0.1 grey,
 * without depth test or blending.  No graphics API is used here.
 * ------------------------------------------------------------------------- */
/* The clip-space positions (3 floats per particle, active-list order) in the context's
 * device buffer, valid until the next call; written asynchronously on its stream. */
mpm_status mpm_render_positions_device(mpm_ctx* ctx, const float** positions);
/* The same positions copied to host memory (3 floats per particle).  Synchronises. */
mpm_status mpm_render_positions(mpm_ctx* ctx, float* positions);
/* RGB8 image (width x height x 3 bytes, rows top to bottom) of the points: pixels whose
 * centres fall inside a point_size square around a point inside the clip volume take
 * `color`, the others `background`.  Synchronises. */
mpm_status mpm_render_points(mpm_ctx* ctx, int32_t width, int32_t height, float point_size, const uint8_t color[3],
                             const uint8_t background[3], uint8_t* rgb);

/* Self-check of failure detection (no counterpart in the reference): one warp waits on
 * an mbarrier that nothing completes, gives up after `polls` polls (1..2^20; each poll
 * may suspend for a hardware-defined interval, microseconds at most) and sets the status
 * word, exactly as the substep kernel does when a tile copy never lands.  Returns
 * MPM_ERR_TIMEOUT (the expected outcome) through mpm_sync; the context stays usable. */
mpm_status mpm_check_wait_timeout(mpm_ctx* ctx, int32_t polls);

/* Copy the last error message (NUL-terminated, truncated to len). */
mpm_status mpm_last_error(const mpm_ctx* ctx, char* buf, size_t len);
/* Kernel launches issued by this context since creation (for accounting). */
int64_t mpm_launch_count(const mpm_ctx* ctx);

/* G2P tile boxes of the fused substep kernel (grid nodes along i x j x k): a box covers
 * the steps whose 32 particles' base cells span at most (box - 2) cells per dimension;
 * other steps gather straight from the velocity grid. */
enum {
  MPM_TILE_4x4x6 = 1, /* the default: one cell, or two neighbours along a sort-brick row */
  MPM_TILE_4x4x4 = 2, /* a third fewer bytes per copy, for steps within 2 x 2 x 2 cells */
  MPM_TILE_4x6x6 = 3  /* also steps across a brick's rows, for sparse scenes (12 warps) */
};
/* Tuning knobs of the fused substep kernel (the reference launches a fixed 64-thread
 * block per 64 particles, src/mpm.cu:217-222):
 *   steps_per_warp: the largest number of 32-particle steps in each range a warp claims
 *     (1..256, default 2); it is halved while each warp would get fewer than 6 ranges;
 *   warps_per_cta: CTA size of the fused kernel, 4, 6 or 12 warps (3, 2 or 1 CTAs per SM,
 *     12 warps resident either way; default 12);
 *   tile_box: MPM_TILE_* (the 4x4x4 and 4x6x6 boxes need 12 warps per CTA).
 * 0 keeps a knob's current value.  Results do not depend on the knobs beyond rounding
 * (the order of the grid's float additions). */
mpm_status mpm_set_tuning(mpm_ctx* ctx, int32_t steps_per_warp, int32_t warps_per_cta, int32_t tile_box);

/* A launch shape of the fused substep kernel (and the sort interval it was measured with). */
typedef struct mpm_tuning {
  int32_t steps_per_warp;
  int32_t warps_per_cta;
  int32_t tile_box;       /* MPM_TILE_* */
  int32_t sort_interval;
  double us_per_substep;  /* measured device time of one substep with this shape (0: not measured) */
  int32_t from_cache;     /* 1: taken from the cache file without measuring */
  int32_t candidates;     /* shapes timed by the search */
} mpm_tuning;

enum {
  MPM_TUNE_SORT_INTERVAL = 1, /* also choose the sort interval (it then replaces params.sort_interval) */
  MPM_TUNE_IGNORE_CACHE = 2   /* measure even when the cache holds an entry (and replace it) */
};

/* Autotuner (no counterpart in the reference, whose launch shape is fixed,
 * src/mpm.cu:217-222): chooses the fused substep's steps per warp, CTA size and tile box
 * (and, with MPM_TUNE_SORT_INTERVAL, the sort interval) for the context's current scene and
 * applies them.  The search is a coordinate descent over those knobs; each candidate is timed
 * with CUDA events over budget_substeps substeps (0: 48; sort intervals over at least two of
 * their periods) on a temporary copy of the context's particles, so the context's own state
 * does not change.  With a cache_path (a JSON file; NULL: no cache), a shape found for the
 * same device, library build and workload class (particle layout, N, particle count to the
 * nearest power of two, material kinds) is reused without measuring, and a new one is
 * stored (MPM_ERR_IO, with the shape applied, when the file cannot be written or is not a
 * tuning cache: another file at that path is never overwritten).  *out (may be NULL)
 * receives the chosen shape.  Synchronises; allocates a copy of the particle arrays while it
 * runs. */
mpm_status mpm_autotune(mpm_ctx* ctx, const char* cache_path, int32_t flags, int32_t budget_substeps,
                        mpm_tuning* out);
/* The context's current launch shape (us_per_substep, from_cache and candidates are 0). */
mpm_status mpm_get_tuning(const mpm_ctx* ctx, mpm_tuning* out);

/* ---------------------------------------------------------------------------
 * Batched scenes.  The reference runs one scene per Simulation; a batch advances many
 * independent scenes (own N, dt, gravity, boundary, material and particle count) with
 * one fused launch per substep for all of them, optionally as a replayed CUDA graph.
 * Particle arrays of a batch are the scenes' particles concatenated in scene order
 * (same per-particle interleaved host layout as mpm_upload_soa).
 * ------------------------------------------------------------------------- */
typedef struct mpm_scene {
  mpm_params params;     /* dt, N, gravity, boundary of this scene (g2p_guard unsupported) */
  mpm_material material; /* the scene's material (particle_volume is per scene) */
  int64_t count;         /* particles of this scene */
} mpm_scene;

typedef struct mpm_batch mpm_batch;

mpm_status mpm_batch_create(const mpm_scene* scenes, int32_t nscenes, int32_t sort_interval, mpm_batch** out);
mpm_status mpm_batch_destroy(mpm_batch* batch);
/* A non-default cudaStream_t for all further work (graphs are re-captured). */
mpm_status mpm_batch_set_stream(mpm_batch* batch, void* cuda_stream);
mpm_status mpm_batch_upload_soa(mpm_batch* batch, const float* x, const float* v, const float* C, const float* F,
                                const float* Jp);
/* nsteps substeps of every scene, one launch each (plus the periodic cell sort). */
mpm_status mpm_batch_substep(mpm_batch* batch, int32_t nsteps);
/* The same as one CUDA graph (captured on first use per phase, then replayed); the
 * particles are cell-sorted at the start of each replayed run and then every sort_interval
 * substeps of it. */
mpm_status mpm_batch_substep_graph(mpm_batch* batch, int32_t nsteps);
mpm_status mpm_batch_sync(mpm_batch* batch);
mpm_status mpm_batch_download_soa(mpm_batch* batch, float* x, float* v, float* C, float* F, float* Jp);
int64_t mpm_batch_particle_count(const mpm_batch* batch);
int64_t mpm_batch_launch_count(const mpm_batch* batch);
mpm_status mpm_batch_last_error(const mpm_batch* batch, char* buf, size_t len);
/* Range size of the batched substep kernel: each warp takes ranges of 32 * steps_per_warp
 * particles of one scene (1..256; default 8).  Rebuilds the range table and drops the
 * captured graphs; synchronises the batch's stream. */
mpm_status mpm_batch_set_steps_per_warp(mpm_batch* batch, int32_t steps_per_warp);
/* Sort interval of a batch (0: never); captured graphs, which sort before their first
 * substep and then every sort_interval substeps, are dropped.  Synchronises the batch's
 * stream. */
mpm_status mpm_batch_set_sort_interval(mpm_batch* batch, int32_t sort_interval);
/* The batch's launch shape: steps_per_warp, warps_per_cta (fixed), tile_box 0 (the batched
 * kernel gathers through L1, without a G2P tile) and the sort interval. */
mpm_status mpm_batch_get_tuning(const mpm_batch* batch, mpm_tuning* out);
/* Autotuner of a batch (no counterpart in the reference): times the batched kernel's range
 * sizes (1, 2, 4, 8, 16 steps per warp) as replayed graphs of budget_substeps substeps
 * (0: 24; rounded up to a multiple of 6) on a temporary copy of the batch, so the batch's own
 * state does not change, and applies the fastest (a change needs a gain above 1%).  With
 * MPM_TUNE_SORT_INTERVAL it then times sort intervals of 8, 12, 16 and 24 substeps over
 * replays of 48.  The cache file, flags and *out are as for mpm_autotune; the
 * workload class is the scene count, the particle count to the nearest power of two, the
 * grid sides and the material kinds.  Synchronises; allocates a second batch while it runs. */
mpm_status mpm_batch_autotune(mpm_batch* batch, const char* cache_path, int32_t flags, int32_t budget_substeps,
                              mpm_tuning* out);

/* ---------------------------------------------------------------------------
 * Differentiable substeps (no counterpart in the reference, which has no gradients).
 * A fixed-corotated (MMFixedCorotated, include/MaterialModel.cuh:40-62) or snow (MMSnow,
 * :67-116) scene is run forward with a checkpoint every `checkpoint_every` substeps; the
 * backward pass recomputes each segment (keeping its states, P2G grids and the polar
 * rotation of each particle's P2G: per segment, checkpoint_every x (34 floats per particle
 * + one N^3 float4 grid) of device memory) and runs hand-written adjoint kernels in
 * reverse.  Host arrays use the interleaved layout of mpm_upload_soa.
 * ------------------------------------------------------------------------- */
typedef struct mpm_diff mpm_diff;
mpm_status mpm_diff_create(const mpm_params* params, const mpm_material* material, int64_t n, int32_t max_steps,
                           int32_t checkpoint_every, mpm_diff** out);
mpm_status mpm_diff_destroy(mpm_diff* diff);
/* Change E / nu and the other material constants (the material kind must stay the same:
 * MPM_ERR_INVALID otherwise). */
mpm_status mpm_diff_set_material(mpm_diff* diff, const mpm_material* material);
/* nsteps substeps from the initial state; writes the final x and v (either may be NULL). */
mpm_status mpm_diff_forward(mpm_diff* diff, const float* x0, const float* v0, const float* C0, const float* F0,
                            const float* Jp0, int32_t nsteps, float* x_out, float* v_out);
/* Adjoint of the last forward run: from dL/dx, dL/dv of the final state to dL/d of the
 * initial x, v, C, F and dL/dmu0, dL/dlambda0 (gmu_glambda[2]); outputs may be NULL. */
mpm_status mpm_diff_backward(mpm_diff* diff, const float* gx_final, const float* gv_final, float* gx0, float* gv0,
                             float* gC0, float* gF0, double* gmu_glambda);

/* Substep entry point that allocates nothing.  It has no counterpart in the reference.
 * For callers that cannot call cudaMalloc: plugins whose host application owns all device
 * memory through its own pool, and embedded or real-time callers that forbid allocation after
 * start-up (an allocation may block, fail or fragment memory at a time they do not choose).
 * It runs `nsteps` substeps on the caller's device state in place, on `stream` (NULL: the
 * legacy default stream), asynchronously:
 *   - state: caller-owned device memory in the library's component-major layout, component k
 *     of particle p at state[k * stride + p]: x 0-2, v 3-5, C 6-14 and F 15-23 (row-major),
 *     Jp 24 (J for a single-liquid table, whose F components are not touched);
 *   - mat: device array of material indices (each < n_materials; a larger index is flagged
 *     in the status word and the particle takes material 0), or NULL for material 0;
 *   - the scratch (three P2G grids, the padded velocity grid and the device status word) is a
 *     static device array of 2.3 MiB that every GPU loading the library holds until exit, so N
 *     is limited to 32 (MPM_ERR_UNSUPPORTED above); g2p_guard is not supported here.
 * Particles are processed in the caller's order (no cell sort; sorted input runs faster).
 * Device-side faults (an expired bounded wait, a non-finite position with check_finite, a
 * material index past the table) set the status word; it is kept across calls until
 * mpm_noalloc_status reads and clears it.
 * The first call on a device looks up the scratch's device address (cudaGetSymbolAddress), so
 * make that first call before any stream capture.  All calls share the scratch, which keeps
 * the last call's contents (each call clears what must start at zero): calls that overlap on
 * the GPU, from any thread or stream, race and must be serialised by the caller. */
mpm_status mpm_substep_noalloc(const mpm_params* params, const mpm_material* materials, int32_t n_materials,
                               float* state, int64_t stride, const uint8_t* mat, int64_t n, int32_t nsteps,
                               void* stream);
/* Status of the no-allocation substeps on the current device (no counterpart in the
 * reference): waits for `stream`, reads the status word in the static scratch and clears it.
 * Returns MPM_ERR_TIMEOUT when a bounded device wait expired (the substep that saw it may
 * have gathered from a grid tile that never arrived), MPM_ERR_STATE for a non-finite particle
 * or a material index past the table, MPM_OK otherwise.  Allocates nothing. */
mpm_status mpm_noalloc_status(void* stream);
/* Self-check of that status path (no counterpart in the reference): one warp on `stream`
 * waits on an mbarrier nothing completes, gives up after `polls` polls (1..2^20) and sets the
 * timeout bit of the no-allocation status word, as the substep does when a tile copy never
 * lands; mpm_noalloc_status then returns MPM_ERR_TIMEOUT.  Allocates nothing. */
mpm_status mpm_noalloc_check_wait_timeout(int32_t polls, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* MPM_GB300_H */
