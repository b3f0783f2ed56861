/*
 * rd_mpm.h - C ABI of the GB300 (sm_103a) explicit APIC / MLS-MPM snow step.
 *
 * Drop-in boundary for the simulation core of brocbyte/realtime-deformations:
 * the class MaterialPointMethod::LagrangeEulerView
 * (realtime-deformations/material_point_method.hpp:174-233), driven by
 * main.cpp:48-54,192-218 and read by drawParticles through getParticles()
 * (main.cpp:255-271).  Each entry point below names the reference interface it
 * replaces.  Plain C: pointers, sizes and POD structs only; no exceptions cross
 * the boundary; every call returns an rd_status.
 *
 * Threading: one handle is used by one host thread at a time.  Each handle owns
 * one CUDA stream and all of its device and host buffers; there is no global
 * mutable state (the reference's global WeightCalculator::h and __constant__
 * devH become per-handle parameters).
 *
 * Element type: every floating-point array crossing the ABI is float when the
 * handle was created with RD_FP32 and double with RD_FP64.  Matrices are 3x3
 * row-major in the math sense, M[3*r + c] = M(r, c) (glm stores the transpose).
 */
#ifndef RD_MPM_H
#define RD_MPM_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum rd_status {
    RD_OK = 0,
    RD_INVALID_ARG = 1,      /* bad pointer, size or parameter */
    RD_OOM = 2,              /* device or pinned-host allocation failed */
    RD_CUDA_ERROR = 3,       /* a CUDA runtime call failed; see rd_last_error */
    RD_DEVICE_FAULT_FLAG = 4,/* a kernel raised a status flag; see rd_get_flags */
    RD_TIMEOUT = 5,          /* a bounded device wait gave up */
    RD_NOT_SUPPORTED = 6,
    RD_TOO_LARGE = 7         /* beyond a fixed capacity (rd_rasterize_noalloc; index ranges) */
} rd_status;

enum { RD_FP32 = 0, RD_FP64 = 1 };
enum { RD_HOST = 0, RD_DEVICE = 1 };
/* Grid boundary condition applied in the grid update.  The reference has no
 * grid boundary; it only clamps particle positions to [3h, (MAX-3)h]
 * (material_point_method.cpp:381-388), which every mode keeps. */
enum { RD_BC_NONE = 0, RD_BC_STICKY = 1 };

/* Device status flags (sticky until rd_clear_flags). */
enum {
    RD_FLAG_OUT_OF_DOMAIN = 1u << 0, /* a stencil node fell outside the grid; dropped */
    RD_FLAG_NONFINITE = 1u << 1,     /* NaN/Inf in particle state after a step */
    RD_FLAG_BAD_WORK = 1u << 2,      /* internal work-list inconsistency */
    RD_FLAG_WAIT_TIMEOUT = 1u << 3   /* a kernel's bounded wait for a tile copy gave up; the step stopped */
};

/* Stage ids for rd_stage, in the order main.cpp:192-218 calls them. */
enum {
    RD_STAGE_RASTERIZE = 0,       /* rasterizeParticlesToGrid, material_point_method.cpp:94-129 */
    RD_STAGE_FORCES = 1,          /* computeExplicitGridForces, :235-254 */
    RD_STAGE_GRID_VELOCITIES = 2, /* gridVelocitiesUpdate(dt), :256-262 (+ rd_params.bc) */
    RD_STAGE_COLLISIONS = 3,      /* gridBasedCollisions(dt, {}), :298-304 (identity) */
    RD_STAGE_DEFORMATION = 4,     /* updateDeformationGradient(dt), :306-330 */
    RD_STAGE_PARTICLE_VELOCITIES = 5, /* updateParticleVelocities, :332-342 */
    RD_STAGE_POSITIONS = 6,       /* updateParticlePositions(dt), :344-350 */
    RD_STAGE_VOLUMES = 7          /* computeParticleVolumesAndDensities, :131-142 */
};

/* Replaces the LagrangeEulerView constructor arguments (material_point_method.hpp:178),
 * the global WeightCalculator::h (material_point_method.cpp:17) and the constants
 * hard-coded in the step (material_point_method.cpp:237-238,260,320;
 * material_point_method.hpp:213).  rd_default_params fills the reference's values. */
typedef struct rd_params {
    int32_t max_i, max_j, max_k;  /* grid nodes per axis (MAX_I, MAX_J, MAX_K) */
    int32_t num_particles;        /* particlesNum */
    double h;                     /* cell size */
    double E, nu, xi;             /* Young's modulus, Poisson ratio, hardening */
    double theta_c, theta_s;      /* singular values clamped to [1-theta_c, 1+theta_s] */
    double gravity[3];
    int32_t bc;                   /* RD_BC_NONE (reference) or RD_BC_STICKY */
    int32_t bc_width;             /* sticky wall width in cells (3) */
    int32_t lagged_b;             /* 1: F update uses B of the previous G2P (reference
                                     order, main.cpp:209-214); 0: textbook order */
    int32_t track_fp;             /* 1: also carry the full plastic F_P (for getParticles);
                                     0: carry J_P = det F_P only */
    int32_t precision;            /* RD_FP32 or RD_FP64 */
    int32_t device;               /* CUDA device ordinal */
} rd_params;

/* Particle arrays, structure of arrays (the reference's Particle,
 * material_point_method.hpp:96-110, without the per-step neighbour list and the
 * viewer's colour/size).  Any pointer may be NULL where noted. */
typedef struct rd_particles {
    void* x;      /* n x 3 positions (required on set) */
    void* v;      /* n x 3 velocities (required on set) */
    void* B;      /* n x 9 APIC B (C = B * DpInverse); NULL on set means 0 */
    void* FE;     /* n x 9 elastic F; NULL on set means identity */
    void* FP;     /* n x 9 plastic F; used only when track_fp; NULL means identity */
    void* Jp;     /* n plastic det; NULL on set means det(FP) or 1 */
    void* mass;   /* n (required on set) */
    void* volume; /* n; NULL on set means 0 (call rd_init_volumes) */
} rd_particles;

typedef struct rd_handle rd_handle;

void rd_default_params(rd_params* p);

/* LagrangeEulerView(max_i, max_j, max_k, particlesNum), material_point_method.cpp:144-154.
 * Allocates every device buffer once; nothing is allocated per step. */
rd_status rd_create(const rd_params* params, rd_handle** out);
/* ~LagrangeEulerView, material_point_method.cpp:156-158 */
rd_status rd_destroy(rd_handle* h);

/* Writes particle state (initializeParticles / writes through getParticles(),
 * material_point_method.cpp:18-63, .hpp:181-183).  where = RD_HOST or RD_DEVICE.
 * RD_HOST: a field in page-locked host memory (cudaHostAlloc, cudaHostRegister)
 * is read in place by the packing kernel over the CPU-GPU link; other host
 * fields are copied to a device staging buffer first.  Either way the call
 * returns once the work is queued: the arrays stay untouched until the
 * handle's stream reaches it (rd_synchronize). */
rd_status rd_set_particles(rd_handle* h, const rd_particles* in, int where);
/* Reads particle state in the caller's original particle order (getParticles()).
 * Fields left NULL are skipped.  RD_HOST: page-locked fields are written in
 * place by the unpacking kernel, the others through a staging buffer; the
 * call returns when the data is there.  RD_DEVICE: returns once queued. */
rd_status rd_get_particles(rd_handle* h, rd_particles* out, int where);

/* rasterizeParticlesToGrid + computeParticleVolumesAndDensities, main.cpp:53-54. */
rd_status rd_init_volumes(rd_handle* h);
/* nsteps x (the seven stage calls of main.cpp:192-218 with no colliders), fused:
 * per step a sort by block and one kernel that runs the grid update, G2P, the
 * plastic SVD and advection of this step and the P2G (MLS force) of the next.
 * The next step's grid is built with this dt; a call with a different dt
 * rebuilds it first. */
rd_status rd_step(rd_handle* h, double dt, int32_t nsteps);
/* One reference stage at the reference's granularity (RD_STAGE_*). */
rd_status rd_stage(rd_handle* h, int32_t stage, double dt);

/* Grid fields as the reference's Cell holds them after the last stage run
 * (material_point_method.hpp:112-117): mass (cells), velocity (cells x 3),
 * force (cells x 3, rd_stage mode only).  Dense, index i*MAX_J*MAX_K + j*MAX_K + k.
 * After rd_step the velocity is the updated grid velocity used by G2P. */
rd_status rd_get_grid(rd_handle* h, void* mass, void* velocity, void* force, int where);

/* Headless stand-in for the viewer's position stream (main.cpp:259-271):
 * float4 (x, y, z, size) per particle in original order, on the device, valid
 * until the next mutating call.  Borrowed pointer. */
rd_status rd_device_xyzs(rd_handle* h, float** xyzs);

/* The colour stream of the same draw (Particle::r, g, b, a): rgba8 per particle in
 * original order, white unless set.  rd_set_colors takes n x 4 bytes. */
rd_status rd_set_colors(rd_handle* h, const uint8_t* rgba, int where);
rd_status rd_device_colors(rd_handle* h, uint8_t** rgba);

/* Point-splat image of the viewer feed, made with CUDA alone (no graphics API; a
 * stand-in for drawParticles' billboards, main.cpp:255-300 and
 * Particle.vertexshader): each particle covers the disc its camera-facing square
 * of side `size` (0.02) projects to, the nearest particle wins each pixel and is
 * shaded as a sphere impostor.  width x height rgba8 pixels, rows from the top,
 * written to `image` (host or device per `where`). */
typedef struct rd_view {
    float view_projection[16]; /* column-major (glm): clip = VP * (x, y, z, 1) */
    float camera_right[3];     /* world-space camera axes (the shader's uniforms) */
    float camera_up[3];
    int32_t width, height;
    uint32_t background;       /* rgba8 */
    int32_t max_radius;        /* pixels; 0 = 32 */
} rd_view;
rd_status rd_splat(rd_handle* h, const rd_view* view, void* image, int where);

/* The reference's diagnostics (material_point_method.cpp:352-443) as device
 * reductions over one scene (0 for a single-scene handle): particleMomentum and
 * the particle mass; gridMass and gridMomentum over the nodes with mass of the
 * grid the last step used (its velocities as G2P read them); the count of such
 * nodes; averageParticleDensity (mean m / V over particles with V > 0);
 * averageDeformationGradient (mean F_E F_P; without the full F_P (track_fp = 0)
 * F_P is taken as J_P^(1/3) I).  All in double. */
typedef struct rd_diagnostics {
    double particle_mass, particle_momentum[3];
    double grid_mass, grid_momentum[3];
    int64_t used_cells;
    double average_particle_density;
    double average_deformation_gradient[9]; /* row-major */
} rd_diagnostics;
rd_status rd_get_diagnostics(rd_handle* h, int32_t scene, rd_diagnostics* out);

rd_status rd_get_flags(rd_handle* h, uint32_t* flags);
rd_status rd_clear_flags(rd_handle* h);
rd_status rd_synchronize(rd_handle* h);
/* The handle's CUDA stream (cudaStream_t), for callers that order their own work. */
rd_status rd_get_stream(rd_handle* h, void** stream);
/* Copies the last error message (NUL-terminated, truncated to len). */
rd_status rd_last_error(rd_handle* h, char* buf, size_t len);
/* Sort diagnostic: sorts the current particles by cell (as every step does)
 * and returns each particle's sort key in original order (n) and the original
 * index of the particle at each sorted position (n).  The key of a particle
 * with base cell b = ivec3(pos / h) (material_point_method.cpp:83) is
 * block * 64 + cell: block = b / 4 per axis linearised x-major like the grid,
 * cell = (b % 4) linearised the same way.  Host or device arrays per `where`. */
rd_status rd_debug_sort(rd_handle* h, uint32_t* keys, uint32_t* order, int where);
/* Exercises the bounded wait of the fused kernel's tile copies: one CTA waits
 * `tries` polls on an mbarrier that nothing arrives at, raises
 * RD_FLAG_WAIT_TIMEOUT and returns; *gave_up = 1 when the wait ran out.  No
 * copy is issued, so nothing is left in flight. */
rd_status rd_debug_wait_timeout(rd_handle* h, int32_t tries, int32_t* gave_up);
/* The bounds-checked build of the library (compiled with RD_BOUNDS_CHECK,
 * librd_mpm_checked.so; no counterpart in the reference) tests the indexes of
 * the fused kernel's and the P2G's shared tiles, records, particles and grid
 * nodes before each access, skips an access out of range and counts it: the
 * count of this process so far into *count, after the handles' work has
 * finished (rd_synchronize), and *checked = 1.  The normal build reports
 * *count = 0 and *checked = 0. */
rd_status rd_debug_bounds_violations(uint64_t* count, int32_t* checked);
/* Kernel ids for the per-kernel event timing below. */
enum {
    RD_KERNEL_KEYS = 0,     /* block keys + histogram (when not fused into G2P) */
    RD_KERNEL_SCAN = 1,     /* scan of the block counts, work items */
    RD_KERNEL_SCATTER = 2,  /* sorted permutation */
    RD_KERNEL_GRID_CLEAR = 3,
    RD_KERNEL_P2G = 4,      /* P2G with the MLS force from the stored state (first step,
                               or after the step size changed) */
    RD_KERNEL_G2P2G = 5,    /* grid update + G2P + F update + advection of this step and
                               the P2G (with the MLS force) of the next, fused */
    RD_KERNEL_ADJ_G2P = 6,  /* reverse of G2P, advection and the plastic split */
    RD_KERNEL_ADJ_P2G = 7,  /* reverse of the grid update and of P2G with the stress */
    RD_KERNEL_COUNT = 8
};
/* Per-kernel timing with CUDA events recorded on the handle's stream around
 * each launch of rd_step (profiling runs; off by default).  rd_kernel_timing
 * synchronises and returns the launches and total milliseconds accumulated
 * since timing was enabled or last reset. */
rd_status rd_set_kernel_timing(rd_handle* h, int enable);
rd_status rd_kernel_timing(rd_handle* h, int kernel, uint64_t* launches, double* total_ms);
/* Number of kernel launches issued by this handle so far. */
rd_status rd_launch_count(rd_handle* h, uint64_t* count);
/* Number of two-step CUDA graphs this handle has replayed (rd_set_graphs). */
rd_status rd_graph_replays(rd_handle* h, uint64_t* count);
/* Bytes of particle state moved by rd_set_particles / rd_get_particles with
 * RD_HOST so far: read or written in place in page-locked host memory, and
 * through the device staging buffer. */
rd_status rd_io_bytes(rd_handle* h, uint64_t* in_place, uint64_t* staged);
/* Page-locked host memory (cudaHostAlloc) for the particle arrays of
 * rd_set_particles / rd_get_particles, which the pack and unpack kernels then
 * read and write in place: the host side of the reference's particle buffer
 * (material_point_method.hpp:181-183) for callers without CUDA headers.
 * bytes = 0 gives NULL.  RD_OOM when the allocation fails. */
rd_status rd_host_alloc(size_t bytes, void** out);
/* Releases memory from rd_host_alloc (NULL: nothing). */
rd_status rd_host_free(void* p);

/* initializeParticles (material_point_method.cpp:18-63) on the device: the cells
 * within radius / h of the origin, 8 points per cell at quarter offsets, each
 * jittered inside a ball of a quarter cell, kept where within `radius` of the
 * origin, placed from the last particle down with this velocity and mass (the
 * reference: radius 0.2, mass 6e-5); particles left over stay at the origin with
 * no mass.  RD_INIT_REFERENCE draws the jitter from the C library's rand()
 * sequence after srand(seed) as the reference does (seed 1 when it never seeds),
 * on one device thread, and reproduces the reference's particles;
 * RD_INIT_PARALLEL draws it from a counter-based hash of (seed, candidate) on one
 * thread per candidate, for large scenes.  *need_more (may be NULL) receives the
 * number of kept points that found no particle.  Single-scene handles. */
enum { RD_INIT_REFERENCE = 0, RD_INIT_PARALLEL = 1 };
typedef struct rd_init_spec {
    double origin[3], velocity[3];
    double radius, mass;
    uint32_t seed;
    int32_t mode;
} rd_init_spec;
rd_status rd_initialize_particles(rd_handle* h, const rd_init_spec* spec, int32_t* need_more);

/* ---- Box colliders (gridBasedCollisions, material_point_method.cpp:264-304) ----
 * The reference's MeshCollider (material_point_method.hpp:74-93) as main.cpp
 * builds it (main.cpp:119-160): a box mesh spanning [-1, 1]^3 placed by
 * matrixWorld = T R S, with a rigid velocity.  Its signed distance is
 * max_i(|p_i| - s_i) in the box frame p = R^T (x - t).  The grid update applies
 * them in order to every node with mass: where the distance is <= 0 and the
 * velocity relative to the box points inwards (v_n = v_rel . n < 0), the
 * relative velocity becomes its tangential part with friction mu = `friction`
 * (0.5 in the reference):
 *   RD_COLLIDE_REFERENCE  as the reference computes it: n = central
 *       differences of the distance with step 0.001 (mathy.hpp:40-56), and
 *       v_t (1 + mu v_n / 3), sticking only when -mu v_n >= 3 - the reference
 *       divides by glm's vec3::length(), which is the component count 3;
 *   RD_COLLIDE_COULOMB    the Coulomb law it intends: n the outward face
 *       normal, v_t (1 + mu v_n / |v_t|), sticking when |v_t| <= -mu v_n.
 * Single-scene handles; up to RD_MAX_COLLIDERS. */
#define RD_MAX_COLLIDERS 16
enum { RD_COLLIDE_REFERENCE = 0, RD_COLLIDE_COULOMB = 1 };
typedef struct rd_collider {
    double translation[3]; /* t: the box centre (mesh.translation) */
    double rotation[4];    /* R as a unit quaternion (w, x, y, z) (mesh.rotation) */
    double scale[3];       /* s: the half extents (mesh.scale) */
    double velocity[3];    /* MeshCollider::velocity */
} rd_collider;
/* Replaces the handle's colliders (count 0 removes them). */
rd_status rd_set_colliders(rd_handle* h, const rd_collider* colliders, int32_t count, int32_t mode, double friction);
/* MeshCollider::move (material_point_method.hpp:89-91) for every collider:
 * t += dt * velocity.  main.cpp:188 calls it once per frame. */
rd_status rd_move_colliders(rd_handle* h, double dt);

/* ---- Batches: many independent scenes stepped together ----
 * No counterpart in the reference, which simulates one LagrangeEulerView per
 * process.  scenes[s] describes scene s exactly as rd_create's params do (its
 * own grid size, cell size, material, gravity, walls and particle count);
 * precision, device, lagged_b and track_fp must agree across scenes and
 * track_fp must be 0 (RD_NOT_SUPPORTED otherwise).  Each step sorts all
 * scenes' particles once and runs one fused kernel over a work list of
 * (scene, block) items; each item reads its scene's parameters.  rd_step,
 * rd_init_volumes, rd_autotune, rd_get_flags, rd_synchronize and
 * rd_device_xyzs act on the whole batch (the xyzs of scene s's particle i
 * are entry first_s + i, first_s = the particle counts of scenes 0..s-1
 * summed); rd_stage, rd_set_particles, rd_get_particles and rd_get_grid are
 * single-scene calls and return RD_NOT_SUPPORTED / RD_INVALID_ARG on a batch.
 * Every scene needs its particles set before rd_init_volumes and rd_step. */
rd_status rd_batch_create(const rd_params* scenes, int32_t nscenes, rd_handle** out);
rd_status rd_batch_num_scenes(rd_handle* h, int32_t* nscenes);
/* rd_set_particles / rd_get_particles / rd_get_grid (mass and velocity) of one scene. */
rd_status rd_batch_set_particles(rd_handle* h, int32_t scene, const rd_particles* in, int where);
rd_status rd_batch_get_particles(rd_handle* h, int32_t scene, rd_particles* out, int where);
rd_status rd_batch_get_grid(rd_handle* h, int32_t scene, void* mass, void* velocity, int where);
/* Same as rd_step. */
rd_status rd_batch_step(rd_handle* h, double dt, int32_t nsteps);

/* CUDA graphs, on by default: within one rd_step call, once the step is steady
 * (positions counted, grid built for this dt), each pair of steps is replayed
 * as one captured graph (scan, scatter, grid clear and the fused kernel, twice)
 * instead of individual launches.  Results are those of the launches. */
rd_status rd_set_graphs(rd_handle* h, int enable);

/* Autotuner: times `steps` steps of the current state (from the same saved
 * state each time) for each work-item size (FP32: 64, 128, 192, 256 particles;
 * FP64: 32, 64, 96, 128), each persistent grid of 1 .. max resident CTAs per SM of
 * the fused kernel and, for FP32 handles with the lagged-B order and without
 * the full F_P, each scatter layout of its P2G (RD_SCATTER_*: how the 64
 * stencil nodes of a record map to a warp's lanes); keeps the fastest and
 * restores the state (the next step re-sorts and rebuilds the grid).
 * Allocates a copy of the particle state for its duration.
 * cache_path (may be NULL): a text file of earlier results, one per line
 * "key<TAB>particles_per_item ctas_per_sm scatter ms_per_step", keyed by
 * rd_tune_key (device architecture and SM count, precision, step options,
 * scene count, particle count and grid size).  When the file holds the
 * handle's key (the last such line counts), that choice is applied without
 * timing anything (from_cache = 1); otherwise the search runs and its result
 * is appended to the file. */
enum { RD_SCATTER_LANE_PAIRS = 0,   /* a lane owns 2 nodes of one record; 32 lanes per record */
       RD_SCATTER_RECORD_PAIRS = 1  /* a lane owns a 4-node column; the half-warps take 2 records of a run */ };
typedef struct rd_tune_result {
    int32_t particles_per_item; /* chosen work-item size */
    int32_t ctas_per_sm;        /* chosen persistent CTAs per SM */
    double ms_per_step;         /* measured for the chosen point (or as cached) */
    int32_t trials;             /* points timed (0 from the cache) */
    int32_t scatter;            /* chosen RD_SCATTER_* */
    int32_t from_cache;         /* 1: taken from cache_path */
} rd_tune_result;
rd_status rd_autotune(rd_handle* h, double dt, int32_t steps, const char* cache_path, rd_tune_result* result);
/* Every point the last rd_autotune timed, in the order timed (up to cap);
 * *count receives how many there were. */
typedef struct rd_tune_trial {
    int32_t particles_per_item, ctas_per_sm, scatter;
    double ms_per_step;
} rd_tune_trial;
rd_status rd_tune_trials(rd_handle* h, rd_tune_trial* out, int32_t cap, int32_t* count);
/* The handle's cache key (NUL-terminated, no tabs or newlines). */
rd_status rd_tune_key(rd_handle* h, char* buf, size_t len);
/* The tuning cache file alone, no device involved: the last line of `path`
 * with this key (*found = 0 when none, or when the file does not exist), and
 * appending one line.  Malformed lines are skipped. */
rd_status rd_tune_cache_get(const char* path, const char* key, rd_tune_result* out, int32_t* found);
rd_status rd_tune_cache_put(const char* path, const char* key, const rd_tune_result* result);
/* Sets the point by hand (0 = default: the largest item, max resident CTAs;
 * scatter RD_SCATTER_*, RD_SCATTER_LANE_PAIRS where it is the only layout). */
rd_status rd_set_tuning(rd_handle* h, int32_t particles_per_item, int32_t ctas_per_sm, int32_t scatter);
rd_status rd_get_tuning(rd_handle* h, int32_t* particles_per_item, int32_t* ctas_per_sm, int32_t* scatter);

/* ---- Reverse mode: gradients of a rollout ----
 * No counterpart in the reference.  rd_adjoint_record runs `steps` steps of
 * rd_step from the current state (of every scene of a batch) and keeps a copy
 * of the state every `checkpoint_every` steps; the handle then holds the final
 * state.  rd_adjoint_backward takes dL/dx (and optionally dL/dv) of the final
 * state, n x 3 in original particle order (scene order for a batch), and
 * returns dL/dv of the recorded start state and, per scene, dL/dE, dL/dnu,
 * dL/dtheta_c, dL/dtheta_s.  It recomputes each segment from its checkpoint
 * (memory: the checkpoints plus one segment of states and grids) and runs
 * hand-written adjoint kernels of every stage per step: advection and the
 * position clamp, G2P (as a scatter), the plastic SVD split (with the clamp's
 * subgradient), the grid update and P2G with the fixed-corotated stress (as a
 * gather).  Volumes and masses are constants; the lagged-B step only
 * (RD_NOT_SUPPORTED otherwise).  The handle keeps the final state afterwards.
 * Any call that changes the state in between invalidates the record. */
typedef struct rd_grads {
    void* v0;         /* n x 3 element type, or NULL; host or device per `where` */
    double* E;        /* one per scene, host, or NULL */
    double* nu;
    double* theta_c;
    double* theta_s;
} rd_grads;
rd_status rd_adjoint_record(rd_handle* h, double dt, int32_t steps, int32_t checkpoint_every);
rd_status rd_adjoint_backward(rd_handle* h, const void* grad_x, const void* grad_v, int where, rd_grads* grads);

/* ---- Implicit time integration (timeIntegration, material_point_method.cpp:212-233) ----
 * The reference writes an implicit grid update that its driver never calls:
 * the grid velocities v of the cells with mass are replaced by the minimiser of
 *   E(v) = sum_i 1/2 m_i |v_i - v*_i|^2 + sum_p V_p Psi(Fhat_p(v), F_P,p)
 * (Energy and ElasticPotential, :160-190), v* = the grid velocities at the
 * call, Fhat_p = (I + dt sum_i v_i grad w_ip^T) F_E,p, Psi = mu ||Fhat - R||^2 +
 * lambda / 2 (J - 1)^2 with R the polar rotation of Fhat (:192-210) and
 * mu = mu0 e, lambda = lambda0 e, where the reference's e is exp(xi * 1 - det F_P)
 * (RD_HARDENING_REFERENCE; RD_HARDENING_INTENDED is exp(xi (1 - det F_P))).  The
 * reference minimises with L-BFGS (history 8, backtracking line search with
 * factor 0.7 and Armijo constant 1e-4, at most 50 iterations, stopping when the
 * gradient's or the step's norm falls below 1e-2) on finite-difference
 * gradients; here the same L-BFGS runs on the device with the analytic gradient
 *   dE/dv_i = m_i (v_i - v*_i) + dt sum_p V_p P_p F_E,p^T grad w_ip,
 *   P = 2 mu (Fhat - R) + lambda (J - 1) J Fhat^-T.
 * It acts on the stage-mode grid: call it after RD_STAGE_RASTERIZE (and the
 * force and grid-velocity stages, as the step order wants); single-scene
 * handles.  opts NULL: the reference's settings and constants (mu0 = lambda0 =
 * 1, xi = 10, material_point_method.hpp:213-216).  Allocates its vectors on
 * the first call (3 reals per cell with mass, times 2 * history + 6). */
enum { RD_HARDENING_REFERENCE = 0, RD_HARDENING_INTENDED = 1 };
typedef struct rd_implicit_opts {
    int32_t max_iters;    /* L-BFGS iterations (50) */
    int32_t history;      /* correction pairs kept, 1..32 (8) */
    double grad_tol;      /* stop when |gradient| < grad_tol (1e-2) ... */
    double step_tol;      /* ... or when |x_k+1 - x_k| < step_tol (1e-2) */
    double mu0, lambda0, xi;
    int32_t hardening;    /* RD_HARDENING_* */
    int32_t ls_max_iters; /* backtracking steps before the line search fails (200) */
} rd_implicit_opts;
void rd_default_implicit_opts(rd_implicit_opts* opts);
typedef struct rd_implicit_result {
    int32_t iterations;   /* L-BFGS iterations taken */
    int32_t evaluations;  /* energy evaluations (with or without gradient) */
    int32_t converged;    /* 1: a tolerance was met; 0: max_iters; -1: the line search failed */
    int32_t unknowns;     /* 3 x cells with mass */
    double energy_start, energy; /* E(v*) and E at the result */
    double grad_norm;     /* |dE/dv| at the result */
} rd_implicit_result;
rd_status rd_time_integration(rd_handle* h, double dt, const rd_implicit_opts* opts, rd_implicit_result* result);
/* E(v) and, when grad is given, dE/dv at the velocity field vel (cells x 3,
 * dense, index i*MAX_J*MAX_K + j*MAX_K + k; only cells with mass count) against
 * the current stage-mode grid (masses, v*); grad is written densely, zero where
 * there is no mass.  Host or device arrays per `where`; the grid is left as it
 * was. */
rd_status rd_implicit_energy(rd_handle* h, double dt, const rd_implicit_opts* opts, const void* vel, void* grad,
                             int where, double* energy);

/* Rasterize without allocating.  No counterpart in the reference: it exists for
 * callers that cannot allocate GPU memory - an engine that has handed the whole
 * device to its own pool allocator, or a real-time frame loop where
 * cudaMalloc's device-wide synchronisation and unbounded latency (or an
 * out-of-memory failure halfway through a frame) cannot be afforded - and
 * therefore cannot create an rd_handle, which owns its buffers.
 *
 * Computes what rasterizeParticlesToGrid (material_point_method.cpp:94-129)
 * accumulates before its velocity division: per grid node the mass sum of
 * w m_p and the momentum sum of w m_p (v_p + B_p D^-1 (x_i - x_p)), written as
 * float4 (m, p_x, p_y, p_z) to grid_out (max_i*max_j*max_k float4, device
 * memory, overwritten; index i*max_j*max_k + j*max_k + k).  in holds device
 * arrays of n = params->num_particles particles: x (n x 3), v (n x 3), mass (n)
 * required, B (n x 9) optional (NULL = 0); other fields are ignored.  FP32 only
 * (RD_NOT_SUPPORTED otherwise).  Work is queued on `stream` (a cudaStream_t;
 * NULL = the legacy default stream); the call returns without waiting.
 *
 * Limits: at most 65,536 particles and 262,144 grid nodes (and 4x4x4-cell
 * blocks x 64 <= 262,144, e.g. a 64^3 grid); larger sizes return RD_TOO_LARGE
 * before anything is queued.  The sort scratch is one fixed device array of
 * about 2.6 MB inside this library, held by every GPU that loads it until the
 * process exits; the call makes no device allocation of its own.  The first
 * call on a device looks up that array's device address (once per device, with
 * the device current); make that first call before any stream capture.  All
 * calls share the array and it keeps the previous call's contents (the call
 * clears what must start at zero), so calls whose work overlaps on the GPU -
 * on different streams, or from different threads - race and must be
 * serialised by the caller.
 *
 * Status: the call returns RD_CUDA_ERROR when a launch fails, and also, queuing
 * nothing, when a CUDA error left by earlier work is pending (it is not
 * consumed).  What the kernels find is recorded in the shared array's flags
 * word, cleared at the start of every call: RD_FLAG_OUT_OF_DOMAIN when a
 * particle's stencil reaches past the grid (those nodes are dropped) and
 * RD_FLAG_BAD_WORK when a particle lies more than a cell outside the grid (the
 * particle is dropped) or the work list overflowed.  Read it with
 * rd_rasterize_noalloc_flags once the stream has been synchronised. */
rd_status rd_rasterize_noalloc(const rd_params* params, const rd_particles* in, float* grid_out, void* stream);
/* The flags word of the last rd_rasterize_noalloc on the current device (0 if
 * none ran there): a blocking 4-byte device-to-host copy, made after the
 * caller has synchronised the stream of that call.  Allocates nothing. */
rd_status rd_rasterize_noalloc_flags(uint32_t* flags);

#ifdef __cplusplus
}
#endif
#endif /* RD_MPM_H */
