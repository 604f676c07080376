/*
 * sph_cuda.h -- C ABI of the GB300 (sm_103a) SPH grid step.
 *
 * This is the drop-in boundary for the uniform-grid SPH step that the reference's
 * CGPUParticleSimulator runs (src/CGPUParticleSimulator.cpp:57-173 with
 * src/CGPUBaseParticleSimulator.cpp:59-97). A CBaseParticleSimulator subclass
 * (include/CBaseParticleSimulator.h:29-110) calls these functions in place of the
 * OpenCL wrapper and kernels. Plain C types only: host pointers, sizes, status codes.
 *
 * Conventions
 *  - Every function returning int returns SPH_OK (0) or a negative SPH_ERR_* code and
 *    never throws; the message of the last failure is sph_last_error(ctx). This replaces
 *    the reference's CLException (src/CLWrapper.cpp:115-121) that
 *    CGPUBaseParticleSimulator::step catches (src/CGPUBaseParticleSimulator.cpp:28-37).
 *  - One context belongs to one host thread at a time; it owns one CUDA stream on one
 *    device. Calls are stream-ordered; download/stat functions synchronise that stream.
 *  - Arrays of particles are scene-major and, within a scene, in id order (ids are
 *    0..n-1 in upload order, then appended particles), float xyz triples.
 *  - A context holds 1..n independent scenes (a batch); every pass covers all scenes
 *    in one launch.
 */
#ifndef SPH_CUDA_H
#define SPH_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SPH_OK 0
#define SPH_ERR_ARG (-1)         /* invalid argument */
#define SPH_ERR_CUDA (-2)        /* CUDA runtime or launch error */
#define SPH_ERR_CAPACITY (-3)    /* more particles than the scene's capacity */
#define SPH_ERR_STATE (-4)       /* call out of order (e.g. step before upload) */
#define SPH_ERR_NOMEM (-5)       /* device or host allocation failed */
#define SPH_ERR_UNSUPPORTED (-6) /* option not available in this build */
#define SPH_ERR_DEVICE (-7)      /* a kernel reported an error status */

/* Arithmetic of the step. */
#define SPH_PLAIN_F32 0 /* all-FP32 state and arithmetic */
#define SPH_F64 1       /* the same method in FP64 (reference run) */
#define SPH_MIXED 2     /* 16-bit cell-relative positions, FP16 velocities, Kahan densities */

/* sph_params.flags */
#define SPH_FLAG_PROFILE 1u    /* record per-pass CUDA-event times (sph_pass_times) */
#define SPH_FLAG_RECORD_ACC 2u /* keep each step's accelerations for sph_download */
/* Density and force passes over every particle of a scene instead of the 27 grid cells: the
 * reference's brute-force simulator (CGPUBruteParticleSimulator, sph_brute.cl:9-57). Visited
 * in the sorted order, the accepted neighbours and their order are the grid form's, so the
 * result is bit-identical to the grid form: an independent check of the grid, for scenes of
 * at most 131,072 particles (SPH_ERR_CAPACITY beyond). Not with SPH_MIXED; no launch variants. */
#define SPH_FLAG_ALL_PAIRS 4u

typedef struct sph_ctx sph_ctx;

/* Physical and numerical parameters; sph_params_default fills the reference's values:
 * h, mass, gas stiffness, rest density, viscosity from include/CParticle.h:80-84;
 * dt = 0.01 from src/CBaseParticleSimulator.cpp:7; gravity (0, -9.80665, 0) from
 * include/CBaseParticleSimulator.h:19; wall constants 10000 / -0.9 from
 * include/CCollisionGeometry.h:20-21 and the 0.01 particle radius of
 * src/CCollisionGeometry.cpp:124. */
typedef struct sph_params {
    uint32_t struct_size; /* sizeof(sph_params) */
    float h;
    float mass;
    float gas_stiffness;
    float rest_density;
    float viscosity;
    float dt;
    float gravity[3];
    float wall_k;
    float wall_damping;
    float wall_radius;
    int32_t precision; /* SPH_PLAIN_F32, SPH_F64 or SPH_MIXED */
    uint32_t flags;    /* SPH_FLAG_* */
    int32_t device;    /* CUDA device ordinal */
} sph_params;

/* One scene of a batch: an axis-aligned box centred on the origin (walls at +-box/2,
 * as CCollisionGeometry builds them from the grid cuboid), a particle capacity, and
 * optional axis-aligned box obstacles (min xyz then max xyz, 6 floats each) that push
 * particles out with the wall spring and damping constants. */
typedef struct sph_scene_desc {
    float box[3];
    uint32_t max_particles;
    uint32_t n_obstacles;
    const float *obstacles; /* 6 * n_obstacles floats, may be NULL when n_obstacles == 0 */
} sph_scene_desc;

/* Fills the reference's constants (see sph_params). */
void sph_params_default(sph_params *p);

/* One scene; replaces the CGPUParticleSimulator constructor + setupKernels
 * (src/CGPUParticleSimulator.cpp:3-55). box: 3 extents (the reference's scalar boxSize
 * is box = {s, s, s}). */
int sph_create(const sph_params *p, const float box[3], uint32_t max_particles, sph_ctx **out);

/* n_scenes independent scenes stepped together (no reference counterpart; one launch
 * per pass over all scenes). */
int sph_batch_create(const sph_params *p, uint32_t n_scenes, const sph_scene_desc *scenes, sph_ctx **out);

/* Device memory a context with these parameters and scenes would allocate (one pool), without
 * creating it or touching a GPU. The optional handoff buffers (24 bytes per particle of
 * capacity, allocated by the first sph_handoff_async or sph_export_positions) are not
 * included. Creating a context fails with SPH_ERR_NOMEM, before any device work, when this
 * exceeds the environment variable SPH_DEVICE_MEMORY_LIMIT (bytes; unset or 0 = no limit). */
int sph_memory_required(const sph_params *params, uint32_t n_scenes, const sph_scene_desc *scenes, uint64_t *bytes);

/* Checked builds (libsph_gb300_checked.so, compiled with SPH_CHECKED). Every counting-sort
 * scatter target, neighbour row range, neighbour index from the masks and id-ordered target is
 * bounds-checked on the device; a failed check skips the access and sets a flag. Every array
 * of the context's pool is followed by a guard region of known bytes. This call waits for the
 * context's work and returns the flags raised since the last call (clearing them), plus
 * SPH_CHECK_CANARY if a guard region changed; 0 = clean. The other library returns
 * SPH_ERR_UNSUPPORTED. */
#define SPH_CHECK_SORT 1u
#define SPH_CHECK_ROW 2u
#define SPH_CHECK_NEIGHBOUR 4u
#define SPH_CHECK_EGRESS 8u
#define SPH_CHECK_CANARY 16u
int sph_debug_check(sph_ctx *ctx, uint32_t *flags);

void sph_destroy(sph_ctx *ctx);

/* Last error message of ctx (or of the last failed create when ctx is NULL). */
const char *sph_last_error(const sph_ctx *ctx);

/* Replaces CGPUBaseParticleSimulator::getSelectedDevice (src/CGPUBaseParticleSimulator.cpp:17-20). */
const char *sph_device_name(const sph_ctx *ctx);

/* The CUDA stream (a cudaStream_t) every call of ctx launches on, for callers that order
 * their own work or record their own events against the step (no reference counterpart:
 * CLWrapper keeps its command queue private, src/CLWrapper.cpp:3-13). The step's kernels are
 * chained launches (programmatic dependent launch): each waits for the complete work before
 * it in the stream, so work a caller enqueues between two calls is ordered as usual. */
void *sph_stream(const sph_ctx *ctx);

/* Replaces every scene's particles: counts[s] particles for scene s, concatenated
 * scene-major; vel may be NULL (zero). Ids restart at 0 in each scene. Mirrors
 * setupScene's addParticle loop (src/CBaseParticleSimulator.cpp:38-74) followed by the
 * first H2D copy of CGPUParticleSimulator::updateGrid (src/CGPUParticleSimulator.cpp:59).
 * Pinned (page-locked) arrays are read by the ingest kernel over the host link, without a
 * staging copy; the call then returns before they are read, so keep them unchanged until
 * the next synchronising call (a download, or sph_stream's work done). Other host memory is
 * copied before the call returns. */
int sph_upload(sph_ctx *ctx, const float *xyz, const float *vel, const uint32_t *counts);

/* Appends n particles to one scene (emitters, e.g. the FOUNTAIN scenario's
 * generateParticles, src/CBaseParticleSimulator.cpp:187-210). */
int sph_append(sph_ctx *ctx, uint32_t scene, const float *xyz, const float *vel, uint32_t n);

/* The disc emitter on the device: appends n particles to a scene like sph_append, generated
 * on the GPU (no host arrays, no host-to-device copy, no host synchronisation). Particle k of
 * emission step `step` lies on the disc of `radius` around center in the plane y = center[1],
 * with velocity (0, speed, 0) + sigma * N(0, I). The particles are bit-identical to
 * sph_scene_fountain_emit's with the same arguments. Generalises the reference's FOUNTAIN
 * source (src/CBaseParticleSimulator.cpp:187-210, 7 particles per step). Same state and
 * capacity errors as sph_append. */
int sph_emit_fountain(sph_ctx *ctx, uint32_t scene, uint64_t seed, uint32_t step, uint32_t n, const float center[3],
                      float radius, float speed, float sigma);

/* CGPUBaseParticleSimulator::setGravityVector (src/CGPUBaseParticleSimulator.cpp:11-15).
 * scene < 0 sets every scene. */
int sph_set_gravity(sph_ctx *ctx, int32_t scene, const float g[3]);

/* nsteps steps of CBaseParticleSimulator::step (src/CBaseParticleSimulator.cpp:116-144):
 * grid build, density/pressure, forces + walls + integration, all on the device. */
int sph_step(sph_ctx *ctx, int32_t nsteps);

/* The three device passes of one step, for the reference's pass-by-pass interface
 * (include/CBaseParticleSimulator.h:92-96): updateGrid (src/CGPUParticleSimulator.cpp:57-139),
 * updateDensityPressure (:141-155), and updateForces (:157-173) fused with
 * updateCollisions and integrate (src/CGPUBaseParticleSimulator.cpp:59-97).
 * Must be called in this order. */
int sph_pass_grid(sph_ctx *ctx);
int sph_pass_density(sph_ctx *ctx);
int sph_pass_forces(sph_ctx *ctx);

/* Milliseconds of the latest passes (grid, density, forces, collisions, integrate), the
 * fields of sProfilingEvent (include/SProfilingEvent.h:8-31). Needs SPH_FLAG_PROFILE; with it
 * each sph_pass_* call waits for its own work, so its time is here when the call returns (the
 * reference's profiled passes each return their own duration). Collisions and integrate are
 * fused into forces and report 0. */
int sph_pass_times(sph_ctx *ctx, double ms[5]);

/* Launch variants of the two neighbour passes. Every variant computes the same bits; only
 * the speed differs (no reference counterpart: the OpenCL kernels have fixed launch shapes,
 * src/CGPUParticleSimulator.cpp:141-173).
 *   density: 0 = one particle per thread; 1, 2, 4 = branchless blocked walk with that many
 *            consecutive sorted particles per thread sharing one candidate scan
 *   forces:  0 = pair terms inside the candidate loop; 1, 2 = accepted neighbours compacted
 *            into a per-thread list of 32 / 64 entries in shared memory, pair terms after;
 *            3..11 = the density pass records each particle's accepted neighbours as bit masks
 *            per row and the force pass visits only those (density_variant is then unused):
 *            3 and 4 one neighbour per iteration (4 capped at 64 registers); 5 and 6 two per
 *            iteration (5 capped at 64); 7 is 6 reading each neighbour from one packed 32-byte
 *            force record written by the density pass; 8 and 9 are 7 capped at 48 and 40
 *            registers (5 and 6 blocks of 256 per SM); 10 and 11 are 9 and 8 launched in
 *            blocks of 128 threads (12 and 10 per SM). SPH_ERR_ARG for other numbers.
 * The mixed form has one density pass (density_variant 0) and force variants 0..3: blocks of
 * 128 threads at up to 64 or 48 registers, blocks of 256 with no cap or 48 registers. On cells
 * of h/2 (sph_set_cell_multiple) the plain form runs density 0 with force variants 7..11. */
int sph_set_variant(sph_ctx *ctx, int32_t density_variant, int32_t forces_variant);
int sph_get_variant(const sph_ctx *ctx, int32_t out[2]);

/* Cell multiple of the step's grid: 1 = the reference's cells of size h and 27-cell stencil
 * (src/CBaseParticleSimulator.cpp:27-31, resources/kernels/sph_grid.cl:124-170); 2 = cells of
 * h/2 with a 125-cell stencil (5 rows of 5 cells in each of 5 planes), which covers 15.6 h^3
 * around a particle instead of 27 h^3, so the density pass tests about 42% fewer candidates.
 * The method and its results are the same within rounding (the candidates are summed in another
 * order). The plain FP32 and mixed forms only (SPH_ERR_UNSUPPORTED for FP64 and all-pairs);
 * between steps only (SPH_ERR_STATE between passes). sph_get_grid still reports the reference's
 * grid of cells of size h. sph_get_cell_multiple returns the current multiple (or SPH_ERR_ARG).
 * The autotuner chooses the multiple with the variants, unless it was set here. */
int sph_set_cell_multiple(sph_ctx *ctx, int32_t cell_multiple);
int sph_get_cell_multiple(const sph_ctx *ctx);

/* Autotuner: one step in which every (cell multiple, density, forces) choice is timed on the
 * current state (per cell multiple the grid pass once, then both neighbour passes re-run from the
 * same sorted inputs per variant pair), the fastest grid + density + forces is kept, and the
 * choice is written to the cache file (SPH_TUNE_CACHE, else $HOME/.cache/sph_gb300/tune.txt)
 * under the device name, precision and particle-count bucket (floor(log2 n)). sph_upload applies
 * a cached choice for its bucket. The simulation advances by exactly one step; reps = timed
 * repetitions per variant (>= 1). */
int sph_autotune(sph_ctx *ctx, int32_t reps);

/* Online tuning of the force variant for a state that changes over a run (a collapsing dam
 * break packs ~4x more neighbours per particle after a few hundred steps than at the start,
 * and the fastest variant changes with it). Every `period` steps (sph_step or the pass
 * calls), one real step runs with each of the record-reading force variants 7, 9, 10 and 11
 * (the mixed form: its variants 0..3), timed with events on the context's stream (one host
 * synchronisation per trial step), and the fastest is kept until the next trial. All of them
 * compute the same bits, so the results do not depend on the choice; the cell multiple stays.
 * Applies while the current force variant is mask-driven (3..11, or any mixed variant).
 * period 0 turns it off (the default); otherwise period >= 4. Not for all-pairs contexts
 * (SPH_ERR_STATE). */
int sph_set_online_tuning(sph_ctx *ctx, int32_t period);

/* Particle count of every scene (n_scenes entries). */
int sph_get_counts(const sph_ctx *ctx, uint32_t *counts);
uint32_t sph_num_scenes(const sph_ctx *ctx);
uint64_t sph_num_particles(const sph_ctx *ctx);
/* Grid resolution of one scene: (int) ceil(box / h) per axis (src/CBaseParticleSimulator.cpp:27-31). */
int sph_get_resolution(const sph_ctx *ctx, uint32_t scene, int32_t res[3]);

/* State after the last call, scene-major and in id order. Any pointer may be NULL.
 * rho / p are the densities and pressures of the last density pass; acc needs
 * SPH_FLAG_RECORD_ACC. Replaces the readback of CGPUBaseParticleSimulator::integrate
 * (src/CGPUBaseParticleSimulator.cpp:84-91). Plain FP32 positions and velocities alone,
 * into 16-byte-aligned pinned arrays, are written there by one gather kernel over the host
 * link (no staging copy); the call returns when the data is in place either way. */
int sph_download(sph_ctx *ctx, float *xyz, float *vel, float *rho, float *p, float *acc);
/* Same in double, for SPH_F64 contexts. */
int sph_download_f64(sph_ctx *ctx, double *xyz, double *vel, double *rho, double *p, double *acc);

/* Front-end handoff without a synchronising download. The reference reads the whole particle
 * buffer back and updates every CParticle after each step (CGPUBaseParticleSimulator::integrate,
 * src/CGPUBaseParticleSimulator.cpp:76-97). sph_handoff_async queues, after the work already
 * queued on the context's stream, the id-ordered float3 positions (and velocities if vel is
 * not NULL) of every particle, and copies them to xyz/vel on a second stream, so that the
 * steps queued next overlap the copy. Use pinned host memory (cudaHostAlloc) for an
 * asynchronous copy. The arrays must stay valid until sph_handoff_ready returns 1 or
 * sph_handoff_wait returns. A handoff waits for the previous handoff's copy before it
 * rewrites the handoff buffers (3 floats x 2 x capacity, allocated by the first call).
 * FP64 and mixed contexts deliver their state rounded to float. */
int sph_handoff_async(sph_ctx *ctx, float *xyz, float *vel);
/* 1 once the last handoff's copy has landed (or none was queued), 0 while it is in flight. */
int sph_handoff_ready(sph_ctx *ctx);
/* Blocks until the last handoff's copy has landed. */
int sph_handoff_wait(sph_ctx *ctx);
/* The same id-ordered float3 positions (and velocities if dev_vel is not NULL) into device
 * arrays of the caller (3 floats per particle each), e.g. a renderer's vertex buffer mapped
 * into CUDA. Queued on the context's stream; consumer_stream (a cudaStream_t, or NULL) is made
 * to wait for it. */
int sph_export_positions(sph_ctx *ctx, float *dev_xyz, float *dev_vel, void *consumer_stream);
/* Headless point splat of one scene, for a front end without a graphics API: an orthographic
 * view along `axis` (0 = x, 1 = y, 2 = z) onto a width x height image covering the box face
 * spanned by the other two axes in increasing order (u, v); row-major, row 0 at the smallest
 * v. A particle lands in pixel floor((p + box/2) * (pixels / box)) per image axis (float,
 * clamped to the image). dev_count (width*height, may be NULL): particles per pixel.
 * dev_depth (width*height floats, may be NULL): the smallest coordinate along axis in the
 * pixel (the particle nearest a viewer on the negative side), +inf where there is none.
 * Deterministic. Queued on the context's stream; consumer_stream (or NULL) waits for it. */
int sph_splat(sph_ctx *ctx, uint32_t scene, int32_t axis, uint32_t width, uint32_t height, uint32_t *dev_count,
              float *dev_depth, void *consumer_stream);

/* The grid of the last grid pass: the cell of every particle (scene-major, id order,
 * cell index local to its scene: x + y*X + z*X*Y), the count of every cell (scene-major),
 * and the ids of each scene's particles in sorted order, ascending (cell, id). Any
 * pointer may be NULL. */
int sph_get_grid(sph_ctx *ctx, uint32_t *cell_of_particle, uint32_t *cell_counts, uint32_t *sorted_ids);

/* FP64 reductions of one scene over the current state: out[0] mass, out[1..3] momentum,
 * out[4] kinetic energy, out[5] mean density, out[6] max density, out[7] particle count. */
int sph_stats(sph_ctx *ctx, uint32_t scene, double out[8]);

/* Grid build that allocates no device memory. No counterpart in the reference: it exists for
 * callers that cannot call cudaMalloc once they are running, such as a host application whose
 * GPU memory is already owned by its own pool allocator, or a per-frame real-time callback
 * where an allocation's implicit device synchronisation would stall the frame.
 * Every array is the caller's device memory:
 *   xyz        3 floats per particle, id order (n particles)
 *   out_cell   n: cell of each particle, x + y*X + z*X*Y with (X, Y, Z) = ceil(box / h)
 *   out_start  X*Y*Z + 1: cell starts, out_start[X*Y*Z] = n
 *   out_order  n: particle ids in ascending (cell, id) order
 * The cells and order equal the grid that sph_pass_grid builds for the same positions and h.
 * Working memory is one fixed device array of about 8 MiB inside this library, held by every
 * GPU that has run a call until the process exits, so n and X*Y*Z are each limited to 1,048,576;
 * larger requests return SPH_ERR_CAPACITY, and a non-finite box or h SPH_ERR_ARG. The first call
 * on a device is its setup: CUDA creates the array there when the library's device code is
 * loaded (under lazy loading, at that call), and the call looks up the array's device address.
 * Make it at the caller's setup, before its pool allocator takes the GPU's memory and before any
 * stream capture; later calls allocate nothing. cudaDeviceReset between calls is not supported
 * (the address found at setup would be stale). All calls share the array: calls whose work
 * overlaps on the GPU race on it and must not be issued. Work is queued on stream (a
 * cudaStream_t; NULL = the legacy default stream); returns a status code only. */
int sph_grid_build_noalloc(const float *xyz, uint32_t n, const float box[3], float h, uint32_t *out_cell,
                           uint32_t *out_start, uint32_t *out_order, void *stream);

/* ---- scene generators (host only, no device needed) ---- */

/* The reference's DAM_BREAK lattice for a cubic box (src/CBaseParticleSimulator.cpp:38-58).
 * Returns the particle count; writes at most cap particles. */
int64_t sph_scene_reference_dam_break(float box, float *xyz, uint64_t cap);

/* A dims[0] x dims[1] x dims[2] lattice of the given spacing anchored at the box's min
 * corner (-box/2), each coordinate jittered by uniform [-jitter, +jitter) * spacing from a
 * seeded splitmix64 stream; particles ordered y outer, x, z inner like the reference. */
int sph_scene_lattice(const uint32_t dims[3], const float box[3], float spacing, float jitter, uint64_t seed, float *xyz);

/* Seeded plan of a batch of dam-break scenes: counts log-uniform in [nmin, nmax], aspect
 * per axis uniform in [amin, amax]; writes lattice dims (3 per scene) and boxes (3 per
 * scene) that keep the fill fraction of the 20^3-lattice, 1.0 x 1.0 x 0.5 m scene. */
int sph_scene_batch_plan(uint32_t n_scenes, uint64_t seed, uint32_t nmin, uint32_t nmax, float amin, float amax,
                         uint32_t *dims, float *boxes);

/* Disc emitter: n particles on a disc of the given radius in the y = center[1] plane,
 * velocity (0, speed, 0) plus N(0, sigma^2) per component. Particle k draws from its own
 * stream seeded by (seed, step, k); sph_emit_fountain generates the same bits on the device. */
int sph_scene_fountain_emit(uint64_t seed, uint32_t step, uint32_t n, const float center[3], float radius, float speed,
                            float sigma, float *xyz, float *vel);

#ifdef __cplusplus
}
#endif

#endif /* SPH_CUDA_H */
