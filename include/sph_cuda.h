/*
 * sph_cuda.h -- libsph_cuda, device-resident fast API.
 *
 * A GB300 (sm_103a) implementation of one TinySPH compute rank's step
 * (fluid.c:270-349): gravity, viscosity impulses, position prediction,
 * uniform-grid neighbour build, double density relaxation with near
 * density, box and mover collision, velocity update.  The particle state
 * lives on the GPU in structure-of-arrays form, kept sorted by
 * (grid cell, particle id); the host keeps the reference's structs.
 *
 * Replaces, for a single-device domain, the compute rank's loop body
 * fluid.c:273-348 (with the MPI halo/migration calls of fluid.c:310-349
 * gone: one domain, no neighbours): the caller creates a handle and uploads
 * its particles once, then calls sph_cuda_step where the loop body was.
 *
 * Conventions
 *  - Every call returns an sph_status (0 = SPH_OK).  On failure
 *    sph_cuda_last_error() returns a message (per host thread).
 *  - A handle is used by one host thread at a time; different handles are
 *    independent (no global state on this API).
 *  - Work is queued on the handle's stream.  Calls that fill host buffers
 *    (download, pack, lists, probes, diagnostics, counters) return only when
 *    the data is in host memory; sph_cuda_step returns once queued.
 *  - Particle "id" is the index in the caller's pointer array
 *    (fluid_particle::id, fluid.h:69); outputs are indexed by id.
 */
#ifndef SPH_CUDA_H
#define SPH_CUDA_H

#include <stddef.h>

#include "sph_types.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sph_cuda sph_cuda_t;

enum sph_status {
    SPH_OK = 0,
    SPH_ERR_INVALID = 1,     /* bad argument (null pointer, n out of range, bad grid) */
    SPH_ERR_CUDA = 2,        /* a CUDA runtime call failed (message has the error) */
    SPH_ERR_ALLOC = 3,       /* device or pinned-host allocation failed */
    SPH_ERR_CAPACITY = 4,    /* n above the handle's capacity or output buffer too small */
    SPH_ERR_STATE = 5,       /* e.g. step before upload */
    SPH_ERR_UNSUPPORTED = 6  /* e.g. halo particles on a single-device domain */
};

/* Device-side event counters, accumulated since the last upload.  None of
 * these events trap or stop the step; the reference drops the same cases
 * silently (hash.c:160-165, 188, 223) or has undefined behaviour. */
typedef struct sph_cuda_counters {
    unsigned long long steps;          /* steps run since the last upload */
    unsigned long long out_of_grid;    /* particle-builds whose cell key fell outside the
                                          grid (negative/NaN coordinate or y == max_y;
                                          undefined behaviour in hash.c:40-44): such a
                                          particle gets no neighbours */
    unsigned long long bucket_overflow;/* particle-builds beyond max_bucket_size in their
                                          cell: dropped from the neighbour search, as
                                          hash.c:160-165 drops them */
    unsigned int max_cell_occupancy;   /* largest cell population seen */
    unsigned int list_cap_risk;        /* nonzero if some half list could have exceeded
                                          max_neighbors (hash.c:188, 223); the cap is not
                                          reproduced: the gathers search the full stencil,
                                          so such a particle keeps neighbours the
                                          reference would have dropped */
} sph_cuda_counters;

/* Creates a handle for up to max_particles particles.
 *   params:   tunable_params.smoothing_radius is h (fluid.c:159); the other
 *             tunables are passed again to every step.
 *   boundary: the global box (fluid.c:118-127); min_x/min_y should be 0 as in
 *             the reference (fluid.c:117: "assumes in various spots min is 0").
 *   grid:     spacing, size_x, size_y, max_bucket_size, max_neighbors as the
 *             reference sets them (fluid.c:173-176, 214-215); its pointers are
 *             ignored (the device owns its own cell lists).
 * Replaces the host allocations of fluid.c:178-235. */
int sph_cuda_create(sph_cuda_t **out, const param *params, const AABB_t *boundary,
                    const neighbor_grid_t *grid, int max_particles);

/* One scene of an ensemble: an independent domain, as one compute rank's
 * set-up would describe it (fluid.c:88-176, 214-215). */
typedef struct sph_scene_desc {
    tunable_parameters params;   /* the scene's tunables (smoothing_radius = its h) */
    AABB_t boundary;             /* its box */
    float spacing;               /* its neighbour-grid spacing */
    unsigned int size_x, size_y; /* its grid dimensions */
    int n;                       /* its particle count */
} sph_scene_desc;

/* No counterpart in the reference (one rank runs one domain there).  Creates
 * a handle holding `nscenes` independent scenes that advance together: every
 * kernel of a step covers the particles of all scenes, each particle using
 * its own scene's grid and tunables.  Particles are uploaded and downloaded
 * concatenated in scene order (scene s holds ids [sum of n of scenes < s,
 * + n_s)); uploads must pass exactly the total count.  max_bucket and
 * max_neighbors apply to every scene.  Each scene's trajectory is identical,
 * bit for bit, to that scene run alone. */
int sph_cuda_create_ensemble(sph_cuda_t **out, const sph_scene_desc *scenes, int nscenes,
                             int max_bucket, int max_neighbors);

/* ---- on-device scene initialisation ---- */

/* A block of particles on a square lattice, generated on the GPU (replaces
 * the host loops of constructFluidVolume / initParticles, geometry.c:29-67,
 * fluid.c:747-768, for the synthetic scenes): particle k of the block sits
 * at row k / cols, column k % cols,
 *   x = float((x0 + column * spacing) + (2 u(2k) - 1) * jitter),
 *   y = float((y0 + row * spacing) + (2 u(2k + 1) - 1) * jitter),
 * with u(c) = top 53 bits of splitmix64(seed + (counter0 + c + 1) * golden)
 * as a double in [0, 1), all in IEEE double arithmetic without fused
 * multiply-adds, and velocity 0. */
typedef struct sph_lattice_block {
    int n;                       /* particles of the block */
    int cols;                    /* particles per lattice row */
    double x0, y0;               /* lower-left lattice point */
    double spacing;              /* lattice spacing */
    double jitter;               /* uniform jitter half-width per axis */
    unsigned long long seed;     /* splitmix64 seed */
    unsigned long long counter0; /* first counter of the block */
} sph_lattice_block;

/* Replaces the handle's particles by the concatenated blocks (ids in block
 * order; for an ensemble, block s is scene s and the counts must match the
 * scenes'), as an upload of the same values would. */
int sph_cuda_init_lattice(sph_cuda_t *h, const sph_lattice_block *blocks, int nblocks);

/* Sets scene `scene`'s tunables for the following steps (all handles). */
int sph_cuda_set_scene_params(sph_cuda_t *h, int scene, const tunable_parameters *tp);

/* Number of scenes of the handle (1 for sph_cuda_create). */
int sph_cuda_num_scenes(sph_cuda_t *h);

/* FP64 mean density, mean near density and kinetic energy per particle of
 * every scene: out[3 s + 0..2]. */
int sph_cuda_scene_diagnostics(sph_cuda_t *h, double *out);

/* Launch shapes of the three gather kernels (viscosity_predict, density,
 * relax_update): shapes[2k] threads per block, shapes[2k+1] 0 for one block
 * per tile of particles or the number of resident blocks per SM for a
 * persistent grid-stride launch.  Any shape gives the same results. */
int sph_cuda_set_launch_shapes(sph_cuda_t *h, const int *shapes);
int sph_cuda_get_launch_shapes(sph_cuda_t *h, int *shapes);

/* Long-row hit masks (off after create): the density pass also records the
 * neighbours among candidates 65..128 of a stencil row, so that the
 * relaxation (and the learned step's message walk) walks hit masks instead
 * of the whole stencil for particles in cells dense enough for such rows.
 * Results are bit for bit the same either way (the same pairs, in the same
 * order); the masks take 24 bytes per particle of device memory, allocated
 * on the first switch on.  They pay in dense scenes and cost a little where
 * long rows are rare; sph_cuda_autotune chooses. */
int sph_cuda_set_long_row_masks(sph_cuda_t *h, int on);
int sph_cuda_get_long_row_masks(sph_cuda_t *h);

/* Autotuner: for each gather in turn (the others at their best so far),
 * times one graph-launched step per candidate shape over trial_steps
 * interleaved rounds and keeps the candidate with the lowest median step
 * time; then chooses long-row masks on or off the same way.  It advances
 * the simulation by 50 x trial_steps steps (each measurement re-captures
 * the step graph with one untimed step first); the chosen shapes go to
 * shapes_out (6 ints) if given. */
int sph_cuda_autotune(sph_cuda_t *h, int trial_steps, int *shapes_out);

/* Frees all device and host resources of the handle. */
int sph_cuda_destroy(sph_cuda_t *h);

/* Queues subsequent work on `stream` (a cudaStream_t, NULL = the handle's own
 * stream).  Re-captures the step graph. */
int sph_cuda_set_stream(sph_cuda_t *h, void *stream);

/* Uploads n particles (id = pointer-array index, fluid.c:197 / geometry.c:57)
 * from the caller's pointer array and sorts them into cells.  Neighbour
 * lists start empty, as after fluid.c:202's calloc: the first step after an
 * upload has no viscosity impulses, exactly like the reference's first step.
 * Replaces initParticles' hand-off (fluid.c:238). */
int sph_cuda_upload(sph_cuda_t *h, fluid_particle *const *particle_pointers, int n);

/* Same, from a contiguous array (particles[i] has id i). */
int sph_cuda_upload_particles(sph_cuda_t *h, const fluid_particle *particles, int n);

/* Same, from structure-of-arrays host buffers (x, y required; vx, vy may be NULL). */
int sph_cuda_upload_soa(sph_cuda_t *h, const float *x, const float *y, const float *vx,
                        const float *vy, int n);

/* Runs nsteps steps with the given tunables (copied at call time; NULL keeps
 * the current ones, and an ensemble takes NULL).  Each step is the reference
 * sequence fluid.c:273-348: apply_gravity, viscosity_impluses,
 * predict_positions, hash_fluid(.., true), double_density_relaxation,
 * updateVelocities, hash_fluid(.., false) -- with viscosity and relaxation as
 * deterministic gathers (Jacobi form).  Captured as one CUDA graph per step. */
int sph_cuda_step(sph_cuda_t *h, const tunable_parameters *tp, int nsteps);

/* Runs nsteps steps, step t using tps[t] (e.g. a moving mover); single scene. */
int sph_cuda_step_schedule(sph_cuda_t *h, const tunable_parameters *tps, int nsteps);

/* One step whose tunables change inside it, where the reference's compute
 * rank receives them: apply_gravity, viscosity_impluses and
 * predict_positions (fluid.c:273-279) run with tp_before (NULL keeps the
 * current ones); then the MPI_Scatterv of fluid.c:293-294 delivers new
 * tunables, and hash_fluid, double_density_relaxation, updateVelocities and
 * the second hash (fluid.c:315-341) run with tp_after, which stay in force
 * for the following steps.  Use it for the first sub-step of each frame
 * (every steps_per_frame-th step) when the render rank sends tunables; the
 * other steps keep sph_cuda_step.  Launched directly (not from the
 * captured graph); single scene. */
int sph_cuda_step_split(sph_cuda_t *h, const tunable_parameters *tp_before,
                        const tunable_parameters *tp_after);

/* Writes the particle state back through the caller's pointer array:
 * x_prev, y_prev, x, y, v_x, v_y, density, density_near, pressure,
 * pressure_near (a_x, a_y and id untouched).  Density and pressure are the
 * values the last step's relaxation used (predicted positions), as in the
 * reference's structs after a step. */
int sph_cuda_download(sph_cuda_t *h, fluid_particle *const *particle_pointers, int n);

/* Same, into a contiguous array indexed by id. */
int sph_cuda_download_particles(sph_cuda_t *h, fluid_particle *particles, int n);

/* Same, into structure-of-arrays host buffers (any pointer may be NULL). */
int sph_cuda_download_soa(sph_cuda_t *h, float *x, float *y, float *vx, float *vy,
                          float *density, float *density_near, int n);

/* Packs the positions as pixel-space shorts for the render rank, by id:
 * coords[2i] = (2 x/max_x - 1) * SHRT_MAX, coords[2i+1] likewise in y.
 * Replaces the packing loop of fluid.c:356-362 (the MPI_Isend of fluid.c:364
 * stays with the caller). */
int sph_cuda_pack_coords_short(sph_cuda_t *h, short *coords, int n);

/* The same packing without waiting: the packed coordinates of the current
 * state are copied into `coords` (page-locked, e.g. from
 * sph_cuda_host_alloc) on a separate copy stream, so the copy overlaps the
 * next sph_cuda_step; sph_cuda_coords_wait(h, coords) returns once they
 * have arrived.  Two copies may be in flight (alternate two buffers, as the
 * reference overlaps its MPI_Isend with the next steps, fluid.c:282-287,
 * 356-364); a third call waits for the oldest.  The two device staging
 * buffers and the copy stream are made with the handle: the call allocates
 * nothing. */
int sph_cuda_pack_coords_async(sph_cuda_t *h, short *coords, int n);
int sph_cuda_coords_wait(sph_cuda_t *h, const short *coords);

/* ---- checkpoint / resume ---- */

/* Writes the handle's particles (the reference's fluid_particle records, by
 * id), its step count and whether the neighbour relation of the current
 * positions exists to a binary file (48-byte header "SPHCKPT1", then the
 * records).  sph_cuda_load_state restores such a file into a handle with the
 * same scenes: the steps that follow are bit-identical to those the saved
 * handle would have taken.  Also the format of the learned relaxation's
 * training trajectories. */
int sph_cuda_save_state(sph_cuda_t *h, const char *path);
int sph_cuda_load_state(sph_cuda_t *h, const char *path);

/* Rebuilds the neighbour relation on the current positions, like
 * hash_fluid(.., false) (fluid.c:341): after it, the next step applies
 * viscosity impulses even if it is the first step after an upload. */
int sph_cuda_rebuild_neighbors(sph_cuda_t *h);

/* Waits for all queued work of the handle. */
int sph_cuda_synchronize(sph_cuda_t *h);

/* Copies the event counters out (synchronises).  Returns SPH_ERR_CUDA (with
 * the counters filled) if a step's cell build found its per-tile particle
 * counts inconsistent with its cell counters -- an internal error after
 * which the steps since the last upload are not valid. */
int sph_cuda_get_counters(sph_cuda_t *h, sph_cuda_counters *out);

/* FP64 diagnostics of the current state: out[0] mean density, out[1] mean
 * near density (both from the last relaxation), out[2] kinetic energy per
 * particle 0.5 |v|^2 (unit mass).  Deterministic reduction order. */
int sph_cuda_diagnostics(sph_cuda_t *h, double out[3]);

/* ---- parity probes: one pass on the CURRENT state, no state change ---- */

/* The reference's half neighbour lists (hash_fluid, hash.c:127-242) on the
 * current positions, in the reference's order: per particle (by id), the
 * later particles of its own cell then the forward cells (0,+1), (+1,-1),
 * (+1,0), (+1,+1), each cell in id order, cut at max_neighbors.
 * counts[id] entries each, concatenated by id into ids (capacity max_total);
 * *total receives the number of entries. */
int sph_cuda_neighbor_lists(sph_cuda_t *h, int *counts, int *ids, long long max_total,
                            long long *total);

/* Density and near density of every particle on the current positions
 * (hash_fluid(.., true) + calculate_density, hash.c:190-194 / fluid.c:527-539). */
int sph_cuda_probe_density(sph_cuda_t *h, const tunable_parameters *tp, float *density,
                           float *density_near);

/* Relaxation displacement of every particle, treating the current positions
 * as the predicted ones (density pass, then the gather form of
 * double_density_relaxation, fluid.c:541-611), before boundary conditions. */
int sph_cuda_probe_relaxation(sph_cuda_t *h, const tunable_parameters *tp, float *dx,
                              float *dy);

/* Viscosity velocity change of every particle on the current positions and
 * velocities (gather form of viscosity_impluses, fluid.c:416-478). */
int sph_cuda_probe_viscosity(sph_cuda_t *h, const tunable_parameters *tp, float *dvx,
                             float *dvy);

/* ---- density without allocation ---- */

/* Largest problem sph_cuda_density_static accepts. */
#define SPH_STATIC_MAX_PARTICLES 65536
#define SPH_STATIC_MAX_CELLS 262144

/* No counterpart in the reference.  For callers that cannot call cudaMalloc
 * (a step loop living inside another framework's fixed device-memory budget,
 * or a real-time loop that cannot take the device-wide synchronisation an
 * allocation may imply): the density and near density of n particles, as
 * sph_cuda_probe_density computes them, from caller-owned DEVICE arrays
 * x[n], y[n] into caller-owned DEVICE arrays density[n], density_near[n]
 * (indexed like the inputs).  grid gives spacing, size_x, size_y,
 * max_bucket_size and max_neighbors; tp gives smoothing_radius.
 *
 * Allocates nothing: every intermediate lives in one fixed-size device
 * array inside the library (about 7 MB, held on every GPU that loads the
 * library until the process exits).  Rejects n > SPH_STATIC_MAX_PARTICLES
 * and size_x * size_y > SPH_STATIC_MAX_CELLS with SPH_ERR_CAPACITY.
 * Each call outside stream capture looks up that array's device address (a
 * call under capture reuses the last one found on the device), so make the
 * first call on a device before any stream capture.  Work is queued on `stream`
 * (NULL = the default stream) and the call returns once it is queued.
 * All calls share the one array: calls whose work overlaps on the GPU (other
 * streams, other host threads) race and corrupt each other's results. */
int sph_cuda_density_static(const float *x, const float *y, int n, const neighbor_grid_t *grid,
                            const tunable_parameters *tp, float *density, float *density_near,
                            void *stream);

/* The event counters of the last sph_cuda_density_static call's neighbour
 * build, written to caller-owned DEVICE memory *d_out on `stream` (steps is
 * 0): out_of_grid counts particles whose cell key fell outside the grid
 * (they get zero density), bucket_overflow the particles dropped beyond
 * max_bucket_size in their cell, max_cell_occupancy the fullest cell, and
 * list_cap_risk is nonzero when a cell held enough particles for a half
 * list to pass max_neighbors (the density pass does not cut lists, so such
 * a particle keeps neighbours the reference would have dropped).  Allocates
 * nothing; queue it after the density call on the same stream, before any
 * other call reuses the shared array. */
int sph_cuda_density_static_counters(sph_cuda_counters *d_out, void *stream);

/* ---- measurement ---- */

/* Runs ONE step (it advances the state) with a CUDA event pair around each
 * kernel on the handle's stream.  ms[k] receives kernel k's time, *count the
 * number of kernels (at most max); names via sph_cuda_step_kernel_name(h, k)
 * (sph_cuda_kernel_name(k) names the kernels of the plain step). */
int sph_cuda_kernel_times(sph_cuda_t *h, const tunable_parameters *tp, float *ms, int max,
                          int *count);
const char *sph_cuda_kernel_name(int k);
const char *sph_cuda_step_kernel_name(sph_cuda_t *h, int k);

/* Kernels launched per step (graph nodes). */
int sph_cuda_launches_per_step(sph_cuda_t *h);

/* Device timer on the handle's stream: start records a CUDA event, stop
 * records a second one, waits for it and returns the elapsed milliseconds. */
int sph_cuda_timer_start(sph_cuda_t *h);
int sph_cuda_timer_stop(sph_cuda_t *h, float *ms);

/* ---- headless liquid-surface image ---- */

/* The render rank's liquid drawing (draw_liquid, liquid_gl.c:305-447, and
 * its shaders) as compute kernels, without a graphics API: metaball sprites
 * of diameter 0.020 x width splatted additively into an 8-bit alpha texture
 * at half the screen resolution, a 15-tap Gaussian blur along y then x,
 * then the threshold/smoothstep composite over black at full resolution.
 * rgb receives width x height x 3 bytes, top row first (a binary PPM body);
 * alpha, if not NULL, the blurred (width/2) x (height/2) alpha texture,
 * bottom row first.
 *   sph_render_liquid        from packed short coordinates (the render
 *                            rank's input, fluid.c:356-362), host memory
 *   sph_cuda_render_liquid   from a handle's current particles (packed on
 *                            the device, no host round trip) */
int sph_render_liquid(const short *coords, int n, int width, int height, unsigned char *rgb,
                      unsigned char *alpha);
int sph_cuda_render_liquid(sph_cuda_t *h, int width, int height, unsigned char *rgb,
                           unsigned char *alpha);

/* Bounds-checked builds (compiled with -DSPH_BOUNDS_CHECK, a stand-in for a
 * memory checker): every data-dependent index of the step's kernels -- a
 * neighbour slot, a cell key, a scatter or permute destination, a cell
 * start -- is tested before its access, and a bad one is skipped and
 * recorded.  sph_cuda_bounds_errors returns the recorded kinds (bit 0
 * neighbour slot, 1 cell key, 2 scatter/permute destination, 3 cell start;
 * always 0 in normal builds), sph_cuda_bounds_checked whether this library
 * is such a build. */
int sph_cuda_bounds_errors(unsigned *flags);
int sph_cuda_bounds_checked(void);

/* Test hook for failure handling: after `after` more successful device or
 * pinned-host allocations of the library (handle creation, scratch and
 * staging buffers), the next one fails as if memory were exhausted (no
 * device fault involved); -1 turns it off.  Process-wide. */
int sph_cuda_debug_fail_allocation(int after);

/* ---- live tunables (host helpers, no device work) ---- */

/* The render rank's fluid presets (controls.c:344-401), applied to a
 * caller's tunables: 'x' standard fluid, 'y' "super goo", 'a' zero g with
 * high surface tension, 'b' spring gas; each sets g, k, k_near, k_spring,
 * sigma, beta and rest_density.  'm' resets the mover to 2 x 2
 * (controls.c:333-339).  SPH_ERR_INVALID for any other letter.  The values
 * reach the device with the next sph_cuda_step / sph_cuda_set_scene_params
 * (a pinned-buffer copy between graph launches). */
int sph_cuda_tunables_preset(tunable_parameters *tp, char which);

/* One frame of the render rank's inactive-mode mover path
 * (renderer.c:493-532): gl_x += 0.01 direction, direction reversed outside
 * [-1, 1], gl_y = sin(3.14 * 5 gl_x) / 10 - 0.6, and the centre in
 * simulation coordinates (renderer.c:397-404) for a box [0, max_x] x
 * [0, max_y].  *gl_x and *direction carry the path's state between frames. */
int sph_cuda_mover_track(float max_x, float max_y, float *gl_x, int *direction,
                         float *center_x, float *center_y);

/* Page-locked host memory for fast transfers (e.g. the packed coordinates
 * buffer of sph_cuda_pack_coords_short), and its release. */
int sph_cuda_host_alloc(void **ptr, size_t bytes);
int sph_cuda_host_free(void *ptr);

/* ---- misc ---- */

/* Message of the last failed call on this host thread ("" if none). */
const char *sph_cuda_last_error(void);

/* sizeof of fluid_particle, neighbor, tunable_parameters, param, bucket_t,
 * neighbor_grid_t, AABB_t as compiled into the library (7 ints). */
int sph_cuda_abi_sizes(int *sizes, int n);

#ifdef __cplusplus
}
#endif

#endif /* SPH_CUDA_H */
