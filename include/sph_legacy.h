/*
 * sph_legacy.h -- libsph_cuda entry points with the reference's own names and
 * signatures, for per-function drop-in and parity checks.
 *
 * Each function does what its reference namesake does to the caller's host
 * structs, computing on the GPU: it copies the particles it reads to the
 * device, runs the kernel, and writes the fields the reference writes back
 * through the same pointers.  They are correct but pay a host<->device round
 * trip per call; a step loop should use sph_cuda_step (sph_cuda.h).
 *
 * Differences from the reference, by design:
 *  - viscosity_impluses and double_density_relaxation evaluate every listed
 *    pair from the state before the call (gather / Jacobi form) instead of
 *    updating in place while sweeping (fluid.c:433-477, 568-610);
 *  - a single-device domain has no halo and no migration: hash_halo and
 *    identify_oob_particles do nothing when there is nothing to exchange and
 *    report SPH_ERR_UNSUPPORTED through sph_legacy_status() otherwise.
 *
 * The functions return void like the reference; sph_legacy_status() gives the
 * sph_status of the last call on this host thread and sph_cuda_last_error()
 * its message.  The library keeps one internal device context for these calls
 * (guarded by a mutex; calls from several threads serialise).
 */
#ifndef SPH_LEGACY_H
#define SPH_LEGACY_H

#include "sph_types.h"

#ifdef __cplusplus
extern "C" {
#endif

/* fluid.h:112 -- mover and box collision of one particle (fluid.c:656-744). */
void boundaryConditions(fluid_particle *p, AABB_t *boundary, param *params);

/* fluid.h:118 -- density contribution of a pair at r/h = ratio (fluid.c:527-539). */
void calculate_density(fluid_particle *p, fluid_particle *q, float ratio);

/* fluid.h:119 -- v_y += -g dt and zero densities, local + halo particles (fluid.c:398-413). */
void apply_gravity(fluid_particle **fluid_particle_pointers, param *params);

/* fluid.h:120 -- viscosity impulses over the given half lists (fluid.c:416-478). */
void viscosity_impluses(fluid_particle **fluid_particle_pointers, neighbor *neighbors,
                        param *params);

/* fluid.h:121 -- x_prev = x, x += v dt, boundary conditions (fluid.c:507-523). */
void predict_positions(fluid_particle **fluid_particle_pointers, AABB_t *boundary_global,
                       param *params);

/* fluid.h:122 -- pressures and relaxation over the given half lists (fluid.c:541-611). */
void double_density_relaxation(fluid_particle **fluid_particle_pointers, neighbor *neighbors,
                               param *params);

/* fluid.h:123 -- v = (x - x_prev)/dt clamped to +-5 (fluid.c:627-639). */
void updateVelocity(fluid_particle *p, param *params);

/* fluid.h:124 -- boundary conditions then updateVelocity for every local
 * particle (fluid.c:642-653); edges is unused, as in the reference. */
void updateVelocities(fluid_particle **fluid_particle_pointers, edge_t *edges,
                      AABB_t *boundary_global, param *params);

/* fluid.h:125 -- clamp a velocity pair to +-5 (fluid.c:613-625). */
void checkVelocity(float *v_x, float *v_y);

/* fluid.h:126 -- out-of-domain particles (fluid.c:481-502): on a single
 * domain none can leave; counts particles outside [node_start_x,
 * node_end_x] and reports SPH_ERR_UNSUPPORTED if there are any. */
void identify_oob_particles(fluid_particle **fluid_particle_pointers,
                            fluid_particle *fluid_particles, oob_t *out_of_bounds,
                            AABB_t *boundary_global, param *params);

/* hash.h:50 -- grid key floor(y/s) * size_x + floor(x/s) (hash.c:35-47);
 * 0xFFFFFFFF for a negative or NaN coordinate (undefined in the reference). */
unsigned int hash_val(float x, float y, neighbor_grid_t *grid, param *params);

/* hash.h:51 -- buckets and half neighbour lists in the reference's order, and
 * with compute_density the pair densities added to each particle's density
 * and density_near (hash.c:127-242). */
void hash_fluid(fluid_particle **fluid_particle_pointers, neighbor_grid_t *grid, param *params,
                bool compute_density);

/* hash.h:52 -- halo particles into the lists (hash.c:51-122): a single-device
 * domain has none; nonzero number_halo_particles is SPH_ERR_UNSUPPORTED. */
void hash_halo(fluid_particle **fluid_particle_pointers, neighbor_grid_t *grid, param *params,
               bool compute_density);

/* No counterpart in the reference: status of the last call above on this
 * host thread (0 = SPH_OK). */
int sph_legacy_status(void);

#ifdef __cplusplus
}
#endif

#endif /* SPH_LEGACY_H */
