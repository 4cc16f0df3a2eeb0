/*
 * sph_types.h -- the reference's data model, as libsph_cuda sees it.
 *
 * The C ABI of libsph_cuda takes the reference's own structs.  A caller that
 * already includes the reference's fluid.h (which pulls in hash.h,
 * geometry.h and communication.h) gets those definitions and this header
 * declares nothing new; a caller without them (tests, other host languages)
 * gets identical layouts from here.  libsph_cuda checks every size and
 * offset at compile time (sph_gb300/csrc/sph_abi.cu).
 *
 *   fluid_particle      fluid.h:56-70    12 floats + int id, 52 bytes
 *   neighbor            fluid.h:72-75    half neighbour list (pointers + count)
 *   tunable_parameters  fluid.h:78-97    15 floats + 3 chars, 64 bytes
 *   param               fluid.h:100-106  tunables + particle counts, 80 bytes
 *   bucket_t            hash.h:35-38     grid bucket (pointers + count)
 *   neighbor_grid_t     hash.h:40-48     grid spacing, size, caps, storage
 *   AABB_t              geometry.h:33-40 axis-aligned box, 6 floats
 *   edge_t, oob_t       communication.h:45-63, only passed through as pointers
 */
#ifndef SPH_TYPES_H
#define SPH_TYPES_H

#ifndef fluid_fluid_h /* the reference's fluid.h is not included */

#include <stdbool.h>

typedef struct FLUID_PARTICLE fluid_particle;
typedef struct NEIGHBOR neighbor;
typedef struct PARAM param;
typedef struct TUNABLE_PARAMETERS tunable_parameters;
typedef struct BUCKET_T bucket_t;
typedef struct NEIGHBOR_GRID_T neighbor_grid_t;
typedef struct AABB_T AABB_t;
typedef struct EDGE_T edge_t; /* opaque here: MPI halo bookkeeping */
typedef struct OOB_T oob_t;   /* opaque here: MPI migration bookkeeping */

#define SPHERE_MOVER 0
#define RECTANGLE_MOVER 1

struct FLUID_PARTICLE {
    float x_prev;
    float y_prev;
    float x;
    float y;
    float v_x;
    float v_y;
    float a_x;
    float a_y;
    float density;
    float density_near;
    float pressure;
    float pressure_near;
    int id; /* index of this particle in the caller's pointer array */
};

struct NEIGHBOR {
    fluid_particle **fluid_neighbors;
    int number_fluid_neighbors;
};

struct TUNABLE_PARAMETERS {
    float rest_density;
    float smoothing_radius;
    float g;
    float k;
    float k_near;
    float k_spring;
    float sigma;
    float beta;
    float time_step;
    float node_start_x;
    float node_end_x;
    float mover_center_x;
    float mover_center_y;
    float mover_width;
    float mover_height;
    char mover_type;
    char kill_sim;
    char active;
};

struct PARAM {
    tunable_parameters tunable_params;
    int number_fluid_particles_global;
    int number_fluid_particles_local;
    int max_fluid_particle_index;
    int number_halo_particles;
};

struct BUCKET_T {
    fluid_particle **fluid_particles;
    unsigned int number_fluid;
};

struct NEIGHBOR_GRID_T {
    float spacing;
    unsigned int size_x;
    unsigned int size_y;
    neighbor *neighbors;
    bucket_t *grid_buckets;
    unsigned int max_neighbors;
    unsigned int max_bucket_size;
};

struct AABB_T {
    float min_x;
    float max_x;
    float min_y;
    float max_y;
    float min_z;
    float max_z;
};

#endif /* fluid_fluid_h */
#endif /* SPH_TYPES_H */
