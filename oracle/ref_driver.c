/*
 * Headless harness around the reference's OWN step functions (test oracle).
 *
 * Compiled by oracle/Makefile together with the unmodified reference sources
 * src/hash.c and src/fluid.c into oracle/_ref/libsph_ref.so.  It replaces
 * start_simulation() (fluid.c:71-395) for a single compute rank with no
 * neighbours: it owns the same host allocations (fluid.c:173-235), and
 * ref_step() calls the reference step functions in the order of the
 * reference loop (fluid.c:270-349) with the MPI calls left out (they move no
 * data on one rank: 0 halo particles, 0 out-of-bounds transfers).
 *
 * Test infrastructure only: the product never links or calls this.
 */
#include "fluid.h"
#include "hash.h"
#include <stdlib.h>
#include <string.h>
#include <limits.h>

typedef struct sim_config {
    float box[4];            /* min_x, max_x, min_y, max_y */
    float spacing;           /* neighbour-grid spacing (fluid.c:176) */
    int size_x, size_y;      /* grid dimensions (fluid.c:214-215) */
    int max_bucket;          /* fluid.c:174 */
    int max_neighbors;       /* fluid.c:175 */
} sim_config;

typedef struct ref_sim {
    param params;
    AABB_t boundary;
    neighbor_grid_t grid;
    edge_t edges;
    fluid_particle *particles;
    fluid_particle **ptrs;
    neighbor *neighbors;
    fluid_particle **nbr_store;
    bucket_t *buckets;
    fluid_particle **bucket_store;
    int n;
} ref_sim;

void *ref_create(int n, const float *x, const float *y, const float *vx, const float *vy,
                 const tunable_parameters *tp, const sim_config *cfg)
{
    ref_sim *s = calloc(1, sizeof(ref_sim));
    int i;
    size_t cells = (size_t)cfg->size_x * cfg->size_y;
    s->n = n;
    s->params.tunable_params = *tp;
    s->params.number_fluid_particles_global = n;
    s->params.number_fluid_particles_local = n;
    s->params.max_fluid_particle_index = n - 1;
    s->params.number_halo_particles = 0;
    s->boundary.min_x = cfg->box[0];
    s->boundary.max_x = cfg->box[1];
    s->boundary.min_y = cfg->box[2];
    s->boundary.max_y = cfg->box[3];
    s->grid.spacing = cfg->spacing;
    s->grid.size_x = cfg->size_x;
    s->grid.size_y = cfg->size_y;
    s->grid.max_bucket_size = cfg->max_bucket;
    s->grid.max_neighbors = cfg->max_neighbors;

    s->particles = calloc((size_t)n, sizeof(fluid_particle));
    s->ptrs = malloc((size_t)n * sizeof(fluid_particle *));
    /* neighbour lists start empty, as fluid.c:202-206 calloc's them */
    s->neighbors = calloc((size_t)n, sizeof(neighbor));
    s->nbr_store = calloc((size_t)n * cfg->max_neighbors, sizeof(fluid_particle *));
    for (i = 0; i < n; i++)
        s->neighbors[i].fluid_neighbors = &s->nbr_store[(size_t)i * cfg->max_neighbors];
    s->grid.neighbors = s->neighbors;
    s->buckets = calloc(cells, sizeof(bucket_t));
    s->bucket_store = calloc(cells * cfg->max_bucket, sizeof(fluid_particle *));
    for (i = 0; i < (int)cells; i++)
        s->buckets[i].fluid_particles = &s->bucket_store[(size_t)i * cfg->max_bucket];
    s->grid.grid_buckets = s->buckets;

    for (i = 0; i < n; i++) {
        fluid_particle *p = &s->particles[i];
        p->x = x[i];
        p->y = y[i];
        p->x_prev = x[i];
        p->y_prev = y[i];
        p->v_x = vx[i];
        p->v_y = vy[i];
        p->id = i;
        s->ptrs[i] = p;
    }
    return s;
}

void ref_destroy(void *h)
{
    ref_sim *s = h;
    if (!s) return;
    free(s->particles);
    free(s->ptrs);
    free(s->neighbors);
    free(s->nbr_store);
    free(s->buckets);
    free(s->bucket_store);
    free(s);
}

void ref_set_tunables(void *h, const tunable_parameters *tp)
{
    ((ref_sim *)h)->params.tunable_params = *tp;
}

static void diagnostics(const ref_sim *s, double *out)
{
    double rho = 0.0, rhon = 0.0, ke = 0.0;
    int i;
    for (i = 0; i < s->n; i++) {
        const fluid_particle *p = s->ptrs[i];
        rho += p->density;
        rhon += p->density_near;
        ke += 0.5 * ((double)p->v_x * p->v_x + (double)p->v_y * p->v_y);
    }
    out[0] = rho / s->n;
    out[1] = rhon / s->n;
    out[2] = ke / s->n;
}

/* One reference step = fluid.c:273-348 without the MPI exchange calls. */
static void one_step(ref_sim *s)
{
    apply_gravity(s->ptrs, &s->params);
    viscosity_impluses(s->ptrs, s->neighbors, &s->params);
    predict_positions(s->ptrs, &s->boundary, &s->params);
    hash_fluid(s->ptrs, &s->grid, &s->params, true);
    hash_halo(s->ptrs, &s->grid, &s->params, true);
    double_density_relaxation(s->ptrs, s->neighbors, &s->params);
    updateVelocities(s->ptrs, &s->edges, &s->boundary, &s->params);
    hash_fluid(s->ptrs, &s->grid, &s->params, false);
    hash_halo(s->ptrs, &s->grid, &s->params, false);
}

/* mover_xy: optional per-step mover centre (2 floats per step, set before the
 * step as the render rank's parameter update would); diag: optional 3 doubles
 * per step (mean density, mean near density, kinetic energy per particle). */
void ref_step(void *h, int nsteps, const float *mover_xy, double *diag)
{
    ref_sim *s = h;
    int t;
    for (t = 0; t < nsteps; t++) {
        if (mover_xy) {
            s->params.tunable_params.mover_center_x = mover_xy[2 * t];
            s->params.tunable_params.mover_center_y = mover_xy[2 * t + 1];
        }
        one_step(s);
        if (diag) diagnostics(s, diag + 3 * t);
    }
}

/* 12 floats per particle in struct order (x_prev .. pressure_near), by id. */
void ref_get(void *h, float *out)
{
    ref_sim *s = h;
    int i;
    for (i = 0; i < s->n; i++) {
        const fluid_particle *p = &s->particles[i];
        memcpy(out + 12 * (size_t)i, p, 12 * sizeof(float));
    }
}

void ref_set_state(void *h, const float *x, const float *y, const float *vx, const float *vy)
{
    ref_sim *s = h;
    int i;
    for (i = 0; i < s->n; i++) {
        fluid_particle *p = &s->particles[i];
        p->x = x[i];
        p->y = y[i];
        if (vx) p->v_x = vx[i];
        if (vy) p->v_y = vy[i];
    }
}

/* Zero the densities (as apply_gravity does, fluid.c:410-411), run the
 * reference hash_fluid() on the current positions and return its neighbour
 * lists as ids: counts[i] entries of list i, concatenated into ids.
 * Returns the total number of list entries, or -1 if max_total is too small. */
int ref_hash(void *h, int compute_density, int *counts, int *ids, int max_total)
{
    ref_sim *s = h;
    int i, j, total = 0;
    for (i = 0; i < s->n; i++) {
        s->ptrs[i]->density = 0.0f;
        s->ptrs[i]->density_near = 0.0f;
    }
    hash_fluid(s->ptrs, &s->grid, &s->params, compute_density != 0);
    for (i = 0; i < s->n; i++) {
        const neighbor *ne = &s->neighbors[i];
        counts[i] = ne->number_fluid_neighbors;
        if (total + ne->number_fluid_neighbors > max_total) return -1;
        for (j = 0; j < ne->number_fluid_neighbors; j++)
            ids[total++] = ne->fluid_neighbors[j]->id;
    }
    return total;
}

/* Run one reference step function by name on the current state, for
 * per-function parity: 0 apply_gravity, 1 viscosity_impluses,
 * 2 predict_positions, 3 double_density_relaxation, 4 updateVelocities. */
void ref_call(void *h, int which)
{
    ref_sim *s = h;
    switch (which) {
    case 0: apply_gravity(s->ptrs, &s->params); break;
    case 1: viscosity_impluses(s->ptrs, s->neighbors, &s->params); break;
    case 2: predict_positions(s->ptrs, &s->boundary, &s->params); break;
    case 3: double_density_relaxation(s->ptrs, s->neighbors, &s->params); break;
    case 4: updateVelocities(s->ptrs, &s->edges, &s->boundary, &s->params); break;
    default: break;
    }
}

/* Packed render coordinates, by id: the expression of fluid.c:360-361
 * (inline in start_simulation there, so restated here as written). */
void ref_pack_coords(void *h, short *out)
{
    ref_sim *s = h;
    int i;
    for (i = 0; i < s->n; i++) {
        const fluid_particle *p = s->ptrs[i];
        out[i * 2] = (2.0f * p->x / s->boundary.max_x - 1.0f) * SHRT_MAX;
        out[i * 2 + 1] = (2.0f * p->y / s->boundary.max_y - 1.0f) * SHRT_MAX;
    }
}

/* Reference hash_val (hash.c:35-47) on one point. */
unsigned int ref_hash_val(void *h, float x, float y)
{
    ref_sim *s = h;
    return hash_val(x, y, &s->grid, &s->params);
}
