/*
 * compute_rank.c -- a compute rank's main loop (start_simulation,
 * fluid.c:71-395) driving libsph_cuda, with the render rank replaced by an
 * in-process stand-in.  It is the end-to-end form of the drop-in: the
 * set-up follows fluid.c:88-176 for one rank (the reference's default
 * tunables, a 15 x 15/aspect box, h = 2 x the initial particle spacing, a
 * 100-particle bucket cap and 400-entry lists), the particles live in the
 * caller's AoS array behind a pointer array as in fluid.c:183-197, and each
 * step is one sph_cuda_step.  The last sub-step of every frame is a split
 * step (sph_cuda_step_split): after its prediction the stand-in render rank
 * hands over new tunables, as the reference's MPI_Scatterv does in that
 * sub-step (fluid.c:293-294), and at its end the packed short coordinates
 * (fluid.c:356-364) go to the stand-in on a copy stream, overlapping the
 * next frame's steps as the reference's MPI_Isend does.  The stand-in moves
 * the mover along the render rank's inactive-mode path (renderer.c:493-532)
 * and cycles the fluid presets x, y, a, b (controls.c:344-401) every
 * `preset_frames` frames.
 *
 * usage: sph_compute_rank N STEPS STEPS_PER_FRAME OUT_PREFIX [PIX_X PIX_Y [PRESET_FRAMES]]
 *
 * Writes OUT_PREFIX.init     n x (x, y) float32: the uploaded particles
 *        OUT_PREFIX.tunables STEPS x 2 tunable_parameters: each step's
 *                            tunables before and after the point where a
 *                            frame's new ones arrive (equal except in the
 *                            last sub-step of a frame)
 *        OUT_PREFIX.frames   header (int32 n, int32 frames, float32 max_x,
 *                            max_y, h, uint32 size_x, size_y) then frames x
 *                            n x 2 int16 coordinates
 * and prints one line of diagnostics.  Exit status 0 on success.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "sph_cuda.h"

static int fail(const char *what)
{
    fprintf(stderr, "compute_rank: %s: %s\n", what, sph_cuda_last_error());
    return 1;
}

/* The stand-in render rank's state. */
typedef struct {
    FILE *frames;
    int nframes;
    float gl_x;
    int direction;
    int preset_frames;
} render_standin;

/* The render rank's tunables for the frame ending now (its MPI_Scatterv,
 * renderer.c:268): the next preset every `preset_frames` frames, and the
 * mover one step further along the inactive-mode path. */
static int render_tunables(render_standin *r, float max_x, float max_y, tunable_parameters *tp)
{
    if (r->preset_frames > 0 && r->nframes > 0 && r->nframes % r->preset_frames == 0) {
        static const char cycle[4] = {'x', 'y', 'a', 'b'};
        if (sph_cuda_tunables_preset(tp, cycle[(r->nframes / r->preset_frames) % 4]) != SPH_OK)
            return 1;
    }
    return sph_cuda_mover_track(max_x, max_y, &r->gl_x, &r->direction, &tp->mover_center_x,
                                &tp->mover_center_y) != SPH_OK;
}

/* Receives one frame of coordinates (the render rank's Irecv, renderer.c:276-282). */
static int render_receive(render_standin *r, const short *coords, int n)
{
    if (fwrite(coords, sizeof(short), 2 * (size_t)n, r->frames) != 2 * (size_t)n) return 1;
    ++r->nframes;
    return 0;
}

int main(int argc, char **argv)
{
    if (argc < 5) {
        fprintf(stderr, "usage: %s N STEPS STEPS_PER_FRAME OUT_PREFIX [PIX_X PIX_Y [PRESET_FRAMES]]\n",
                argv[0]);
        return 2;
    }
    const int n_global = atoi(argv[1]);
    const int steps = atoi(argv[2]);
    const int steps_per_frame = atoi(argv[3]);
    const char *prefix = argv[4];
    const int pix_x = argc > 6 ? atoi(argv[5]) : 1920;
    const int pix_y = argc > 6 ? atoi(argv[6]) : 1080;
    const int preset_frames = argc > 7 ? atoi(argv[7]) : 0;
    if (n_global <= 0 || steps < 0 || steps_per_frame <= 0 || pix_x <= 0 || pix_y <= 0) {
        fprintf(stderr, "compute_rank: bad arguments\n");
        return 2;
    }

    /* set-up of one compute rank (fluid.c:88-176) */
    param params;
    memset(&params, 0, sizeof(params));
    tunable_parameters *tp = &params.tunable_params;
    tp->kill_sim = 0;
    tp->active = 1;
    tp->g = 6.0f;
    tp->time_step = 1.0f / 30.0f / (float)steps_per_frame;
    tp->k = 0.2f;
    tp->k_near = 6.0f;
    tp->k_spring = 10.0f;
    tp->sigma = 5.0f;
    tp->beta = 0.5f;
    tp->rest_density = 30.0f;
    tp->mover_width = 2.0f;
    tp->mover_height = 2.0f;
    tp->mover_type = SPHERE_MOVER;

    AABB_t box;
    memset(&box, 0, sizeof(box));
    box.max_x = 15.0f;
    box.max_y = box.max_x / ((float)pix_x / (float)pix_y);
    const float area = box.max_x * box.max_y;
    const float spacing = sqrtf(area / (float)n_global);
    tp->smoothing_radius = 2.0f * spacing;
    tp->node_start_x = 0.0f;
    tp->node_end_x = box.max_x;

    /* the water volume is the whole box: a lattice of `spacing`, row by row
     * from the floor, cell centres, as many particles as fit up to N */
    const int nx = (int)(box.max_x / spacing);
    const int ny = (int)(box.max_y / spacing);
    int n = nx * ny < n_global ? nx * ny : n_global;
    params.number_fluid_particles_global = n;
    params.number_fluid_particles_local = n;
    params.max_fluid_particle_index = n - 1;
    params.number_halo_particles = 0;

    neighbor_grid_t grid;
    memset(&grid, 0, sizeof(grid));
    grid.max_bucket_size = 100;
    grid.max_neighbors = grid.max_bucket_size * 4;
    grid.spacing = tp->smoothing_radius;
    grid.size_x = (unsigned)ceilf(box.max_x / grid.spacing);
    grid.size_y = (unsigned)ceilf(box.max_y / grid.spacing);

    fluid_particle *particles = calloc((size_t)n, sizeof(fluid_particle));
    fluid_particle **ptrs = calloc((size_t)n, sizeof(fluid_particle *));
    if (!particles || !ptrs) return 1;
    for (int i = 0; i < n; ++i) {
        fluid_particle *p = &particles[i];
        p->x = ((float)(i % nx) + 0.5f) * spacing;
        p->y = ((float)(i / nx) + 0.5f) * spacing;
        p->x_prev = p->x;
        p->y_prev = p->y;
        p->id = i;
        ptrs[i] = p;
    }
    /* the mover starts where the inactive path starts */
    render_standin r = {NULL, 0, 0.0f, 1, preset_frames};
    float gl_y = sinf(3.14f * 5.0f * r.gl_x) / 10.0f - 0.6f;
    tp->mover_center_x = r.gl_x * box.max_x * 0.5f + box.max_x * 0.5f;
    tp->mover_center_y = gl_y * box.max_y * 0.5f + box.max_y * 0.5f;

    char path[4096];
    snprintf(path, sizeof(path), "%s.init", prefix);
    FILE *f = fopen(path, "wb");
    if (!f) return 1;
    for (int i = 0; i < n; ++i) {
        const float xy[2] = {particles[i].x, particles[i].y};
        fwrite(xy, sizeof(float), 2, f);
    }
    fclose(f);
    snprintf(path, sizeof(path), "%s.tunables", prefix);
    FILE *ftp = fopen(path, "wb");
    snprintf(path, sizeof(path), "%s.frames", prefix);
    r.frames = fopen(path, "wb");
    if (!ftp || !r.frames) return 1;
    const int32_t hdr_i[2] = {n, 0};
    const float hdr_f[3] = {box.max_x, box.max_y, tp->smoothing_radius};
    const uint32_t hdr_g[2] = {grid.size_x, grid.size_y};
    fwrite(hdr_i, sizeof(hdr_i), 1, r.frames);
    fwrite(hdr_f, sizeof(hdr_f), 1, r.frames);
    fwrite(hdr_g, sizeof(hdr_g), 1, r.frames);

    /* the device replaces the host allocations of fluid.c:178-235 */
    sph_cuda_t *sim = NULL;
    if (sph_cuda_create(&sim, &params, &box, &grid, n) != SPH_OK) return fail("create");
    if (sph_cuda_upload(sim, ptrs, n) != SPH_OK) return fail("upload");
    /* two page-locked frames: frame f is copied while the steps of frame
     * f + 1 run, as the reference overlaps its MPI_Isend of the coordinates
     * with the next steps and waits for it before packing again
     * (fluid.c:282-287, 356-364); the render stand-in answers each frame
     * with the tunables of the steps after the next frame boundary, one
     * frame behind, as the render rank's MPI_Scatterv does
     * (fluid.c:293-294) */
    short *coords[2] = {NULL, NULL};
    for (int b = 0; b < 2; ++b)
        if (sph_cuda_host_alloc((void **)&coords[b], 2 * (size_t)n * sizeof(short)) != SPH_OK)
            return fail("host_alloc");
    int frame = 0, pending = -1;

    int sub_step = 0;
    for (int t = 0; t < steps; ++t) {
        if (tp->kill_sim) break;
        fwrite(tp, sizeof(*tp), 1, ftp);
        if (sub_step == steps_per_frame - 1) {
            /* the previous frame's coordinates have arrived at the render
             * rank (its copy overlapped this frame's steps); it answers with
             * this frame's tunables, which act from the hash of this
             * sub-step on */
            if (pending >= 0) {
                if (sph_cuda_coords_wait(sim, coords[pending]) != SPH_OK) return fail("wait");
                if (render_receive(&r, coords[pending], n)) return fail("render stand-in");
            }
            tunable_parameters after = *tp;
            if (render_tunables(&r, box.max_x, box.max_y, &after)) return fail("render stand-in");
            fwrite(&after, sizeof(after), 1, ftp);
            if (sph_cuda_step_split(sim, tp, &after) != SPH_OK) return fail("split step");
            *tp = after;
            pending = frame & 1;
            if (sph_cuda_pack_coords_async(sim, coords[pending], n) != SPH_OK) return fail("pack");
            ++frame;
        } else {
            fwrite(tp, sizeof(*tp), 1, ftp);
            if (sph_cuda_step(sim, tp, 1) != SPH_OK) return fail("step");
        }
        sub_step = sub_step == steps_per_frame - 1 ? 0 : sub_step + 1;
    }
    if (pending >= 0) {
        if (sph_cuda_coords_wait(sim, coords[pending]) != SPH_OK) return fail("wait");
        if (render_receive(&r, coords[pending], n)) return fail("render stand-in");
    }
    if (sph_cuda_download(sim, ptrs, n) != SPH_OK) return fail("download");
    double diag[3];
    if (sph_cuda_diagnostics(sim, diag) != SPH_OK) return fail("diagnostics");
    sph_cuda_counters cnt;
    if (sph_cuda_get_counters(sim, &cnt) != SPH_OK) return fail("counters");

    /* frame count into the header */
    fseek(r.frames, sizeof(int32_t), SEEK_SET);
    const int32_t nf = r.nframes;
    fwrite(&nf, sizeof(nf), 1, r.frames);
    fclose(r.frames);
    fclose(ftp);
    printf("particles %d steps %llu frames %d mean_density %.6f kinetic_energy %.6f "
           "max_cell_occupancy %u\n",
           n, (unsigned long long)cnt.steps, r.nframes, diag[0], diag[2], cnt.max_cell_occupancy);
    sph_cuda_host_free(coords[0]);
    sph_cuda_host_free(coords[1]);
    sph_cuda_destroy(sim);
    free(ptrs);
    free(particles);
    return 0;
}
