/*
 * sph_oracle.c -- CPU restatement of the TinySPH compute step.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker for the CUDA library:
 * tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * it; the product library (libsph_cuda) never links, calls or falls back to
 * it.
 *
 * Three parts, all written from the reference sources (file:line cited):
 *
 *  1. orc_* "reference order" step (Gauss-Seidel).  A restatement of
 *     hash.c:35-242 and fluid.c:398-744 that keeps the reference's visiting
 *     order and its float/double mix, so that, compiled with
 *     -O2 -ffp-contract=off, it reproduces the compiled reference
 *     (oracle/_ref) bit for bit.  tests/test_oracle_pin.py checks exactly
 *     that, and against the committed golden vectors, which is what pins it.
 *     On machines where the reference sources are absent this restatement is
 *     the CPU baseline.
 *
 *  2. orc_*_f64 gather oracles.  The same physics recast as a Jacobi gather
 *     (every pair term evaluated from the state before the pass), in FP64,
 *     over the symmetric closure of the reference's own half neighbour lists.
 *     These are the parity targets of the GPU's density, viscosity and
 *     relaxation passes.
 *
 *  3. orc_step_jacobi: a float Jacobi step (what the GPU computes), used to
 *     measure Jacobi-vs-Gauss-Seidel drift on the CPU.
 *
 * Cell keys outside the grid (negative or NaN coordinates, or y == max_y)
 * are undefined behaviour in the reference (an out-of-range unsigned
 * conversion or an out-of-bounds bucket write, hash.c:40-44 and
 * hash.c:158-163).  Here such a particle is simply not inserted into any
 * bucket: it gets no neighbours.  The CUDA library does the same.
 */
#include <limits.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

/* Same layout as the reference's tunable_parameters (fluid.h:78-97). */
typedef struct orc_tunables {
    float rest_density, smoothing_radius, g, k, k_near, k_spring, sigma, beta, time_step;
    float node_start_x, node_end_x, mover_center_x, mover_center_y, mover_width, mover_height;
    char mover_type, kill_sim, active;
} orc_tunables;

#define ORC_SPHERE_MOVER 0     /* fluid.h:48 */
#define ORC_RECTANGLE_MOVER 1  /* fluid.h:49 */
#define ORC_NO_CELL 0xFFFFFFFFu

typedef struct sim_config {
    float box[4];            /* min_x, max_x, min_y, max_y (AABB_t, geometry.h:33-40) */
    float spacing;           /* grid spacing (fluid.c:176: = h) */
    int size_x, size_y;      /* fluid.c:214-215 */
    int max_bucket;          /* fluid.c:174 */
    int max_neighbors;       /* fluid.c:175 */
} sim_config;

typedef struct orc_sim {
    int n;
    orc_tunables tp;
    sim_config cfg;
    /* particle state, SoA by id (fields of fluid_particle, fluid.h:56-70) */
    float *xp, *yp, *x, *y, *vx, *vy, *rho, *rhon, *P, *Pn;
    /* half neighbour lists: list i holds lst_cnt[i] ids at lst[i*max_neighbors] */
    int *lst_cnt, *lst;
    /* buckets: bkt_cnt[c] ids at bkt[c*max_bucket], insertion (id) order */
    int *bkt_cnt, *bkt;
    /* symmetric closure of the half lists (CSR), rebuilt on demand */
    int *sym_off, *sym_idx, *sym_own;
    long sym_cap;
} orc_sim;

/* ------------------------------------------------------------------ */
/* small helpers                                                        */
/* ------------------------------------------------------------------ */

/* checkVelocity, fluid.c:613-625 */
static void clamp5(float *a, float *b)
{
    const float v_max = 5.0f;
    if (*a > v_max) *a = v_max;
    else if (*a < -v_max) *a = -v_max;
    if (*b > v_max) *b = v_max;
    else if (*b < -v_max) *b = -v_max;
}

/* hash_val, hash.c:35-47: key = floor(y/s)*size_x + floor(x/s) in unsigned
 * arithmetic.  x == size_x*s therefore aliases cell (0, gy+1), as in the
 * reference.  Out-of-grid keys (see file header) return ORC_NO_CELL. */
unsigned int orc_cell_key(float x, float y, const sim_config *c)
{
    double fx = floor(x / c->spacing);
    double fy = floor(y / c->spacing);
    unsigned int gx, gy, key;
    if (!(fx >= 0.0) || !(fy >= 0.0) || fx >= 4294967296.0 || fy >= 4294967296.0)
        return ORC_NO_CELL;
    gx = (unsigned int)fx;
    gy = (unsigned int)fy;
    key = gy * (unsigned int)c->size_x + gx;
    if ((double)gy * c->size_x + gx >= (double)c->size_x * c->size_y) return ORC_NO_CELL;
    return key;
}

/* boundaryConditions, fluid.c:656-744, on one particle */
static void boundary(float *px, float *py, const orc_tunables *tp, const float *box)
{
    float x = *px, y = *py;
    float cx = tp->mover_center_x, cy = tp->mover_center_y;
    if (tp->mover_type == ORC_SPHERE_MOVER) {
        float radius = tp->mover_width * 0.5f;
        float d2 = (x - cx) * (x - cx) + (y - cy) * (y - cy);
        if (d2 <= radius * radius && d2 > 0.0f) {
            float d = (float)sqrt((double)d2);
            float nx = (cx - x) / d;
            float ny = (cy - y) / d;
            float pen = radius - d;
            x -= pen * nx;
            y -= pen * ny;
        }
    } else if (tp->mover_type == ORC_RECTANGLE_MOVER) {
        float hw = (float)(tp->mover_width * 0.5);
        float hh = (float)(tp->mover_height * 0.5);
        float pcx = x - cx, pcy = y - cy;
        float dcx = (float)fabs((double)pcx), dcy = (float)fabs((double)pcy);
        if (dcx < hw && dcy < hh) {
            float penx = hw - dcx, peny = hh - dcy;
            if (penx < peny) {
                if (pcx < 0.0f) x -= penx; else x += penx;
            } else {
                if (pcy < 0.0f) y -= peny; else y += peny;
            }
        }
    }
    if (x < box[0]) x = box[0];
    else if (x > box[1]) x = box[1] - 0.001f;
    if (y < box[2]) y = box[2];
    else if (y > box[3]) y = box[3] - 0.001f;
    *px = x;
    *py = y;
}

/* ------------------------------------------------------------------ */
/* lifecycle                                                            */
/* ------------------------------------------------------------------ */

void *orc_create(int n, const float *x, const float *y, const float *vx, const float *vy,
                 const orc_tunables *tp, const sim_config *cfg)
{
    orc_sim *s = calloc(1, sizeof(orc_sim));
    size_t cells = (size_t)cfg->size_x * cfg->size_y;
    int i;
    s->n = n;
    s->tp = *tp;
    s->cfg = *cfg;
    s->xp = calloc((size_t)n, sizeof(float));
    s->yp = calloc((size_t)n, sizeof(float));
    s->x = calloc((size_t)n, sizeof(float));
    s->y = calloc((size_t)n, sizeof(float));
    s->vx = calloc((size_t)n, sizeof(float));
    s->vy = calloc((size_t)n, sizeof(float));
    s->rho = calloc((size_t)n, sizeof(float));
    s->rhon = calloc((size_t)n, sizeof(float));
    s->P = calloc((size_t)n, sizeof(float));
    s->Pn = calloc((size_t)n, sizeof(float));
    s->lst_cnt = calloc((size_t)n, sizeof(int));    /* empty lists at start, fluid.c:202 */
    s->lst = calloc((size_t)n * cfg->max_neighbors, sizeof(int));
    s->bkt_cnt = calloc(cells, sizeof(int));
    s->bkt = calloc(cells * cfg->max_bucket, sizeof(int));
    s->sym_off = calloc((size_t)n + 1, sizeof(int));
    for (i = 0; i < n; i++) {
        s->x[i] = s->xp[i] = x[i];
        s->y[i] = s->yp[i] = y[i];
        s->vx[i] = vx ? vx[i] : 0.0f;
        s->vy[i] = vy ? vy[i] : 0.0f;
    }
    return s;
}

void orc_destroy(void *h)
{
    orc_sim *s = h;
    if (!s) return;
    free(s->xp); free(s->yp); free(s->x); free(s->y); free(s->vx); free(s->vy);
    free(s->rho); free(s->rhon); free(s->P); free(s->Pn);
    free(s->lst_cnt); free(s->lst); free(s->bkt_cnt); free(s->bkt);
    free(s->sym_off); free(s->sym_idx); free(s->sym_own);
    free(s);
}

void orc_set_tunables(void *h, const orc_tunables *tp) { ((orc_sim *)h)->tp = *tp; }

void orc_set_state(void *h, const float *x, const float *y, const float *vx, const float *vy)
{
    orc_sim *s = h;
    int i;
    for (i = 0; i < s->n; i++) {
        s->x[i] = x[i];
        s->y[i] = y[i];
        if (vx) s->vx[i] = vx[i];
        if (vy) s->vy[i] = vy[i];
    }
}

/* Replace the half neighbour lists (counts + concatenated ids), e.g. with
 * lists produced by another implementation. */
void orc_set_lists(void *h, const int *counts, const int *ids)
{
    orc_sim *s = h;
    long off = 0;
    int i, j;
    for (i = 0; i < s->n; i++) {
        s->lst_cnt[i] = counts[i];
        for (j = 0; j < counts[i]; j++) s->lst[(size_t)i * s->cfg.max_neighbors + j] = ids[off++];
    }
}

/* 12 floats per particle in fluid_particle field order, by id. */
void orc_get(void *h, float *out)
{
    orc_sim *s = h;
    int i;
    for (i = 0; i < s->n; i++) {
        float *o = out + 12 * (size_t)i;
        o[0] = s->xp[i]; o[1] = s->yp[i]; o[2] = s->x[i]; o[3] = s->y[i];
        o[4] = s->vx[i]; o[5] = s->vy[i]; o[6] = 0.0f; o[7] = 0.0f;
        o[8] = s->rho[i]; o[9] = s->rhon[i]; o[10] = s->P[i]; o[11] = s->Pn[i];
    }
}

/* ------------------------------------------------------------------ */
/* 1. reference-order (Gauss-Seidel) restatement                        */
/* ------------------------------------------------------------------ */

/* calculate_density, fluid.c:527-539 */
static void add_density(orc_sim *s, int p, int q, float ratio)
{
    float omr2 = (1.0f - ratio) * (1.0f - ratio);
    if (ratio < 1.0f) {
        s->rho[p] += omr2;
        s->rhon[p] += omr2 * (1.0f - ratio);
        s->rho[q] += omr2;
        s->rhon[q] += omr2 * (1.0f - ratio);
    }
}

/* Appends `other` to the half list of `owner` (hash.c:188-195, 223-230). */
static void list_append(orc_sim *s, int owner, int other, float r2, int dens, float h_recip,
                        int density_owner_first)
{
    int *cnt = &s->lst_cnt[owner];
    if (*cnt < s->cfg.max_neighbors) {
        s->lst[(size_t)owner * s->cfg.max_neighbors + (*cnt)++] = other;
        if (dens) {
            float r = (float)sqrt((double)r2);
            float ratio = r * h_recip;
            if (density_owner_first) add_density(s, owner, other, ratio);
            else add_density(s, other, owner, ratio);
        }
    }
}

/* hash_fluid, hash.c:127-242.  Buckets are filled in id (pointer-array)
 * order with the bucket cap; the sweep visits cells row-major and, per
 * cell, first the same-cell pairs (c < n) and then the forward cells
 * (0,+1), (+1,-1), (+1,0), (+1,+1), bounds-checked.  Inclusive cutoff
 * r2 <= h2, list cap max_neighbors. */
void orc_hash(void *h, int compute_density)
{
    orc_sim *s = h;
    const sim_config *c = &s->cfg;
    const int sx = c->size_x, sy = c->size_y, cap = c->max_bucket;
    const float hh = s->tp.smoothing_radius;
    const float h_recip = 1.0f / hh;
    const float h2 = hh * hh;
    static const int fwd[4][2] = {{0, 1}, {1, -1}, {1, 0}, {1, 1}};
    int i, gx, gy, a, b, f;

    memset(s->bkt_cnt, 0, (size_t)sx * sy * sizeof(int));
    for (i = 0; i < s->n; i++) {
        unsigned int key = orc_cell_key(s->x[i], s->y[i], c);
        s->lst_cnt[i] = 0;
        if (key == ORC_NO_CELL) continue;
        if (s->bkt_cnt[key] < cap) s->bkt[(size_t)key * cap + s->bkt_cnt[key]++] = i;
    }
    for (gy = 0; gy < sy; gy++) {
        for (gx = 0; gx < sx; gx++) {
            const int cell = gy * sx + gx;
            const int m = s->bkt_cnt[cell];
            const int *mem = &s->bkt[(size_t)cell * cap];
            if (m == 0) continue;
            for (a = 0; a < m; a++) {
                const int p = mem[a];
                for (b = a + 1; b < m; b++) {
                    const int q = mem[b];
                    float r2 = (s->x[p] - s->x[q]) * (s->x[p] - s->x[q]) +
                               (s->y[p] - s->y[q]) * (s->y[p] - s->y[q]);
                    if (r2 > h2) continue;
                    list_append(s, p, q, r2, compute_density, h_recip, 1);
                }
            }
            for (f = 0; f < 4; f++) {
                const int nx = gx + fwd[f][0], ny = gy + fwd[f][1];
                int ncell, mn;
                const int *nmem;
                if (ny < 0 || nx < 0 || nx >= sx || ny >= sy) continue;
                ncell = ny * sx + nx;
                mn = s->bkt_cnt[ncell];
                nmem = &s->bkt[(size_t)ncell * cap];
                for (a = 0; a < m; a++) {
                    const int q = mem[a];
                    for (b = 0; b < mn; b++) {
                        const int qn = nmem[b];
                        float r2 = (s->x[qn] - s->x[q]) * (s->x[qn] - s->x[q]) +
                                   (s->y[qn] - s->y[q]) * (s->y[qn] - s->y[q]);
                        if (r2 > h2) continue;
                        list_append(s, q, qn, r2, compute_density, h_recip, 0);
                    }
                }
            }
        }
    }
}

/* apply_gravity, fluid.c:398-413 */
static void gs_gravity(orc_sim *s)
{
    const float dt = s->tp.time_step;
    const float g = -s->tp.g;
    int i;
    for (i = 0; i < s->n; i++) {
        s->vy[i] += g * dt;
        s->rho[i] = 0.0f;
        s->rhon[i] = 0.0f;
    }
}

/* viscosity_impluses, fluid.c:416-478: reverse particle order, in-place */
static void gs_viscosity(orc_sim *s)
{
    const float h_recip = 1.0f / s->tp.smoothing_radius;
    const float sigma = s->tp.sigma, beta = s->tp.beta, dt = s->tp.time_step;
    int i, j;
    for (i = s->n; i-- > 0;) {
        const float px = s->x[i], py = s->y[i];
        const int *l = &s->lst[(size_t)i * s->cfg.max_neighbors];
        for (j = 0; j < s->lst_cnt[i]; j++) {
            const int q = l[j];
            float qmpx = s->x[q] - px, qmpy = s->y[q] - py;
            float r = (float)sqrt((double)(qmpx * qmpx + qmpy * qmpy));
            float r_recip = 1.0f / r;
            float ratio = r * h_recip;
            float u = ((s->vx[i] - s->vx[q]) * qmpx + (s->vy[i] - s->vy[q]) * qmpy) * r_recip;
            if (u > 0.0f) {
                float imp = dt * (1 - ratio) * (sigma * u + beta * u * u);
                float ix = imp * qmpx * r_recip, iy = imp * qmpy * r_recip;
                clamp5(&ix, &iy);
                s->vx[i] -= ix * 0.5f;
                s->vy[i] -= iy * 0.5f;
                s->vx[q] += ix * 0.5f;
                s->vy[q] += iy * 0.5f;
            }
        }
    }
}

/* predict_positions, fluid.c:507-523 */
static void gs_predict(orc_sim *s)
{
    const float dt = s->tp.time_step;
    int i;
    for (i = 0; i < s->n; i++) {
        s->xp[i] = s->x[i];
        s->yp[i] = s->y[i];
        s->x[i] += s->vx[i] * dt;
        s->y[i] += s->vy[i] * dt;
        boundary(&s->x[i], &s->y[i], &s->tp, s->cfg.box);
    }
}

/* double_density_relaxation, fluid.c:541-611: reverse order, in-place,
 * with the double-precision tail of D (the 0.5 literal, fluid.c:591) */
static void gs_relax(orc_sim *s)
{
    const float k = s->tp.k, k_near = s->tp.k_near, k_spring = s->tp.k_spring;
    const float hh = s->tp.smoothing_radius, h_recip = 1.0f / hh;
    const float dt = s->tp.time_step, rest = s->tp.rest_density;
    int i, j;
    for (i = 0; i < s->n; i++) {
        s->P[i] = k * (s->rho[i] - rest);
        s->Pn[i] = k_near * s->rhon[i];
    }
    for (i = s->n; i-- > 0;) {
        const float pp = s->P[i], ppn = s->Pn[i];
        const int *l = &s->lst[(size_t)i * s->cfg.max_neighbors];
        for (j = 0; j < s->lst_cnt[i]; j++) {
            const int q = l[j];
            float r = (float)sqrt((double)((s->x[i] - s->x[q]) * (s->x[i] - s->x[q]) +
                                           (s->y[i] - s->y[q]) * (s->y[i] - s->y[q])));
            float r_recip = 1.0f / r;
            float ratio = r * h_recip;
            float omr = 1.0f - ratio;
            if (r <= 0.000001f) {
                s->x[i] += 0.000001f;
                s->y[i] += 0.000001f;
            }
            if (ratio < 1.0f && r > 0.0f) {
                float ab = (pp + s->P[q]) * omr + (ppn + s->Pn[q]) * omr * omr;
                float D = (float)((double)(dt * dt) *
                                  ((double)ab + (double)(k_spring * (hh - r)) * 0.5));
                float Dx = D * (s->x[q] - s->x[i]) * r_recip;
                float Dy = D * (s->y[q] - s->y[i]) * r_recip;
                s->x[q] += Dx;
                s->y[q] += Dy;
                s->x[i] -= Dx;
                s->y[i] -= Dy;
            }
        }
    }
}

/* updateVelocities / updateVelocity, fluid.c:627-653 */
static void gs_update_velocities(orc_sim *s)
{
    const float dt = s->tp.time_step;
    int i;
    for (i = 0; i < s->n; i++) {
        float vx, vy;
        boundary(&s->x[i], &s->y[i], &s->tp, s->cfg.box);
        vx = (s->x[i] - s->xp[i]) / dt;
        vy = (s->y[i] - s->yp[i]) / dt;
        clamp5(&vx, &vy);
        s->vx[i] = vx;
        s->vy[i] = vy;
    }
}

static void diagnostics(const orc_sim *s, double *out)
{
    double rho = 0.0, rhon = 0.0, ke = 0.0;
    int i;
    for (i = 0; i < s->n; i++) {
        rho += s->rho[i];
        rhon += s->rhon[i];
        ke += 0.5 * ((double)s->vx[i] * s->vx[i] + (double)s->vy[i] * s->vy[i]);
    }
    out[0] = rho / s->n;
    out[1] = rhon / s->n;
    out[2] = ke / s->n;
}

void orc_diagnostics(void *h, double *out) { diagnostics((orc_sim *)h, out); }

/* One step in the reference loop's order (fluid.c:273-348, single domain). */
void orc_step(void *h, int nsteps, const float *mover_xy, double *diag)
{
    orc_sim *s = h;
    int t;
    for (t = 0; t < nsteps; t++) {
        if (mover_xy) {
            s->tp.mover_center_x = mover_xy[2 * t];
            s->tp.mover_center_y = mover_xy[2 * t + 1];
        }
        gs_gravity(s);
        gs_viscosity(s);
        gs_predict(s);
        orc_hash(s, 1);
        gs_relax(s);
        gs_update_velocities(s);
        orc_hash(s, 0);
        if (diag) diagnostics(s, diag + 3 * t);
    }
}

/* Per-function entry, same numbering as the harness around the reference:
 * 0 gravity, 1 viscosity, 2 predict, 3 relaxation, 4 velocity update. */
void orc_call(void *h, int which)
{
    orc_sim *s = h;
    switch (which) {
    case 0: gs_gravity(s); break;
    case 1: gs_viscosity(s); break;
    case 2: gs_predict(s); break;
    case 3: gs_relax(s); break;
    case 4: gs_update_velocities(s); break;
    default: break;
    }
}

/* Copies the current half lists out (counts + concatenated ids). */
long orc_get_lists(void *h, int *counts, int *ids, long max_total)
{
    orc_sim *s = h;
    long total = 0;
    int i, j;
    for (i = 0; i < s->n; i++) {
        counts[i] = s->lst_cnt[i];
        if (total + s->lst_cnt[i] > max_total) return -1;
        for (j = 0; j < s->lst_cnt[i]; j++) ids[total++] = s->lst[(size_t)i * s->cfg.max_neighbors + j];
    }
    return total;
}

/* Packed render coordinates (fluid.c:356-362), by id. */
void orc_pack_coords(void *h, short *out)
{
    orc_sim *s = h;
    int i;
    for (i = 0; i < s->n; i++) {
        out[2 * i] = (short)((2.0f * s->x[i] / s->cfg.box[1] - 1.0f) * SHRT_MAX);
        out[2 * i + 1] = (short)((2.0f * s->y[i] / s->cfg.box[3] - 1.0f) * SHRT_MAX);
    }
}

/* ------------------------------------------------------------------ */
/* 2. FP64 gather (Jacobi) oracles over the symmetric closure           */
/* ------------------------------------------------------------------ */

/* Builds S_i = both directions of every listed pair.  sym_own[e] is 1 when
 * particle i holds the pair in its own half list (i.e. plays "p" in the
 * reference's loops), 0 when it is the listed neighbour "q". */
static void build_closure(orc_sim *s)
{
    const int n = s->n, mn = s->cfg.max_neighbors;
    long total = 0;
    int i, j;
    int *fill;
    for (i = 0; i <= n; i++) s->sym_off[i] = 0;
    for (i = 0; i < n; i++) {
        s->sym_off[i + 1] += s->lst_cnt[i];
        for (j = 0; j < s->lst_cnt[i]; j++) s->sym_off[s->lst[(size_t)i * mn + j] + 1]++;
    }
    for (i = 0; i < n; i++) s->sym_off[i + 1] += s->sym_off[i];
    total = s->sym_off[n];
    if (total > s->sym_cap) {
        free(s->sym_idx);
        free(s->sym_own);
        s->sym_cap = total + 1;
        s->sym_idx = malloc((size_t)s->sym_cap * sizeof(int));
        s->sym_own = malloc((size_t)s->sym_cap * sizeof(int));
    }
    fill = calloc((size_t)n, sizeof(int));
    for (i = 0; i < n; i++) {
        for (j = 0; j < s->lst_cnt[i]; j++) {
            const int q = s->lst[(size_t)i * mn + j];
            long e = s->sym_off[i] + fill[i]++;
            s->sym_idx[e] = q;
            s->sym_own[e] = 1;
            e = s->sym_off[q] + fill[q]++;
            s->sym_idx[e] = i;
            s->sym_own[e] = 0;
        }
    }
    free(fill);
}

/* Density and near density (fluid.c:527-539 summed over S_i), FP64. */
void orc_density_f64(void *h, double *rho, double *rhon)
{
    orc_sim *s = h;
    const double hh = s->tp.smoothing_radius;
    int i;
    long e;
    build_closure(s);
    for (i = 0; i < s->n; i++) {
        double a = 0.0, b = 0.0;
        for (e = s->sym_off[i]; e < s->sym_off[i + 1]; e++) {
            const int j = s->sym_idx[e];
            double dx = (double)s->x[i] - s->x[j], dy = (double)s->y[i] - s->y[j];
            double ratio = sqrt(dx * dx + dy * dy) / hh;
            if (ratio < 1.0) {
                a += (1.0 - ratio) * (1.0 - ratio);
                b += (1.0 - ratio) * (1.0 - ratio) * (1.0 - ratio);
            }
        }
        rho[i] = a;
        rhon[i] = b;
    }
}

/* Relaxation displacement in gather form (fluid.c:541-611 recast):
 *   dx_i = sum_{j in S_i, 0 < r < h} D_ij (x_i - x_j) / r
 *          + (1e-6, 1e-6) * #{j in S_i owned by i with r <= 1e-6}
 * with D_ij = dt^2 [ (P_i+P_j)(1-r/h) + (Pn_i+Pn_j)(1-r/h)^2 + k_spring (h-r)/2 ],
 * P = k (rho - rest), Pn = k_near rho_near, evaluated in FP64 from the given
 * float densities and the current float positions.  scale[i] bounds the
 * magnitude of the summed terms (absolute values), for relative tolerances. */
void orc_relax_f64(void *h, const float *rho, const float *rhon, double *dx, double *dy,
                   double *scale)
{
    orc_sim *s = h;
    const double k = s->tp.k, k_near = s->tp.k_near, k_spring = s->tp.k_spring;
    const double hh = s->tp.smoothing_radius, dt = s->tp.time_step, rest = s->tp.rest_density;
    int i;
    long e;
    build_closure(s);
    for (i = 0; i < s->n; i++) {
        const double Pi = k * ((double)rho[i] - rest), Pni = k_near * rhon[i];
        double ax = 0.0, ay = 0.0, sc = 0.0;
        int nudges = 0;
        for (e = s->sym_off[i]; e < s->sym_off[i + 1]; e++) {
            const int j = s->sym_idx[e];
            const double ex = (double)s->x[i] - s->x[j], ey = (double)s->y[i] - s->y[j];
            const double r = sqrt(ex * ex + ey * ey);
            const double omr = 1.0 - r / hh;
            if (r <= 0.000001 && s->sym_own[e]) nudges++;
            if (r / hh < 1.0 && r > 0.0) {
                const double Pj = k * ((double)rho[j] - rest), Pnj = k_near * rhon[j];
                const double D = dt * dt * ((Pi + Pj) * omr + (Pni + Pnj) * omr * omr +
                                            k_spring * (hh - r) * 0.5);
                ax += D * ex / r;
                ay += D * ey / r;
                sc += dt * dt * ((k * (fabs((double)rho[i]) + rest) +
                                  k * (fabs((double)rho[j]) + rest)) * omr +
                                 k_near * (fabs((double)rhon[i]) + fabs((double)rhon[j])) * omr * omr +
                                 fabs(k_spring) * (hh - r) * 0.5);
            }
        }
        dx[i] = ax + nudges * 0.000001;
        dy[i] = ay + nudges * 0.000001;
        scale[i] = sc + nudges * 0.000001;
    }
}

/* Viscosity velocity change in gather form (fluid.c:416-478 recast):
 *   dv_i = -1/2 sum_{j in S_i, u > 0} clamp5(I_ij),
 *   I_ij = dt (1 - r/h)(sigma u + beta u^2) (x_j - x_i)/r,
 *   u = ((v_i - v_j) . (x_j - x_i)) / r, from the velocities before the pass.
 * scale[i] = 1/2 sum |I_ij| (per-component bound, for relative tolerances). */
void orc_viscosity_f64(void *h, double *dvx, double *dvy, double *scale)
{
    orc_sim *s = h;
    const double hh = s->tp.smoothing_radius, dt = s->tp.time_step;
    const double sigma = s->tp.sigma, beta = s->tp.beta;
    int i;
    long e;
    build_closure(s);
    for (i = 0; i < s->n; i++) {
        double ax = 0.0, ay = 0.0, sc = 0.0;
        for (e = s->sym_off[i]; e < s->sym_off[i + 1]; e++) {
            const int j = s->sym_idx[e];
            const double qx = (double)s->x[j] - s->x[i], qy = (double)s->y[j] - s->y[i];
            const double r = sqrt(qx * qx + qy * qy);
            double u, imp, ix, iy;
            if (!(r > 0.0)) continue;
            u = (((double)s->vx[i] - s->vx[j]) * qx + ((double)s->vy[i] - s->vy[j]) * qy) / r;
            if (!(u > 0.0)) continue;
            imp = dt * (1.0 - r / hh) * (sigma * u + beta * u * u);
            ix = imp * qx / r;
            iy = imp * qy / r;
            if (ix > 5.0) ix = 5.0; else if (ix < -5.0) ix = -5.0;
            if (iy > 5.0) iy = 5.0; else if (iy < -5.0) iy = -5.0;
            ax -= 0.5 * ix;
            ay -= 0.5 * iy;
            sc += 0.5 * (fabs(ix) + fabs(iy)) + 0.5 * fabs(imp);
        }
        dvx[i] = ax;
        dvy[i] = ay;
        scale[i] = sc;
    }
}

/* ------------------------------------------------------------------ */
/* 3. float Jacobi step (the GPU's formulation) for drift studies       */
/* ------------------------------------------------------------------ */

static void jacobi_viscosity(orc_sim *s, float *nvx, float *nvy)
{
    const float h_recip = 1.0f / s->tp.smoothing_radius;
    const float sigma = s->tp.sigma, beta = s->tp.beta, dt = s->tp.time_step;
    int i;
    long e;
    build_closure(s);
    for (i = 0; i < s->n; i++) {
        float ax = 0.0f, ay = 0.0f;
        for (e = s->sym_off[i]; e < s->sym_off[i + 1]; e++) {
            const int j = s->sym_idx[e];
            float qx = s->x[j] - s->x[i], qy = s->y[j] - s->y[i];
            float r = sqrtf(qx * qx + qy * qy);
            float r_recip = 1.0f / r, ratio = r * h_recip;
            float u = ((s->vx[i] - s->vx[j]) * qx + (s->vy[i] - s->vy[j]) * qy) * r_recip;
            if (u > 0.0f) {
                float imp = dt * (1.0f - ratio) * (sigma * u + beta * u * u);
                float ix = imp * qx * r_recip, iy = imp * qy * r_recip;
                clamp5(&ix, &iy);
                ax -= ix * 0.5f;
                ay -= iy * 0.5f;
            }
        }
        nvx[i] = s->vx[i] + ax;
        nvy[i] = s->vy[i] + ay;
    }
}

static void jacobi_density(orc_sim *s)
{
    const float hh = s->tp.smoothing_radius, h_recip = 1.0f / hh;
    int i;
    long e;
    build_closure(s);
    for (i = 0; i < s->n; i++) {
        float a = 0.0f, b = 0.0f;
        for (e = s->sym_off[i]; e < s->sym_off[i + 1]; e++) {
            const int j = s->sym_idx[e];
            float dx = s->x[i] - s->x[j], dy = s->y[i] - s->y[j];
            float ratio = sqrtf(dx * dx + dy * dy) * h_recip;
            if (ratio < 1.0f) {
                float omr = 1.0f - ratio;
                a += omr * omr;
                b += omr * omr * omr;
            }
        }
        s->rho[i] = a;
        s->rhon[i] = b;
    }
}

static void jacobi_relax(orc_sim *s, float *nx, float *ny)
{
    const float k = s->tp.k, k_near = s->tp.k_near, k_spring = s->tp.k_spring;
    const float hh = s->tp.smoothing_radius, h_recip = 1.0f / hh;
    const float dt = s->tp.time_step, rest = s->tp.rest_density;
    int i;
    long e;
    for (i = 0; i < s->n; i++) {
        s->P[i] = k * (s->rho[i] - rest);
        s->Pn[i] = k_near * s->rhon[i];
    }
    for (i = 0; i < s->n; i++) {
        float ax = 0.0f, ay = 0.0f;
        int nudges = 0;
        for (e = s->sym_off[i]; e < s->sym_off[i + 1]; e++) {
            const int j = s->sym_idx[e];
            float ex = s->x[i] - s->x[j], ey = s->y[i] - s->y[j];
            float r = sqrtf(ex * ex + ey * ey);
            float ratio = r * h_recip, omr = 1.0f - ratio;
            if (r <= 0.000001f && s->sym_own[e]) nudges++;
            if (ratio < 1.0f && r > 0.0f) {
                float D = dt * dt * ((s->P[i] + s->P[j]) * omr + (s->Pn[i] + s->Pn[j]) * omr * omr +
                                     k_spring * (hh - r) * 0.5f);
                ax += D * ex / r;
                ay += D * ey / r;
            }
        }
        nx[i] = s->x[i] + ax + nudges * 0.000001f;
        ny[i] = s->y[i] + ay + nudges * 0.000001f;
    }
}

/* Same sequence as orc_step with the viscosity, density and relaxation
 * passes in gather (Jacobi) form: the formulation the CUDA library uses. */
/* One float Jacobi step.  With `after`, the tunables are replaced after
 * predict_positions and before the hash, the relaxation and the velocity
 * update, where the reference's compute rank receives new tunables inside a
 * step (the MPI_Scatterv of fluid.c:293-294). */
static void jacobi_step(orc_sim *s, float *ta, float *tb, const orc_tunables *after)
{
    int i;
    gs_gravity(s);
    jacobi_viscosity(s, ta, tb);
    memcpy(s->vx, ta, (size_t)s->n * sizeof(float));
    memcpy(s->vy, tb, (size_t)s->n * sizeof(float));
    gs_predict(s);
    if (after) s->tp = *after;
    orc_hash(s, 0);
    jacobi_density(s);
    jacobi_relax(s, ta, tb);
    for (i = 0; i < s->n; i++) {
        s->x[i] = ta[i];
        s->y[i] = tb[i];
    }
    gs_update_velocities(s);
    orc_hash(s, 0);
}

void orc_step_jacobi(void *h, int nsteps, const float *mover_xy, double *diag)
{
    orc_sim *s = h;
    float *ta = malloc((size_t)s->n * sizeof(float));
    float *tb = malloc((size_t)s->n * sizeof(float));
    int t;
    for (t = 0; t < nsteps; t++) {
        if (mover_xy) {
            s->tp.mover_center_x = mover_xy[2 * t];
            s->tp.mover_center_y = mover_xy[2 * t + 1];
        }
        jacobi_step(s, ta, tb, NULL);
        if (diag) diagnostics(s, diag + 3 * t);
    }
    free(ta);
    free(tb);
}

/* One Jacobi step whose tunables switch inside it: `before` (NULL keeps the
 * current ones) for gravity, viscosity and prediction, `after` from the
 * hash on, and for the steps that follow. */
void orc_step_jacobi_split(void *h, const orc_tunables *before, const orc_tunables *after)
{
    orc_sim *s = h;
    float *ta = malloc((size_t)s->n * sizeof(float));
    float *tb = malloc((size_t)s->n * sizeof(float));
    if (before) s->tp = *before;
    jacobi_step(s, ta, tb, after);
    free(ta);
    free(tb);
}

/* Zeroes the densities (as apply_gravity does, fluid.c:410-411) and runs
 * the hash on the current positions: the same contract as ref_hash(). */
void orc_hash_fresh(void *h, int compute_density)
{
    orc_sim *s = h;
    int i;
    for (i = 0; i < s->n; i++) {
        s->rho[i] = 0.0f;
        s->rhon[i] = 0.0f;
    }
    orc_hash(s, compute_density);
}
