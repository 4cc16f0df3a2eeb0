// sph_legacy.cu -- the reference-named entry points (include/sph_legacy.h).
//
// Each call gathers the fields it reads from the caller's structs into a
// pinned staging buffer, copies them to the device, runs its kernel, and
// writes the fields the reference writes back through the same pointers.
// The arithmetic is the step kernels' (sph_device.cuh); the only host work is
// packing/unpacking the structs and turning pointer lists into index lists.
#include <cstring>
#include <mutex>
#include <vector>

#include "sph_device.cuh"
#include "sph_legacy.h"

namespace sph {
namespace {

thread_local int g_status = SPH_OK;

struct LegacyCtx {
    std::mutex mu;
    cudaStream_t stream = nullptr;
    void *dbuf = nullptr;
    size_t dbytes = 0;
    void *hbuf = nullptr;
    size_t hbytes = 0;
    sph_cuda *hash = nullptr;  // handle used by hash_fluid
    float spacing = 0.0f;
    unsigned sx = 0, sy = 0, mb = 0, mn = 0;
    int cap = 0;
};

LegacyCtx &ctx()
{
    static LegacyCtx c;
    return c;
}

int set(int st)
{
    g_status = st;
    return st;
}

int prepare(LegacyCtx &c, size_t dev_bytes, size_t host_bytes)
{
    if (!c.stream) {
        const int rc = cuda_fail(cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking),
                                 "cudaStreamCreate");
        if (rc) return rc;
    }
    if (dev_bytes > c.dbytes) {
        if (c.dbuf) cudaFree(c.dbuf);
        c.dbuf = nullptr;
        c.dbytes = 0;
        const int rc = cuda_fail(cudaMalloc(&c.dbuf, dev_bytes), "cudaMalloc");
        if (rc) return rc;
        c.dbytes = dev_bytes;
    }
    if (host_bytes > c.hbytes) {
        if (c.hbuf) cudaFreeHost(c.hbuf);
        c.hbuf = nullptr;
        c.hbytes = 0;
        const int rc = cuda_fail(cudaHostAlloc(&c.hbuf, host_bytes, cudaHostAllocDefault),
                                 "cudaHostAlloc");
        if (rc) return rc;
        c.hbytes = host_bytes;
    }
    return SPH_OK;
}

float4 box_grid(const AABB_t *b) { return make_float4(b->min_x, b->max_x, b->min_y, b->max_y); }

inline int blocks(int n) { return (n + kBlock - 1) / kBlock; }

// ---- kernels ---------------------------------------------------------------

__global__ void kl_gravity(int n, float g, float dt, float2 *vel, float2 *rho)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    vel[i].y = __fadd_rn(vel[i].y, __fmul_rn(-g, dt));
    rho[i] = make_float2(0.0f, 0.0f);
}

__global__ void kl_predict(int n, tunable_parameters P, float4 g, float2 *pos, const float2 *vel,
                           float2 *prev)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float2 p = pos[i], v = vel[i];
    prev[i] = p;
    float x = __fadd_rn(p.x, __fmul_rn(v.x, P.time_step));
    float y = __fadd_rn(p.y, __fmul_rn(v.y, P.time_step));
    boundary(x, y, P, g);
    pos[i] = make_float2(x, y);
}

// updateVelocity (fluid.c:627-639), after boundaryConditions when `bc`.
__global__ void kl_velocity(int n, tunable_parameters P, float4 g, int bc, float2 *pos,
                            const float2 *prev, float2 *vel)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    float x = pos[i].x, y = pos[i].y;
    if (bc) boundary(x, y, P, g);
    pos[i] = make_float2(x, y);
    const float2 q = prev[i];
    vel[i] = make_float2(clamp5(__fdiv_rn(__fsub_rn(x, q.x), P.time_step)),
                         clamp5(__fdiv_rn(__fsub_rn(y, q.y), P.time_step)));
}

__global__ void kl_boundary(tunable_parameters P, float4 g, float2 *pos)
{
    float x = pos->x, y = pos->y;
    boundary(x, y, P, g);
    *pos = make_float2(x, y);
}

__global__ void kl_clamp(float2 *v) { *v = make_float2(clamp5(v->x), clamp5(v->y)); }

// calculate_density (fluid.c:527-539) on the pair's two density records.
__global__ void kl_pair_density(float ratio, float2 *rp, float2 *rq)
{
    const float omr2 = __fmul_rn(__fsub_rn(1.0f, ratio), __fsub_rn(1.0f, ratio));
    if (ratio < 1.0f) {
        const float omr3 = __fmul_rn(omr2, __fsub_rn(1.0f, ratio));
        *rp = make_float2(__fadd_rn(rp->x, omr2), __fadd_rn(rp->y, omr3));
        *rq = make_float2(__fadd_rn(rq->x, omr2), __fadd_rn(rq->y, omr3));
    }
}

// hash_val (hash.c:35-47) with its unsigned arithmetic; negative/NaN -> ~0u.
__global__ void kl_hash_val(float x, float y, float spacing, unsigned size_x, unsigned *out)
{
    const float fx = floorf(__fdiv_rn(x, spacing)), fy = floorf(__fdiv_rn(y, spacing));
    if (!(fx >= 0.0f) || !(fy >= 0.0f) || fx >= 4294967296.0f || fy >= 4294967296.0f) {
        *out = 0xFFFFFFFFu;
        return;
    }
    *out = (unsigned)fy * size_x + (unsigned)fx;
}

__global__ void kl_count_outside(int n, float lo, float hi, const float2 *pos, unsigned *count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float x = pos[i].x;
    if (x < lo || x > hi) atomicAdd(count, 1u);
}

// Viscosity in gather form over explicit lists (CSR of the symmetric closure
// of the caller's half lists): dv_i = -1/2 sum_j clamp5(I_ij).
__global__ void kl_list_viscosity(int n, tunable_parameters P, const float2 *pos,
                                  const float2 *vel, const int *off, const int *nbr,
                                  float2 *vel_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float dt = P.time_step, h_recip = __fdiv_rn(1.0f, P.smoothing_radius);
    const float2 p = pos[i], v = vel[i];
    float dvx = 0.0f, dvy = 0.0f;
    for (int e = off[i]; e < off[i + 1]; ++e) {
        const int j = nbr[e];
        const float2 q = pos[j], w = vel[j];
        const float qx = q.x - p.x, qy = q.y - p.y;
        const float r2 = dist2(qx, qy);
        if (!(r2 > 0.0f)) continue;
        const float r_recip = rsqrtf(r2), r = r2 * r_recip;
        const float u = ((v.x - w.x) * qx + (v.y - w.y) * qy) * r_recip;
        if (u > 0.0f) {
            const float imp = dt * (1.0f - r * h_recip) * (P.sigma * u + P.beta * u * u);
            dvx -= 0.5f * clamp5(imp * qx * r_recip);
            dvy -= 0.5f * clamp5(imp * qy * r_recip);
        }
    }
    vel_out[i] = make_float2(__fadd_rn(v.x, dvx), __fadd_rn(v.y, dvy));
}

// Relaxation in gather form over explicit lists; own[e] marks pairs the
// particle holds in its own half list (it receives the r <= 1e-6 nudge).
// Also writes the pressures (fluid.c:560-565).
__global__ void kl_list_relax(int n, tunable_parameters P, const float2 *pos, const float2 *rho,
                              const int *off, const int *nbr, const unsigned char *own,
                              float2 *pos_out, float2 *press_out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float hh = P.smoothing_radius, h_recip = __fdiv_rn(1.0f, hh);
    const float dt2 = P.time_step * P.time_step, half_spring = 0.5f * P.k_spring;
    const float2 p = pos[i], rp = rho[i];
    const float Pi = __fmul_rn(P.k, __fsub_rn(rp.x, P.rest_density));
    const float Pni = __fmul_rn(P.k_near, rp.y);
    press_out[i] = make_float2(Pi, Pni);
    float ax = 0.0f, ay = 0.0f;
    int nudges = 0;
    for (int e = off[i]; e < off[i + 1]; ++e) {
        const int j = nbr[e];
        const float2 q = pos[j], rq = rho[j];
        const float ex = p.x - q.x, ey = p.y - q.y;
        const float r2 = dist2(ex, ey);
        const float r = r2 > 0.0f ? __fsqrt_rn(r2) : 0.0f;
        if (r <= 0.000001f && own[e]) ++nudges;
        const float ratio = r * h_recip;
        if (ratio < 1.0f && r > 0.0f) {
            const float omr = 1.0f - ratio;
            const float Pj = __fmul_rn(P.k, __fsub_rn(rq.x, P.rest_density));
            const float Pnj = __fmul_rn(P.k_near, rq.y);
            const float D = dt2 * ((Pi + Pj) * omr + (Pni + Pnj) * omr * omr + half_spring * (hh - r));
            ax += D * ex / r;
            ay += D * ey / r;
        }
    }
    const float nd = (float)nudges * 0.000001f;
    pos_out[i] = make_float2(__fadd_rn(__fadd_rn(p.x, ax), nd), __fadd_rn(__fadd_rn(p.y, ay), nd));
}

// ---- host helpers -----------------------------------------------------------

template <class T>
T *carve(char *&p, size_t count)
{
    T *r = reinterpret_cast<T *>(p);
    p += ((count * sizeof(T)) + 255) & ~(size_t)255;
    return r;
}

size_t span(size_t count, size_t elem) { return ((count * elem) + 255) & ~(size_t)255; }

// Symmetric closure of the caller's half lists as CSR over particle indices.
int build_closure(fluid_particle *const *ptrs, const neighbor *nb, int n, std::vector<int> &off,
                  std::vector<int> &idx, std::vector<unsigned char> &own)
{
    off.assign((size_t)n + 1, 0);
    for (int i = 0; i < n; ++i) {
        for (int k = 0; k < nb[i].number_fluid_neighbors; ++k) {
            const fluid_particle *q = nb[i].fluid_neighbors[k];
            if (!q || q->id < 0 || q->id >= n) {
                set_error("neighbour %d of particle %d is not a local particle (halo particles are "
                          "not supported on a single-device domain)", k, i);
                return SPH_ERR_UNSUPPORTED;
            }
            off[i + 1]++;
            off[q->id + 1]++;
        }
    }
    for (int i = 0; i < n; ++i) off[i + 1] += off[i];
    idx.assign((size_t)off[n], 0);
    own.assign((size_t)off[n], 0);
    std::vector<int> fill(off.begin(), off.end() - 1);
    for (int i = 0; i < n; ++i) {
        for (int k = 0; k < nb[i].number_fluid_neighbors; ++k) {
            const int j = nb[i].fluid_neighbors[k]->id;
            idx[fill[i]] = j;
            own[fill[i]++] = 1;
            idx[fill[j]] = i;
            own[fill[j]++] = 0;
        }
    }
    return SPH_OK;
}

int sync(LegacyCtx &c) { return cuda_fail(cudaStreamSynchronize(c.stream), "legacy sync"); }

int check_ptrs(fluid_particle *const *ptrs, int n)
{
    if (n < 0) {
        set_error("negative particle count %d", n);
        return SPH_ERR_INVALID;
    }
    if (n > 0 && !ptrs) {
        set_error("null particle pointer array");
        return SPH_ERR_INVALID;
    }
    for (int i = 0; i < n; ++i)
        if (!ptrs[i]) {
            set_error("particle pointer %d is NULL", i);
            return SPH_ERR_INVALID;
        }
    return SPH_OK;
}

#define LTRY(expr)                        \
    do {                                  \
        const int _rc = (expr);           \
        if (_rc != SPH_OK) return set(_rc); \
    } while (0)

}  // namespace
}  // namespace sph

using namespace sph;

extern "C" {

int sph_legacy_status(void) { return g_status; }

void apply_gravity(fluid_particle **ptrs, param *params)
{
    [&]() -> int {
        if (!params) return set(SPH_ERR_INVALID);
        const int n = params->number_fluid_particles_local + params->number_halo_particles;
        LTRY(check_ptrs(ptrs, n));
        if (n == 0) return set(SPH_OK);
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        LTRY(prepare(c, 2 * span(n, sizeof(float2)), 2 * (size_t)n * sizeof(float2)));
        float2 *hv = (float2 *)c.hbuf, *hr = hv + n;
        for (int i = 0; i < n; ++i) hv[i] = make_float2(ptrs[i]->v_x, ptrs[i]->v_y);
        char *d = (char *)c.dbuf;
        float2 *dv = carve<float2>(d, n), *dr = carve<float2>(d, n);
        LTRY(cuda_fail(cudaMemcpyAsync(dv, hv, n * sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        kl_gravity<<<blocks(n), kBlock, 0, c.stream>>>(n, params->tunable_params.g,
                                                       params->tunable_params.time_step, dv, dr);
        LTRY(cuda_fail(cudaMemcpyAsync(hv, dv, n * sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(cuda_fail(cudaMemcpyAsync(hr, dr, n * sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(sync(c));
        for (int i = 0; i < n; ++i) {
            ptrs[i]->v_y = hv[i].y;
            ptrs[i]->density = hr[i].x;
            ptrs[i]->density_near = hr[i].y;
        }
        return set(SPH_OK);
    }();
}

void predict_positions(fluid_particle **ptrs, AABB_t *boundary_global, param *params)
{
    [&]() -> int {
        if (!params || !boundary_global) return set(SPH_ERR_INVALID);
        const int n = params->number_fluid_particles_local;
        LTRY(check_ptrs(ptrs, n));
        if (n == 0) return set(SPH_OK);
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        LTRY(prepare(c, 3 * span(n, sizeof(float2)), 3 * (size_t)n * sizeof(float2)));
        float2 *hp = (float2 *)c.hbuf, *hv = hp + n, *hq = hv + n;
        for (int i = 0; i < n; ++i) {
            hp[i] = make_float2(ptrs[i]->x, ptrs[i]->y);
            hv[i] = make_float2(ptrs[i]->v_x, ptrs[i]->v_y);
        }
        char *d = (char *)c.dbuf;
        float2 *dp = carve<float2>(d, n), *dv = carve<float2>(d, n), *dq = carve<float2>(d, n);
        LTRY(cuda_fail(cudaMemcpyAsync(dp, hp, 2 * n * sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        LTRY(cuda_fail(cudaMemcpyAsync(dv, hv, n * sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        kl_predict<<<blocks(n), kBlock, 0, c.stream>>>(n, params->tunable_params,
                                                       box_grid(boundary_global), dp, dv, dq);
        LTRY(cuda_fail(cudaMemcpyAsync(hp, dp, n * sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(cuda_fail(cudaMemcpyAsync(hq, dq, n * sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(sync(c));
        for (int i = 0; i < n; ++i) {
            ptrs[i]->x_prev = hq[i].x;
            ptrs[i]->y_prev = hq[i].y;
            ptrs[i]->x = hp[i].x;
            ptrs[i]->y = hp[i].y;
        }
        return set(SPH_OK);
    }();
}

void updateVelocities(fluid_particle **ptrs, edge_t *edges, AABB_t *boundary_global, param *params)
{
    (void)edges;
    [&]() -> int {
        if (!params || !boundary_global) return set(SPH_ERR_INVALID);
        const int n = params->number_fluid_particles_local;
        LTRY(check_ptrs(ptrs, n));
        if (n == 0) return set(SPH_OK);
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        LTRY(prepare(c, 3 * span(n, sizeof(float2)), 3 * (size_t)n * sizeof(float2)));
        float2 *hp = (float2 *)c.hbuf, *hq = hp + n, *hv = hq + n;
        for (int i = 0; i < n; ++i) {
            hp[i] = make_float2(ptrs[i]->x, ptrs[i]->y);
            hq[i] = make_float2(ptrs[i]->x_prev, ptrs[i]->y_prev);
        }
        char *d = (char *)c.dbuf;
        float2 *dp = carve<float2>(d, n), *dq = carve<float2>(d, n), *dv = carve<float2>(d, n);
        LTRY(cuda_fail(cudaMemcpyAsync(dp, hp, n * sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        LTRY(cuda_fail(cudaMemcpyAsync(dq, hq, n * sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        kl_velocity<<<blocks(n), kBlock, 0, c.stream>>>(n, params->tunable_params,
                                                        box_grid(boundary_global), 1, dp, dq, dv);
        LTRY(cuda_fail(cudaMemcpyAsync(hp, dp, n * sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(cuda_fail(cudaMemcpyAsync(hv, dv, n * sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(sync(c));
        for (int i = 0; i < n; ++i) {
            ptrs[i]->x = hp[i].x;
            ptrs[i]->y = hp[i].y;
            ptrs[i]->v_x = hv[i].x;
            ptrs[i]->v_y = hv[i].y;
        }
        return set(SPH_OK);
    }();
}

void viscosity_impluses(fluid_particle **ptrs, neighbor *neighbors, param *params)
{
    [&]() -> int {
        if (!params || !neighbors) return set(SPH_ERR_INVALID);
        const int n = params->number_fluid_particles_local;
        LTRY(check_ptrs(ptrs, n));
        if (n == 0) return set(SPH_OK);
        std::vector<int> off, idx;
        std::vector<unsigned char> own;
        LTRY(build_closure(ptrs, neighbors, n, off, idx, own));
        const size_t ne = idx.size();
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        LTRY(prepare(c, 3 * span(n, sizeof(float2)) + span(n + 1, 4) + span(ne + 1, 4),
                     3 * (size_t)n * sizeof(float2)));
        float2 *hp = (float2 *)c.hbuf, *hv = hp + n;
        for (int i = 0; i < n; ++i) {
            hp[i] = make_float2(ptrs[i]->x, ptrs[i]->y);
            hv[i] = make_float2(ptrs[i]->v_x, ptrs[i]->v_y);
        }
        char *d = (char *)c.dbuf;
        float2 *dp = carve<float2>(d, n), *dv = carve<float2>(d, n), *dout = carve<float2>(d, n);
        int *doff = carve<int>(d, n + 1), *didx = carve<int>(d, ne + 1);
        LTRY(cuda_fail(cudaMemcpyAsync(dp, hp, n * sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        LTRY(cuda_fail(cudaMemcpyAsync(dv, hv, n * sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        LTRY(cuda_fail(cudaMemcpyAsync(doff, off.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice, c.stream), "H2D"));
        if (ne) LTRY(cuda_fail(cudaMemcpyAsync(didx, idx.data(), ne * sizeof(int), cudaMemcpyHostToDevice, c.stream), "H2D"));
        kl_list_viscosity<<<blocks(n), kBlock, 0, c.stream>>>(n, params->tunable_params, dp, dv,
                                                              doff, didx, dout);
        LTRY(cuda_fail(cudaMemcpyAsync(hv, dout, n * sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(sync(c));  // also orders the pageable index copies before vector release
        for (int i = 0; i < n; ++i) {
            ptrs[i]->v_x = hv[i].x;
            ptrs[i]->v_y = hv[i].y;
        }
        return set(SPH_OK);
    }();
}

void double_density_relaxation(fluid_particle **ptrs, neighbor *neighbors, param *params)
{
    [&]() -> int {
        if (!params || !neighbors) return set(SPH_ERR_INVALID);
        if (params->number_halo_particles != 0) {
            set_error("halo particles are not supported on a single-device domain");
            return set(SPH_ERR_UNSUPPORTED);
        }
        const int n = params->number_fluid_particles_local;
        LTRY(check_ptrs(ptrs, n));
        if (n == 0) return set(SPH_OK);
        std::vector<int> off, idx;
        std::vector<unsigned char> own;
        LTRY(build_closure(ptrs, neighbors, n, off, idx, own));
        const size_t ne = idx.size();
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        LTRY(prepare(c, 4 * span(n, sizeof(float2)) + span(n + 1, 4) + span(ne + 1, 4) + span(ne + 1, 1),
                     4 * (size_t)n * sizeof(float2)));
        float2 *hp = (float2 *)c.hbuf, *hr = hp + n, *hpr = hr + n;
        for (int i = 0; i < n; ++i) {
            hp[i] = make_float2(ptrs[i]->x, ptrs[i]->y);
            hr[i] = make_float2(ptrs[i]->density, ptrs[i]->density_near);
        }
        char *d = (char *)c.dbuf;
        float2 *dp = carve<float2>(d, n), *dr = carve<float2>(d, n), *dout = carve<float2>(d, n);
        float2 *dpr = carve<float2>(d, n);
        int *doff = carve<int>(d, n + 1), *didx = carve<int>(d, ne + 1);
        unsigned char *down = carve<unsigned char>(d, ne + 1);
        LTRY(cuda_fail(cudaMemcpyAsync(dp, hp, n * sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        LTRY(cuda_fail(cudaMemcpyAsync(dr, hr, n * sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        LTRY(cuda_fail(cudaMemcpyAsync(doff, off.data(), (n + 1) * sizeof(int), cudaMemcpyHostToDevice, c.stream), "H2D"));
        if (ne) {
            LTRY(cuda_fail(cudaMemcpyAsync(didx, idx.data(), ne * sizeof(int), cudaMemcpyHostToDevice, c.stream), "H2D"));
            LTRY(cuda_fail(cudaMemcpyAsync(down, own.data(), ne, cudaMemcpyHostToDevice, c.stream), "H2D"));
        }
        kl_list_relax<<<blocks(n), kBlock, 0, c.stream>>>(n, params->tunable_params, dp, dr, doff,
                                                          didx, down, dout, dpr);
        LTRY(cuda_fail(cudaMemcpyAsync(hp, dout, n * sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(cuda_fail(cudaMemcpyAsync(hpr, dpr, n * sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(sync(c));
        for (int i = 0; i < n; ++i) {
            ptrs[i]->x = hp[i].x;
            ptrs[i]->y = hp[i].y;
            ptrs[i]->pressure = hpr[i].x;
            ptrs[i]->pressure_near = hpr[i].y;
        }
        return set(SPH_OK);
    }();
}

void hash_fluid(fluid_particle **ptrs, neighbor_grid_t *grid, param *params, bool compute_density)
{
    [&]() -> int {
        if (!params || !grid || !grid->neighbors || !grid->grid_buckets) return set(SPH_ERR_INVALID);
        const int n = params->number_fluid_particles_local;
        LTRY(check_ptrs(ptrs, n));
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        const bool same = c.hash && c.spacing == grid->spacing && c.sx == grid->size_x &&
                          c.sy == grid->size_y && c.mb == grid->max_bucket_size &&
                          c.mn == grid->max_neighbors && c.cap >= n;
        if (!same) {
            if (c.hash) sph_cuda_destroy(c.hash);
            c.hash = nullptr;
            AABB_t box{};
            box.max_x = grid->spacing * grid->size_x;
            box.max_y = grid->spacing * grid->size_y;
            param p = *params;
            p.number_halo_particles = 0;
            LTRY(sph_cuda_create(&c.hash, &p, &box, grid, n > 0 ? n : 1));
            c.spacing = grid->spacing;
            c.sx = grid->size_x;
            c.sy = grid->size_y;
            c.mb = grid->max_bucket_size;
            c.mn = grid->max_neighbors;
            c.cap = n > 0 ? n : 1;
        }
        sph_cuda *h = c.hash;
        LTRY(sph_cuda_upload(h, ptrs, n));
        // half lists in the reference's order (hash.c:169-234)
        std::vector<int> counts((size_t)n + 1), off((size_t)n + 1, 0);
        long long total = 0;
        if (n > 0) {
            const int rc = sph_cuda_neighbor_lists(h, counts.data(), nullptr, 0, &total);
            if (rc != SPH_OK && rc != SPH_ERR_CAPACITY) return set(rc);
        }
        std::vector<int> ids((size_t)total + 1);
        if (n > 0) LTRY(sph_cuda_neighbor_lists(h, counts.data(), ids.data(), total, &total));
        long long o = 0;
        for (int i = 0; i < n; ++i) {
            neighbor *ne = &grid->neighbors[i];
            ne->number_fluid_neighbors = counts[i];
            for (int k = 0; k < counts[i]; ++k) ne->fluid_neighbors[k] = ptrs[ids[o + k]];
            o += counts[i];
        }
        // buckets (hash.c:147-166): each cell's first max_bucket_size members, id order
        const size_t cells = (size_t)grid->size_x * grid->size_y;
        std::vector<int> start(cells + 2), sorted((size_t)n + 1);
        LTRY(cuda_fail(cudaMemcpyAsync(start.data(), h->start_a, (cells + 2) * sizeof(int),
                                       cudaMemcpyDeviceToHost, h->stream), "D2H"));
        if (n > 0)
            LTRY(cuda_fail(cudaMemcpyAsync(sorted.data(), h->id_a, (size_t)n * sizeof(int),
                                           cudaMemcpyDeviceToHost, h->stream), "D2H"));
        LTRY(cuda_fail(cudaStreamSynchronize(h->stream), "D2H sync"));
        for (size_t cc = 0; cc < cells; ++cc) {
            bucket_t *b = &grid->grid_buckets[cc];
            const int m0 = start[cc + 1] - start[cc];
            const int m = m0 < (int)grid->max_bucket_size ? m0 : (int)grid->max_bucket_size;
            b->number_fluid = (unsigned)m;
            for (int k = 0; k < m; ++k) b->fluid_particles[k] = ptrs[sorted[start[cc] + k]];
        }
        if (compute_density && n > 0) {
            std::vector<float> rho((size_t)n), rhon((size_t)n);
            LTRY(sph_cuda_probe_density(h, &params->tunable_params, rho.data(), rhon.data()));
            // calculate_density accumulates into the existing values (fluid.c:532-536)
            for (int i = 0; i < n; ++i) {
                ptrs[i]->density += rho[i];
                ptrs[i]->density_near += rhon[i];
            }
        }
        return set(SPH_OK);
    }();
}

void hash_halo(fluid_particle **ptrs, neighbor_grid_t *grid, param *params, bool compute_density)
{
    (void)ptrs;
    (void)grid;
    (void)compute_density;
    if (!params) {
        set(SPH_ERR_INVALID);
        return;
    }
    if (params->number_halo_particles != 0) {
        set_error("hash_halo: %d halo particles; a single-device domain has none",
                  params->number_halo_particles);
        set(SPH_ERR_UNSUPPORTED);
        return;
    }
    set(SPH_OK);
}

void identify_oob_particles(fluid_particle **ptrs, fluid_particle *fluid_particles,
                            oob_t *out_of_bounds, AABB_t *boundary_global, param *params)
{
    (void)fluid_particles;
    (void)out_of_bounds;
    (void)boundary_global;
    [&]() -> int {
        if (!params) return set(SPH_ERR_INVALID);
        const int n = params->number_fluid_particles_local;
        LTRY(check_ptrs(ptrs, n));
        if (n == 0) return set(SPH_OK);
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        LTRY(prepare(c, span(n, sizeof(float2)) + span(1, 4), (size_t)n * sizeof(float2) + 16));
        float2 *hp = (float2 *)c.hbuf;
        for (int i = 0; i < n; ++i) hp[i] = make_float2(ptrs[i]->x, ptrs[i]->y);
        char *d = (char *)c.dbuf;
        float2 *dp = carve<float2>(d, n);
        unsigned *dc = carve<unsigned>(d, 1);
        LTRY(cuda_fail(cudaMemsetAsync(dc, 0, sizeof(unsigned), c.stream), "memset"));
        LTRY(cuda_fail(cudaMemcpyAsync(dp, hp, n * sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        kl_count_outside<<<blocks(n), kBlock, 0, c.stream>>>(n, params->tunable_params.node_start_x,
                                                             params->tunable_params.node_end_x, dp, dc);
        unsigned outside = 0;
        LTRY(cuda_fail(cudaMemcpyAsync(&outside, dc, sizeof(unsigned), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(sync(c));
        if (outside) {
            set_error("%u particles left [node_start_x, node_end_x]; a single-device domain has no "
                      "neighbour to send them to", outside);
            return set(SPH_ERR_UNSUPPORTED);
        }
        return set(SPH_OK);
    }();
}

// ---- single-particle functions --------------------------------------------

void boundaryConditions(fluid_particle *p, AABB_t *boundary, param *params)
{
    [&]() -> int {
        if (!p || !boundary || !params) return set(SPH_ERR_INVALID);
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        LTRY(prepare(c, 256, 64));
        float2 *hp = (float2 *)c.hbuf;
        *hp = make_float2(p->x, p->y);
        float2 *dp = (float2 *)c.dbuf;
        LTRY(cuda_fail(cudaMemcpyAsync(dp, hp, sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        kl_boundary<<<1, 1, 0, c.stream>>>(params->tunable_params, box_grid(boundary), dp);
        LTRY(cuda_fail(cudaMemcpyAsync(hp, dp, sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(sync(c));
        p->x = hp->x;
        p->y = hp->y;
        return set(SPH_OK);
    }();
}

void updateVelocity(fluid_particle *p, param *params)
{
    [&]() -> int {
        if (!p || !params) return set(SPH_ERR_INVALID);
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        LTRY(prepare(c, 3 * 256, 64));
        float2 *h = (float2 *)c.hbuf;
        h[0] = make_float2(p->x, p->y);
        h[1] = make_float2(p->x_prev, p->y_prev);
        char *d = (char *)c.dbuf;
        float2 *dp = carve<float2>(d, 1), *dq = carve<float2>(d, 1), *dv = carve<float2>(d, 1);
        LTRY(cuda_fail(cudaMemcpyAsync(dp, &h[0], sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        LTRY(cuda_fail(cudaMemcpyAsync(dq, &h[1], sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        kl_velocity<<<1, 32, 0, c.stream>>>(1, params->tunable_params, float4{}, 0, dp, dq, dv);
        LTRY(cuda_fail(cudaMemcpyAsync(&h[2], dv, sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(sync(c));
        p->v_x = h[2].x;
        p->v_y = h[2].y;
        return set(SPH_OK);
    }();
}

void checkVelocity(float *v_x, float *v_y)
{
    [&]() -> int {
        if (!v_x || !v_y) return set(SPH_ERR_INVALID);
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        LTRY(prepare(c, 256, 64));
        float2 *h = (float2 *)c.hbuf;
        *h = make_float2(*v_x, *v_y);
        float2 *dv = (float2 *)c.dbuf;
        LTRY(cuda_fail(cudaMemcpyAsync(dv, h, sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        kl_clamp<<<1, 1, 0, c.stream>>>(dv);
        LTRY(cuda_fail(cudaMemcpyAsync(h, dv, sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(sync(c));
        *v_x = h->x;
        *v_y = h->y;
        return set(SPH_OK);
    }();
}

void calculate_density(fluid_particle *p, fluid_particle *q, float ratio)
{
    [&]() -> int {
        if (!p || !q) return set(SPH_ERR_INVALID);
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        LTRY(prepare(c, 2 * 256, 64));
        float2 *h = (float2 *)c.hbuf;
        h[0] = make_float2(p->density, p->density_near);
        h[1] = make_float2(q->density, q->density_near);
        char *d = (char *)c.dbuf;
        float2 *dp = carve<float2>(d, 1), *dq = carve<float2>(d, 1);
        LTRY(cuda_fail(cudaMemcpyAsync(dp, &h[0], sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        LTRY(cuda_fail(cudaMemcpyAsync(dq, &h[1], sizeof(float2), cudaMemcpyHostToDevice, c.stream), "H2D"));
        kl_pair_density<<<1, 1, 0, c.stream>>>(ratio, dp, dq);
        LTRY(cuda_fail(cudaMemcpyAsync(&h[0], dp, sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(cuda_fail(cudaMemcpyAsync(&h[1], dq, sizeof(float2), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(sync(c));
        p->density = h[0].x;
        p->density_near = h[0].y;
        q->density = h[1].x;
        q->density_near = h[1].y;
        return set(SPH_OK);
    }();
}

unsigned int hash_val(float x, float y, neighbor_grid_t *grid, param *params)
{
    (void)params;
    unsigned out = 0xFFFFFFFFu;
    [&]() -> int {
        if (!grid) return set(SPH_ERR_INVALID);
        LegacyCtx &c = ctx();
        std::lock_guard<std::mutex> lock(c.mu);
        LTRY(prepare(c, 256, 64));
        unsigned *d = (unsigned *)c.dbuf;
        kl_hash_val<<<1, 1, 0, c.stream>>>(x, y, grid->spacing, grid->size_x, d);
        LTRY(cuda_fail(cudaMemcpyAsync(c.hbuf, d, sizeof(unsigned), cudaMemcpyDeviceToHost, c.stream), "D2H"));
        LTRY(sync(c));
        out = *(unsigned *)c.hbuf;
        return set(SPH_OK);
    }();
    return out;
}

}  // extern "C"
