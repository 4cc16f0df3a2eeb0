// sph_capi.cu -- handle lifecycle and the device-resident C API of libsph_cuda.
#include <algorithm>
#include <atomic>
#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cmath>
#include <cstring>
#include <new>

#include "sph_internal.h"

namespace sph {

// kernels.cu
int launch_unpermute(sph_cuda *h, float2 *out);
int launch_pack(sph_cuda *h, short2 *out);
int launch_diagnostics(sph_cuda *h, double *d_out);
int launch_scene_diagnostics(sph_cuda *h, double *d_out);
int launch_probe(sph_cuda *h, int which, void *scratch, float2 *out);
size_t probe_scratch_bytes(int n);
int launch_half_lists(sph_cuda *h, unsigned *d_counts, int *d_off, int *d_ids, bool write);
const char *kernel_name(int k);
int step_kernel_count();

static thread_local char g_err[512] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_fail(cudaError_t e, const char *what)
{
    if (e == cudaSuccess) return SPH_OK;
    set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    return e == cudaErrorMemoryAllocation ? SPH_ERR_ALLOC : SPH_ERR_CUDA;
}

#define SPH_TRY(expr)                          \
    do {                                       \
        const int _rc = (expr);                \
        if (_rc != SPH_OK) return _rc;         \
    } while (0)
#define SPH_CUDA(call) SPH_TRY(cuda_fail((call), #call))

// Test hook (sph_cuda_debug_fail_allocation): the allocation after `after`
// more successful ones reports cudaErrorMemoryAllocation without
// allocating; -1 = off.  Process-wide, host-side only.
static std::atomic<int> g_alloc_fail_after{-1};

static cudaError_t device_alloc(void **p, size_t bytes)
{
    int k = g_alloc_fail_after.load();
    while (k >= 0) {
        if (g_alloc_fail_after.compare_exchange_weak(k, k - 1)) {
            if (k == 0) {
                *p = nullptr;
                return cudaErrorMemoryAllocation;
            }
            break;
        }
    }
    return cudaMalloc(p, bytes);
}

static cudaError_t host_alloc(void **p, size_t bytes)
{
    int k = g_alloc_fail_after.load();
    while (k >= 0) {
        if (g_alloc_fail_after.compare_exchange_weak(k, k - 1)) {
            if (k == 0) {
                *p = nullptr;
                return cudaErrorMemoryAllocation;
            }
            break;
        }
    }
    return cudaHostAlloc(p, bytes, cudaHostAllocDefault);
}

template <class T>
static int dalloc(T **p, size_t count)
{
    *p = nullptr;
    if (count == 0) count = 1;
    return cuda_fail(device_alloc((void **)p, count * sizeof(T)), "cudaMalloc");
}

int ensure_scratch(sph_cuda *h, size_t bytes)
{
    if (bytes <= h->d_scratch_bytes) return SPH_OK;
    if (h->d_scratch) cudaFree(h->d_scratch);
    h->d_scratch = nullptr;
    h->d_scratch_bytes = 0;
    SPH_CUDA(device_alloc(&h->d_scratch, bytes));
    h->d_scratch_bytes = bytes;
    return SPH_OK;
}

int ensure_stage(sph_cuda *h, size_t bytes)
{
    if (bytes <= h->h_stage_bytes) return SPH_OK;
    if (h->h_stage) cudaFreeHost(h->h_stage);
    h->h_stage = nullptr;
    h->h_stage_bytes = 0;
    SPH_CUDA(host_alloc(&h->h_stage, bytes));
    h->h_stage_bytes = bytes;
    return SPH_OK;
}

static void destroy_graph(sph_cuda *h)
{
    if (h->exec) cudaGraphExecDestroy(h->exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->exec = nullptr;
    h->graph = nullptr;
    h->graph_n = -1;
}

// One step as a graph (captured on the handle's stream).
static int capture_step(sph_cuda *h)
{
    destroy_graph(h);
    SPH_CUDA(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    int nk = 0;
    int rc = enqueue_step(h, nullptr, &nk);
    cudaGraph_t g = nullptr;
    const cudaError_t ce = cudaStreamEndCapture(h->stream, &g);
    if (rc != SPH_OK) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    SPH_CUDA(ce);
    h->graph = g;
    SPH_CUDA(cudaGraphInstantiate(&h->exec, g, 0));
    h->graph_n = h->n;
    h->launches_per_step = nk;
    return SPH_OK;
}

// Copies a scene's tunables into its record of the device scene table
// through a pinned ring slot, so that the copy is asynchronous and the
// caller's struct can be reused at once.  Skipped when unchanged.
int set_scene_params(sph_cuda *h, int scene, const tunable_parameters *tp)
{
    if (h->tp_valid[scene] && std::memcmp(&h->last_tp[scene], tp, sizeof(*tp)) == 0) return SPH_OK;
    const int s = h->params_next;
    h->params_next = (s + 1) % h->params_ring;
    SPH_CUDA(cudaEventSynchronize(h->params_ev[s]));
    h->h_params_ring[s] = *tp;
    SPH_CUDA(cudaMemcpyAsync(&h->d_scenes[scene].P, &h->h_params_ring[s], sizeof(*tp),
                             cudaMemcpyHostToDevice, h->stream));
    SPH_CUDA(cudaEventRecord(h->params_ev[s], h->stream));
    h->last_tp[scene] = *tp;
    h->tp_valid[scene] = 1;
    h->scenes[scene].P = *tp;
    return SPH_OK;
}

int run_steps(sph_cuda *h, int nsteps)
{
    if (h->n == 0) return SPH_OK;
    if (h->graph_n != h->n) SPH_TRY(capture_step(h));
    for (int t = 0; t < nsteps; ++t) SPH_CUDA(cudaGraphLaunch(h->exec, h->stream));
    return SPH_OK;
}

static int validate_tp(const tunable_parameters *tp)
{
    if (!tp) {
        set_error("tunable parameters are NULL");
        return SPH_ERR_INVALID;
    }
    if (!(tp->smoothing_radius > 0.0f) || !(tp->time_step > 0.0f)) {
        set_error("smoothing_radius and time_step must be positive (got %g, %g)",
                  (double)tp->smoothing_radius, (double)tp->time_step);
        return SPH_ERR_INVALID;
    }
    return SPH_OK;
}

static int validate_grid(float spacing, unsigned sx, unsigned sy)
{
    if (!(spacing > 0.0f) || sx == 0 || sy == 0 || (unsigned long long)sx * sy >= (1ull << 30)) {
        set_error("invalid neighbour grid (spacing %g, %u x %u)", (double)spacing, sx, sy);
        return SPH_ERR_INVALID;
    }
    return SPH_OK;
}

static int check_handle(sph_cuda *h)
{
    if (!h) {
        set_error("null handle");
        return SPH_ERR_INVALID;
    }
    return SPH_OK;
}

static int check_n(sph_cuda *h, int n)
{
    if (n < 0 || n > h->capacity) {
        set_error("particle count %d outside [0, %d]", n, h->capacity);
        return n < 0 ? SPH_ERR_INVALID : SPH_ERR_CAPACITY;
    }
    if (h->nscenes > 1 && n != h->capacity) {
        set_error("an ensemble of %d scenes holds exactly %d particles (got %d)", h->nscenes,
                  h->capacity, n);
        return SPH_ERR_INVALID;
    }
    return SPH_OK;
}

static void free_all(sph_cuda *h)
{
    destroy_graph(h);
    free_learned_buffers(h);
    if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
    for (int k = 0; k < 2; ++k) {
        if (h->d_coords[k]) cudaFree(h->d_coords[k]);
        if (h->pack_ev[k]) cudaEventDestroy(h->pack_ev[k]);
        if (h->copy_ev[k]) cudaEventDestroy(h->copy_ev[k]);
    }
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    void *ptrs[] = {h->pos_a, h->vel_a, h->id_a, h->pos_b, h->prev_b, h->vel_b, h->kr_b,
                    h->pos_c, h->prev_c, h->xr_c, h->mask01_c, h->mask2_c, h->maskx_c, h->rows_c, h->id_c,
                    h->tmp_id, h->cnt, h->start_a, h->start_c, h->tile_sums, h->build_tiles, h->d_scenes,
                    h->d_p_off, h->d_nocell, h->d_state, h->d_partials, h->d_scratch};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (h->h_stage) cudaFreeHost(h->h_stage);
    if (h->h_params_ring) cudaFreeHost(h->h_params_ring);
    if (h->params_ev) {
        for (int i = 0; i < h->params_ring; ++i)
            if (h->params_ev[i]) cudaEventDestroy(h->params_ev[i]);
        delete[] h->params_ev;
    }
    for (cudaEvent_t e : h->timer)
        if (e) cudaEventDestroy(e);
    if (h->own_stream) cudaStreamDestroy(h->own_stream);
}

// Uploads the scene table and the slot offsets (scene particle counts may
// change between uploads of a single-scene handle).
static int push_scenes(sph_cuda *h)
{
    std::vector<int> off(h->nscenes + 1);
    int p = 0;
    for (int s = 0; s < h->nscenes; ++s) {
        h->scenes[s].p_off = p;
        off[s] = p;
        p += h->scenes[s].n;
    }
    off[h->nscenes] = p;
    SPH_CUDA(cudaMemcpyAsync(h->d_scenes, h->scenes.data(), h->nscenes * sizeof(Scene),
                             cudaMemcpyHostToDevice, h->stream));
    SPH_CUDA(cudaMemcpyAsync(h->d_p_off, off.data(), (h->nscenes + 1) * sizeof(int),
                             cudaMemcpyHostToDevice, h->stream));
    SPH_CUDA(cudaStreamSynchronize(h->stream));  // host vectors go out of scope
    for (int s = 0; s < h->nscenes; ++s) {
        h->last_tp[s] = h->scenes[s].P;
        h->tp_valid[s] = 1;
    }
    return SPH_OK;
}

// Allocates a handle for `scenes` (cell offsets filled in here).
// The coordinate frames' resources: two device staging buffers of
// capacity + 1 packed coordinates, their pack and copy events, and the copy
// stream.  Made with the handle (so a frame loop allocates nothing), all or
// nothing.
static int ensure_frames(sph_cuda *h)
{
    if (h->copy_stream) return SPH_OK;
    auto undo = [&]() {
        for (int k = 0; k < 2; ++k) {
            if (h->d_coords[k]) cudaFree(h->d_coords[k]);
            if (h->pack_ev[k]) cudaEventDestroy(h->pack_ev[k]);
            if (h->copy_ev[k]) cudaEventDestroy(h->copy_ev[k]);
            h->d_coords[k] = nullptr;
            h->pack_ev[k] = h->copy_ev[k] = nullptr;
        }
    };
    int rc = SPH_OK;
    for (int k = 0; k < 2 && !rc; ++k) {
        rc = cuda_fail(device_alloc((void **)&h->d_coords[k],
                                    ((size_t)h->capacity + 1) * sizeof(short2)), "cudaMalloc");
        if (!rc) rc = cuda_fail(cudaEventCreateWithFlags(&h->pack_ev[k], cudaEventDisableTiming),
                                "cudaEventCreate");
        if (!rc) rc = cuda_fail(cudaEventCreateWithFlags(&h->copy_ev[k], cudaEventDisableTiming),
                                "cudaEventCreate");
    }
    if (!rc) rc = cuda_fail(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking),
                            "cudaStreamCreate");
    if (rc) undo();
    return rc;
}

static int build_handle(sph_cuda **out, std::vector<Scene> &&scenes, int capacity, int max_bucket,
                        int max_neighbors)
{
    *out = nullptr;
    sph_cuda *h = new (std::nothrow) sph_cuda();
    if (!h) {
        set_error("host allocation failed");
        return SPH_ERR_ALLOC;
    }
    auto fail = [&](int rc) {
        free_all(h);
        delete h;
        return rc;
    };
    h->scenes = std::move(scenes);
    h->nscenes = (int)h->scenes.size();
    h->capacity = capacity;
    h->max_bucket = max_bucket;
    h->max_neighbors = max_neighbors;
    h->last_tp.resize(h->nscenes);
    h->tp_valid.assign(h->nscenes, 0);
    long long m = 0;
    for (Scene &s : h->scenes) {
        s.c_off = (int)m;
        s.max_bucket = max_bucket;
        s.max_neighbors = max_neighbors;
        m += (long long)s.ncells + 1;
    }
    if (m >= (1ll << 30)) {
        set_error("%lld grid cells in total: above 2^30", m);
        return fail(SPH_ERR_INVALID);
    }
    h->M = (int)m;
    int dev = 0;
    int rc = cuda_fail(cudaGetDevice(&dev), "cudaGetDevice");
    if (!rc) rc = cuda_fail(cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, dev),
                            "cudaDeviceGetAttribute");
    if (rc) return fail(rc);
    rc = cuda_fail(cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking),
                   "cudaStreamCreate");
    if (rc) return fail(rc);
    h->stream = h->own_stream;
    const size_t N = (size_t)capacity;
    const size_t M = (size_t)h->M;
    const size_t scan_items = std::max(M, N) + 1;
    h->ntiles = (int)((scan_items + kScanTile - 1) / kScanTile);
    h->npartials = 148 * 2;
    const size_t nwords = (M + 31) / 32 + 1;
    if ((rc = dalloc(&h->pos_a, N)) || (rc = dalloc(&h->vel_a, N)) || (rc = dalloc(&h->id_a, N)) ||
        (rc = dalloc(&h->pos_b, N)) || (rc = dalloc(&h->prev_b, N)) ||
        (rc = dalloc(&h->vel_b, N)) || (rc = dalloc(&h->kr_b, N)) || (rc = dalloc(&h->pos_c, N)) ||
        (rc = dalloc(&h->prev_c, N)) || (rc = dalloc(&h->xr_c, N)) ||
        (rc = dalloc(&h->mask01_c, N)) || (rc = dalloc(&h->mask2_c, N)) || (rc = dalloc(&h->rows_c, N)) ||
        (rc = dalloc(&h->id_c, N)) || (rc = dalloc(&h->tmp_id, N)) ||
        (rc = dalloc(&h->cnt, std::max(M, N + 1))) ||
        (rc = dalloc(&h->start_a, std::max(M + 1, N + 1))) || (rc = dalloc(&h->start_c, M + 1)) ||
        (rc = dalloc(&h->tile_sums, (size_t)h->ntiles)) ||
        (rc = dalloc(&h->build_tiles, (size_t)h->ntiles)) ||
        (rc = dalloc(&h->d_scenes, (size_t)h->nscenes)) ||
        (rc = dalloc(&h->d_p_off, (size_t)h->nscenes + 1)) || (rc = dalloc(&h->d_nocell, nwords)) ||
        (rc = dalloc(&h->d_state, 1)) || (rc = dalloc(&h->d_partials, (size_t)h->npartials * 3 + 3)))
        return fail(rc);
    rc = cuda_fail(cudaMemsetAsync(h->cnt, 0, std::max(M, N + 1) * sizeof(unsigned), h->stream),
                   "cudaMemset");
    if (!rc) rc = cuda_fail(cudaMemsetAsync(h->d_state, 0, sizeof(DevState), h->stream), "cudaMemset");
    if (!rc)
        rc = cuda_fail(cudaMemsetAsync(h->build_tiles, 0, (size_t)h->ntiles * sizeof(unsigned), h->stream),
                       "cudaMemset");
    if (rc) return fail(rc);
    {
        std::vector<unsigned> bits(nwords, 0u);
        for (const Scene &s : h->scenes) {
            const size_t k = (size_t)s.c_off + s.ncells;
            bits[k >> 5] |= 1u << (k & 31);
        }
        rc = cuda_fail(cudaMemcpy(h->d_nocell, bits.data(), nwords * sizeof(unsigned),
                                  cudaMemcpyHostToDevice),
                       "no-cell bitmap");
        if (rc) return fail(rc);
    }
    h->params_ring = 64;
    rc = cuda_fail(host_alloc((void **)&h->h_params_ring,
                              h->params_ring * sizeof(tunable_parameters)),
                   "cudaHostAlloc");
    if (rc) return fail(rc);
    h->params_ev = new (std::nothrow) cudaEvent_t[h->params_ring]();
    if (!h->params_ev) return fail(SPH_ERR_ALLOC);
    for (int i = 0; i < h->params_ring; ++i) {
        rc = cuda_fail(cudaEventCreateWithFlags(&h->params_ev[i], cudaEventDisableTiming),
                       "cudaEventCreate");
        if (rc) return fail(rc);
    }
    for (cudaEvent_t &e : h->timer) {
        rc = cuda_fail(cudaEventCreate(&e), "cudaEventCreate");
        if (rc) return fail(rc);
    }
    rc = push_scenes(h);
    if (!rc) rc = ensure_frames(h);
    if (rc) return fail(rc);
    *out = h;
    return SPH_OK;
}

// The common tail of every upload: the particle count, a fresh device state,
// zero tile counts and the sort into the A order (upload_soa_device).
static int upload_finish(sph_cuda *h, int n)
{
    if (h->nscenes == 1 && h->scenes[0].n != n) {
        h->scenes[0].n = n;
        SPH_TRY(push_scenes(h));
    }
    h->n = n;
    SPH_CUDA(cudaMemsetAsync(h->d_state, 0, sizeof(DevState), h->stream));
    SPH_TRY(upload_soa_device(h, n));
    SPH_CUDA(cudaStreamSynchronize(h->stream));  // the caller's buffers are free again
    return SPH_OK;
}

// Host particles reached through a pointer array -> device, then sort.
// `fill(i, rec)` writes particle i's 8 floats (x, y, vx, vy, x_prev, y_prev,
// rho, rho_near) into a page-locked staging buffer, copied as four arrays.
template <class Fill>
static int upload_common(sph_cuda *h, int n, Fill fill)
{
    SPH_TRY(check_n(h, n));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    SPH_TRY(ensure_stage(h, (size_t)n * 5 * sizeof(float2) + 16));
    float4 *xr = (float4 *)h->h_stage;
    float2 *pos = (float2 *)(xr + n), *vel = pos + n, *prev = vel + n;
    for (int i = 0; i < n; ++i) {
        float r[8];
        fill(i, r);
        pos[i] = make_float2(r[0], r[1]);
        vel[i] = make_float2(r[2], r[3]);
        prev[i] = make_float2(r[4], r[5]);
        xr[i] = make_float4(r[0], r[1], r[6], r[7]);
    }
    const size_t b = (size_t)n * sizeof(float2);
    if (n > 0) {
        SPH_CUDA(cudaMemcpyAsync(h->pos_b, pos, b, cudaMemcpyHostToDevice, h->stream));
        SPH_CUDA(cudaMemcpyAsync(h->vel_b, vel, b, cudaMemcpyHostToDevice, h->stream));
        SPH_CUDA(cudaMemcpyAsync(h->prev_c, prev, b, cudaMemcpyHostToDevice, h->stream));
        SPH_CUDA(cudaMemcpyAsync(h->xr_c, xr, 2 * b, cudaMemcpyHostToDevice, h->stream));
    }
    return upload_finish(h, n);
}

// Sorted state -> id-order host SoA in the staging buffer (5 n float2:
// pos, vel, prev, rho, pressure).  Synchronous.
static int download_common(sph_cuda *h, int n, float2 **host)
{
    if (n != h->n) {
        set_error("download of %d particles, handle holds %d", n, h->n);
        return SPH_ERR_INVALID;
    }
    const size_t b = (size_t)n * 5 * sizeof(float2);
    SPH_TRY(ensure_scratch(h, b + 16));
    SPH_TRY(ensure_stage(h, b + 16));
    SPH_TRY(launch_unpermute(h, (float2 *)h->d_scratch));
    if (n > 0)
        SPH_CUDA(cudaMemcpyAsync(h->h_stage, h->d_scratch, b, cudaMemcpyDeviceToHost, h->stream));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    *host = (float2 *)h->h_stage;
    return SPH_OK;
}

// The tunables a single-scene call passes (NULL = keep the current ones);
// ensembles take their per-scene tunables from sph_cuda_set_scene_params.
static int apply_tp(sph_cuda *h, const tunable_parameters *tp)
{
    if (!tp) return SPH_OK;
    if (h->nscenes != 1) {
        set_error("an ensemble takes per-scene tunables (sph_cuda_set_scene_params); pass NULL");
        return SPH_ERR_INVALID;
    }
    SPH_TRY(validate_tp(tp));
    return set_scene_params(h, 0, tp);
}

}  // namespace sph

using namespace sph;

extern "C" {

const char *sph_cuda_last_error(void) { return sph::g_err; }

int sph_cuda_create(sph_cuda_t **out, const param *params, const AABB_t *boundary,
                    const neighbor_grid_t *grid, int max_particles)
{
    if (!out || !params || !boundary || !grid) {
        set_error("sph_cuda_create: null argument");
        return SPH_ERR_INVALID;
    }
    *out = nullptr;
    if (max_particles < 0) {
        set_error("max_particles %d < 0", max_particles);
        return SPH_ERR_INVALID;
    }
    SPH_TRY(validate_grid(grid->spacing, grid->size_x, grid->size_y));
    if (grid->max_bucket_size == 0 || grid->max_neighbors == 0) {
        set_error("max_bucket_size and max_neighbors must be positive");
        return SPH_ERR_INVALID;
    }
    if (params->number_halo_particles != 0) {
        set_error("halo particles (%d) are not supported: libsph_cuda runs a single-device domain",
                  params->number_halo_particles);
        return SPH_ERR_UNSUPPORTED;
    }
    SPH_TRY(validate_tp(&params->tunable_params));
    Scene s{};
    s.P = params->tunable_params;
    s.spacing = grid->spacing;
    s.size_x = (int)grid->size_x;
    s.size_y = (int)grid->size_y;
    s.ncells = s.size_x * s.size_y;
    s.n = 0;
    s.min_x = boundary->min_x;
    s.max_x = boundary->max_x;
    s.min_y = boundary->min_y;
    s.max_y = boundary->max_y;
    std::vector<Scene> v(1, s);
    return build_handle(out, std::move(v), max_particles, (int)grid->max_bucket_size,
                        (int)grid->max_neighbors);
}

int sph_cuda_create_ensemble(sph_cuda_t **out, const sph_scene_desc *descs, int nscenes,
                             int max_bucket, int max_neighbors)
{
    if (!out || !descs || nscenes <= 0) {
        set_error("sph_cuda_create_ensemble: null argument or no scenes");
        return SPH_ERR_INVALID;
    }
    *out = nullptr;
    if (max_bucket <= 0 || max_neighbors <= 0) {
        set_error("max_bucket and max_neighbors must be positive");
        return SPH_ERR_INVALID;
    }
    std::vector<Scene> v((size_t)nscenes);
    long long total = 0;
    for (int i = 0; i < nscenes; ++i) {
        const sph_scene_desc &d = descs[i];
        SPH_TRY(validate_grid(d.spacing, d.size_x, d.size_y));
        SPH_TRY(validate_tp(&d.params));
        if (d.n < 0) {
            set_error("scene %d has %d particles", i, d.n);
            return SPH_ERR_INVALID;
        }
        Scene &s = v[i];
        s = Scene{};
        s.P = d.params;
        s.spacing = d.spacing;
        s.size_x = (int)d.size_x;
        s.size_y = (int)d.size_y;
        s.ncells = s.size_x * s.size_y;
        s.n = d.n;
        s.min_x = d.boundary.min_x;
        s.max_x = d.boundary.max_x;
        s.min_y = d.boundary.min_y;
        s.max_y = d.boundary.max_y;
        total += d.n;
    }
    if (total >= (1ll << 31)) {
        set_error("%lld particles in total: above 2^31", total);
        return SPH_ERR_INVALID;
    }
    return build_handle(out, std::move(v), (int)total, max_bucket, max_neighbors);
}

int sph_cuda_set_scene_params(sph_cuda_t *h, int scene, const tunable_parameters *tp)
{
    SPH_TRY(check_handle(h));
    if (scene < 0 || scene >= h->nscenes) {
        set_error("scene %d outside [0, %d)", scene, h->nscenes);
        return SPH_ERR_INVALID;
    }
    SPH_TRY(validate_tp(tp));
    return set_scene_params(h, scene, tp);
}

int sph_cuda_num_scenes(sph_cuda_t *h) { return h ? h->nscenes : 0; }

int sph_cuda_destroy(sph_cuda_t *h)
{
    if (!h) return SPH_OK;
    cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return SPH_OK;
}

int sph_cuda_set_stream(sph_cuda_t *h, void *stream)
{
    SPH_TRY(check_handle(h));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    h->stream = stream ? (cudaStream_t)stream : h->own_stream;
    destroy_graph(h);
    return SPH_OK;
}

int sph_cuda_upload(sph_cuda_t *h, fluid_particle *const *ptrs, int n)
{
    SPH_TRY(check_handle(h));
    if (!ptrs && n > 0) {
        set_error("null particle pointer array");
        return SPH_ERR_INVALID;
    }
    for (int i = 0; i < n; ++i)
        if (!ptrs[i]) {
            set_error("particle pointer %d is NULL", i);
            return SPH_ERR_INVALID;
        }
    return upload_common(h, n, [&](int i, float *r) {
        const fluid_particle *p = ptrs[i];
        r[0] = p->x; r[1] = p->y; r[2] = p->v_x; r[3] = p->v_y;
        r[4] = p->x_prev; r[5] = p->y_prev; r[6] = p->density; r[7] = p->density_near;
    });
}

// The caller's contiguous arrays go to the device as they are (one copy
// each, no host-side repacking) and a kernel lays them out.
int sph_cuda_upload_particles(sph_cuda_t *h, const fluid_particle *ps, int n)
{
    SPH_TRY(check_handle(h));
    if (!ps && n > 0) {
        set_error("null particle array");
        return SPH_ERR_INVALID;
    }
    SPH_TRY(check_n(h, n));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    if (n > 0) {
        const size_t b = (size_t)n * sizeof(fluid_particle);
        SPH_TRY(ensure_scratch(h, b));
        auto *recs = static_cast<fluid_particle *>(h->d_scratch);
        SPH_CUDA(cudaMemcpyAsync(recs, ps, b, cudaMemcpyHostToDevice, h->stream));
        SPH_TRY(launch_upload_layout(h, n, nullptr, nullptr, nullptr, nullptr, recs));
    }
    return upload_finish(h, n);
}

int sph_cuda_upload_soa(sph_cuda_t *h, const float *x, const float *y, const float *vx,
                        const float *vy, int n)
{
    SPH_TRY(check_handle(h));
    if ((!x || !y) && n > 0) {
        set_error("x and y are required");
        return SPH_ERR_INVALID;
    }
    SPH_TRY(check_n(h, n));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    if (n > 0) {
        // the A-state arrays are free until the sort rewrites them
        const size_t b = (size_t)n * sizeof(float);
        float *dx = reinterpret_cast<float *>(h->pos_a), *dy = dx + n;
        float *dvx = reinterpret_cast<float *>(h->vel_a), *dvy = dvx + n;
        SPH_CUDA(cudaMemcpyAsync(dx, x, b, cudaMemcpyHostToDevice, h->stream));
        SPH_CUDA(cudaMemcpyAsync(dy, y, b, cudaMemcpyHostToDevice, h->stream));
        if (vx) SPH_CUDA(cudaMemcpyAsync(dvx, vx, b, cudaMemcpyHostToDevice, h->stream));
        if (vy) SPH_CUDA(cudaMemcpyAsync(dvy, vy, b, cudaMemcpyHostToDevice, h->stream));
        SPH_TRY(launch_upload_layout(h, n, dx, dy, vx ? dvx : nullptr, vy ? dvy : nullptr,
                                     nullptr));
    }
    return upload_finish(h, n);
}

int sph_cuda_step(sph_cuda_t *h, const tunable_parameters *tp, int nsteps)
{
    SPH_TRY(check_handle(h));
    if (nsteps < 0) {
        set_error("nsteps %d < 0", nsteps);
        return SPH_ERR_INVALID;
    }
    SPH_TRY(apply_tp(h, tp));
    return run_steps(h, nsteps);
}

int sph_cuda_step_schedule(sph_cuda_t *h, const tunable_parameters *tps, int nsteps)
{
    SPH_TRY(check_handle(h));
    if (nsteps < 0 || (!tps && nsteps > 0)) {
        set_error("bad schedule (%d steps)", nsteps);
        return SPH_ERR_INVALID;
    }
    for (int t = 0; t < nsteps; ++t) {
        SPH_TRY(apply_tp(h, &tps[t]));
        SPH_TRY(run_steps(h, 1));
    }
    return SPH_OK;
}

int sph_cuda_step_split(sph_cuda_t *h, const tunable_parameters *tp_before,
                        const tunable_parameters *tp_after)
{
    SPH_TRY(check_handle(h));
    if (h->nscenes != 1) {
        set_error("a split step takes the tunables of one scene");
        return SPH_ERR_INVALID;
    }
    SPH_TRY(validate_tp(tp_after));
    SPH_TRY(apply_tp(h, tp_before));
    if (h->n == 0) return set_scene_params(h, 0, tp_after);
    int nk = 0;
    return enqueue_step(h, nullptr, &nk, tp_after);
}

int sph_cuda_download(sph_cuda_t *h, fluid_particle *const *ptrs, int n)
{
    SPH_TRY(check_handle(h));
    if (!ptrs && n > 0) {
        set_error("null particle pointer array");
        return SPH_ERR_INVALID;
    }
    float2 *s = nullptr;
    SPH_TRY(download_common(h, n, &s));
    for (int i = 0; i < n; ++i) {
        fluid_particle *p = ptrs[i];
        if (!p) continue;
        p->x = s[i].x; p->y = s[i].y;
        p->v_x = s[n + i].x; p->v_y = s[n + i].y;
        p->x_prev = s[2 * n + i].x; p->y_prev = s[2 * n + i].y;
        p->density = s[3 * n + i].x; p->density_near = s[3 * n + i].y;
        p->pressure = s[4 * n + i].x; p->pressure_near = s[4 * n + i].y;
    }
    return SPH_OK;
}

int sph_cuda_download_particles(sph_cuda_t *h, fluid_particle *ps, int n)
{
    SPH_TRY(check_handle(h));
    if (!ps && n > 0) {
        set_error("null particle array");
        return SPH_ERR_INVALID;
    }
    float2 *s = nullptr;
    SPH_TRY(download_common(h, n, &s));
    for (int i = 0; i < n; ++i) {
        fluid_particle *p = &ps[i];
        p->x = s[i].x; p->y = s[i].y;
        p->v_x = s[n + i].x; p->v_y = s[n + i].y;
        p->x_prev = s[2 * n + i].x; p->y_prev = s[2 * n + i].y;
        p->density = s[3 * n + i].x; p->density_near = s[3 * n + i].y;
        p->pressure = s[4 * n + i].x; p->pressure_near = s[4 * n + i].y;
    }
    return SPH_OK;
}

// Laid out on the device and copied straight into the caller's arrays (no
// host-side repacking).
int sph_cuda_download_soa(sph_cuda_t *h, float *x, float *y, float *vx, float *vy, float *rho,
                          float *rho_near, int n)
{
    SPH_TRY(check_handle(h));
    if (n != h->n) {
        set_error("download of %d particles, handle holds %d", n, h->n);
        return SPH_ERR_INVALID;
    }
    if (n == 0) return SPH_OK;
    const size_t rec = (size_t)n * 5 * sizeof(float2), col = (size_t)n * sizeof(float);
    SPH_TRY(ensure_scratch(h, rec + 6 * col + 16));
    float2 *s = static_cast<float2 *>(h->d_scratch);
    float *cols = reinterpret_cast<float *>(s + 5 * (size_t)n);
    SPH_TRY(launch_unpermute(h, s));
    SPH_TRY(launch_split_soa(h, n, s, cols));
    float *dst[6] = {x, y, vx, vy, rho, rho_near};
    for (int k = 0; k < 6; ++k)
        if (dst[k])
            SPH_CUDA(cudaMemcpyAsync(dst[k], cols + k * (size_t)n, col, cudaMemcpyDeviceToHost,
                                     h->stream));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    return SPH_OK;
}

int sph_cuda_pack_coords_short(sph_cuda_t *h, short *coords, int n)
{
    SPH_TRY(check_handle(h));
    if (n != h->n || (!coords && n > 0)) {
        set_error("pack: n %d (handle holds %d) or null buffer", n, h->n);
        return SPH_ERR_INVALID;
    }
    const size_t b = (size_t)n * sizeof(short2);
    SPH_TRY(ensure_scratch(h, b + 16));
    SPH_TRY(launch_pack(h, (short2 *)h->d_scratch));
    if (n > 0) SPH_CUDA(cudaMemcpyAsync(coords, h->d_scratch, b, cudaMemcpyDeviceToHost, h->stream));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    return SPH_OK;
}

int sph_cuda_pack_coords_async(sph_cuda_t *h, short *coords, int n)
{
    SPH_TRY(check_handle(h));
    if (n != h->n || (!coords && n > 0)) {
        set_error("pack: n %d (handle holds %d) or null buffer", n, h->n);
        return SPH_ERR_INVALID;
    }
    SPH_TRY(ensure_frames(h));
    const int k = h->pack_slot;
    // the copy made from this staging buffer two calls ago must be complete
    if (h->copy_dst[k]) SPH_CUDA(cudaEventSynchronize(h->copy_ev[k]));
    SPH_TRY(launch_pack(h, h->d_coords[k]));
    SPH_CUDA(cudaEventRecord(h->pack_ev[k], h->stream));
    SPH_CUDA(cudaStreamWaitEvent(h->copy_stream, h->pack_ev[k], 0));
    if (n > 0)
        SPH_CUDA(cudaMemcpyAsync(coords, h->d_coords[k], (size_t)n * sizeof(short2),
                                 cudaMemcpyDeviceToHost, h->copy_stream));
    SPH_CUDA(cudaEventRecord(h->copy_ev[k], h->copy_stream));
    h->copy_dst[k] = coords;
    h->pack_slot = k ^ 1;
    return SPH_OK;
}

int sph_cuda_coords_wait(sph_cuda_t *h, const short *coords)
{
    SPH_TRY(check_handle(h));
    for (int k = 0; k < 2; ++k)
        if (h->copy_dst[k] && h->copy_dst[k] == (const void *)coords) {
            SPH_CUDA(cudaEventSynchronize(h->copy_ev[k]));
            h->copy_dst[k] = nullptr;
            return SPH_OK;
        }
    set_error("no pending coordinate copy into %p", (const void *)coords);
    return SPH_ERR_STATE;
}

// Checkpoint file: header, then n fluid_particle records by id.
struct CheckpointHeader {
    char magic[8];           // "SPHCKPT1"
    uint32_t version;        // 1
    int32_t n;               // particles (all scenes)
    int32_t nscenes;
    uint32_t lists_valid;    // the neighbour relation of the positions exists
    uint64_t steps;          // steps since the last upload
    uint32_t record_bytes;   // sizeof(fluid_particle)
    uint32_t reserved[3];
};
static_assert(sizeof(CheckpointHeader) == 48, "checkpoint header layout");

int sph_cuda_save_state(sph_cuda_t *h, const char *path)
{
    SPH_TRY(check_handle(h));
    if (!path) {
        set_error("null path");
        return SPH_ERR_INVALID;
    }
    const int n = h->n;
    std::vector<fluid_particle> ps((size_t)n + 1);
    SPH_TRY(sph_cuda_download_particles(h, ps.data(), n));
    DevState st;
    SPH_CUDA(cudaMemcpy(&st, h->d_state, sizeof(st), cudaMemcpyDeviceToHost));
    CheckpointHeader hd;
    std::memset(&hd, 0, sizeof(hd));
    std::memcpy(hd.magic, "SPHCKPT1", 8);
    hd.version = 1;
    hd.n = n;
    hd.nscenes = h->nscenes;
    hd.lists_valid = st.lists_valid;
    hd.steps = st.steps;
    hd.record_bytes = sizeof(fluid_particle);
    FILE *f = std::fopen(path, "wb");
    if (!f) {
        set_error("cannot open %s for writing", path);
        return SPH_ERR_INVALID;
    }
    const bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1 &&
                    (n == 0 || std::fwrite(ps.data(), sizeof(fluid_particle), (size_t)n, f) == (size_t)n);
    const bool closed = std::fclose(f) == 0;
    if (!ok || !closed) {
        set_error("writing %s failed", path);
        return SPH_ERR_INVALID;
    }
    return SPH_OK;
}

int sph_cuda_load_state(sph_cuda_t *h, const char *path)
{
    SPH_TRY(check_handle(h));
    if (!path) {
        set_error("null path");
        return SPH_ERR_INVALID;
    }
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        set_error("cannot open %s", path);
        return SPH_ERR_INVALID;
    }
    CheckpointHeader hd;
    std::vector<fluid_particle> ps;
    bool ok = std::fread(&hd, sizeof(hd), 1, f) == 1 && std::memcmp(hd.magic, "SPHCKPT1", 8) == 0 &&
              hd.version == 1 && hd.record_bytes == sizeof(fluid_particle) && hd.n >= 0;
    if (ok && (hd.nscenes != h->nscenes || hd.n > h->capacity)) {
        std::fclose(f);
        set_error("checkpoint of %d particles in %d scenes does not fit this handle (%d scenes, "
                  "capacity %d)", hd.n, hd.nscenes, h->nscenes, h->capacity);
        return SPH_ERR_INVALID;
    }
    if (ok) {
        ps.resize((size_t)hd.n + 1);
        ok = hd.n == 0 || std::fread(ps.data(), sizeof(fluid_particle), (size_t)hd.n, f) == (size_t)hd.n;
    }
    std::fclose(f);
    if (!ok) {
        set_error("%s is not a libsph_cuda checkpoint (or is truncated)", path);
        return SPH_ERR_INVALID;
    }
    SPH_TRY(sph_cuda_upload_particles(h, ps.data(), hd.n));
    // the upload starts counters afresh: restore the step count and whether
    // the next step applies viscosity
    SPH_CUDA(cudaMemcpy(&h->d_state->steps, &hd.steps, sizeof(hd.steps), cudaMemcpyHostToDevice));
    SPH_CUDA(cudaMemcpy(&h->d_state->lists_valid, &hd.lists_valid, sizeof(hd.lists_valid),
                        cudaMemcpyHostToDevice));
    return SPH_OK;
}

int sph_cuda_rebuild_neighbors(sph_cuda_t *h)
{
    SPH_TRY(check_handle(h));
    // The sorted state always carries the cell lists of its current
    // positions, so the relation exists already: enable it.
    const unsigned one = 1u;
    SPH_CUDA(cudaMemcpyAsync(&h->d_state->lists_valid, &one, sizeof(one), cudaMemcpyHostToDevice,
                             h->stream));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    return SPH_OK;
}

int sph_cuda_synchronize(sph_cuda_t *h)
{
    SPH_TRY(check_handle(h));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    return SPH_OK;
}

int sph_cuda_get_counters(sph_cuda_t *h, sph_cuda_counters *out)
{
    SPH_TRY(check_handle(h));
    if (!out) {
        set_error("null counters");
        return SPH_ERR_INVALID;
    }
    DevState s;
    SPH_CUDA(cudaMemcpyAsync(&s, h->d_state, sizeof(s), cudaMemcpyDeviceToHost, h->stream));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    out->steps = s.steps;
    out->out_of_grid = s.out_of_grid;
    out->bucket_overflow = s.bucket_overflow;
    out->max_cell_occupancy = s.max_occ;
    out->list_cap_risk = s.list_cap_risk;
    if (s.tile_count_mismatch) {
        set_error("internal: a cell build's tile counts disagreed with its cell counters");
        return SPH_ERR_CUDA;
    }
    return SPH_OK;
}

int sph_cuda_diagnostics(sph_cuda_t *h, double out[3])
{
    SPH_TRY(check_handle(h));
    if (!out) {
        set_error("null output");
        return SPH_ERR_INVALID;
    }
    if (h->n == 0) {
        out[0] = out[1] = out[2] = 0.0;
        return SPH_OK;
    }
    double *d_out = h->d_partials + 3 * h->npartials;
    SPH_TRY(launch_diagnostics(h, d_out));
    SPH_CUDA(cudaMemcpyAsync(out, d_out, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    return SPH_OK;
}

int sph_cuda_scene_diagnostics(sph_cuda_t *h, double *out)
{
    SPH_TRY(check_handle(h));
    if (!out) {
        set_error("null output");
        return SPH_ERR_INVALID;
    }
    if (h->n == 0) {
        for (int s = 0; s < 3 * h->nscenes; ++s) out[s] = 0.0;
        return SPH_OK;
    }
    const size_t b = (size_t)h->nscenes * 3 * sizeof(double);
    SPH_TRY(ensure_scratch(h, b + 16));
    SPH_TRY(launch_scene_diagnostics(h, (double *)h->d_scratch));
    SPH_CUDA(cudaMemcpyAsync(out, h->d_scratch, b, cudaMemcpyDeviceToHost, h->stream));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    return SPH_OK;
}

int sph_cuda_neighbor_lists(sph_cuda_t *h, int *counts, int *ids, long long max_total,
                            long long *total)
{
    SPH_TRY(check_handle(h));
    if (!counts || !total) {
        set_error("null output");
        return SPH_ERR_INVALID;
    }
    const int n = h->n;
    *total = 0;
    if (n == 0) return SPH_OK;
    // scratch: counts (n+1 words) | offsets (n+1 ints), each 256-byte aligned
    const size_t part = (((size_t)(n + 1) * sizeof(int)) + 255) & ~(size_t)255;
    SPH_TRY(ensure_scratch(h, 2 * part));
    unsigned *d_counts = (unsigned *)h->d_scratch;
    int *d_off = (int *)((char *)h->d_scratch + part);
    SPH_CUDA(cudaMemsetAsync(d_counts, 0, (size_t)(n + 1) * sizeof(unsigned), h->stream));
    SPH_TRY(launch_half_lists(h, d_counts, d_off, nullptr, false));
    SPH_CUDA(cudaMemcpyAsync(counts, d_counts, (size_t)n * sizeof(int), cudaMemcpyDeviceToHost,
                             h->stream));
    int tot = 0;
    SPH_CUDA(cudaMemcpyAsync(&tot, d_off + n, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    *total = tot;
    if (tot > max_total || (!ids && tot > 0)) {
        set_error("neighbour list buffer holds %lld entries, %d needed", max_total, tot);
        return SPH_ERR_CAPACITY;
    }
    if (tot == 0) return SPH_OK;
    int *d_ids = nullptr;
    SPH_CUDA(cudaMallocAsync((void **)&d_ids, (size_t)tot * sizeof(int), h->stream));
    int rc = launch_half_lists(h, nullptr, d_off, d_ids, true);
    if (rc == SPH_OK)
        rc = cuda_fail(cudaMemcpyAsync(ids, d_ids, (size_t)tot * sizeof(int),
                                       cudaMemcpyDeviceToHost, h->stream),
                       "list copy");
    cudaFreeAsync(d_ids, h->stream);
    if (rc == SPH_OK) rc = cuda_fail(cudaStreamSynchronize(h->stream), "list sync");
    return rc;
}

static int probe(sph_cuda *h, const tunable_parameters *tp, int which, float *a, float *b)
{
    SPH_TRY(check_handle(h));
    if (tp) SPH_TRY(validate_tp(tp));
    if (tp && h->nscenes != 1) {
        set_error("probes of an ensemble use each scene's own tunables; pass NULL");
        return SPH_ERR_INVALID;
    }
    const int n = h->n;
    if (n == 0) return SPH_OK;
    if (!a || !b) {
        set_error("null output");
        return SPH_ERR_INVALID;
    }
    const size_t sb = probe_scratch_bytes(n);
    SPH_TRY(ensure_scratch(h, sb + (size_t)n * sizeof(float2) + 256));
    SPH_TRY(ensure_stage(h, (size_t)n * sizeof(float2) + 16));
    float2 *out = (float2 *)((char *)h->d_scratch + sb);
    // probes use their own parameters without disturbing the step's
    const tunable_parameters saved = h->scenes[0].P;
    if (tp) SPH_TRY(set_scene_params(h, 0, tp));
    SPH_TRY(launch_probe(h, which, h->d_scratch, out));
    SPH_CUDA(cudaMemcpyAsync(h->h_stage, out, (size_t)n * sizeof(float2), cudaMemcpyDeviceToHost,
                             h->stream));
    if (tp) SPH_TRY(set_scene_params(h, 0, &saved));
    SPH_CUDA(cudaStreamSynchronize(h->stream));
    const float2 *s = (const float2 *)h->h_stage;
    for (int i = 0; i < n; ++i) {
        a[i] = s[i].x;
        b[i] = s[i].y;
    }
    return SPH_OK;
}

int sph_cuda_probe_density(sph_cuda_t *h, const tunable_parameters *tp, float *rho, float *rho_near)
{
    return probe(h, tp, 0, rho, rho_near);
}

int sph_cuda_probe_relaxation(sph_cuda_t *h, const tunable_parameters *tp, float *dx, float *dy)
{
    return probe(h, tp, 1, dx, dy);
}

int sph_cuda_probe_viscosity(sph_cuda_t *h, const tunable_parameters *tp, float *dvx, float *dvy)
{
    return probe(h, tp, 2, dvx, dvy);
}

int sph_cuda_kernel_times(sph_cuda_t *h, const tunable_parameters *tp, float *ms, int max,
                          int *count)
{
    SPH_TRY(check_handle(h));
    if (!ms || !count) {
        set_error("null output");
        return SPH_ERR_INVALID;
    }
    *count = 0;
    SPH_TRY(apply_tp(h, tp));
    if (h->n == 0) return SPH_OK;
    cudaEvent_t ev[kMaxKernelsPerStep + 1];
    const int ne = step_kernel_count(h) + 1;
    for (int i = 0; i < ne; ++i) SPH_CUDA(cudaEventCreate(&ev[i]));
    int nk = 0;
    int rc = enqueue_step(h, ev, &nk);
    if (rc == SPH_OK) rc = cuda_fail(cudaEventSynchronize(ev[nk]), "timing sync");
    if (rc == SPH_OK) {
        for (int k = 0; k < nk && k < max; ++k) cudaEventElapsedTime(&ms[k], ev[k], ev[k + 1]);
        *count = nk < max ? nk : max;
    }
    for (int i = 0; i < ne; ++i) cudaEventDestroy(ev[i]);
    return rc;
}

const char *sph_cuda_kernel_name(int k) { return sph::kernel_name(k); }

const char *sph_cuda_step_kernel_name(sph_cuda_t *h, int k) { return sph::step_kernel_name(h, k); }

int sph_cuda_launches_per_step(sph_cuda_t *h)
{
    if (!h) return 0;
    return step_kernel_count(h);
}

int sph_cuda_set_launch_shapes(sph_cuda_t *h, const int *shapes)
{
    SPH_TRY(check_handle(h));
    if (!shapes) {
        set_error("null shapes");
        return SPH_ERR_INVALID;
    }
    for (int k = 0; k < kGathers; ++k) {
        const int b = shapes[2 * k], p = shapes[2 * k + 1];
        const int max_b = k == 2 ? kBlock : kMaxBlock;  // relax_update is built for <= 256
        if (b < 32 || b > max_b || (b & 31) || p < 0 || p > 32) {
            set_error("launch shape %d: block %d (32..%d, multiple of 32), persistent %d (0..32)",
                      k, b, max_b, p);
            return SPH_ERR_INVALID;
        }
    }
    for (int k = 0; k < kGathers; ++k) {
        h->shape[k].block = shapes[2 * k];
        h->shape[k].persistent = shapes[2 * k + 1];
    }
    destroy_graph(h);
    return SPH_OK;
}

int sph_cuda_set_long_row_masks(sph_cuda_t *h, int on)
{
    SPH_TRY(check_handle(h));
    if (on && !long_masks_supported()) {
        set_error("long-row masks are not built with the shared-memory staged gathers");
        return SPH_ERR_UNSUPPORTED;
    }
    if (on && !h->maskx_c) SPH_TRY(dalloc(&h->maskx_c, 3 * (size_t)h->capacity + 3));
    if ((on != 0) != h->long_masks) {
        SPH_CUDA(cudaStreamSynchronize(h->stream));
        h->long_masks = on != 0;
        destroy_graph(h);
    }
    return SPH_OK;
}

int sph_cuda_get_long_row_masks(sph_cuda_t *h) { return h && h->long_masks ? 1 : 0; }

int sph_cuda_get_launch_shapes(sph_cuda_t *h, int *shapes)
{
    SPH_TRY(check_handle(h));
    if (!shapes) {
        set_error("null shapes");
        return SPH_ERR_INVALID;
    }
    for (int k = 0; k < kGathers; ++k) {
        shapes[2 * k] = h->shape[k].block;
        shapes[2 * k + 1] = h->shape[k].persistent;
    }
    return SPH_OK;
}

// Tries each candidate launch shape on the three gathers for `trial_steps`
// steps (which advance the simulation) and keeps, per gather, the shape with
// the lowest median CUDA-event time.
int sph_cuda_autotune(sph_cuda_t *h, int trial_steps, int *shapes_out)
{
    SPH_TRY(check_handle(h));
    if (trial_steps <= 0) trial_steps = 3;
    if (h->n == 0) {
        if (shapes_out) SPH_TRY(sph_cuda_get_launch_shapes(h, shapes_out));
        return SPH_OK;
    }
    static const Shape cands[] = {{128, 0}, {256, 0}, {512, 0}, {256, 2}, {256, 4},
                                  {128, 8}, {512, 1}, {512, 2}};
    const int nc = (int)(sizeof(cands) / sizeof(cands[0]));
    // What is measured is what runs: one graph-launched step per candidate,
    // CUDA events around it.  One gather at a time (coordinate descent, the
    // others at their best so far); the candidates of a gather are
    // interleaved, one step each per round, so that the state's drift (the
    // gathers slow down as a scene compresses) reaches all of them alike;
    // the lowest median wins.
    Shape pick[kGathers];
    for (int k = 0; k < kGathers; ++k) pick[k] = h->shape[k];
    for (int k = 0; k < kGathers; ++k) {
        std::vector<float> t[sizeof(cands) / sizeof(cands[0])];
        for (int r = 0; r < trial_steps; ++r)
            for (int c = 0; c < nc; ++c) {
                Shape sc = cands[c];
                if (k == 2 && sc.block > kBlock) sc.block = kBlock;  // relax_update: <= 256
                for (int q = 0; q < kGathers; ++q) h->shape[q] = pick[q];
                h->shape[k] = sc;
                destroy_graph(h);
                SPH_TRY(run_steps(h, 1));  // captures the graph with these shapes
                SPH_CUDA(cudaEventRecord(h->timer[0], h->stream));
                SPH_TRY(run_steps(h, 1));
                SPH_CUDA(cudaEventRecord(h->timer[1], h->stream));
                SPH_CUDA(cudaEventSynchronize(h->timer[1]));
                float ms = 0.0f;
                SPH_CUDA(cudaEventElapsedTime(&ms, h->timer[0], h->timer[1]));
                t[c].push_back(ms);
            }
        float best = 3.4e38f;
        for (int c = 0; c < nc; ++c) {
            std::sort(t[c].begin(), t[c].end());
            const float med = t[c][t[c].size() / 2];
            if (med < best) {
                best = med;
                Shape sc = cands[c];
                if (k == 2 && sc.block > kBlock) sc.block = kBlock;
                pick[k] = sc;
            }
        }
    }
    for (int k = 0; k < kGathers; ++k) h->shape[k] = pick[k];
    // then the long-row hit masks, on or off, the same way (they pay where
    // stencil rows of more than 64 candidates are common, and cost a little
    // where they are not)
    if (long_masks_supported()) {
        const bool was = h->long_masks;
        if (sph_cuda_set_long_row_masks(h, 1) == SPH_OK) {
            std::vector<float> t[2];
            for (int r = 0; r < trial_steps; ++r)
                for (int v = 0; v < 2; ++v) {
                    h->long_masks = v != 0;
                    destroy_graph(h);
                    SPH_TRY(run_steps(h, 1));
                    SPH_CUDA(cudaEventRecord(h->timer[0], h->stream));
                    SPH_TRY(run_steps(h, 1));
                    SPH_CUDA(cudaEventRecord(h->timer[1], h->stream));
                    SPH_CUDA(cudaEventSynchronize(h->timer[1]));
                    float ms = 0.0f;
                    SPH_CUDA(cudaEventElapsedTime(&ms, h->timer[0], h->timer[1]));
                    t[v].push_back(ms);
                }
            for (auto &v : t) std::sort(v.begin(), v.end());
            h->long_masks = t[1][t[1].size() / 2] < t[0][t[0].size() / 2];
        } else {
            h->long_masks = was;
        }
    }
    destroy_graph(h);
    if (shapes_out) SPH_TRY(sph_cuda_get_launch_shapes(h, shapes_out));
    return SPH_OK;
}

int sph_cuda_timer_start(sph_cuda_t *h)
{
    SPH_TRY(check_handle(h));
    SPH_CUDA(cudaEventRecord(h->timer[0], h->stream));
    return SPH_OK;
}

int sph_cuda_timer_stop(sph_cuda_t *h, float *ms)
{
    SPH_TRY(check_handle(h));
    if (!ms) {
        set_error("null output");
        return SPH_ERR_INVALID;
    }
    SPH_CUDA(cudaEventRecord(h->timer[1], h->stream));
    SPH_CUDA(cudaEventSynchronize(h->timer[1]));
    SPH_CUDA(cudaEventElapsedTime(ms, h->timer[0], h->timer[1]));
    return SPH_OK;
}

int sph_cuda_host_alloc(void **ptr, size_t bytes)
{
    if (!ptr) {
        set_error("null output");
        return SPH_ERR_INVALID;
    }
    *ptr = nullptr;
    SPH_CUDA(cudaHostAlloc(ptr, bytes ? bytes : 1, cudaHostAllocDefault));
    return SPH_OK;
}

int sph_cuda_bounds_errors(unsigned *flags)
{
    if (!flags) {
        set_error("null output");
        return SPH_ERR_INVALID;
    }
    *flags = bounds_flags_kernels() | bounds_flags_learned();
    return SPH_OK;
}

int sph_cuda_bounds_checked(void)
{
#ifdef SPH_BOUNDS_CHECK
    return 1;
#else
    return 0;
#endif
}

int sph_cuda_debug_fail_allocation(int after)
{
    g_alloc_fail_after.store(after < 0 ? -1 : after);
    return SPH_OK;
}

int sph_cuda_host_free(void *ptr)
{
    if (ptr) SPH_CUDA(cudaFreeHost(ptr));
    return SPH_OK;
}

int sph_cuda_tunables_preset(tunable_parameters *tp, char which)
{
    if (!tp) {
        set_error("null tunables");
        return SPH_ERR_INVALID;
    }
    struct Preset {
        char id;
        float g, k, k_near, k_spring, sigma, beta, rest;
    };
    // the render rank's presets, controls.c:344-401
    static const Preset presets[] = {
        {'x', 6.0f, 0.2f, 6.0f, 10.0f, 5.0f, 0.5f, 30.0f},
        {'y', 6.0f, 0.1f, 3.0f, -30.0f, 100.0f, 10.0f, 30.0f},
        {'a', 0.0f, 0.2f, 6.0f, 10.0f, 20.0f, 2.0f, 55.0f},
        {'b', 6.0f, 0.0f, 0.0f, 115.0f, 20.0f, 2.0f, 0.0f},
    };
    if (which == 'm') {
        tp->mover_width = 2.0f;
        tp->mover_height = 2.0f;
        return SPH_OK;
    }
    for (const Preset &p : presets)
        if (p.id == which) {
            tp->g = p.g;
            tp->k = p.k;
            tp->k_near = p.k_near;
            tp->k_spring = p.k_spring;
            tp->sigma = p.sigma;
            tp->beta = p.beta;
            tp->rest_density = p.rest;
            return SPH_OK;
        }
    set_error("unknown preset '%c' (x, y, a, b or m)", which);
    return SPH_ERR_INVALID;
}

int sph_cuda_mover_track(float max_x, float max_y, float *gl_x, int *direction, float *center_x,
                         float *center_y)
{
    if (!gl_x || !direction || !center_x || !center_y) {
        set_error("null argument");
        return SPH_ERR_INVALID;
    }
    float x = *gl_x + 0.01f * (float)*direction;
    if (x > 1.0f || x < -1.0f) *direction = -*direction;
    const float y = sinf(3.14f * 5.0f * x) / 10.0f - 0.6f;
    *gl_x = x;
    const float hw = max_x * 0.5f, hh = max_y * 0.5f;
    *center_x = x * hw + hw;
    *center_y = y * hh + hh;
    return SPH_OK;
}

}  // extern "C"
