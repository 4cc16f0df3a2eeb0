// sph_internal.h -- shared between the translation units of libsph_cuda.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "sph_cuda.h"

namespace sph {

// One scene -- an independent domain with its own box, grid and tunables --
// as the kernels see it.  A handle holds one scene (the compute rank's
// domain) or many (an ensemble).  Cell keys are global: a scene's local key
// gy * size_x + gx (hash.c:35-47) is offset by c_off, and local key
// `ncells` is the scene's own "no cell" bucket for particles whose key falls
// outside its grid.  Sorting by global key keeps each scene's particles in
// the contiguous slot range [p_off, p_off + n), in the id range of the same
// bounds.
struct Scene {
    tunable_parameters P;  // first member: per-step updates copy into it
    float spacing;
    int size_x, size_y;
    int ncells;
    int c_off;
    int p_off;
    int n;
    float min_x, max_x, min_y, max_y;
    int max_bucket;
    int max_neighbors;
    int pad[3];
};
static_assert(sizeof(Scene) % 16 == 0, "Scene is loaded as an aligned record");

// What every particle kernel receives by value.
struct Ctx {
    const Scene *scenes;
    const int *p_off;  // nscenes + 1 slot offsets (p_off[s] = scenes[s].p_off)
    int nscenes;
    int n;             // particles of all scenes
    int max_bucket;    // bucket cap, the same in every scene
    int M;             // cell counters of all scenes (cells + no-cell buckets)
    // particles per scan tile of the build that the kernel's cell keys feed,
    // counted by the step's key producers (null: not counted)
    unsigned *tile_cnt = nullptr;
    // long-row hit masks (kernels built for them only): per particle, 3
    // words holding the hit bits of candidates kMaskRow..2 kMaskRow - 1 of
    // each stencil row (null: rows longer than kMaskRow are not masked)
    unsigned long long *maskx = nullptr;
};

// Device-resident counters and flags of one handle.
struct DevState {
    unsigned long long steps;
    unsigned long long out_of_grid;
    unsigned long long bucket_overflow;
    unsigned int max_occ;          // largest cell population ever seen
    unsigned int list_cap_risk;
    unsigned int lists_valid;      // a neighbour relation exists: viscosity is on
    unsigned int build_max_occ[4]; // per build slot, reset by the build's key producer
    unsigned int fb_count;         // learned step: fallback particles with masked rows (list front)
    unsigned int fb_long;          // ... and with rows too long for a mask (list back)
    unsigned int tile_count_mismatch;  // a build's tile counts disagreed with its counters
    unsigned int pad[2];
    unsigned long long learned_steps;     // steps run with a learned model attached
    unsigned long long learned_fallback;  // particle-steps of those that used the plain relaxation
};

enum BuildSlot { SLOT_PREDICTED = 0, SLOT_RELAXED = 1, SLOT_UPLOAD = 2, SLOT_PROBE = 3 };

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;                        // per thread
constexpr int kScanTile = kScanThreads * kScanItems;  // cells per scan tile
// tiles of a step's cell build (k_cell_starts), counted by the key producers
#ifndef SPH_BUILD_THREADS
#define SPH_BUILD_THREADS 256
#endif
#ifndef SPH_BUILD_ITEMS
#define SPH_BUILD_ITEMS 16
#endif
constexpr int kBuildThreads = SPH_BUILD_THREADS;  // cell-starts CTA
constexpr int kBuildItems = SPH_BUILD_ITEMS;      // cell counters per thread
constexpr int kBuildTile = kBuildThreads * kBuildItems;
static_assert(kBuildTile >= kScanTile, "the build's tile counts fit the scan tile buffer");
constexpr int kBlock = 256;                           // default particle-kernel block
constexpr int kMaxBlock = 512;                        // largest block an autotuner may pick
constexpr int kRankScanMax = 1024;  // cells above this population use atomic order
constexpr int kMaxKernelsPerStep = 16;
constexpr int kGathers = 3;         // viscosity_predict, density, relax_update

// Launch shape of one gather kernel: threads per block, and 0 for one block
// per tile of particles or the number of resident blocks per SM for a
// persistent grid-stride launch.
struct Shape {
    int block = kBlock;
    int persistent = 0;
};

struct LearnedModel;

}  // namespace sph

// The handle.  Arrays named by the order they are kept in:
//   *_a : sorted by (cell of pos_a, id)  -- the state between steps
//   *_b : scratch in the order of the pass that wrote it
//   *_c : sorted by (cell of the predicted position, id)
struct sph_cuda {
    std::vector<sph::Scene> scenes;  // host copy of the scene table
    int nscenes = 0;
    int M = 0;                       // cell counters of all scenes (cells + no-cell buckets)
    int max_bucket = 0, max_neighbors = 0;
    int capacity = 0;
    int n = 0;
    int num_sms = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;

    sph::Scene *d_scenes = nullptr;
    int *d_p_off = nullptr;
    unsigned *d_nocell = nullptr;  // bit per cell counter: set for the no-cell buckets

    float2 *pos_a = nullptr, *vel_a = nullptr;
    int *id_a = nullptr;
    float2 *pos_b = nullptr, *prev_b = nullptr, *vel_b = nullptr;
    uint2 *kr_b = nullptr;  // (cell key, arrival rank) per particle
    float2 *pos_c = nullptr, *prev_c = nullptr;
    float4 *xr_c = nullptr;               // (x, y, rho, rho_near) of the density pass
    ulonglong2 *mask01_c = nullptr;       // neighbour hit masks of stencil rows 0, 1
    unsigned long long *mask2_c = nullptr;  // ... and row 2
    // long-row hit masks (sph_cuda_set_long_row_masks): 3 words per particle
    bool long_masks = false;
    unsigned long long *maskx_c = nullptr;
    int4 *rows_c = nullptr;               // the stencil rows' first slots and walk mode
    int *id_c = nullptr;
    int *tmp_id = nullptr;
    unsigned int *cnt = nullptr;  // M counters, zero between builds
    int *start_a = nullptr;       // M + 1 cell starts for the *_a order
    int *start_c = nullptr;       // M + 1 cell starts for the *_c order
    int *tile_sums = nullptr;
    unsigned *build_tiles = nullptr;  // particles per build tile of a step's build (kept zero between builds)
    int ntiles = 0;

    sph::DevState *d_state = nullptr;
    double *d_partials = nullptr;
    int npartials = 0;

    // output scratch (device) and pinned staging (host), grown on demand
    void *d_scratch = nullptr;
    size_t d_scratch_bytes = 0;
    void *h_stage = nullptr;
    size_t h_stage_bytes = 0;

    // pinned ring of tunables for asynchronous parameter updates
    tunable_parameters *h_params_ring = nullptr;
    cudaEvent_t *params_ev = nullptr;
    int params_ring = 0;
    int params_next = 0;
    std::vector<tunable_parameters> last_tp;  // per scene, as last copied
    std::vector<char> tp_valid;

    sph::Shape shape[sph::kGathers];  // launch shapes of the gathers (autotuned)

    // learned relaxation (attached model, its threshold and per-step buffers in C order)
    sph::LearnedModel *learned = nullptr;
    float learned_thr = 0.01f;
    void *feat_c = nullptr;          // BF16 feature rows, 32 per particle
    unsigned short *nbc_c = nullptr;  // neighbour counts (65535: never use the network)
    float4 *net_c = nullptr;         // network outputs (dx / s, dy / s, error, 0)
    int *fb_list = nullptr;          // slots that take the plain relaxation this step

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_n = -1;
    cudaEvent_t timer[2] = {nullptr, nullptr};
    int launches_per_step = 0;

    // asynchronous coordinate hand-off: two device staging buffers, copied to
    // the caller's host buffers on their own stream
    cudaStream_t copy_stream = nullptr;
    short2 *d_coords[2] = {nullptr, nullptr};
    cudaEvent_t pack_ev[2] = {nullptr, nullptr};
    cudaEvent_t copy_ev[2] = {nullptr, nullptr};
    const void *copy_dst[2] = {nullptr, nullptr};
    int pack_slot = 0;
};

namespace sph {

// Error reporting (per host thread).
void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

inline Ctx make_ctx(const sph_cuda *h)
{
    Ctx c;
    c.scenes = h->d_scenes;
    c.p_off = h->d_p_off;
    c.nscenes = h->nscenes;
    c.n = h->n;
    c.max_bucket = h->max_bucket;
    c.M = h->M;
    c.tile_cnt = h->build_tiles;
    c.maskx = h->long_masks ? h->maskx_c : nullptr;
    return c;
}

// Core operations shared by the fast API and the legacy entry points.
int ensure_scratch(sph_cuda *h, size_t bytes);
int ensure_stage(sph_cuda *h, size_t bytes);
int upload_soa_device(sph_cuda *h, int n);  // pos_b/vel_b (id order) + xr_c -> state
int launch_upload_layout(sph_cuda *h, int n, const float *x, const float *y, const float *vx,
                         const float *vy, const fluid_particle *recs);
int launch_split_soa(sph_cuda *h, int n, const float2 *rec, float *out);
int set_scene_params(sph_cuda *h, int scene, const tunable_parameters *tp);
int enqueue_step(sph_cuda *h, cudaEvent_t *events, int *nkernels,
                 const tunable_parameters *mid_tp = nullptr);
unsigned bounds_flags_kernels();  // checked builds (SPH_BOUNDS_CHECK): recorded index faults
unsigned bounds_flags_learned();
int enqueue_predicted_state(sph_cuda *h);       // first half of a step: C order + density
int launch_density_pass(sph_cuda *h);            // the density pass on the C order
bool long_masks_supported();
int launch_learned_passes(sph_cuda *h, cudaEvent_t *events);  // features + network (C order)
int launch_learned_relax(sph_cuda *h, float2 *probe_out, cudaEvent_t *events = nullptr);
void free_learned_buffers(sph_cuda *h);
const char *step_kernel_name(const sph_cuda *h, int k);
int step_kernel_count(const sph_cuda *h);
int run_steps(sph_cuda *h, int nsteps);

}  // namespace sph
