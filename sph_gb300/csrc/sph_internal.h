// sph_internal.h -- shared between the translation units of libsph_cuda.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_cuda.h"

namespace sph {

// Neighbour grid as the kernels see it.  Cell key = gy * size_x + gx
// (hash.c:35-47); key `ncells` is the "no cell" bucket that collects
// particles whose key falls outside the grid.
struct Grid {
    float spacing;
    int size_x, size_y;
    int ncells;
    float min_x, max_x, min_y, max_y;
    int max_bucket;
    int max_neighbors;
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
    unsigned int pad[5];
};

enum BuildSlot { SLOT_PREDICTED = 0, SLOT_RELAXED = 1, SLOT_UPLOAD = 2, SLOT_PROBE = 3 };

constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;                        // per thread
constexpr int kScanTile = kScanThreads * kScanItems;  // cells per scan tile
constexpr int kBlock = 256;                           // particle kernels
constexpr int kRankScanMax = 1024;  // cells above this population use atomic order
constexpr int kMaxKernelsPerStep = 16;

}  // namespace sph

// The handle.  Arrays named by the order they are kept in:
//   *_a : sorted by (cell of pos_a, id)  -- the state between steps
//   *_b : scratch in the order of the pass that wrote it
//   *_c : sorted by (cell of the predicted position, id)
struct sph_cuda {
    sph::Grid g;
    int capacity = 0;
    int n = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;

    float2 *pos_a = nullptr, *vel_a = nullptr;
    int *id_a = nullptr;
    float2 *pos_b = nullptr, *prev_b = nullptr, *vel_b = nullptr;
    uint2 *kr_b = nullptr;  // (cell key, arrival rank) per particle
    float2 *pos_c = nullptr, *prev_c = nullptr;
    float4 *xr_c = nullptr;               // (x, y, rho, rho_near) of the density pass
    ulonglong2 *mask01_c = nullptr;       // neighbour hit masks of stencil rows 0, 1
    unsigned long long *mask2_c = nullptr;  // ... and row 2
    int *id_c = nullptr;
    int *tmp_id = nullptr;
    unsigned int *cnt = nullptr;  // ncells + 1 counters, zero between builds
    int *start_a = nullptr;       // ncells + 2 cell starts for the *_a order
    int *start_c = nullptr;       // ncells + 2 cell starts for the *_c order
    int *tile_sums = nullptr;
    int ntiles = 0;

    tunable_parameters *d_params = nullptr;
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
    tunable_parameters last_tp;
    bool tp_valid = false;

    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    int graph_n = -1;
    cudaEvent_t timer[2] = {nullptr, nullptr};
    int launches_per_step = 0;
};

namespace sph {

// Error reporting (per host thread).
void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

// Core operations shared by the fast API and the legacy entry points.
int ensure_scratch(sph_cuda *h, size_t bytes);
int ensure_stage(sph_cuda *h, size_t bytes);
int upload_soa_device(sph_cuda *h, int n);  // pos_b/vel_b (id order) + xr_c -> state
int set_params(sph_cuda *h, const tunable_parameters *tp);
int enqueue_step(sph_cuda *h, cudaEvent_t *events, int *nkernels);
int run_steps(sph_cuda *h, int nsteps);
int neighbor_lists(sph_cuda *h, int *counts, int *ids, long long max_total, long long *total);

}  // namespace sph
