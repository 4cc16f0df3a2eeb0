// sph_noalloc.cu -- a density pass that allocates no memory.
//
// Some callers of this library cannot call cudaMalloc: a step loop that owns
// a fixed device-memory budget handed out by another framework's allocator,
// or a real-time loop (the render-driven compute rank) that must not take the
// device-wide synchronisation a cudaMalloc/cudaFree can imply.  For them,
// sph_cuda_density_static() computes the reference's density and near
// density (hash_fluid(.., true) + calculate_density, hash.c:127-242 /
// fluid.c:527-539) of caller-owned device arrays, keeping every intermediate
// (cell keys, histogram, cell starts, sorted copies) in the file-scope array
// below, whose size is fixed at compile time.  Every GPU that loads the
// library holds that array (about 7 MB) until the process exits.
#include <mutex>

#include "sph_internal.h"

namespace sph {

// Kernels of sph_kernels.cu, launched here unchanged.
__global__ void k_keys(Ctx c, const float2 *__restrict__ pos, uint2 *__restrict__ kr,
                       unsigned *__restrict__ cnt, unsigned *occ_reset);
__global__ void k_scan_reduce(const unsigned *__restrict__ in, int M,
                              const unsigned *__restrict__ nocell, int *__restrict__ tile_sums,
                              DevState *__restrict__ st, unsigned *occ, int max_bucket,
                              int max_neighbors);
__global__ void k_scan_apply(unsigned *__restrict__ in, int M, const int *__restrict__ tile_sums,
                             int *__restrict__ out, int zero_input);
__global__ void k_scatter_ids(int n, const uint2 *__restrict__ kr, const int *__restrict__ id_src,
                              const int *__restrict__ start, int *__restrict__ tmp,
                              unsigned *tile_cnt, int ntiles);
__global__ void k_permute(int n, const uint2 *__restrict__ kr, const int *__restrict__ start,
                          const int *__restrict__ tmp, const int *__restrict__ id_src,
                          const float2 *__restrict__ a_src, const float2 *__restrict__ b_src,
                          int *__restrict__ id_dst, float2 *__restrict__ a_dst,
                          float2 *__restrict__ b_dst, DevState *__restrict__ end_step);
__global__ void k_density(Ctx c, const float2 *__restrict__ pos, const int *__restrict__ start,
                          const unsigned *__restrict__ occ_in, float4 *__restrict__ xr_out,
                          ulonglong2 *__restrict__ mask01, unsigned long long *__restrict__ mask2,
                          int4 *__restrict__ rows_out);

namespace {

constexpr size_t kAlign = 256;
constexpr size_t up(size_t b) { return (b + kAlign - 1) / kAlign * kAlign; }

constexpr size_t kN = SPH_STATIC_MAX_PARTICLES;
constexpr size_t kC = SPH_STATIC_MAX_CELLS;
constexpr size_t kTiles = ((kC + 1 > kN ? kC + 1 : kN) + 1 + kScanTile - 1) / kScanTile;

// Layout of the scratch array (byte offsets, each 256-byte aligned).
constexpr size_t kNocellWords = (kC + 1 + 31) / 32 + 1;
constexpr size_t kOffScene = 0;
constexpr size_t kOffPoff = kOffScene + up(sizeof(Scene));
constexpr size_t kOffNocell = kOffPoff + up(2 * sizeof(int));
constexpr size_t kOffState = kOffNocell + up(kNocellWords * sizeof(unsigned));
constexpr size_t kOffCnt = kOffState + up(sizeof(DevState));
constexpr size_t kOffStart = kOffCnt + up((kC + 1) * sizeof(unsigned));
constexpr size_t kOffTiles = kOffStart + up((kC + 2) * sizeof(int));
constexpr size_t kOffPosIn = kOffTiles + up(kTiles * sizeof(int));
constexpr size_t kOffKr = kOffPosIn + up(kN * sizeof(float2));
constexpr size_t kOffTmp = kOffKr + up(kN * sizeof(uint2));
constexpr size_t kOffPosS = kOffTmp + up(kN * sizeof(int));
constexpr size_t kOffIdS = kOffPosS + up(kN * sizeof(float2));
constexpr size_t kOffXr = kOffIdS + up(kN * sizeof(int));
constexpr size_t kOffM01 = kOffXr + up(kN * sizeof(float4));
constexpr size_t kOffM2 = kOffM01 + up(kN * sizeof(ulonglong2));
constexpr size_t kScratchBytes = kOffM2 + up(kN * sizeof(unsigned long long));

}  // namespace

// The scratch of sph_cuda_density_static: shared by every call on a device.
static __device__ __align__(256) unsigned char g_static_scratch[kScratchBytes];

namespace {

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
void *g_scratch_addr[kMaxDevices] = {};

// Device address of g_static_scratch on the current device (the host-side
// name of the array is only a stand-in).  Looked up again on every call that
// is not being captured into a graph, so that a context torn down and
// recreated (cudaDeviceReset) is seen; a call under stream capture uses the
// address of the last call on this device outside capture, which must
// exist.
int scratch_address(cudaStream_t stream, void **out)
{
    int dev = 0;
    int rc = cuda_fail(cudaGetDevice(&dev), "cudaGetDevice");
    if (rc != SPH_OK) return rc;
    if (dev < 0 || dev >= kMaxDevices) {
        set_error("device ordinal %d above %d", dev, kMaxDevices - 1);
        return SPH_ERR_UNSUPPORTED;
    }
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    rc = cuda_fail(cudaStreamIsCapturing(stream, &cap), "cudaStreamIsCapturing");
    if (rc != SPH_OK) return rc;
    std::lock_guard<std::mutex> lock(g_setup_mu);
    if (cap == cudaStreamCaptureStatusNone) {
        void *p = nullptr;
        rc = cuda_fail(cudaGetSymbolAddress(&p, g_static_scratch), "cudaGetSymbolAddress");
        if (rc != SPH_OK) return rc;
        g_scratch_addr[dev] = p;
    } else if (!g_scratch_addr[dev]) {
        set_error("sph_cuda_density_static: the first call on a device must come before any "
                  "stream capture");
        return SPH_ERR_STATE;
    }
    *out = g_scratch_addr[dev];
    return SPH_OK;
}

// The one-scene table of the call: scene record, slot offsets {0, n} and
// the scene's no-cell bucket in the (cleared) no-cell bitmap.
__global__ void k_static_scene(Scene s)
{
    *reinterpret_cast<Scene *>(g_static_scratch + kOffScene) = s;
    int *p_off = reinterpret_cast<int *>(g_static_scratch + kOffPoff);
    p_off[0] = 0;
    p_off[1] = s.n;
    unsigned *bits = reinterpret_cast<unsigned *>(g_static_scratch + kOffNocell);
    bits[s.ncells >> 5] |= 1u << (s.ncells & 31);
}

__global__ void __launch_bounds__(kBlock)
k_static_gather(int n, const float *__restrict__ x, const float *__restrict__ y,
                float2 *__restrict__ pos)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) pos[i] = make_float2(x[i], y[i]);
}

__global__ void __launch_bounds__(kBlock)
k_static_scatter(int n, const int *__restrict__ ids, const float4 *__restrict__ xr,
                 float *__restrict__ rho, float *__restrict__ rho_near)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = xr[i];
    const int id = ids[i];
    rho[id] = v.z;
    rho_near[id] = v.w;
}

// The counters of the last call's cell build, into caller device memory.
__global__ void k_static_counters(sph_cuda_counters *out)
{
    const DevState *st = reinterpret_cast<const DevState *>(g_static_scratch + kOffState);
    sph_cuda_counters c;
    c.steps = 0ull;
    c.out_of_grid = st->out_of_grid;
    c.bucket_overflow = st->bucket_overflow;
    c.max_cell_occupancy = st->max_occ;
    c.list_cap_risk = st->list_cap_risk;
    *out = c;
}

}  // namespace
}  // namespace sph

using namespace sph;

extern "C" int sph_cuda_density_static_counters(sph_cuda_counters *d_out, void *stream)
{
    if (!d_out) {
        set_error("sph_cuda_density_static_counters: null device output");
        return SPH_ERR_INVALID;
    }
    // the kernel names the array itself: no device address is needed here
    k_static_counters<<<1, 1, 0, static_cast<cudaStream_t>(stream)>>>(d_out);
    return cuda_fail(cudaGetLastError(), "sph_cuda_density_static_counters launch");
}

extern "C" int sph_cuda_density_static(const float *x, const float *y, int n,
                                       const neighbor_grid_t *grid, const tunable_parameters *tp,
                                       float *density, float *density_near, void *stream)
{
    if (!grid || !tp) {
        set_error("sph_cuda_density_static: null grid or tunables");
        return SPH_ERR_INVALID;
    }
    if (n < 0 || n > SPH_STATIC_MAX_PARTICLES) {
        set_error("sph_cuda_density_static: %d particles, the static scratch holds at most %d", n,
                  SPH_STATIC_MAX_PARTICLES);
        return n < 0 ? SPH_ERR_INVALID : SPH_ERR_CAPACITY;
    }
    const unsigned long long cells = (unsigned long long)grid->size_x * grid->size_y;
    if (!(grid->spacing > 0.0f) || cells == 0 || grid->max_bucket_size == 0 ||
        grid->max_neighbors == 0) {
        set_error("sph_cuda_density_static: invalid neighbour grid");
        return SPH_ERR_INVALID;
    }
    if (cells > SPH_STATIC_MAX_CELLS) {
        set_error("sph_cuda_density_static: %llu grid cells, the static scratch holds at most %d",
                  cells, SPH_STATIC_MAX_CELLS);
        return SPH_ERR_CAPACITY;
    }
    if (!(tp->smoothing_radius > 0.0f)) {
        set_error("sph_cuda_density_static: smoothing_radius must be positive");
        return SPH_ERR_INVALID;
    }
    if (n > 0 && (!x || !y || !density || !density_near)) {
        set_error("sph_cuda_density_static: null device array");
        return SPH_ERR_INVALID;
    }
    void *base_v = nullptr;
    int rc = scratch_address(static_cast<cudaStream_t>(stream), &base_v);
    if (rc != SPH_OK) return rc;
    if (n == 0) return SPH_OK;

    char *base = static_cast<char *>(base_v);
    const Scene *scene = reinterpret_cast<const Scene *>(base + kOffScene);
    const int *p_off = reinterpret_cast<const int *>(base + kOffPoff);
    unsigned *nocell = reinterpret_cast<unsigned *>(base + kOffNocell);
    DevState *state = reinterpret_cast<DevState *>(base + kOffState);
    unsigned *cnt = reinterpret_cast<unsigned *>(base + kOffCnt);
    int *start = reinterpret_cast<int *>(base + kOffStart);
    int *tiles = reinterpret_cast<int *>(base + kOffTiles);
    float2 *pos_in = reinterpret_cast<float2 *>(base + kOffPosIn);
    uint2 *kr = reinterpret_cast<uint2 *>(base + kOffKr);
    int *tmp = reinterpret_cast<int *>(base + kOffTmp);
    float2 *pos_s = reinterpret_cast<float2 *>(base + kOffPosS);
    int *id_s = reinterpret_cast<int *>(base + kOffIdS);
    float4 *xr = reinterpret_cast<float4 *>(base + kOffXr);
    ulonglong2 *m01 = reinterpret_cast<ulonglong2 *>(base + kOffM01);
    unsigned long long *m2 = reinterpret_cast<unsigned long long *>(base + kOffM2);

    Scene sc{};
    sc.P = *tp;
    sc.spacing = grid->spacing;
    sc.size_x = (int)grid->size_x;
    sc.size_y = (int)grid->size_y;
    sc.ncells = (int)cells;
    sc.c_off = 0;
    sc.p_off = 0;
    sc.n = n;
    sc.max_bucket = (int)grid->max_bucket_size;
    sc.max_neighbors = (int)grid->max_neighbors;
    Ctx c;
    c.scenes = scene;
    c.p_off = p_off;
    c.nscenes = 1;
    c.n = n;
    c.max_bucket = sc.max_bucket;
    c.M = (int)cells + 1;

    cudaStream_t s = static_cast<cudaStream_t>(stream);
    const int M = sc.ncells + 1;
    const int nt = (M + kScanTile - 1) / kScanTile;
    const int nb = (n + kBlock - 1) / kBlock;
    // The array keeps the previous call's contents: the histogram and the
    // counters must start from zero.
    rc = cuda_fail(cudaMemsetAsync(cnt, 0, (size_t)M * sizeof(unsigned), s), "cudaMemsetAsync");
    if (rc != SPH_OK) return rc;
    rc = cuda_fail(cudaMemsetAsync(state, 0, sizeof(DevState), s), "cudaMemsetAsync");
    if (rc != SPH_OK) return rc;
    rc = cuda_fail(cudaMemsetAsync(nocell, 0, ((size_t)M + 31) / 32 * sizeof(unsigned), s),
                   "cudaMemsetAsync");
    if (rc != SPH_OK) return rc;
    unsigned *occ = &state->build_max_occ[SLOT_PROBE];
    k_static_scene<<<1, 1, 0, s>>>(sc);
    k_static_gather<<<nb, kBlock, 0, s>>>(n, x, y, pos_in);
    k_keys<<<nb, kBlock, 0, s>>>(c, pos_in, kr, cnt, occ);
    k_scan_reduce<<<nt, kScanThreads, 0, s>>>(cnt, M, nocell, tiles, state, occ, sc.max_bucket,
                                              sc.max_neighbors);
    k_scan_apply<<<nt, kScanThreads, 0, s>>>(cnt, M, tiles, start, 1);
    k_scatter_ids<<<nb, kBlock, 0, s>>>(n, kr, nullptr, start, tmp, nullptr, 0);
    k_permute<<<nb, kBlock, 0, s>>>(n, kr, start, tmp, nullptr, pos_in, nullptr, id_s, pos_s,
                                    nullptr, nullptr);
    k_density<<<nb, kBlock, 0, s>>>(c, pos_s, start, occ, xr, m01, m2, nullptr);
    k_static_scatter<<<nb, kBlock, 0, s>>>(n, id_s, xr, density, density_near);
    return cuda_fail(cudaGetLastError(), "sph_cuda_density_static launch");
}
