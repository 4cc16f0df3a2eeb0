// sph_kernels.cu -- the step kernels of libsph_cuda (sm_103a).
//
// One step (fluid.c:273-348) is eleven kernels on one stream, captured as a
// CUDA graph:
//
//   viscosity_predict   gravity + viscosity gather + predict + BCs + cell key   (A -> B)
//   scan_reduce/apply   exclusive scan of the cell histogram -> cell starts      (C cells)
//   scatter, permute    counting-sort scatter, then in-cell order by id          (B -> C)
//   density             density / near-density gather                           (C)
//   relax_update        relaxation gather + BCs + velocity update + cell key     (C -> B)
//   scan_reduce/apply   cell starts of the relaxed positions                     (A cells)
//   scatter, permute    back into (cell, id) order                              (B -> A)
//
// A handle holds one scene or many (an ensemble): every kernel runs over the
// particles of all scenes at once, each particle reading its own scene's
// grid and tunables from the scene table.
//
// Every pass is a gather: a thread owns one particle (in sorted order) and
// reads its 3x3 cell stencil, so no floating-point atomics exist and every
// sum is taken in a fixed order: the results are deterministic.  The only
// atomics are the integer cell-histogram increments, whose arrival rank is
// used solely to give each particle a distinct scratch slot; the final
// in-cell order is by id, recomputed deterministically in `permute`.
#include <algorithm>
#include <type_traits>
#include <utility>
#include <cstdio>

#include "sph_device.cuh"
#include "sph_learned.h"

// Unroll factors of the candidate filter loops and the relaxation's
// register budget (tuned on GB300).
#ifndef SPH_VISC_UNROLL
#define SPH_VISC_UNROLL 4
#endif
#ifndef SPH_DENS_UNROLL
#define SPH_DENS_UNROLL 2
#endif
#ifndef SPH_RELAX_MIN_BLOCKS
#define SPH_RELAX_MIN_BLOCKS 4  // resident 256-thread CTAs per SM the relaxation is built for
#endif
#ifndef SPH_RELAX_SMEM
#define SPH_RELAX_SMEM 0  // relaxation reads its stencil rows from a shared-memory copy
#endif
#ifndef SPH_DENS_SMEM
#define SPH_DENS_SMEM 0   // density pass likewise
#endif
#ifndef SPH_VISC_SMEM
#define SPH_VISC_SMEM 0   // viscosity pass likewise
#endif

namespace sph {
// Shared-memory elements a gather CTA stages per thread of the CTA (the
// three stencil-row runs of a CTA in one grid row are about 3.2 per thread).
#ifndef SPH_STAGE_PER_THREAD
#define SPH_STAGE_PER_THREAD 4
#endif
constexpr int kStagePerThread = SPH_STAGE_PER_THREAD;
constexpr int kViscUnroll = SPH_VISC_UNROLL;
constexpr int kDensUnroll = SPH_DENS_UNROLL;
}  // namespace sph

namespace sph {

// ---------------------------------------------------------------------------
// block-wide helpers
// ---------------------------------------------------------------------------

template <class T>
__device__ __forceinline__ T warp_sum(T v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ unsigned warp_max(unsigned v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Counts one particle with cell key `key` into its build tile: the lanes of
// the warp that reach this call together and share a tile add with one
// atomic (the particles of a warp are neighbours in cell order, so almost
// every warp issues one).
__device__ __forceinline__ void add_tile_count(unsigned *tile_cnt, unsigned key)
{
    if (!tile_cnt) return;
    const unsigned active = __activemask();
    const unsigned t = key / (unsigned)kBuildTile;
    const unsigned lane = threadIdx.x & 31;
    const int first = __ffs(active) - 1;
    // nearly every warp's particles share one tile: a broadcast and a vote
    // settle it; the rest group their lanes by tile
    const unsigned t0 = __shfl_sync(active, t, first);
    if (__all_sync(active, t == t0)) {
        if (lane == (unsigned)first) atomicAdd(tile_cnt + t0, (unsigned)__popc(active));
        return;
    }
    const unsigned peers = __match_any_sync(active, t);
    if (lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(tile_cnt + t, (unsigned)__popc(peers));
}

// The same count for a whole CTA, called once by every thread of it (t: the
// build tile of the key the thread made, -1 for none): warps whose keys
// share one tile report it to thread 0, which adds runs of equal tiles with
// one atomic each.  The particles a CTA advances lie in one or two tiles,
// and the CTAs running at any moment in a narrow range of them: in a light
// kernel (the learned relaxation) one atomic per warp makes those few
// counters a hot spot, one per CTA does not.  The gathers keep the warp
// form: the barrier here would hold each CTA until its slowest warp.
__device__ __forceinline__ void cta_tile_count(unsigned *tile_cnt, int t)
{
    __shared__ int s_t[kMaxBlock / 32];
    __shared__ unsigned s_c[kMaxBlock / 32];
    const unsigned lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned made = __ballot_sync(0xffffffffu, t >= 0);
    int t0 = -1;
    bool uniform = true;
    if (made) {
        t0 = __shfl_sync(0xffffffffu, t, __ffs(made) - 1);
        uniform = __all_sync(0xffffffffu, t < 0 || t == t0);
    }
    if (!uniform && t >= 0) {
        const unsigned peers = __match_any_sync(made, t);
        if (lane == (unsigned)(__ffs(peers) - 1)) atomicAdd(tile_cnt + t, (unsigned)__popc(peers));
    }
    if (lane == 0) {
        s_t[warp] = (made && uniform) ? t0 : -1;
        s_c[warp] = (unsigned)__popc(made);
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        int cur = -1;
        unsigned acc = 0u;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            const int tw = s_t[w];
            if (tw < 0) continue;
            if (tw != cur) {
                if (cur >= 0) atomicAdd(tile_cnt + cur, acc);
                cur = tw;
                acc = 0u;
            }
            acc += s_c[w];
        }
        if (cur >= 0) atomicAdd(tile_cnt + cur, acc);
    }
}

// Exclusive scan over the block; returns the thread's exclusive prefix and
// the block total.  `sh` holds one word per warp.
__device__ __forceinline__ unsigned block_exclusive_scan(unsigned v, unsigned *sh, unsigned &total)
{
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    unsigned x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) sh[warp] = x;
    __syncthreads();
    if (warp == 0) {
        unsigned w = lane < nw ? sh[lane] : 0u;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < nw) sh[lane] = w;
    }
    __syncthreads();
    total = sh[nw - 1];
    const unsigned before = warp ? sh[warp - 1] : 0u;
    __syncthreads();
    return before + x - v;
}

// ---------------------------------------------------------------------------
// cell build: histogram scan, scatter, permute
// ---------------------------------------------------------------------------

// Per-tile sums of the histogram, and occupancy statistics of the in-grid
// cells (`nocell` has a bit set for every scene's no-cell bucket).
__global__ void __launch_bounds__(kScanThreads)
k_scan_reduce(const unsigned *__restrict__ in, int M, const unsigned *__restrict__ nocell,
              int *__restrict__ tile_sums, DevState *__restrict__ st, unsigned *occ,
              int max_bucket, int max_neighbors)
{
    __shared__ unsigned sh_s[kScanThreads / 32], sh_m[kScanThreads / 32];
    __shared__ unsigned long long sh_e[kScanThreads / 32], sh_o[kScanThreads / 32];
    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    unsigned s = 0, mx = 0;
    unsigned long long excess = 0, outside = 0;
    unsigned v[kScanItems];
    if (base + kScanItems <= M) {
        const uint4 *p = reinterpret_cast<const uint4 *>(in + base);
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            const uint4 t = p[q];
            v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
        }
    } else {
#pragma unroll
        for (int e = 0; e < kScanItems; ++e) v[e] = base + e < M ? in[base + e] : 0u;
    }
    // the thread's 16 counters lie in one 32-bit word of the no-cell bitmap
    const unsigned bits = (nocell && base < M) ? (__ldg(nocell + (base >> 5)) >> (base & 31)) : 0u;
#pragma unroll
    for (int e = 0; e < kScanItems; ++e) {
        s += v[e];
        if ((bits >> e) & 1u) {
            outside += v[e];
        } else {
            mx = max(mx, v[e]);
            if (v[e] > (unsigned)max_bucket) excess += v[e] - max_bucket;
        }
    }
    s = warp_sum(s);
    mx = warp_max(mx);
    excess = warp_sum(excess);
    outside = warp_sum(outside);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { sh_s[warp] = s; sh_m[warp] = mx; sh_e[warp] = excess; sh_o[warp] = outside; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned ts = 0, tm = 0;
        unsigned long long te = 0, to = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) {
            ts += sh_s[w]; tm = max(tm, sh_m[w]); te += sh_e[w]; to += sh_o[w];
        }
        tile_sums[blockIdx.x] = (int)ts;
        if (occ) {
            atomicMax(occ, tm);
            atomicMax(&st->max_occ, tm);
            if (te) atomicAdd(&st->bucket_overflow, te);
            if (to) atomicAdd(&st->out_of_grid, to);
            const unsigned m = tm < (unsigned)max_bucket ? tm : (unsigned)max_bucket;
            if (m > 0 && 5u * m - 1u > (unsigned)max_neighbors) atomicOr(&st->list_cap_risk, 1u);
        }
    }
}

// Exclusive scan: out[i] = sum(in[0..i)), out[M] = total.  Zeroes `in` when
// asked (the histogram must be zero before the next build).
__global__ void __launch_bounds__(kScanThreads)
k_scan_apply(unsigned *__restrict__ in, int M, const int *__restrict__ tile_sums,
             int *__restrict__ out, int zero_input)
{
    __shared__ unsigned sh[kScanThreads / 32];
    __shared__ unsigned sh_prefix;
    // prefix of all earlier tiles
    unsigned acc = 0;
    for (int t = threadIdx.x; t < (int)blockIdx.x; t += blockDim.x) acc += (unsigned)tile_sums[t];
    acc = warp_sum(acc);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned p = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) p += sh[w];
        sh_prefix = p;
    }
    __syncthreads();
    const unsigned prefix = sh_prefix;
    __syncthreads();

    const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    unsigned v[kScanItems];
    const bool full = base + kScanItems <= M;
    if (full) {
        const uint4 *p = reinterpret_cast<const uint4 *>(in + base);
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            const uint4 t = p[q];
            v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
        }
    } else {
#pragma unroll
        for (int e = 0; e < kScanItems; ++e) v[e] = base + e < M ? in[base + e] : 0u;
    }
    unsigned local = 0;
#pragma unroll
    for (int e = 0; e < kScanItems; ++e) local += v[e];
    unsigned total;
    unsigned run = prefix + block_exclusive_scan(local, sh, total);
    if (full) {
        int4 *o = reinterpret_cast<int4 *>(out + base);
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            int4 t;
            t.x = (int)run; run += v[4 * q];
            t.y = (int)run; run += v[4 * q + 1];
            t.z = (int)run; run += v[4 * q + 2];
            t.w = (int)run; run += v[4 * q + 3];
            o[q] = t;
        }
        if (zero_input) {
            uint4 *p = reinterpret_cast<uint4 *>(in + base);
#pragma unroll
            for (int q = 0; q < kScanItems / 4; ++q) p[q] = make_uint4(0, 0, 0, 0);
        }
    } else {
#pragma unroll
        for (int e = 0; e < kScanItems; ++e) {
            if (base + e < M) {
                out[base + e] = (int)run;
                run += v[e];
                if (zero_input) in[base + e] = 0u;
            }
        }
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[M] = (int)(prefix + total);
}

// Cell starts of a step's build in one pass over the counters: the key
// producers of a step (viscosity_predict, the relaxations) also count their
// particles per build tile (add_tile_count), so each CTA takes the prefix of
// the tiles before it from those counts, scans its own tile of counters
// into starts, zeroes the counters and gathers the occupancy statistics of
// k_scan_reduce -- with one barrier, so that a CTA's life is one round of
// loads and one of stores.  It checks its tile's total against the
// producers' count (DevState::tile_count_mismatch); the build's scatter
// zeroes the counts afterwards.
__global__ void __launch_bounds__(kBuildThreads, 1536 / kBuildThreads)
k_cell_starts(unsigned *__restrict__ in, int M, const unsigned *__restrict__ nocell,
              const unsigned *__restrict__ tile_cnt, int *__restrict__ out, DevState *st,
              unsigned *occ, int max_bucket, int max_neighbors)
{
    constexpr int ITEMS = kBuildItems, NW = ITEMS >= 32 ? ITEMS / 32 : 1;
    constexpr int WARPS = kBuildThreads / 32;
    static_assert(ITEMS % 4 == 0 && (ITEMS == 16 || ITEMS % 32 == 0), "items per thread");
    __shared__ unsigned sh_sum[WARPS], sh_pre[WARPS], sh_m[WARPS];
    __shared__ unsigned long long sh_e[WARPS], sh_o[WARPS];
    pdl_enter();
    const int tile = blockIdx.x;
    const int base = tile * kBuildTile + threadIdx.x * ITEMS;
    // prefix of all earlier tiles, from the producers' counts: the loads go
    // out together with the tile's own counters
    unsigned acc = 0;
    {
        constexpr int kBatch = 4;
        for (int t0 = 0; t0 < tile; t0 += kBatch * kBuildThreads) {
            unsigned x[kBatch];
#pragma unroll
            for (int j = 0; j < kBatch; ++j) {
                const int t = t0 + j * kBuildThreads + threadIdx.x;
                x[j] = t < tile ? __ldcg(tile_cnt + t) : 0u;
            }
#pragma unroll
            for (int j = 0; j < kBatch; ++j) acc += x[j];
        }
    }
    // a tile no producer counted a particle into holds only zero counters:
    // its counters are neither read nor zeroed again (most tiles of a
    // sparse scene); the others check their total against the count below
    const unsigned expect = __ldcg(tile_cnt + tile);
    unsigned v[ITEMS];
    const bool full = base + ITEMS <= M;
    if (expect == 0u) {
#pragma unroll
        for (int e = 0; e < ITEMS; ++e) v[e] = 0u;
    } else if (full) {
        const uint4 *p = reinterpret_cast<const uint4 *>(in + base);
#pragma unroll
        for (int q = 0; q < ITEMS / 4; ++q) {
            const uint4 t = p[q];
            v[4 * q] = t.x; v[4 * q + 1] = t.y; v[4 * q + 2] = t.z; v[4 * q + 3] = t.w;
        }
    } else {
#pragma unroll
        for (int e = 0; e < ITEMS; ++e) v[e] = base + e < M ? in[base + e] : 0u;
    }
    // the thread's counters in the no-cell bitmap
    unsigned bits[NW];
#pragma unroll
    for (int j = 0; j < NW; ++j)
        bits[j] = (nocell && base + 32 * j < M) ? __ldg(nocell + (base >> 5) + j) : 0u;
    if (ITEMS < 32) bits[0] >>= (base & 31);
    unsigned local = 0, mx = 0;
    unsigned long long excess = 0, outside = 0;
#pragma unroll
    for (int e = 0; e < ITEMS; ++e) {
        local += v[e];
        if ((bits[e >> 5] >> (e & 31)) & 1u) {
            outside += v[e];
        } else {
            mx = max(mx, v[e]);
            if (v[e] > (unsigned)max_bucket) excess += v[e] - max_bucket;
        }
    }
    // warp-level: inclusive scan of the thread sums, reductions of the rest
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned x = local;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const unsigned y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    acc = warp_sum(acc);
    mx = warp_max(mx);
    excess = warp_sum(excess);
    outside = warp_sum(outside);
    if (lane == 31) sh_sum[warp] = x;
    if (lane == 0) { sh_pre[warp] = acc; sh_m[warp] = mx; sh_e[warp] = excess; sh_o[warp] = outside; }
    __syncthreads();
    // every thread combines the per-warp words itself (no second barrier)
    unsigned before = 0, total = 0, prefix = 0;
#pragma unroll
    for (int w = 0; w < WARPS; ++w) {
        const unsigned sw = sh_sum[w];
        before += w < warp ? sw : 0u;
        total += sw;
        prefix += sh_pre[w];
    }
    unsigned run = prefix + before + x - local;
    if (full) {
        int4 *o = reinterpret_cast<int4 *>(out + base);
        uint4 *z = reinterpret_cast<uint4 *>(in + base);
#pragma unroll
        for (int q = 0; q < ITEMS / 4; ++q) {
            int4 t;
            t.x = (int)run; run += v[4 * q];
            t.y = (int)run; run += v[4 * q + 1];
            t.z = (int)run; run += v[4 * q + 2];
            t.w = (int)run; run += v[4 * q + 3];
            o[q] = t;
            if (expect != 0u) z[q] = make_uint4(0, 0, 0, 0);
        }
    } else {
#pragma unroll
        for (int e = 0; e < ITEMS; ++e) {
            if (base + e < M) {
                out[base + e] = (int)run;
                run += v[e];
                if (expect != 0u) in[base + e] = 0u;
            }
        }
    }
    if (tile == (int)gridDim.x - 1 && threadIdx.x == blockDim.x - 1) out[M] = (int)(prefix + total);
    if (threadIdx.x == 0) {
        if (total != expect) atomicOr(&st->tile_count_mismatch, 1u);
        if (occ) {
            unsigned tm = 0;
            unsigned long long te = 0, to = 0;
#pragma unroll
            for (int w = 0; w < WARPS; ++w) {
                tm = max(tm, sh_m[w]); te += sh_e[w]; to += sh_o[w];
            }
            atomicMax(occ, tm);
            atomicMax(&st->max_occ, tm);
            if (te) atomicAdd(&st->bucket_overflow, te);
            if (to) atomicAdd(&st->out_of_grid, to);
            const unsigned m = tm < (unsigned)max_bucket ? tm : (unsigned)max_bucket;
            if (m > 0 && 5u * m - 1u > (unsigned)max_neighbors) atomicOr(&st->list_cap_risk, 1u);
        }
    }
}

// Scratch slot per particle: cell start + arrival rank.
__global__ void __launch_bounds__(kBlock)
k_scatter_ids(int n, const uint2 *__restrict__ kr, const int *__restrict__ id_src,
              const int *__restrict__ start, int *__restrict__ tmp, unsigned *tile_cnt, int ntiles)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    // the build's tile counts have been read (k_cell_starts): zero them for
    // the next build
    for (int t = i; t < ntiles; t += gridDim.x * blockDim.x) tile_cnt[t] = 0u;
    if (i >= n) return;
    const uint2 k = kr[i];
    const int d = __ldg(start + k.x) + (int)k.y;
    if (in_bounds(d, n, kBadScatter)) tmp[d] = id_src ? id_src[i] : i;
}

// Final position = cell start + number of cell members with a smaller id, so
// that each cell holds its particles in id order -- the order hash.c:153-163
// inserts them into a bucket (pointer-array order).
__global__ void __launch_bounds__(kBlock)
k_permute(int n, const uint2 *__restrict__ kr, const int *__restrict__ start,
          const int *__restrict__ tmp, const int *__restrict__ id_src,
          const float2 *__restrict__ a_src, const float2 *__restrict__ b_src,
          int *__restrict__ id_dst, float2 *__restrict__ a_dst, float2 *__restrict__ b_dst,
          DevState *__restrict__ end_step)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (end_step && i == 0) {
        // last kernel of a step: the neighbour relation of the new positions
        // now exists (viscosity is on from the next step), one more step done
        end_step->lists_valid = 1u;
        end_step->steps += 1ull;
    }
    if (i >= n) return;
    const uint2 k = kr[i];
    const int s0 = __ldg(start + k.x), s1 = __ldg(start + k.x + 1);
    const int myid = id_src ? id_src[i] : i;
    int r;
    if (s1 - s0 <= kRankScanMax) {
        r = 0;
        for (int j = s0; j < s1; ++j)
            if (in_bounds(j, n, kBadScatter)) r += __ldg(tmp + j) < myid;
    } else {
        r = (int)k.y;  // pathological cell: arrival order
    }
    const int d = s0 + r;
    if (!in_bounds(d, n, kBadScatter)) return;
    id_dst[d] = myid;
    a_dst[d] = a_src[i];
    if (b_src) b_dst[d] = b_src[i];
}

// The step's forms of k_scatter_ids and k_permute: K particles per thread
// (strided by the block size, so the loads stay coalesced), their loads
// issued together, so that each thread has K dependent chains (key -> cell
// start -> slot) in flight instead of one.
template <int K>
__global__ void __launch_bounds__(kBlock)
k_scatter_ids_x(int n, const uint2 *__restrict__ kr, const int *__restrict__ id_src,
                const int *__restrict__ start, int *__restrict__ tmp, unsigned *tile_cnt,
                int ntiles)
{
    pdl_enter();
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    for (int t = g; t < ntiles; t += gridDim.x * blockDim.x) tile_cnt[t] = 0u;
    const int i0 = blockIdx.x * blockDim.x * K + threadIdx.x;
    uint2 k[K];
    int id[K], st[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        const int i = i0 + j * blockDim.x;
        if (i < n) {
            k[j] = kr[i];
            id[j] = id_src ? id_src[i] : i;
        }
    }
#pragma unroll
    for (int j = 0; j < K; ++j)
        if (i0 + j * (int)blockDim.x < n) st[j] = __ldg(start + k[j].x);
#pragma unroll
    for (int j = 0; j < K; ++j) {
        if (i0 + j * (int)blockDim.x >= n) continue;
        const int d = st[j] + (int)k[j].y;
        if (in_bounds(d, n, kBadScatter)) tmp[d] = id[j];
    }
}

template <int K>
__global__ void __launch_bounds__(kBlock)
k_permute_x(int n, const uint2 *__restrict__ kr, const int *__restrict__ start,
            const int *__restrict__ tmp, const int *__restrict__ id_src,
            const float2 *__restrict__ a_src, const float2 *__restrict__ b_src,
            int *__restrict__ id_dst, float2 *__restrict__ a_dst, float2 *__restrict__ b_dst,
            DevState *__restrict__ end_step)
{
    pdl_enter();
    if (end_step && blockIdx.x == 0 && threadIdx.x == 0) {
        end_step->lists_valid = 1u;
        end_step->steps += 1ull;
    }
    const int i0 = blockIdx.x * blockDim.x * K + threadIdx.x;
    uint2 k[K];
    int id[K], s0[K], s1[K];
    float2 a[K], b[K];
#pragma unroll
    for (int j = 0; j < K; ++j) {
        const int i = i0 + j * blockDim.x;
        if (i < n) {
            k[j] = kr[i];
            id[j] = id_src ? id_src[i] : i;
            a[j] = a_src[i];
            if (b_src) b[j] = b_src[i];
        }
    }
#pragma unroll
    for (int j = 0; j < K; ++j)
        if (i0 + j * (int)blockDim.x < n) {
            s0[j] = __ldg(start + k[j].x);
            s1[j] = __ldg(start + k[j].x + 1);
        }
#pragma unroll
    for (int j = 0; j < K; ++j) {
        if (i0 + j * (int)blockDim.x >= n) continue;
        int r;
        if (s1[j] - s0[j] <= kRankScanMax) {
            r = 0;
            for (int q = s0[j]; q < s1[j]; ++q)
                if (in_bounds(q, n, kBadScatter)) r += __ldg(tmp + q) < id[j];
        } else {
            r = (int)k[j].y;  // pathological cell: arrival order
        }
        const int d = s0[j] + r;
        if (!in_bounds(d, n, kBadScatter)) continue;
        id_dst[d] = id[j];
        a_dst[d] = a[j];
        if (b_src) b_dst[d] = b[j];
    }
}

// Cell keys of uploaded positions (id order, no step before them).
__global__ void __launch_bounds__(kBlock)
k_keys(Ctx c, const float2 *__restrict__ pos, uint2 *__restrict__ kr, unsigned *__restrict__ cnt,
       unsigned *occ_reset)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && occ_reset) *occ_reset = 0u;
    if (i >= c.n) return;
    const SG g = load_grid(c.scenes + scene_of(c, i));
    const float2 p = pos[i];
    const unsigned key = cell_key(p.x, p.y, g);
    kr[i] = make_uint2(key, in_bounds(key, c.M, kBadKey) ? atomicAdd(cnt + key, 1u) : 0u);
}

// ---------------------------------------------------------------------------
// pass 1: gravity + viscosity (gather) + predict + boundary + cell key
// ---------------------------------------------------------------------------

// apply_gravity (fluid.c:398-413), viscosity_impluses (fluid.c:416-478) in
// gather form, predict_positions (fluid.c:507-523) with boundaryConditions.
// Gather form of the viscosity: dv_i = -1/2 sum_j clamp5(I_ij),
// I_ij = dt (1 - r/h)(sigma u + beta u^2) (x_j - x_i)/r for u > 0,
// u = ((v_i - v_j).(x_j - x_i))/r, all from the velocities after gravity.
// PROBE writes dv instead of advancing.
// STAGED: every thread of the CTA calls this (valid = false for a thread
// without a particle), and the CTA first copies the union of its stencil
// rows' positions and velocities to shared memory (sm_p, sm_v; cap
// elements each; stage_rows).
template <bool PROBE, bool STAGED = false>
__device__ __forceinline__ void viscosity_predict_one(
    int i, const Ctx &c, const DevState *__restrict__ st, const float2 *__restrict__ pos,
    const float2 *__restrict__ vel, const int *__restrict__ start, bool capped,
    float2 *__restrict__ pos_out, float2 *__restrict__ prev_out, uint2 *__restrict__ kr_out,
    unsigned *__restrict__ cnt, float2 *__restrict__ probe_out, int *tile_made = nullptr,
    bool valid = true, float2 *sm_p = nullptr, float2 *sm_v = nullptr, int cap = 0)
{
    const Scene *S = c.scenes + (valid ? scene_of(c, i) : 0);
    const SG g = load_grid(S);
    const float dt = __ldg(&S->P.time_step);
    const float gdt = __fmul_rn(-__ldg(&S->P.g), dt);
    const float hh = __ldg(&S->P.smoothing_radius);
    const float h2 = __fmul_rn(hh, hh);
    const float h_recip = __fdiv_rn(1.0f, hh);
    const float sigma = __ldg(&S->P.sigma), beta = __ldg(&S->P.beta);
    const float dt_h = dt * h_recip;

    const float2 p = valid ? pos[i] : make_float2(-1.0f, -1.0f);
    const float2 v0 = valid ? vel[i] : make_float2(0.0f, 0.0f);  // before gravity: velocity differences need none
    float2 v = make_float2(v0.x, __fadd_rn(v0.y, gdt));
    float2 dv = make_float2(0.0f, 0.0f);
    const unsigned key = cell_key(p.x, p.y, g);
    // One pair's impulse on this particle; self (and any coincident
    // particle) has r2 == 0 and gives none, as u is NaN in the reference for
    // r == 0 (fluid.c:446-451).  IN_RANGE: the caller has established
    // r2 <= h2 (a hit-mask walk recomputes the same r2).
    const float2 mp = make_float2(-p.x, -p.y);
    auto impulse_core = [&](const float4 &d, bool in_range) {
        float2 e;
        const float r2 = dist2_packed(mp, make_float2(d.x, d.y), e);
        const float qx = e.x, qy = e.y;
        if ((!in_range && r2 > h2) || r2 == 0.0f) return;
        const float r_recip = rsqrtf(r2);
        const float r = r2 * r_recip;
        // gravity adds the same amount to both velocities: the difference
        // is taken before it (one packed subtraction)
        const float2 w = __fadd2_rn(v0, make_float2(-d.z, -d.w));
        const float u0 = (w.x * qx + w.y * qy) * r_recip;
        // only approaching pairs (u > 0) push; the others run the same
        // instructions with u = 0, whose impulse is +-0 and leaves dv's bits
        // as they are (no divergent branch: about half the pairs of every
        // warp approach)
        const float u = u0 > 0.0f ? u0 : 0.0f;
        // dt (1 - r/h) (sigma u + beta u^2) = (dt - (dt/h) r) u (sigma + beta u)
        const float imp = fmaf(-dt_h, r, dt) * u * fmaf(beta, u, sigma);
        // per component imp * q * r_recip, clamped, halved and subtracted
        // (packed FP32x2, each operation rounded as the scalar form)
        const float2 t = __fmul2_rn(__fmul2_rn(make_float2(imp, imp), e),
                                    make_float2(r_recip, r_recip));
        dv = __ffma2_rn(make_float2(-0.5f, -0.5f), make_float2(clamp5(t.x), clamp5(t.y)), dv);
    };
    auto impulse_with = [&](const float4 &d) { impulse_core(d, false); };
    auto load_pv = [&](int j) {
        const float2 q = __ldg(pos + j), w = __ldg(vel + j);
        return make_float4(q.x, q.y, w.x, w.y);
    };
    auto impulse = [&](int j) { impulse_with(load_pv(j)); };
    const bool search = valid && (PROBE || st->lists_valid) &&
                        searchable(key, i, start, g, capped, c.max_bucket);
    int ra[3] = {0, 0, 0}, rl[3] = {0, 0, 0};
    if (search && !capped) stencil_rows(key, start, g, ra, rl, c.n);
    const bool masked = search && !capped && rl[0] <= kMaskRow && rl[1] <= kMaskRow &&
                        rl[2] <= kMaskRow;
    int d[3] = {0, 0, 0};
    bool staged = false;
    if (STAGED) {
        int lo[3], hi[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const bool use = masked && rl[r] > 0;
            lo[r] = use ? ra[r] : INT_MAX;
            hi[r] = use ? ra[r] + rl[r] : INT_MIN;
        }
        staged = stage_rows(lo, hi, pos, sm_p, cap, d, vel, sm_v);
    }
    if (!valid) return;
    if (masked) {
        // two phases: a cheap scan marks the neighbours of each stencil
        // row, then only they pay for the impulse (less SIMT waste)
        auto two_phase = [&](auto SMc, const float2 *bp, const float2 *bv) {
            constexpr bool SM = decltype(SMc)::value;
            unsigned long long m[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const float2 *row = bp + ra[r] + (SM ? d[r] : 0);
                auto at = [&](int t) { return SM ? row[t] : __ldg(row + t); };
                const int len = rl[r];
                // 32-bit halves: cheaper bit operations than one 64-bit mask
                unsigned lo = 0u, hi = 0u;
                const int n0 = min(len, 32);
#pragma unroll kViscUnroll
                for (int t = 0; t < n0; ++t) {
                    float2 e;
                    const float r2 = dist2_packed(mp, at(t), e);
                    // self and coincident particles are marked too; the
                    // impulse skips them (r2 == 0)
                    lo |= (unsigned)(r2 <= h2) << t;
                }
#pragma unroll kViscUnroll
                for (int t = 32; t < len; ++t) {
                    float2 e;
                    const float r2 = dist2_packed(mp, at(t), e);
                    hi |= (unsigned)(r2 <= h2) << (t - 32);
                }
                m[r] = ((unsigned long long)hi << 32) | lo;
            }
            m[1] &= ~(1ull << (i - ra[1]));  // self
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const int dd = SM ? d[r] : 0;
                walk_mask<float4>(
                    m[r], ra[r], c.n,
                    [&](int j) {
                        if (SM) {
                            const float2 q = bp[j + dd], w = bv[j + dd];
                            return make_float4(q.x, q.y, w.x, w.y);
                        }
                        return load_pv(j);
                    },
                    [&](int, const float4 &dq) { impulse_core(dq, true); });
            }
        };
        if (STAGED && staged)
            two_phase(std::integral_constant<bool, true>(), sm_p, sm_v);
        else
            two_phase(std::integral_constant<bool, false>(), pos, vel);
    } else if (search) {
        for_each_candidate(key, start, g, capped, c.max_bucket, c.n, impulse);
    }
    if (PROBE) {
        probe_out[i] = dv;
        return;
    }
    v.x = __fadd_rn(v.x, dv.x);
    v.y = __fadd_rn(v.y, dv.y);
    float nx = __fadd_rn(p.x, __fmul_rn(v.x, dt));
    float ny = __fadd_rn(p.y, __fmul_rn(v.y, dt));
    boundary_of(nx, ny, S);
    const unsigned k2 = cell_key(nx, ny, g);
    unsigned rank = 0u;
    if (in_bounds(k2, c.M, kBadKey)) {
        rank = atomicAdd(cnt + k2, 1u);
        if (tile_made)
            *tile_made = (int)(k2 / (unsigned)kBuildTile);
        else
            add_tile_count(c.tile_cnt, k2);
    }
    pos_out[i] = make_float2(nx, ny);
    prev_out[i] = p;
    kr_out[i] = make_uint2(k2, rank);
}

// The viscosity pass with the CTA's stencil rows (positions and velocities)
// staged in shared memory.
template <bool PERSIST>
__global__ void __maxnreg__(48)
k_viscosity_predict_sm(Ctx c, const DevState *__restrict__ st, const float2 *__restrict__ pos,
                       const float2 *__restrict__ vel, const int *__restrict__ start,
                       const unsigned *__restrict__ occ_in, unsigned *occ_reset,
                       float2 *__restrict__ pos_out, float2 *__restrict__ prev_out,
                       uint2 *__restrict__ kr_out, unsigned *__restrict__ cnt)
{
    extern __shared__ float2 sm_pv[];
    pdl_enter();
    if (blockIdx.x == 0 && threadIdx.x == 0) *occ_reset = 0u;
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    const int cap = kStagePerThread * (int)blockDim.x;
    const int ntiles = (c.n + blockDim.x - 1) / blockDim.x;
    for (int tile = blockIdx.x; tile < ntiles; tile += PERSIST ? gridDim.x : ntiles) {
        const int i = tile * blockDim.x + threadIdx.x;
        viscosity_predict_one<false, true>(i, c, st, pos, vel, start, capped, pos_out, prev_out,
                                           kr_out, cnt, nullptr, nullptr, i < c.n, sm_pv,
                                           sm_pv + cap, cap);
    }
}

// 48 registers: more resident warps than the compiler's free choice (55),
// without spills.
template <bool PROBE, bool PERSIST = false>
__global__ void __maxnreg__(48)
k_viscosity_predict(Ctx c, const DevState *__restrict__ st, const float2 *__restrict__ pos,
                    const float2 *__restrict__ vel, const int *__restrict__ start,
                    const unsigned *__restrict__ occ_in, unsigned *occ_reset,
                    float2 *__restrict__ pos_out, float2 *__restrict__ prev_out,
                    uint2 *__restrict__ kr_out, unsigned *__restrict__ cnt,
                    float2 *__restrict__ probe_out)
{
    pdl_enter();
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (!PROBE && i0 == 0) *occ_reset = 0u;
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    if (!PERSIST) {
        if (i0 < c.n)
            viscosity_predict_one<PROBE>(i0, c, st, pos, vel, start, capped, pos_out, prev_out,
                                         kr_out, cnt, probe_out);
        return;
    }
    for (int i = i0; i < c.n; i += gridDim.x * blockDim.x)
        viscosity_predict_one<PROBE>(i, c, st, pos, vel, start, capped, pos_out, prev_out, kr_out,
                                     cnt, probe_out);
}

// ---------------------------------------------------------------------------
// pass 2: density and near density (gather)
// ---------------------------------------------------------------------------

// rho_i = sum_j (1 - r/h)^2, rho_near_i = sum_j (1 - r/h)^3 over neighbours
// j != i with r/h < 1 (calculate_density, fluid.c:527-539; the pairs of
// hash_fluid, hash.c:185/221: r2 <= h2 inclusive).
// Writes xr = (x, y, rho, rho_near) and, per stencil row, the bit mask of the
// candidates that are neighbours (r2 <= h2, self excluded), which the
// relaxation pass of the same positions walks instead of the whole stencil.
// The candidate filter of one particle over its three stencil rows (slots
// [ra[r], ra[r] + rl[r])), reading the rows from global memory or, SM, from
// the CTA's shared-memory copy (slot j of row r at base[j + d[r]]).
// mx (long-row masks): where the hit bits of candidates kMaskRow..
// 2 kMaskRow - 1 of each row go (3 words; null: nowhere).
template <bool SM>
__device__ __forceinline__ void density_filter(int i, float2 mp, float h2, float h_recip,
                                               const int (&ra)[3], const int (&rl)[3],
                                               const float2 *base, const int (&d)[3],
                                               float2 &ab, unsigned long long (&m)[3],
                                               unsigned long long *mx = nullptr)
{
    // the particle's own slot in its row (row 1): never a neighbour of
    // itself (hash.c pairs distinct particles only)
    const int self = i - ra[1];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const float2 *row = base + ra[r] + (SM ? d[r] : 0);
        auto at = [&](int t) { return SM ? row[t] : __ldg(row + t); };
        const int len = rl[r];
        unsigned mh[2] = {0u, 0u};  // 32-bit halves of the row's hit mask
#pragma unroll
        for (int hh = 0; hh < 2; ++hh) {
            const int t1 = hh == 0 ? min(len, 32) : min(len, kMaskRow);
#pragma unroll kDensUnroll
            for (int t = 32 * hh; t < t1; ++t) {
                float2 e;
                const float r2 = dist2_packed(mp, at(t), e);
                if (r2 <= h2 && (r != 1 || t != self)) {
                    mh[hh] |= 1u << (t & 31);
                    add_density(ab, r2, h_recip);
                }
            }
        }
        // rows longer than the mask: with long-row masks the next kMaskRow
        // candidates' bits go to mx; the rest have no mask bits (the
        // relaxation then walks the whole stencil)
        int t2 = kMaskRow;
        if (mx != nullptr && len > kMaskRow) {
            unsigned long long hx = 0ull;
            t2 = min(len, 2 * kMaskRow);
            for (int t = kMaskRow; t < t2; ++t) {
                float2 e;
                const float r2 = dist2_packed(mp, at(t), e);
                if (r2 <= h2 && (r != 1 || t != self)) {
                    hx |= 1ull << (t - kMaskRow);
                    add_density(ab, r2, h_recip);
                }
            }
            mx[r] = hx;
        }
        for (int t = t2; t < len; ++t) {
            float2 e;
            const float r2 = dist2_packed(mp, at(t), e);
            if (r2 <= h2 && (r != 1 || t != self)) add_density(ab, r2, h_recip);
        }
        m[r] = ((unsigned long long)mh[1] << 32) | mh[0];
    }
}

// STAGED: every thread of the CTA calls this (also those with no particle,
// valid = false), and the CTA first copies the union of its stencil rows to
// shared memory `sm` (cap elements; stage_rows).
// LM: long-row masks (rows of up to 2 kMaskRow candidates recorded as
// kRowsMasked2, their second masks in c.maskx).
template <bool STAGED = false, bool LM = false>
__device__ __forceinline__ void density_one(int i, const Ctx &c, const float2 *__restrict__ pos,
                                            const int *__restrict__ start, bool capped,
                                            float4 *__restrict__ xr_out,
                                            ulonglong2 *__restrict__ mask01,
                                            unsigned long long *__restrict__ mask2,
                                            int4 *__restrict__ rows_out, bool valid = true,
                                            float2 *sm = nullptr, int cap = 0)
{
    const Scene *S = c.scenes + (valid ? scene_of(c, i) : 0);
    const SG g = load_grid(S);
    const float hh = __ldg(&S->P.smoothing_radius);
    const float h2 = __fmul_rn(hh, hh);
    const float h_recip = __fdiv_rn(1.0f, hh);
    const float2 p = valid ? pos[i] : make_float2(-1.0f, -1.0f);
    const float2 mp = make_float2(-p.x, -p.y);
    const unsigned key = cell_key(p.x, p.y, g);
    float2 ab = make_float2(0.0f, 0.0f);  // (rho, rho_near)
    unsigned long long m[3] = {0ull, 0ull, 0ull};
    int4 rec = make_int4(0, 0, 0, kRowsNone);
    const bool search = valid && searchable(key, i, start, g, capped, c.max_bucket);
    int ra[3] = {0, 0, 0}, rl[3] = {0, 0, 0};
    if (search && !capped) stencil_rows(key, start, g, ra, rl, c.n);
    int d[3] = {0, 0, 0};
    bool staged = false;
    if (STAGED) {
        int lo[3], hi[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            const bool use = search && !capped && rl[r] > 0;
            lo[r] = use ? ra[r] : INT_MAX;
            hi[r] = use ? ra[r] + rl[r] : INT_MIN;
        }
        staged = stage_rows(lo, hi, pos, sm, cap, d);
    }
    if (!valid) return;
    if (search) {
        rec.w = kRowsFull;
        if (!capped) {
            unsigned long long *mx = nullptr;
            if (rl[0] <= kMaskRow && rl[1] <= kMaskRow && rl[2] <= kMaskRow) {
                rec = make_int4(ra[0], ra[1], ra[2], kRowsMasked);
            } else if (LM && !STAGED && c.maskx && rl[0] <= 2 * kMaskRow &&
                       rl[1] <= 2 * kMaskRow && rl[2] <= 2 * kMaskRow) {
                rec = make_int4(ra[0], ra[1], ra[2], kRowsMasked2);
                mx = c.maskx + 3 * (size_t)i;
                mx[0] = mx[1] = mx[2] = 0ull;  // rows of kMaskRow or fewer leave theirs
            }
            if (STAGED && staged)
                density_filter<true>(i, mp, h2, h_recip, ra, rl, sm, d, ab, m);
            else
                density_filter<false>(i, mp, h2, h_recip, ra, rl, pos, d, ab, m, LM ? mx : nullptr);
        } else {
            for_each_candidate(key, start, g, true, c.max_bucket, c.n, [&](int j) {
                if (j == i) return;
                const float2 q = __ldg(pos + j);
                const float r2 = dist2(p.x - q.x, p.y - q.y);
                if (r2 > h2) return;
                add_density(ab, r2, h_recip);
            });
        }
    }
    xr_out[i] = make_float4(p.x, p.y, ab.x, ab.y);
    mask01[i] = make_ulonglong2(m[0], m[1]);
    mask2[i] = m[2];
    if (rows_out) rows_out[i] = rec;
}

// The density pass with the CTA's stencil rows staged in shared memory
// (one tile of blockDim.x particles per CTA, or grid-stride over tiles).
template <bool PERSIST>
__global__ void __launch_bounds__(kMaxBlock, 4)
k_density_sm(Ctx c, const float2 *__restrict__ pos, const int *__restrict__ start,
             const unsigned *__restrict__ occ_in, float4 *__restrict__ xr_out,
             ulonglong2 *__restrict__ mask01, unsigned long long *__restrict__ mask2,
             int4 *__restrict__ rows_out)
{
    extern __shared__ float2 sm_pos[];
    pdl_enter();
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    const int ntiles = (c.n + blockDim.x - 1) / blockDim.x;
    for (int tile = blockIdx.x; tile < ntiles; tile += PERSIST ? gridDim.x : ntiles) {
        const int i = tile * blockDim.x + threadIdx.x;
        density_one<true>(i, c, pos, start, capped, xr_out, mask01, mask2, rows_out, i < c.n,
                          sm_pos, kStagePerThread * (int)blockDim.x);
    }
}

// 32 registers (four 512-thread CTAs' worth per SM): full occupancy for this
// issue-bound pass outweighs the few spilled values of its rare paths.
#ifndef SPH_DENS_MIN_BLOCKS
#define SPH_DENS_MIN_BLOCKS 4  // resident 512-thread CTAs per SM the density pass is built for
#endif
template <bool PERSIST, bool LM = false>
__global__ void __launch_bounds__(kMaxBlock, SPH_DENS_MIN_BLOCKS)
k_density_t(Ctx c, const float2 *__restrict__ pos, const int *__restrict__ start,
            const unsigned *__restrict__ occ_in, float4 *__restrict__ xr_out,
            ulonglong2 *__restrict__ mask01, unsigned long long *__restrict__ mask2,
            int4 *__restrict__ rows_out)
{
    pdl_enter();
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (!PERSIST) {
        if (i0 < c.n)
            density_one<false, LM>(i0, c, pos, start, capped, xr_out, mask01, mask2, rows_out);
        return;
    }
    for (int i = i0; i < c.n; i += gridDim.x * blockDim.x)
        density_one<false, LM>(i, c, pos, start, capped, xr_out, mask01, mask2, rows_out);
}

// One density launch per block (the form other translation units call).
__global__ void __launch_bounds__(kMaxBlock)
k_density(Ctx c, const float2 *__restrict__ pos, const int *__restrict__ start,
          const unsigned *__restrict__ occ_in, float4 *__restrict__ xr_out,
          ulonglong2 *__restrict__ mask01, unsigned long long *__restrict__ mask2,
          int4 *__restrict__ rows_out)
{
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (i0 < c.n) density_one(i0, c, pos, start, capped, xr_out, mask01, mask2, rows_out);
}

// ---------------------------------------------------------------------------
// pass 3: relaxation (gather) + boundary + velocity update + cell key
// ---------------------------------------------------------------------------

// Whether particle (slot i, id_i, cell ki) holds the pair with (slot j) in
// its own half list in the reference: same cell and smaller id
// (hash.c:178-199), or j's cell is one of i's forward cells
// (0,+1), (+1,-1), (+1,0), (+1,+1) (hash.c:203-234).
__device__ __noinline__ bool owns_pair(unsigned ki, int id_i, float2 qj, int id_j, const SG &g)
{
    const unsigned kj = cell_key(qj.x, qj.y, g);
    if (kj == ki) return id_i < id_j;
    const int li = (int)ki - g.c_off, lj = (int)kj - g.c_off;
    const int yi = li / g.size_x, xi = li - yi * g.size_x;
    const int yj = lj / g.size_x, xj = lj - yj * g.size_x;
    const int dx = xj - xi, dy = yj - yi;
    return (dx == 0 && dy == 1) || (dx == 1 && dy >= -1 && dy <= 1);
}

struct RelaxConsts {
    float h2, hh, h_recip, dt2, k, k_near, rest, half_spring;
};

// One neighbour's contribution to the displacement (r2 <= h2 known), with
// the constants pre-multiplied by dt^2; the rare r <= 1e-6 path computes
// the grid and cell key it needs itself, so that they are not live across
// the neighbour walk.
struct WalkConsts {
    float h_recip, kd, knd, hsd, hshd, Pd, Pnd;
};

// The scene's relaxation constants, and the walk's for particle record me =
// (x, y, rho, rho_near): P = k (rho - rest), Pn = k_near rho_near
// (fluid.c:563-564), pre-multiplied by dt^2.  One definition for every
// relaxation path, so that their pair terms round identically.
__device__ __forceinline__ RelaxConsts relax_consts(const Scene *__restrict__ S)
{
    RelaxConsts c;
    c.hh = __ldg(&S->P.smoothing_radius);
    c.h2 = __fmul_rn(c.hh, c.hh);
    c.h_recip = __fdiv_rn(1.0f, c.hh);
    const float dt = __ldg(&S->P.time_step);
    c.dt2 = __fmul_rn(dt, dt);
    c.k = __ldg(&S->P.k);
    c.k_near = __ldg(&S->P.k_near);
    c.rest = __ldg(&S->P.rest_density);
    c.half_spring = __fmul_rn(0.5f, __ldg(&S->P.k_spring));
    return c;
}

__device__ __forceinline__ WalkConsts walk_consts(const RelaxConsts &c, float4 me)
{
    const float Pi = __fmul_rn(c.k, __fsub_rn(me.z, c.rest));
    const float Pni = __fmul_rn(c.k_near, me.w);
    WalkConsts wc;
    wc.h_recip = c.h_recip;
    wc.kd = __fmul_rn(c.dt2, c.k);
    wc.knd = __fmul_rn(c.dt2, c.k_near);
    wc.hsd = __fmul_rn(c.dt2, c.half_spring);
    wc.hshd = __fmul_rn(wc.hsd, c.hh);
    wc.Pd = __fmul_rn(c.dt2, __fsub_rn(Pi, __fmul_rn(c.k, c.rest)));
    wc.Pnd = __fmul_rn(c.dt2, Pni);
    return wc;
}

__device__ __noinline__ bool owns_pair_of(const Scene *S, float2 p, const int *__restrict__ ids,
                                          int i, float2 q, int j)
{
    const SG g = load_grid(S);
    return owns_pair(cell_key(p.x, p.y, g), ids[i], q, ids[j], g);
}

// The pair term of one neighbour (r2 <= h2 known): returns whether it
// displaces the particle, by s (p - q) with d = q - p (the caller adds
// -s d with one packed FMA), and counts a nudge of the pair's owner.
__device__ __forceinline__ bool relax_pair_term(const WalkConsts &c, float2 p, float4 q, int i,
                                                int j, const Scene *S,
                                                const int *__restrict__ ids, float &s, float2 &d,
                                                int &nudges)
{
    // d = q - p: the negated pair offset, rounded as p - q is
    const float r2 = dist2_packed(make_float2(-p.x, -p.y), make_float2(q.x, q.y), d);
    if (r2 <= 2e-12f) {
        // r <= 1e-6 (rare): the owner of the pair is nudged (fluid.c:583-586)
        const float r = r2 > 0.0f ? __fsqrt_rn(r2) : 0.0f;
        if (j != i && r <= 0.000001f && owns_pair_of(S, p, ids, i, make_float2(q.x, q.y), j))
            ++nudges;
        if (!(r > 0.0f)) return false;
    }
    const float r_recip = rsqrtf(r2);
    const float r = r2 * r_recip;
    const float ratio = r * c.h_recip;
    if (!(ratio < 1.0f)) return false;
    const float omr = 1.0f - ratio;
    const float D = (c.Pd + c.kd * q.z) * omr + (c.Pnd + c.knd * q.w) * omr * omr +
                    (c.hshd - c.hsd * r);
    s = D * r_recip;
    return true;
}

__device__ __forceinline__ void relax_pair_walk(const WalkConsts &c, float2 p, float4 q, int i,
                                                int j, const Scene *S,
                                                const int *__restrict__ ids, float2 &a,
                                                int &nudges)
{
    float s;
    float2 d;
    if (relax_pair_term(c, p, q, i, j, S, ids, s, d, nudges))
        a = __ffma2_rn(make_float2(-s, -s), d, a);  // += s (p - q), per component
}

// double_density_relaxation (fluid.c:541-611) in gather form:
//   dx_i = sum_{j: 0 < r < h} D_ij (x_i - x_j)/r,
//   D_ij = dt^2 [(P_i + P_j)(1 - r/h) + (Pn_i + Pn_j)(1 - r/h)^2 + k_spring (h - r)/2],
//   P = k (rho - rest_density), Pn = k_near rho_near (fluid.c:560-565),
// plus the reference's (1e-6, 1e-6) nudge for each pair with r <= 1e-6 that
// the particle owns (fluid.c:583-586).  Then updateVelocities
// (fluid.c:642-653): boundaryConditions, v = (x - x_prev)/dt clamped to +-5.
// Walks the density pass's hit masks; rows longer than kMaskRow (or
// overflowing buckets) fall back to the whole stencil.
// PROBE writes the displacement instead of advancing.
// The network's output for a learned step: particle i takes the displacement
// (net.x, net.y) * s, s = h dt^2 (k + k_near + k_spring), when it has at most
// max_nb neighbours (counts of 65535 mark particles the network must not
// take) and the predicted density error net.z (percent of rest density) is
// at most thr_pct; every other particle runs the plain relaxation.
struct LearnedIn {
    const float4 *net = nullptr;
    const unsigned short *nbc = nullptr;
    float thr_pct = 0.0f;
    int max_nb = 0;
    bool defer = false;  // leave the fallback particles to a second pass
};

// Where a masked walk reads its neighbours' (x, y, rho, rho_near) records:
// global memory, or the CTA's shared-memory copy of its stencil rows
// (stage_rows: slot j of row r at sm[j + d[r]]).
struct RowsIn {
    const float4 *sm = nullptr;
    int d[3] = {0, 0, 0};
};

// The end of a particle's relaxation: x += the displacement and the owner's
// nudges, boundaryConditions, then updateVelocity (fluid.c:627-653):
// v = (x - x_prev)/dt clamped to +-5, and the new position's cell key
// counted into the build of the relaxed positions.
__device__ __forceinline__ void relax_finish(int i, const Ctx &cx, const Scene *S, float2 p,
                                             float2 acc, int nudges,
                                             const float2 *__restrict__ prev,
                                             float2 *__restrict__ pos_out,
                                             float2 *__restrict__ vel_out,
                                             uint2 *__restrict__ kr_out,
                                             unsigned *__restrict__ cnt, int *tile_made)
{
    const float nd = (float)nudges * 0.000001f;
    float nx = __fadd_rn(__fadd_rn(p.x, acc.x), nd);
    float ny = __fadd_rn(__fadd_rn(p.y, acc.y), nd);
    boundary_of(nx, ny, S);
    const float2 pv = prev[i];
    const float dt_end = __ldg(&S->P.time_step);
    const float vx = clamp5(__fdiv_rn(__fsub_rn(nx, pv.x), dt_end));
    const float vy = clamp5(__fdiv_rn(__fsub_rn(ny, pv.y), dt_end));
    const unsigned k2 = cell_key(nx, ny, load_grid(S));
    unsigned rank = 0u;
    if (in_bounds(k2, cx.M, kBadKey)) {
        rank = atomicAdd(cnt + k2, 1u);
        if (tile_made)
            *tile_made = (int)(k2 / (unsigned)kBuildTile);
        else
            add_tile_count(cx.tile_cnt, k2);
    }
    pos_out[i] = make_float2(nx, ny);
    vel_out[i] = make_float2(vx, vy);
    kr_out[i] = make_uint2(k2, rank);
}

template <bool PROBE, bool LEARNED = false, bool LONG_ROWS = false, bool LM = false>
__device__ __forceinline__ void relax_update_one(
    int i, const Ctx &cx, const float4 *__restrict__ xr, const ulonglong2 *__restrict__ mask01,
    const unsigned long long *__restrict__ mask2, const int4 *__restrict__ rows,
    const float2 *__restrict__ prev, const int *__restrict__ ids, const int *__restrict__ start,
    bool capped, float2 *__restrict__ pos_out, float2 *__restrict__ vel_out,
    uint2 *__restrict__ kr_out, unsigned *__restrict__ cnt, float2 *__restrict__ probe_out,
    const LearnedIn &L = LearnedIn(), bool *used_net = nullptr, int *tile_made = nullptr,
    const RowsIn &R = RowsIn())
{
    const Scene *S = cx.scenes + scene_of(cx, i);
    const SG g = load_grid(S);
    const RelaxConsts c = relax_consts(S);

    const float4 me = xr[i];
    // the plain pass requests the hit masks with the record and prefetches
    // the previous position, so that their DRAM latencies overlap instead of
    // following one another (the record decides whether the masks are used;
    // relax_finish reads the previous position): 7% off this latency-bound
    // pass
    constexpr bool kHoist = !LEARNED;
    ulonglong2 m01h = make_ulonglong2(0ull, 0ull);
    unsigned long long m2h = 0ull;
    if (kHoist && rows) {
        m01h = __ldg(mask01 + i);
        m2h = __ldg(mask2 + i);
        asm volatile("prefetch.global.L1 [%0];" ::"l"(prev + i));
    }
    const float2 p = make_float2(me.x, me.y);
    const WalkConsts wc = walk_consts(c, me);
    float2 acc = make_float2(0.0f, 0.0f);  // the displacement
    int nudges = 0;
    bool net = false;
    if (LEARNED) {
        // the network's output requested with the count (not after it), and
        // the previous position prefetched for relax_finish: one DRAM latency
        // for a network particle instead of three in a row
        const float4 y = __ldg(L.net + i);
        asm volatile("prefetch.global.L1 [%0];" ::"l"(prev + i));
        if ((int)__ldg(L.nbc + i) <= L.max_nb && y.z <= L.thr_pct) {
            const float s = c.hh * c.dt2 * (c.k + c.k_near + 2.0f * c.half_spring);
            acc = make_float2(y.x * s, y.y * s);
            net = true;
        }
    }
    if (LEARNED && used_net) *used_net = net;
    if (LEARNED && !net && L.defer) return;
    // the density pass's row record: the stencil rows' first slots, so the
    // walk needs neither the cell key nor the cell starts (without one, the
    // rows are found here)
    int mode = net ? kRowsNone : kRowsFull;
    int ra[3] = {0, 0, 0};
    if (!net && rows) {
        const int4 rw = __ldg(rows + i);
        mode = rw.w;
        ra[0] = rw.x; ra[1] = rw.y; ra[2] = rw.z;
    }
    unsigned key = 0u;
    if (mode == kRowsFull) {
        key = cell_key(p.x, p.y, g);
        if (!searchable(key, i, start, g, capped, cx.max_bucket)) {
            mode = kRowsNone;
        } else if (!capped) {
            int rl[3];
            stencil_rows(key, start, g, ra, rl, cx.n);
            if (rl[0] <= kMaskRow && rl[1] <= kMaskRow && rl[2] <= kMaskRow) {
                mode = kRowsMasked;
            } else if (LONG_ROWS) {
                // a row longer than one mask (dense cells): filter and walk
                // 64 candidates at a time, in slot order -- for the fallback
                // pass, whose particles are the dense ones (in the full pass
                // the extra code costs the common path more than it saves)
                const float2 mp = make_float2(-p.x, -p.y);
                auto xr_pos = [&](int j) {
                    const float4 q = __ldg(xr + j);
                    return make_float2(q.x, q.y);
                };
                for (int r = 0; r < 3; ++r)
                    walk_row_hits<float4>(
                        ra[r], rl[r], r == 1 ? i : -1, cx.n, mp, c.h2, xr_pos,
                        [&](int j) { return __ldg(xr + j); },
                        [&](int j, const float4 &q) {
                            relax_pair_walk(wc, p, q, i, j, S, ids, acc, nudges);
                        });
                mode = kRowsNone;
            }
        }
    }
    if (LM && mode == kRowsMasked2) {
        // rows of up to 2 kMaskRow candidates: each row's two masks in slot
        // order (the visiting order of the whole-stencil walk)
        const ulonglong2 m01 = kHoist ? m01h : mask01[i];
        const unsigned long long mm[3] = {m01.x, m01.y, kHoist ? m2h : mask2[i]};
        const unsigned long long *mx = cx.maskx + 3 * (size_t)i;
        const unsigned long long mh[3] = {__ldg(mx), __ldg(mx + 1), __ldg(mx + 2)};
#pragma unroll
        for (int r = 0; r < 3; ++r) {
#pragma unroll
            for (int q = 0; q < 2; ++q)
                walk_mask<float4>(
                    q ? mh[r] : mm[r], ra[r] + q * kMaskRow, cx.n,
                    [&](int j) { return __ldg(xr + j); },
                    [&](int j, const float4 &qv) {
                        relax_pair_walk(wc, p, qv, i, j, S, ids, acc, nudges);
                    });
        }
    } else if (mode == kRowsMasked) {
        const ulonglong2 m01 = kHoist ? m01h : mask01[i];
        const unsigned long long mm[3] = {m01.x, m01.y, kHoist ? m2h : mask2[i]};
        if (R.sm) {
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                const float4 *row = R.sm + R.d[r];
                walk_mask<float4>(
                    mm[r], ra[r], cx.n, [&](int j) { return row[j]; },
                    [&](int j, const float4 &q) {
                        relax_pair_walk(wc, p, q, i, j, S, ids, acc, nudges);
                    });
            }
        } else {
#pragma unroll
            for (int r = 0; r < 3; ++r)
                walk_mask<float4>(
                    mm[r], ra[r], cx.n, [&](int j) { return __ldg(xr + j); },
                    [&](int j, const float4 &q) {
                        relax_pair_walk(wc, p, q, i, j, S, ids, acc, nudges);
                    });
        }
    } else if (mode == kRowsFull) {
        for_each_candidate(key, start, g, capped, cx.max_bucket, cx.n, [&](int j) {
            if (j == i) return;
            const float4 q = __ldg(xr + j);
            if (dist2(p.x - q.x, p.y - q.y) > c.h2) return;
            relax_pair_walk(wc, p, q, i, j, S, ids, acc, nudges);
        });
    }
    if (PROBE) {
        const float nd = (float)nudges * 0.000001f;
        probe_out[i] = make_float2(acc.x + nd, acc.y + nd);
        return;
    }
    relax_finish(i, cx, S, p, acc, nudges, prev, pos_out, vel_out, kr_out, cnt, tile_made);
}


// The slot ranges a thread's masked walk reads (stage_rows' lo, hi): for row
// r, [ra[r], ra[r] + index of the highest hit + 1); nothing for rows without
// hits or particles that do not walk masks.
__device__ __forceinline__ void mask_ranges(int4 rw, unsigned long long m0, unsigned long long m1,
                                            unsigned long long m2, int (&lo)[3], int (&hi)[3])
{
    const int ra[3] = {rw.x, rw.y, rw.z};
    const unsigned long long mm[3] = {m0, m1, m2};
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const bool use = rw.w == kRowsMasked && mm[r] != 0ull;
        lo[r] = use ? ra[r] : INT_MAX;
        hi[r] = use ? ra[r] + 64 - __clzll(mm[r]) : INT_MIN;
    }
}

template <bool PROBE, bool PERSIST = false>
__global__ void __launch_bounds__(kBlock, SPH_RELAX_MIN_BLOCKS)
k_relax_update_sm(Ctx c, const float4 *__restrict__ xr, const ulonglong2 *__restrict__ mask01,
                  const unsigned long long *__restrict__ mask2, const int4 *__restrict__ rows,
                  const float2 *__restrict__ prev,
                  const int *__restrict__ ids, const int *__restrict__ start,
                  const unsigned *__restrict__ occ_in, unsigned *occ_reset,
                  float2 *__restrict__ pos_out, float2 *__restrict__ vel_out,
                  uint2 *__restrict__ kr_out, unsigned *__restrict__ cnt,
                  float2 *__restrict__ probe_out)
{
    extern __shared__ float4 sm_rows[];
    pdl_enter();
    if (!PROBE && blockIdx.x == 0 && threadIdx.x == 0) *occ_reset = 0u;
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    const int ntiles = (c.n + blockDim.x - 1) / blockDim.x;
    for (int tile = blockIdx.x; tile < ntiles; tile += PERSIST ? gridDim.x : ntiles) {
        const int i = tile * blockDim.x + threadIdx.x;
        int lo[3] = {INT_MAX, INT_MAX, INT_MAX}, hi[3] = {INT_MIN, INT_MIN, INT_MIN};
        if (i < c.n) {
            const int4 rw = __ldg(rows + i);
            const ulonglong2 m01 = __ldg(mask01 + i);
            mask_ranges(rw, m01.x, m01.y, __ldg(mask2 + i), lo, hi);
        }
        RowsIn R;
        if (stage_rows(lo, hi, xr, sm_rows, kStagePerThread * (int)blockDim.x, R.d)) R.sm = sm_rows;
        if (i < c.n)
            relax_update_one<PROBE>(i, c, xr, mask01, mask2, rows, prev, ids, start, capped,
                                    pos_out, vel_out, kr_out, cnt, probe_out, LearnedIn(), nullptr,
                                    nullptr, R);
    }
}

template <bool PROBE, bool PERSIST = false, bool LM = false>
__global__ void __launch_bounds__(kBlock, SPH_RELAX_MIN_BLOCKS)
k_relax_update(Ctx c, const float4 *__restrict__ xr, const ulonglong2 *__restrict__ mask01,
               const unsigned long long *__restrict__ mask2, const int4 *__restrict__ rows,
               const float2 *__restrict__ prev,
               const int *__restrict__ ids, const int *__restrict__ start,
               const unsigned *__restrict__ occ_in, unsigned *occ_reset,
               float2 *__restrict__ pos_out, float2 *__restrict__ vel_out,
               uint2 *__restrict__ kr_out, unsigned *__restrict__ cnt,
               float2 *__restrict__ probe_out)
{
    pdl_enter();
    const int i0 = blockIdx.x * blockDim.x + threadIdx.x;
    if (!PROBE && i0 == 0) *occ_reset = 0u;
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    if (!PERSIST) {
        if (i0 < c.n)
            relax_update_one<PROBE, false, false, LM>(i0, c, xr, mask01, mask2, rows, prev, ids,
                                                      start, capped, pos_out, vel_out, kr_out,
                                                      cnt, probe_out);
        return;
    }
    for (int i = i0; i < c.n; i += gridDim.x * blockDim.x)
        relax_update_one<PROBE, false, false, LM>(i, c, xr, mask01, mask2, rows, prev, ids, start,
                                                  capped, pos_out, vel_out, kr_out, cnt,
                                                  probe_out);
}

// The relaxation pass of a learned step (one particle per thread).  PROBE:
// every particle's displacement, fallback included.  Otherwise the particles
// that take the network are advanced here and the others are appended to
// fb_list (one atomic per warp that has any) for k_relax_fallback, so that
// the rare plain gathers do not hold up whole warps.  Block 0 counts the step.
template <bool PROBE, bool LM = false>
__global__ void __launch_bounds__(kBlock, 4)
k_relax_learned(Ctx c, const float4 *__restrict__ xr, const ulonglong2 *__restrict__ mask01,
                const unsigned long long *__restrict__ mask2, const int4 *__restrict__ rows,
                const float2 *__restrict__ prev,
                const int *__restrict__ ids, const int *__restrict__ start,
                const unsigned *__restrict__ occ_in, unsigned *occ_reset,
                float2 *__restrict__ pos_out, float2 *__restrict__ vel_out,
                uint2 *__restrict__ kr_out, unsigned *__restrict__ cnt,
                float2 *__restrict__ probe_out, LearnedIn L, DevState *st, int *__restrict__ fb_list)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (!PROBE && i == 0) {
        *occ_reset = 0u;
        atomicAdd(&st->learned_steps, 1ull);
    }
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    bool used = true;
    L.defer = !PROBE;
    int t = -1;
    if (i < c.n)
        relax_update_one<PROBE, true, false, LM>(i, c, xr, mask01, mask2, rows, prev, ids, start, capped, pos_out,
                                      vel_out, kr_out, cnt, probe_out, L, &used, &t);
    if (PROBE) return;
    if (c.tile_cnt) cta_tile_count(c.tile_cnt, t);
    // fallback particles: those whose stencil rows fit the hit masks go to
    // the front of fb_list (one thread each in k_relax_fallback), those with
    // a row too long for a mask to the back (one warp each)
    const bool longrow = !used && __ldg(rows + i).w == kRowsFull;
    const unsigned lane = threadIdx.x & 31u;
    const unsigned fbs = __ballot_sync(0xffffffffu, !used && !longrow);
    const unsigned fbl = __ballot_sync(0xffffffffu, longrow);
    if (fbs) {
        const int leader = __ffs(fbs) - 1;
        unsigned base = 0;
        if (lane == (unsigned)leader) base = atomicAdd(&st->fb_count, (unsigned)__popc(fbs));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (!used && !longrow) fb_list[base + __popc(fbs & ((1u << lane) - 1u))] = i;
    }
    if (fbl) {
        const int leader = __ffs(fbl) - 1;
        unsigned base = 0;
        if (lane == (unsigned)leader) base = atomicAdd(&st->fb_long, (unsigned)__popc(fbl));
        base = __shfl_sync(0xffffffffu, base, leader);
        if (longrow) fb_list[c.n - 1 - (int)(base + __popc(fbl & ((1u << lane) - 1u)))] = i;
    }
}

// The plain relaxation and update of particle i by a whole warp: the lanes
// test 32 stencil candidates at a time and evaluate the pair terms of the
// hits in parallel; the displacement is then accumulated from them in slot
// order, row by row, with the same packed FMA as the one-thread walk, so the
// result is bit for bit the one-thread result (the plain step's).  Lane 0
// finishes the particle.  The learned step's fallback particles are its
// dense ones (long stencil rows): one thread each made them a long tail.
__device__ __forceinline__ void relax_warp_one(
    int i, const Ctx &cx, const float4 *__restrict__ xr, const ulonglong2 *__restrict__ mask01,
    const unsigned long long *__restrict__ mask2, const int4 *__restrict__ rows,
    const float2 *__restrict__ prev, const int *__restrict__ ids, const int *__restrict__ start,
    bool capped, float2 *__restrict__ pos_out, float2 *__restrict__ vel_out,
    uint2 *__restrict__ kr_out, unsigned *__restrict__ cnt)
{
    const unsigned lane = threadIdx.x & 31u;
    if (capped) {
        // overflowing buckets (pathological): the one-thread form
        if (lane == 0)
            relax_update_one<false, false, true>(i, cx, xr, mask01, mask2, rows, prev, ids, start,
                                                 capped, pos_out, vel_out, kr_out, cnt, nullptr);
        return;
    }
    const Scene *S = cx.scenes + scene_of(cx, i);
    const SG g = load_grid(S);
    const RelaxConsts c = relax_consts(S);
    const float h2 = c.h2;
    const float4 me = xr[i];
    const float2 p = make_float2(me.x, me.y);
    const WalkConsts wc = walk_consts(c, me);  // as relax_update_one's
    float2 acc = make_float2(0.0f, 0.0f);
    int nudges = 0;
    const unsigned key = cell_key(p.x, p.y, g);
    if (searchable(key, i, start, g, false, cx.max_bucket)) {
        int ra[3], rl[3];
        stencil_rows(key, start, g, ra, rl, cx.n);
        const float2 mp = make_float2(-p.x, -p.y);
        for (int r = 0; r < 3; ++r) {
            for (int c0 = 0; c0 < rl[r]; c0 += 32) {
                const int t = c0 + (int)lane;
                const int j = ra[r] + t;
                float s = 0.0f;
                float2 d = make_float2(0.0f, 0.0f);
                bool apply = false;
                if (t < rl[r] && j != i && in_bounds(j, cx.n, kBadSlot)) {
                    const float4 q = __ldg(xr + j);
                    float2 e;
                    if (dist2_packed(mp, make_float2(q.x, q.y), e) <= h2)
                        apply = relax_pair_term(wc, p, q, i, j, S, ids, s, d, nudges);
                }
                unsigned hits = __ballot_sync(0xffffffffu, apply);
                while (hits) {
                    const int b = __ffs(hits) - 1;
                    hits &= hits - 1u;
                    const float sb = __shfl_sync(0xffffffffu, s, b);
                    const float dx = __shfl_sync(0xffffffffu, d.x, b);
                    const float dy = __shfl_sync(0xffffffffu, d.y, b);
                    acc = __ffma2_rn(make_float2(-sb, -sb), make_float2(dx, dy), acc);
                }
            }
        }
        nudges = __reduce_add_sync(0xffffffffu, nudges);
    }
    if (lane == 0) relax_finish(i, cx, S, p, acc, nudges, prev, pos_out, vel_out, kr_out, cnt,
                                nullptr);
}

// The fallback particles of a learned step: the plain relaxation + update
// for each slot on fb_list -- one thread per particle for those at its front
// (rows within the hit masks), then one warp per particle for those at its
// back (a row too long for a mask: the densest, whose one-thread walks were
// the long tail).  Grid-stride loops: the counts are known on the device
// only.  Block 0 adds the counts to the fallback statistics.
template <bool LM = false>
__global__ void __launch_bounds__(kBlock, 4)
k_relax_fallback(Ctx c, const float4 *__restrict__ xr, const ulonglong2 *__restrict__ mask01,
                 const unsigned long long *__restrict__ mask2, const int4 *__restrict__ rows,
                 const float2 *__restrict__ prev,
                 const int *__restrict__ ids, const int *__restrict__ start,
                 const unsigned *__restrict__ occ_in, float2 *__restrict__ pos_out,
                 float2 *__restrict__ vel_out, uint2 *__restrict__ kr_out,
                 unsigned *__restrict__ cnt, DevState *st, const int *__restrict__ fb_list)
{
    const unsigned total = st->fb_count, total_long = st->fb_long;
    if (blockIdx.x == 0 && threadIdx.x == 0)
        atomicAdd(&st->learned_fallback, (unsigned long long)(total + total_long));
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    const unsigned t0 = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned nt = gridDim.x * blockDim.x;
    for (unsigned k = t0; k < total; k += nt)
        relax_update_one<false, false, true, LM>(fb_list[k], c, xr, mask01, mask2, rows, prev,
                                                 ids, start, capped, pos_out, vel_out, kr_out,
                                                 cnt, nullptr);
    // the long-row particles: a warp each when they are few enough for one
    // pass of the grid's warps (the long tail of a step with a few dense
    // spots), else a thread each (many dense particles: a warp each would
    // leave most of them waiting).  Both sum in slot order: the same bits.
    const unsigned w0 = t0 >> 5, nw = nt >> 5;
    if (total_long <= nw) {
        for (unsigned k = w0; k < total_long; k += nw)
            relax_warp_one(fb_list[c.n - 1 - (int)k], c, xr, mask01, mask2, rows, prev, ids,
                           start, capped, pos_out, vel_out, kr_out, cnt);
    } else {
        for (unsigned k = t0; k < total_long; k += nt)
            relax_update_one<false, false, true, LM>(fb_list[c.n - 1 - (int)k], c, xr, mask01,
                                                     mask2, rows, prev, ids, start, capped,
                                                     pos_out, vel_out, kr_out, cnt, nullptr);
    }
}

// ---------------------------------------------------------------------------
// state I/O, diagnostics, neighbour lists
// ---------------------------------------------------------------------------

// Sorted state -> id order: out = [pos | vel | prev | rho | pressure] (5 n float2).
__global__ void __launch_bounds__(kBlock)
k_unpermute(Ctx c, const int *__restrict__ id_a, const float2 *__restrict__ pos_a,
            const float2 *__restrict__ vel_a, const int *__restrict__ id_c,
            const float2 *__restrict__ prev_c, const float4 *__restrict__ xr_c,
            float2 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const size_t n = (size_t)c.n;
    const int ia = id_a[i], ic = id_c[i];
    out[ia] = pos_a[i];
    out[n + ia] = vel_a[i];
    out[2 * n + ic] = prev_c[i];
    const float4 x4 = xr_c[i];
    const float2 r = make_float2(x4.z, x4.w);
    out[3 * n + ic] = r;
    // pressure and near pressure, fluid.c:563-564, with the scene's tunables
    const Scene *S = c.scenes + scene_of(c, i);
    const float k = __ldg(&S->P.k), rest = __ldg(&S->P.rest_density), kn = __ldg(&S->P.k_near);
    out[4 * n + ic] = make_float2(__fmul_rn(k, __fsub_rn(r.x, rest)), __fmul_rn(kn, r.y));
}

// (rho, rho_near) of the (x, y, rho, rho_near) records.
__global__ void __launch_bounds__(kBlock)
k_xr_density(int n, const float4 *__restrict__ xr, float2 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 v = xr[i];
    out[i] = make_float2(v.z, v.w);
}

// Sorted per-particle values -> id order.
__global__ void __launch_bounds__(kBlock)
k_by_id(int n, const int *__restrict__ ids, const float2 *__restrict__ in, float2 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    out[ids[i]] = in[i];
}

// Identity id map for the *_c slots that download reads before the first step.
__global__ void __launch_bounds__(kBlock)
k_iota(int n, int *__restrict__ ids)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) ids[i] = i;
}

// Pixel-space shorts for the render rank (fluid.c:360-361), by id.
__global__ void __launch_bounds__(kBlock)
k_pack_coords(Ctx c, const int *__restrict__ id_a, const float2 *__restrict__ pos_a,
              short2 *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const Scene *S = c.scenes + scene_of(c, i);
    const float max_x = __ldg(&S->max_x), max_y = __ldg(&S->max_y);
    const float2 p = pos_a[i];
    const float cx = __fmul_rn(__fsub_rn(__fdiv_rn(__fmul_rn(2.0f, p.x), max_x), 1.0f), 32767.0f);
    const float cy = __fmul_rn(__fsub_rn(__fdiv_rn(__fmul_rn(2.0f, p.y), max_y), 1.0f), 32767.0f);
    out[id_a[i]] = make_short2((short)__float2int_rz(cx), (short)__float2int_rz(cy));
}

// FP64 sums of density, near density and 0.5|v|^2, per block (fixed order).
__global__ void __launch_bounds__(kBlock)
k_diag_partial(int n, const float4 *__restrict__ xr_c, const float2 *__restrict__ vel_a,
               double *__restrict__ partials)
{
    __shared__ double sh[3][kBlock / 32];
    double a = 0.0, b = 0.0, c = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float4 r = xr_c[i];
        const float2 v = vel_a[i];
        a += r.z;
        b += r.w;
        c += 0.5 * ((double)v.x * v.x + (double)v.y * v.y);
    }
    a = warp_sum(a); b = warp_sum(b); c = warp_sum(c);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { sh[0][warp] = a; sh[1][warp] = b; sh[2][warp] = c; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0, s1 = 0, s2 = 0;
        for (int w = 0; w < kBlock / 32; ++w) { s0 += sh[0][w]; s1 += sh[1][w]; s2 += sh[2][w]; }
        partials[3 * blockIdx.x] = s0;
        partials[3 * blockIdx.x + 1] = s1;
        partials[3 * blockIdx.x + 2] = s2;
    }
}

__global__ void k_diag_final(int nparts, int n, const double *__restrict__ partials, double *out)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s0 = 0, s1 = 0, s2 = 0;
    for (int b = 0; b < nparts; ++b) {
        s0 += partials[3 * b];
        s1 += partials[3 * b + 1];
        s2 += partials[3 * b + 2];
    }
    out[0] = n ? s0 / n : 0.0;
    out[1] = n ? s1 / n : 0.0;
    out[2] = n ? s2 / n : 0.0;
}

// Per-scene FP64 means (one block per scene, fixed order).  The density
// records are in C order and the velocities in A order; both keep every
// scene in its own slot range.
__global__ void __launch_bounds__(kBlock)
k_diag_scenes(Ctx c, const float4 *__restrict__ xr_c, const float2 *__restrict__ vel_a,
              double *__restrict__ out)
{
    __shared__ double sh[3][kBlock / 32];
    const int s = blockIdx.x;
    const int b0 = __ldg(c.p_off + s), b1 = __ldg(c.p_off + s + 1);
    double a = 0.0, b = 0.0, k = 0.0;
    for (int i = b0 + threadIdx.x; i < b1; i += blockDim.x) {
        const float4 r = xr_c[i];
        const float2 v = vel_a[i];
        a += r.z;
        b += r.w;
        k += 0.5 * ((double)v.x * v.x + (double)v.y * v.y);
    }
    a = warp_sum(a); b = warp_sum(b); k = warp_sum(k);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { sh[0][warp] = a; sh[1][warp] = b; sh[2][warp] = k; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double s0 = 0, s1 = 0, s2 = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { s0 += sh[0][w]; s1 += sh[1][w]; s2 += sh[2][w]; }
        const int m = b1 - b0;
        out[3 * s] = m ? s0 / m : 0.0;
        out[3 * s + 1] = m ? s1 / m : 0.0;
        out[3 * s + 2] = m ? s2 / m : 0.0;
    }
}

// The reference's half list of one particle, in its order (hash.c:169-234):
// later members of its own cell, then the forward cells (0,+1), (+1,-1),
// (+1,0), (+1,+1), each in id order, r2 <= h2, cut at max_neighbors.
// WRITE = false counts, WRITE = true writes ids at out + off[id].
template <bool WRITE>
__global__ void __launch_bounds__(kBlock)
k_half_lists(Ctx c, const float2 *__restrict__ pos, const int *__restrict__ ids,
             const int *__restrict__ start, const unsigned *__restrict__ occ_in,
             unsigned *__restrict__ counts, const int *__restrict__ off, int *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const Scene *S = c.scenes + scene_of(c, i);
    const SG g = load_grid(S);
    const float hh = __ldg(&S->P.smoothing_radius);
    const int max_neighbors = __ldg(&S->max_neighbors);
    const float h2 = __fmul_rn(hh, hh);
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    const float2 p = pos[i];
    const unsigned key = cell_key(p.x, p.y, g);
    const int myid = ids[i];
    int cnum = 0;
    int *dst = WRITE ? out + off[myid] : nullptr;
    if (searchable(key, i, start, g, capped, c.max_bucket)) {
        const int lk = (int)key - g.c_off;
        const int gy = lk / g.size_x, gx = lk - gy * g.size_x;
#pragma unroll
        for (int f = 0; f < 5; ++f) {
            const int x = gx + (f >= 2 ? 1 : 0);
            const int y = gy + (f == 0 ? 0 : (f == 1 ? 1 : f - 3));
            if (x < 0 || y < 0 || x >= g.size_x || y >= g.size_y) continue;
            const int cell = g.c_off + y * g.size_x + x;
            const int a = start[cell], e = start[cell + 1];
            const int b = capped && e - a > c.max_bucket ? a + c.max_bucket : e;
            for (int j = f == 0 ? i + 1 : a; j < b; ++j) {
                const float2 q = pos[j];
                if (dist2(p.x - q.x, p.y - q.y) > h2) continue;
                if (cnum < max_neighbors) {
                    if (WRITE) dst[cnum] = ids[j];
                    ++cnum;
                }
            }
        }
    }
    if (!WRITE) counts[myid] = (unsigned)cnum;
}

// ---------------------------------------------------------------------------
// host-side launchers
// ---------------------------------------------------------------------------

static inline int blocks_for(int n, int bs = kBlock) { return (n + bs - 1) / bs; }

// Launches one kernel of a step on the handle's stream.  With SPH_PDL it is
// a programmatic dependent launch: the kernel may start launching while
// its predecessor's last CTAs still run, and waits for the predecessor's
// results in pdl_enter (in stream capture this becomes a programmatic edge
// of the step's graph).
#ifndef SPH_PDL
#define SPH_PDL 1
#endif
template <typename... KArgs, typename... Args>
static void launch_step(void (*kern)(KArgs...), dim3 grid, dim3 block, size_t smem,
                        cudaStream_t stream, Args &&...args)
{
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = stream;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = SPH_PDL ? 1 : 0;
    (void)cudaLaunchKernelEx(&cfg, kern, std::forward<Args>(args)...);
}

// Grid of a gather launch for shape s.
static inline dim3 gather_grid(const sph_cuda *h, const Shape &s)
{
    const int tiles = blocks_for(h->n, s.block);
    if (s.persistent <= 0) return dim3(tiles);
    const int p = h->num_sms * s.persistent;
    return dim3(p < tiles ? p : tiles);
}

// Exclusive scan of `in` (M entries) into out (M + 1 entries).  Both arrays
// must be 16-byte aligned: the scan kernels move 16-byte vectors.
static int launch_scan(sph_cuda *h, unsigned *in, int M, int *out, unsigned *occ, bool zero,
                       const unsigned *nocell)
{
    if (((uintptr_t)in | (uintptr_t)out) & 15u) {
        set_error("internal: scan arrays not 16-byte aligned");
        return SPH_ERR_INVALID;
    }
    const int tiles = (M + kScanTile - 1) / kScanTile;
    if (tiles > h->ntiles) {
        set_error("internal: scan of %d items exceeds the tile buffer", M);
        return SPH_ERR_INVALID;
    }
    k_scan_reduce<<<tiles, kScanThreads, 0, h->stream>>>(in, M, nocell, h->tile_sums, h->d_state,
                                                         occ, h->max_bucket, h->max_neighbors);
    k_scan_apply<<<tiles, kScanThreads, 0, h->stream>>>(in, M, h->tile_sums, out, zero ? 1 : 0);
    return SPH_OK;
}

// The cell starts of a step's build (all M counters, zeroed after) into
// `out` (M + 1 entries); the build's key producer counted its particles per
// build tile into build_tiles, which the build's scatter zeroes again.
static int build_tiles_of(const sph_cuda *h) { return (h->M + kBuildTile - 1) / kBuildTile; }
// particles per thread of the step's scatter and permute
constexpr int kBuildPerThread = 2;

static void enqueue_cell_starts(sph_cuda *h, int *out, unsigned *occ)
{
    launch_step(k_cell_starts, build_tiles_of(h), kBuildThreads, 0, h->stream, h->cnt, h->M,
                (const unsigned *)h->d_nocell, (const unsigned *)h->build_tiles, out, h->d_state,
                occ, h->max_bucket, h->max_neighbors);
}

static const char *const kKernelNames[] = {
    "viscosity_predict", "cell_starts_1", "cell_scatter_1", "cell_permute_1", "density",
    "relax_update",      "cell_starts_2", "cell_scatter_2", "cell_permute_2"};
static const int kStepKernels = 9;
// A step with a learned model: density becomes the feature pass, then the
// network, then the relaxation with fallback.
static const char *const kLearnedKernelNames[] = {
    "viscosity_predict", "cell_starts_1",  "cell_scatter_1", "cell_permute_1",
    "features",          "mlp",            "relax_learned",  "relax_fallback",
    "cell_starts_2",     "cell_scatter_2", "cell_permute_2"};
static const int kLearnedStepKernels = 11;

// Viscosity + prediction, the rebuild into the C order (kernels 0-3 of a step).
template <class Mark>
static void enqueue_predict_sort(sph_cuda *h, Mark &mark)
{
    const int n = h->n;
    const int nb = blocks_for(n);
    const Ctx c = make_ctx(h);
    DevState *st = h->d_state;
    {
#if SPH_VISC_SMEM
        auto kv = h->shape[0].persistent ? k_viscosity_predict_sm<true>
                                         : k_viscosity_predict_sm<false>;
        const size_t smem = 2 * (size_t)kStagePerThread * h->shape[0].block * sizeof(float2);
        launch_step(kv, gather_grid(h, h->shape[0]), h->shape[0].block, smem, h->stream, c,
                    (const DevState *)st, (const float2 *)h->pos_a, (const float2 *)h->vel_a,
                    (const int *)h->start_a, (const unsigned *)&st->build_max_occ[SLOT_RELAXED],
                    &st->build_max_occ[SLOT_PREDICTED], h->pos_b, h->prev_b, h->kr_b, h->cnt);
#else
        auto kv = h->shape[0].persistent ? k_viscosity_predict<false, true>
                                         : k_viscosity_predict<false, false>;
        launch_step(kv, gather_grid(h, h->shape[0]), h->shape[0].block, 0, h->stream, c,
                    (const DevState *)st, (const float2 *)h->pos_a, (const float2 *)h->vel_a,
                    (const int *)h->start_a, (const unsigned *)&st->build_max_occ[SLOT_RELAXED],
                    &st->build_max_occ[SLOT_PREDICTED], h->pos_b, h->prev_b, h->kr_b, h->cnt,
                    (float2 *)nullptr);
#endif
    }
    mark();
    enqueue_cell_starts(h, h->start_c, &st->build_max_occ[SLOT_PREDICTED]);
    mark();
    const int nbx = blocks_for(n, kBlock * kBuildPerThread);
    launch_step(k_scatter_ids_x<kBuildPerThread>, nbx, kBlock, 0, h->stream, n,
                (const uint2 *)h->kr_b, (const int *)h->id_a, (const int *)h->start_c, h->tmp_id,
                h->build_tiles, build_tiles_of(h));
    mark();
    launch_step(k_permute_x<kBuildPerThread>, nbx, kBlock, 0, h->stream, n,
                (const uint2 *)h->kr_b, (const int *)h->start_c, (const int *)h->tmp_id,
                (const int *)h->id_a, (const float2 *)h->pos_b, (const float2 *)h->prev_b,
                h->id_c, h->pos_c, h->prev_c, (DevState *)nullptr);
    mark();
}

static void enqueue_density(sph_cuda *h)
{
    DevState *st = h->d_state;
#if SPH_DENS_SMEM
    auto kd = h->shape[1].persistent ? k_density_sm<true> : k_density_sm<false>;
    const size_t smem = (size_t)kStagePerThread * h->shape[1].block * sizeof(float2);
#else
    auto kd = h->shape[1].persistent
                  ? (h->long_masks ? k_density_t<true, true> : k_density_t<true, false>)
                  : (h->long_masks ? k_density_t<false, true> : k_density_t<false, false>);
    const size_t smem = 0;
#endif
    launch_step(kd, gather_grid(h, h->shape[1]), h->shape[1].block, smem, h->stream, make_ctx(h),
                (const float2 *)h->pos_c, (const int *)h->start_c,
                (const unsigned *)&st->build_max_occ[SLOT_PREDICTED], h->xr_c, h->mask01_c,
                h->mask2_c, h->rows_c);
}

// Whether this build's gathers support long-row hit masks (not with the
// shared-memory staged forms).
bool long_masks_supported() { return !(SPH_DENS_SMEM || SPH_RELAX_SMEM); }

// The density pass of a step (the learned step's features start with it).
int launch_density_pass(sph_cuda *h)
{
    if (h->n == 0) return SPH_OK;
    enqueue_density(h);
    return cuda_fail(cudaGetLastError(), "density");
}

// The C-order state of the next step's relaxation -- predicted positions,
// their cell starts, density records and hit masks -- without advancing:
// the A state is left as it is (the last step's density record in xr_c is
// replaced).
int enqueue_predicted_state(sph_cuda *h)
{
    if (h->n == 0) return SPH_OK;
    auto none = []() {};
    enqueue_predict_sort(h, none);
    enqueue_density(h);
    return cuda_fail(cudaGetLastError(), "predicted state");
}

// The relaxation passes of a learned step (network particles, then the
// fallback list); with probe_out, one pass writes every particle's
// displacement (C order) instead of advancing.  `events` (two) are recorded
// after each pass.
int launch_learned_relax(sph_cuda *h, float2 *probe_out, cudaEvent_t *events)
{
    const Ctx c = make_ctx(h);
    DevState *st = h->d_state;
    LearnedIn L;
    L.net = h->net_c;
    L.nbc = h->nbc_c;
    L.thr_pct = h->learned_thr * 100.0f;
    // a negative threshold sends every particle to the plain relaxation
    L.max_nb = h->learned_thr < 0.0f ? -1 : SPH_LEARNED_MAX_NEIGHBORS;
    const int nb = blocks_for(h->n);
    const unsigned *occ = &st->build_max_occ[SLOT_PREDICTED];
    const bool lm = h->long_masks;
    if (probe_out) {
        (lm ? k_relax_learned<true, true> : k_relax_learned<true, false>)<<<nb, kBlock, 0,
                                                                          h->stream>>>(
            c, h->xr_c, h->mask01_c, h->mask2_c, h->rows_c, h->prev_c, h->id_c, h->start_c, occ,
            nullptr, nullptr, nullptr, nullptr, nullptr, probe_out, L, st, nullptr);
        return cuda_fail(cudaGetLastError(), "learned relaxation probe");
    }
    (lm ? k_relax_learned<false, true> : k_relax_learned<false, false>)<<<nb, kBlock, 0,
                                                                        h->stream>>>(
        c, h->xr_c, h->mask01_c, h->mask2_c, h->rows_c, h->prev_c, h->id_c, h->start_c, occ,
        &st->build_max_occ[SLOT_RELAXED], h->pos_b, h->vel_b, h->kr_b, h->cnt, nullptr, L, st,
        h->fb_list);
    if (events) cudaEventRecord(events[0], h->stream);
    const int fb_blocks = std::min(nb, 4 * h->num_sms);
    (lm ? k_relax_fallback<true> : k_relax_fallback<false>)<<<fb_blocks, kBlock, 0, h->stream>>>(
        c, h->xr_c, h->mask01_c, h->mask2_c, h->rows_c, h->prev_c, h->id_c, h->start_c, occ,
        h->pos_b, h->vel_b, h->kr_b, h->cnt, st, h->fb_list);
    if (events) cudaEventRecord(events[1], h->stream);
    return cuda_fail(cudaGetLastError(), "learned relaxation");
}

// Queues one step.  With `events` (one per kernel + 1) each kernel is
// bracketed for timing.  With `mid_tp`, the scene's tunables are replaced
// by *mid_tp after the first half (gravity, viscosity, prediction and the
// cell build of the predicted positions) and before the density pass, the
// relaxation and the velocity update -- where the reference's compute rank
// receives new tunables inside a step (fluid.c:293-294, between
// predict_positions at :279 and hash_fluid at :315).  Single-scene handles.
int enqueue_step(sph_cuda *h, cudaEvent_t *events, int *nkernels, const tunable_parameters *mid_tp)
{
    const int n = h->n;
    const int nb = blocks_for(n);
    const Ctx c = make_ctx(h);
    DevState *st = h->d_state;
    int e = 0;
    auto mark = [&]() {
        if (events) cudaEventRecord(events[e], h->stream);
        ++e;
    };
    mark();
    enqueue_predict_sort(h, mark);
    if (mid_tp) {
        const int rc = set_scene_params(h, 0, mid_tp);
        if (rc != SPH_OK) return rc;
    }
    if (h->learned) {
        int rc = launch_learned_passes(h, events ? events + e : nullptr);
        if (rc != SPH_OK) return rc;
        e += 2;
        rc = launch_learned_relax(h, nullptr, events ? events + e : nullptr);
        if (rc != SPH_OK) return rc;
        e += 2;
    } else {
        enqueue_density(h);
        mark();
#if SPH_RELAX_SMEM
        auto kr = h->shape[2].persistent ? k_relax_update_sm<false, true>
                                         : k_relax_update_sm<false, false>;
        const size_t smem = (size_t)kStagePerThread * h->shape[2].block * sizeof(float4);
#else
        auto kr = h->shape[2].persistent
                      ? (h->long_masks ? k_relax_update<false, true, true>
                                       : k_relax_update<false, true, false>)
                      : (h->long_masks ? k_relax_update<false, false, true>
                                       : k_relax_update<false, false, false>);
        const size_t smem = 0;
#endif
        launch_step(kr, gather_grid(h, h->shape[2]), h->shape[2].block, smem, h->stream, c,
                    (const float4 *)h->xr_c, (const ulonglong2 *)h->mask01_c,
                    (const unsigned long long *)h->mask2_c, (const int4 *)h->rows_c,
                    (const float2 *)h->prev_c, (const int *)h->id_c, (const int *)h->start_c,
                    (const unsigned *)&st->build_max_occ[SLOT_PREDICTED],
                    &st->build_max_occ[SLOT_RELAXED], h->pos_b, h->vel_b, h->kr_b, h->cnt,
                    (float2 *)nullptr);
        mark();
    }
    enqueue_cell_starts(h, h->start_a, &st->build_max_occ[SLOT_RELAXED]);
    mark();
    const int nbx = blocks_for(n, kBlock * kBuildPerThread);
    launch_step(k_scatter_ids_x<kBuildPerThread>, nbx, kBlock, 0, h->stream, n,
                (const uint2 *)h->kr_b, (const int *)h->id_c, (const int *)h->start_a, h->tmp_id,
                h->build_tiles, build_tiles_of(h));
    mark();
    launch_step(k_permute_x<kBuildPerThread>, nbx, kBlock, 0, h->stream, n,
                (const uint2 *)h->kr_b, (const int *)h->start_a, (const int *)h->tmp_id,
                (const int *)h->id_c, (const float2 *)h->pos_b, (const float2 *)h->vel_b,
                h->id_a, h->pos_a, h->vel_a, st);
    mark();
    if (nkernels) *nkernels = e - 1;
    return cuda_fail(cudaGetLastError(), "step launch");
}

unsigned bounds_flags_kernels() { return read_bounds_flag(); }

const char *kernel_name(int k)
{
    return (k >= 0 && k < kStepKernels) ? kKernelNames[k] : "";
}
const char *step_kernel_name(const sph_cuda *h, int k)
{
    if (h && h->learned) return (k >= 0 && k < kLearnedStepKernels) ? kLearnedKernelNames[k] : "";
    return kernel_name(k);
}
int step_kernel_count() { return kStepKernels; }
int step_kernel_count(const sph_cuda *h)
{
    return (h && h->learned) ? kLearnedStepKernels : kStepKernels;
}

// Host-layout particles, already on the device, -> the upload arrays in id
// order: pos_b, vel_b, prev_c and xr_c = (x, y, rho, rho_near).  From
// structure-of-arrays (vx, vy may be null: zero) or from the reference's
// fluid_particle records.
__global__ void __launch_bounds__(kBlock)
k_upload_soa(int n, const float *__restrict__ x, const float *__restrict__ y,
             const float *__restrict__ vx, const float *__restrict__ vy, float2 *__restrict__ pos,
             float2 *__restrict__ vel, float2 *__restrict__ prev, float4 *__restrict__ xr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float px = x[i], py = y[i];
    pos[i] = make_float2(px, py);
    vel[i] = make_float2(vx ? vx[i] : 0.0f, vy ? vy[i] : 0.0f);
    prev[i] = make_float2(px, py);
    xr[i] = make_float4(px, py, 0.0f, 0.0f);
}

__global__ void __launch_bounds__(kBlock)
k_upload_records(int n, const fluid_particle *__restrict__ ps, float2 *__restrict__ pos,
                 float2 *__restrict__ vel, float2 *__restrict__ prev, float4 *__restrict__ xr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const fluid_particle &p = ps[i];
    pos[i] = make_float2(p.x, p.y);
    vel[i] = make_float2(p.v_x, p.v_y);
    prev[i] = make_float2(p.x_prev, p.y_prev);
    xr[i] = make_float4(p.x, p.y, p.density, p.density_near);
}

// Launches one of the two above on device copies of the caller's arrays
// (x, y, vx, vy or recs; the others null).
int launch_upload_layout(sph_cuda *h, int n, const float *x, const float *y, const float *vx,
                         const float *vy, const fluid_particle *recs)
{
    if (n == 0) return SPH_OK;
    const int nb = blocks_for(n);
    if (recs)
        k_upload_records<<<nb, kBlock, 0, h->stream>>>(n, recs, h->pos_b, h->vel_b, h->prev_c,
                                                       h->xr_c);
    else
        k_upload_soa<<<nb, kBlock, 0, h->stream>>>(n, x, y, vx, vy, h->pos_b, h->vel_b, h->prev_c,
                                                   h->xr_c);
    return cuda_fail(cudaGetLastError(), "upload layout");
}

// The id-order records of k_unpermute (pos, vel, prev, (rho, rho_near),
// pressures; n float2 each) -> six float arrays x, y, vx, vy, rho, rho_near
// (n each, in that order), for copies straight into the caller's arrays.
__global__ void __launch_bounds__(kBlock)
k_split_soa(int n, const float2 *__restrict__ rec, float *__restrict__ out)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const size_t m = (size_t)n;
    const float2 p = rec[i], v = rec[m + i], r = rec[3 * m + i];
    out[i] = p.x;
    out[m + i] = p.y;
    out[2 * m + i] = v.x;
    out[3 * m + i] = v.y;
    out[4 * m + i] = r.x;
    out[5 * m + i] = r.y;
}

int launch_split_soa(sph_cuda *h, int n, const float2 *rec, float *out)
{
    if (n == 0) return SPH_OK;
    k_split_soa<<<blocks_for(n), kBlock, 0, h->stream>>>(n, rec, out);
    return cuda_fail(cudaGetLastError(), "split");
}

// Upload tail: pos_b / vel_b (id order) -> sorted A state; prev_c / xr_c
// already hold the uploaded values in id order.
int upload_soa_device(sph_cuda *h, int n)
{
    const int nb = blocks_for(n);
    DevState *st = h->d_state;
    if (n > 0) {
        // a fresh state starts every step's build from zero tile counts,
        // whatever an interrupted step left
        cudaMemsetAsync(h->build_tiles, 0, (size_t)h->ntiles * sizeof(unsigned), h->stream);
        k_iota<<<nb, kBlock, 0, h->stream>>>(n, h->id_c);
        k_keys<<<nb, kBlock, 0, h->stream>>>(make_ctx(h), h->pos_b, h->kr_b, h->cnt,
                                             &st->build_max_occ[SLOT_RELAXED]);
        const int rc = launch_scan(h, h->cnt, h->M, h->start_a, &st->build_max_occ[SLOT_RELAXED],
                                   true, h->d_nocell);
        if (rc != SPH_OK) return rc;
        k_scatter_ids<<<nb, kBlock, 0, h->stream>>>(n, h->kr_b, nullptr, h->start_a, h->tmp_id,
                                                    nullptr, 0);
        k_permute<<<nb, kBlock, 0, h->stream>>>(n, h->kr_b, h->start_a, h->tmp_id, nullptr,
                                                h->pos_b, h->vel_b, h->id_a, h->pos_a, h->vel_a,
                                                nullptr);
    }
    return cuda_fail(cudaGetLastError(), "upload kernels");
}

int launch_unpermute(sph_cuda *h, float2 *out)
{
    if (h->n == 0) return SPH_OK;
    k_unpermute<<<blocks_for(h->n), kBlock, 0, h->stream>>>(make_ctx(h), h->id_a, h->pos_a,
                                                            h->vel_a, h->id_c, h->prev_c, h->xr_c,
                                                            out);
    return cuda_fail(cudaGetLastError(), "unpermute");
}

int launch_pack(sph_cuda *h, short2 *out)
{
    if (h->n == 0) return SPH_OK;
    k_pack_coords<<<blocks_for(h->n), kBlock, 0, h->stream>>>(make_ctx(h), h->id_a, h->pos_a, out);
    return cuda_fail(cudaGetLastError(), "pack coords");
}

int launch_diagnostics(sph_cuda *h, double *d_out)
{
    const int parts = h->npartials;
    k_diag_partial<<<parts, kBlock, 0, h->stream>>>(h->n, h->xr_c, h->vel_a, h->d_partials);
    k_diag_final<<<1, 32, 0, h->stream>>>(parts, h->n, h->d_partials, d_out);
    return cuda_fail(cudaGetLastError(), "diagnostics");
}

int launch_scene_diagnostics(sph_cuda *h, double *d_out)
{
    if (h->nscenes == 0) return SPH_OK;
    k_diag_scenes<<<h->nscenes, kBlock, 0, h->stream>>>(make_ctx(h), h->xr_c, h->vel_a, d_out);
    return cuda_fail(cudaGetLastError(), "scene diagnostics");
}

// Probes on the A state.  which: 0 density, 1 relaxation displacement,
// 2 viscosity velocity change.  `scratch` (probe_scratch_bytes(n), 256-byte
// aligned) holds the sorted records; out: n float2 by id (device).
size_t probe_scratch_bytes(int n)
{
    const size_t a = ((size_t)n * 16 + 255) & ~(size_t)255;
    return 4 * a + (((size_t)n * 8 + 255) & ~(size_t)255);
}

int launch_probe(sph_cuda *h, int which, void *scratch, float2 *out)
{
    const int n = h->n;
    if (n == 0) return SPH_OK;
    const int nb = blocks_for(n);
    const Ctx c = make_ctx(h);
    DevState *st = h->d_state;
    const unsigned *occ = &st->build_max_occ[SLOT_RELAXED];
    const size_t a = ((size_t)n * 16 + 255) & ~(size_t)255;
    char *base = (char *)scratch;
    float4 *xr = (float4 *)base;
    ulonglong2 *m01 = (ulonglong2 *)(base + a);
    unsigned long long *m2 = (unsigned long long *)(base + 2 * a);
    int4 *rw = (int4 *)(base + 3 * a);
    float2 *sorted = (float2 *)(base + 4 * a);
    if (which == 0 || which == 1) {
        k_density<<<nb, kBlock, 0, h->stream>>>(c, h->pos_a, h->start_a, occ, xr, m01, m2, rw);
        if (which == 1)
            k_relax_update<true><<<nb, kBlock, 0, h->stream>>>(
                c, xr, m01, m2, rw, nullptr, h->id_a, h->start_a, occ, nullptr, nullptr, nullptr,
                nullptr, nullptr, sorted);
        else
            k_xr_density<<<nb, kBlock, 0, h->stream>>>(n, xr, sorted);
    } else {
        k_viscosity_predict<true><<<nb, kBlock, 0, h->stream>>>(
            c, st, h->pos_a, h->vel_a, h->start_a, occ, nullptr, nullptr, nullptr, nullptr,
            nullptr, sorted);
    }
    k_by_id<<<nb, kBlock, 0, h->stream>>>(n, h->id_a, sorted, out);
    return cuda_fail(cudaGetLastError(), "probe");
}

// Half lists in the reference's order on the A state.  d_counts: n + 1
// words, d_off: n + 1 ints (both 16-byte aligned).
int launch_half_lists(sph_cuda *h, unsigned *d_counts, int *d_off, int *d_ids, bool write)
{
    const int n = h->n;
    if (n == 0) return SPH_OK;
    const int nb = blocks_for(n);
    const Ctx c = make_ctx(h);
    const unsigned *occ = &h->d_state->build_max_occ[SLOT_RELAXED];
    if (!write) {
        k_half_lists<false><<<nb, kBlock, 0, h->stream>>>(c, h->pos_a, h->id_a, h->start_a, occ,
                                                          d_counts, nullptr, nullptr);
        const int rc = launch_scan(h, d_counts, n, d_off, nullptr, false, nullptr);
        if (rc != SPH_OK) return rc;
    } else {
        k_half_lists<true><<<nb, kBlock, 0, h->stream>>>(c, h->pos_a, h->id_a, h->start_a, occ,
                                                         nullptr, d_off, d_ids);
    }
    return cuda_fail(cudaGetLastError(), "half lists");
}

}  // namespace sph
