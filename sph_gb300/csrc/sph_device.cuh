// sph_device.cuh -- device helpers shared by the libsph_cuda kernels.
#pragma once

#include <climits>

#include "sph_internal.h"

namespace sph {

// The scene of a particle slot (slots of a scene are contiguous, and ids
// follow the same ranges): the last s with p_off[s] <= i.
__device__ __forceinline__ int scene_of(const Ctx &c, int i)
{
    if (c.nscenes == 1) return 0;
    int lo = 0, hi = c.nscenes;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(c.p_off + mid) <= i) lo = mid;
        else hi = mid;
    }
    return lo;
}

// Programmatic dependent launch between the kernels of a step: a kernel
// lets the next one start launching as soon as all of its own CTAs are
// running (pdl_trigger), and waits for its predecessor's results before
// touching them (pdl_wait).  Both are no-ops for a kernel launched without
// the programmatic-serialization attribute.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;"); }
__device__ __forceinline__ void pdl_enter()
{
    pdl_wait();
    pdl_trigger();
}

// A scene's grid, as the cell keys and stencils use it.  inv is 1/spacing
// when spacing is a power of two (then x / spacing == x * inv exactly: both
// round the same real number), 0 otherwise.
struct SG {
    float spacing, inv;
    int size_x, size_y, ncells, c_off;
};

__device__ __forceinline__ SG load_grid(const Scene *__restrict__ S)
{
    SG g;
    g.spacing = __ldg(&S->spacing);
    const unsigned b = __float_as_uint(g.spacing);
    const unsigned e = (b >> 23) & 0xFFu;
    // a normal power of two whose reciprocal is normal too
    g.inv = ((b & 0x807FFFFFu) == 0u && e > 1u && e < 253u) ? __uint_as_float((254u - e) << 23)
                                                           : 0.0f;
    g.size_x = __ldg(&S->size_x);
    g.size_y = __ldg(&S->size_y);
    g.ncells = __ldg(&S->ncells);
    g.c_off = __ldg(&S->c_off);
    return g;
}

// A scene's box: min_x, max_x, min_y, max_y.
__device__ __forceinline__ float4 load_box(const Scene *__restrict__ S)
{
    return make_float4(__ldg(&S->min_x), __ldg(&S->max_x), __ldg(&S->min_y), __ldg(&S->max_y));
}

__device__ __forceinline__ tunable_parameters load_params(const Scene *__restrict__ S)
{
    tunable_parameters P;
    const float4 *src = reinterpret_cast<const float4 *>(&S->P);
    float4 *dst = reinterpret_cast<float4 *>(&P);
#pragma unroll
    for (int k = 0; k < 4; ++k) dst[k] = __ldg(src + k);
    return P;
}

// hash_val (hash.c:35-47): local key = floor(y/s) * size_x + floor(x/s), with
// the IEEE float division of the reference, returned as a global key
// (c_off + local).  x == size_x * s aliases cell (0, gy+1) exactly as in the
// reference.  Keys outside [0, ncells) -- a negative or NaN coordinate, or
// y == size_y * s -- are undefined behaviour there; here they map to the
// scene's "no cell" bucket c_off + ncells.
__device__ __forceinline__ unsigned cell_key(float x, float y, const SG &g)
{
    const bool p2 = g.inv != 0.0f;
    const float fx = floorf(p2 ? __fmul_rn(x, g.inv) : __fdiv_rn(x, g.spacing));
    const float fy = floorf(p2 ? __fmul_rn(y, g.inv) : __fdiv_rn(y, g.spacing));
    if (!(fx >= 0.0f) || !(fy >= 0.0f) || fx > 1073741824.0f || fy > 1073741824.0f)
        return (unsigned)(g.c_off + g.ncells);
    const long long k = (long long)(unsigned)fy * g.size_x + (long long)(unsigned)fx;
    return (unsigned)(g.c_off + (k < g.ncells ? (int)k : g.ncells));
}

// checkVelocity, fluid.c:613-625
__device__ __forceinline__ float clamp5(float v)
{
    return v > 5.0f ? 5.0f : (v < -5.0f ? -5.0f : v);
}

// boundaryConditions, fluid.c:656-744.  Rounded step by step (no fused
// multiply-add) so the per-particle arithmetic equals the reference's.
__device__ __forceinline__ void boundary(float &x, float &y, const tunable_parameters &P,
                                         const float4 &box)
{
    const float cx = P.mover_center_x, cy = P.mover_center_y;
    if (P.mover_type == SPHERE_MOVER) {
        const float radius = __fmul_rn(P.mover_width, 0.5f);
        const float ex = __fsub_rn(x, cx), ey = __fsub_rn(y, cy);
        const float d2 = __fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey));
        if (d2 <= __fmul_rn(radius, radius) && d2 > 0.0f) {
            const float d = __fsqrt_rn(d2);
            const float nx = __fdiv_rn(__fsub_rn(cx, x), d);
            const float ny = __fdiv_rn(__fsub_rn(cy, y), d);
            const float pen = __fsub_rn(radius, d);
            x = __fsub_rn(x, __fmul_rn(pen, nx));
            y = __fsub_rn(y, __fmul_rn(pen, ny));
        }
    } else if (P.mover_type == RECTANGLE_MOVER) {
        const float hw = __fmul_rn(P.mover_width, 0.5f);
        const float hh = __fmul_rn(P.mover_height, 0.5f);
        const float pcx = __fsub_rn(x, cx), pcy = __fsub_rn(y, cy);
        const float dcx = fabsf(pcx), dcy = fabsf(pcy);
        if (dcx < hw && dcy < hh) {
            const float penx = __fsub_rn(hw, dcx), peny = __fsub_rn(hh, dcy);
            if (penx < peny) {
                x = pcx < 0.0f ? __fsub_rn(x, penx) : __fadd_rn(x, penx);
            } else {
                y = pcy < 0.0f ? __fsub_rn(y, peny) : __fadd_rn(y, peny);
            }
        }
    }
    if (x < box.x) x = box.x;
    else if (x > box.y) x = __fsub_rn(box.y, 0.001f);
    if (y < box.z) y = box.z;
    else if (y > box.w) y = __fsub_rn(box.w, 0.001f);
}

// boundaryConditions with the scene's mover and box, read at the call (kept
// out of the registers of the gather loops that precede it).
__device__ __forceinline__ void boundary_of(float &x, float &y, const Scene *__restrict__ S)
{
    tunable_parameters P;
    P.mover_center_x = __ldg(&S->P.mover_center_x);
    P.mover_center_y = __ldg(&S->P.mover_center_y);
    P.mover_width = __ldg(&S->P.mover_width);
    P.mover_height = __ldg(&S->P.mover_height);
    P.mover_type = (char)__ldg(reinterpret_cast<const signed char *>(&S->P.mover_type));
    boundary(x, y, P, load_box(S));
}

// r^2 rounded exactly as the reference computes it (two products, one sum,
// no contraction): the neighbour test r2 <= h2 must agree bit for bit.
__device__ __forceinline__ float dist2(float dx, float dy)
{
    return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
}

// One neighbour's share of (rho, rho_near): ((1 - r/h)^2, (1 - r/h)^3) for
// r/h < 1 (calculate_density, fluid.c:527-539), each term rounded exactly as
// the reference rounds it: r = sqrt(r2) correctly rounded (hash.c:190 takes
// the double root of the float r2 and stores it as a float, which is the
// correctly rounded float root), ratio = r * (1/h) (hash.c:191), w = 1 -
// ratio, then w*w and (w*w)*w.  Near r = h the subtraction w = 1 - ratio
// cancels, so a root that is off by one unit would change a sparse
// particle's density by far more than 1e-5; with the same terms, only the
// order of the (positive) sum differs from the reference.
__device__ __forceinline__ void add_density(float2 &ab, float r2, float h_recip)
{
    const float ratio = __fmul_rn(__fsqrt_rn(r2), h_recip);
    if (ratio < 1.0f) {
        const float omr = __fsub_rn(1.0f, ratio);
        const float omr2 = __fmul_rn(omr, omr);
        ab = __fadd2_rn(ab, make_float2(omr2, __fmul_rn(omr2, omr)));
    }
}

// dist2 of p and q in packed FP32x2 arithmetic (sm_100+): d = q - p per
// component (given mp = -p), r2 = d.x^2 + d.y^2, each operation rounded
// exactly as dist2(p.x - q.x, p.y - q.y) rounds it (the squares of +-dx
// are equal), in three instructions instead of five.
__device__ __forceinline__ float dist2_packed(float2 mp, float2 q, float2 &d)
{
    d = __fadd2_rn(q, mp);
    const float2 s = __fmul2_rn(d, d);
    return __fadd_rn(s.x, s.y);
}

// Checked builds (-DSPH_BOUNDS_CHECK, the stand-in for a memory checker):
// every index that comes from data -- neighbour slots from cell starts and
// hit masks, cell keys, scatter and permute destinations -- is tested
// before its access; a bad one records its kind in a per-translation-unit
// device flag and the access is skipped (no trap, no fault).  Normal builds
// compile the tests away.
enum BoundsKind : unsigned {
    kBadSlot = 1u,      // neighbour slot outside [0, n)
    kBadKey = 2u,       // cell key outside [0, M)
    kBadScatter = 4u,   // scatter / permute destination outside [0, n)
    kBadStart = 8u      // cell start index outside [0, M]
};
#ifdef SPH_BOUNDS_CHECK
static __device__ unsigned g_bounds_flag;
__device__ __forceinline__ bool in_bounds(long long i, long long n, unsigned kind)
{
    if (i >= 0 && i < n) return true;
    atomicOr(&g_bounds_flag, kind);
    return false;
}
// Host side, per translation unit: the flags recorded by its kernels.
static inline unsigned read_bounds_flag()
{
    unsigned v = 0;
    cudaMemcpyFromSymbol(&v, g_bounds_flag, sizeof(v));
    return v;
}
#else
__device__ __forceinline__ bool in_bounds(long long, long long, unsigned) { return true; }
static inline unsigned read_bounds_flag() { return 0u; }
#endif

// Visits the candidate slots of the 3x3 cell stencil around `key` in sorted
// order.  Without bucket overflow, the three cells of a stencil row are
// contiguous in the sorted arrays, so each row is one range
// [start[row+x0], start[row+x1+1]).  With overflow (`capped`), each cell is
// cut to its first max_bucket members in id order, as hash.c:160-165 keeps
// only the first max_bucket_size particles of a bucket.
template <class F>
__device__ __forceinline__ void for_each_candidate(unsigned key, const int *__restrict__ start,
                                                   const SG &g, bool capped, int max_bucket,
                                                   int n, F &&f)
{
    const int lk = (int)key - g.c_off;
    const int gy = lk / g.size_x;
    const int gx = lk - gy * g.size_x;
    const int x0 = gx > 0 ? gx - 1 : 0;
    const int x1 = gx + 1 < g.size_x ? gx + 1 : g.size_x - 1;
    const int y0 = gy > 0 ? gy - 1 : 0;
    const int y1 = gy + 1 < g.size_y ? gy + 1 : g.size_y - 1;
    for (int y = y0; y <= y1; ++y) {
        const int row = g.c_off + y * g.size_x;
        if (!capped) {
            const int a = __ldg(start + row + x0), b = __ldg(start + row + x1 + 1);
            for (int j = a; j < b; ++j)
                if (in_bounds(j, n, kBadSlot)) f(j);
        } else {
            for (int x = x0; x <= x1; ++x) {
                const int a = __ldg(start + row + x);
                const int e = __ldg(start + row + x + 1);
                const int b = e - a > max_bucket ? a + max_bucket : e;
                for (int j = a; j < b; ++j)
                    if (in_bounds(j, n, kBadSlot)) f(j);
            }
        }
    }
}

// A particle takes part in the neighbour search if its key is in its
// scene's grid and, when some cell overflowed, it is among its cell's first
// max_bucket.
__device__ __forceinline__ bool searchable(unsigned key, int slot, const int *__restrict__ start,
                                           const SG &g, bool capped, int max_bucket)
{
    if ((int)key - g.c_off >= g.ncells) return false;
    return !capped || slot - __ldg(start + key) < max_bucket;
}

// The three stencil rows of a cell (slot 0: gy-1, 1: gy, 2: gy+1), each the
// contiguous range [a[r], a[r] + len[r]) of sorted slots (empty outside the
// grid).  Valid when no cell overflowed its bucket cap.
__device__ __forceinline__ void stencil_rows(unsigned key, const int *__restrict__ start,
                                             const SG &g, int (&a)[3], int (&len)[3], int n)
{
    const int lk = (int)key - g.c_off;
    const int gy = lk / g.size_x;
    const int gx = lk - gy * g.size_x;
    const int x0 = gx > 0 ? gx - 1 : 0;
    const int x1 = gx + 1 < g.size_x ? gx + 1 : g.size_x - 1;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const int y = gy + r - 1;
        if (y < 0 || y >= g.size_y) {
            a[r] = 0;
            len[r] = 0;
        } else {
            const int row = g.c_off + y * g.size_x;
            a[r] = __ldg(start + row + x0);
            len[r] = __ldg(start + row + x1 + 1) - a[r];
            // checked builds: a row outside [0, n) is reported and emptied
            if (len[r] > 0 && !(in_bounds(a[r], n, kBadStart) && in_bounds(a[r] + len[r] - 1, n, kBadSlot)))
                len[r] = 0;
        }
    }
}

// ---------------------------------------------------------------------------
// CTA staging of stencil rows in shared memory
// ---------------------------------------------------------------------------

// The particles of a CTA are consecutive in cell order, so the stencil rows
// its threads read are three short, heavily overlapping runs of slots: for
// each row r, the union of the threads' ranges [lo, hi) is one contiguous run
// a little longer than the CTA.  stage_rows copies those three runs of `src`
// into shared memory once (coalesced 8- or 16-byte loads), so that every
// neighbour read of the gather that follows is a shared-memory load instead
// of an L1/L2 round trip.  Each thread passes its own ranges (lo = INT_MAX,
// hi = INT_MIN for a row it does not read); every thread of the CTA must
// call it (it has two CTA barriers).  Returns true when the runs fit `cap`
// elements, in which case slot j of row r is at sm[j + delta[r]] (and, when
// a second array src2 is given, at sm2[j + delta[r]]); otherwise nothing is
// staged and the gather reads global memory as before.
constexpr int kStageWarpsMax = kMaxBlock / 32;

__device__ __forceinline__ int warp_min_i(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = min(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

__device__ __forceinline__ int warp_max_i(int v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = max(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

template <class T, class U = T>
__device__ __forceinline__ bool stage_rows(const int (&lo)[3], const int (&hi)[3],
                                           const T *__restrict__ src, T *sm, int cap,
                                           int (&delta)[3], const U *__restrict__ src2 = nullptr,
                                           U *sm2 = nullptr)
{
    __shared__ int4 s_red[kStageWarpsMax][2];  // per warp: (lo0, lo1, lo2, -), (hi0, hi1, hi2, -)
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    int l[3], h[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        l[r] = warp_min_i(lo[r]);
        h[r] = warp_max_i(hi[r]);
    }
    if (lane == 0) {
        s_red[warp][0] = make_int4(l[0], l[1], l[2], 0);
        s_red[warp][1] = make_int4(h[0], h[1], h[2], 0);
    }
    __syncthreads();
    // every thread combines the per-warp words itself (no second reduction barrier)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        l[r] = INT_MAX;
        h[r] = INT_MIN;
    }
    for (int w = 0; w < nw; ++w) {
        const int4 a = s_red[w][0], b = s_red[w][1];
        l[0] = min(l[0], a.x); l[1] = min(l[1], a.y); l[2] = min(l[2], a.z);
        h[0] = max(h[0], b.x); h[1] = max(h[1], b.y); h[2] = max(h[2], b.z);
    }
    int len[3], off[3], total = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        len[r] = h[r] > l[r] ? h[r] - l[r] : 0;
        off[r] = total;
        total += len[r];
        delta[r] = off[r] - l[r];
    }
    const bool ok = total <= cap;  // the same in every thread of the CTA
    if (ok) {
#pragma unroll
        for (int r = 0; r < 3; ++r)
            for (int k = threadIdx.x; k < len[r]; k += blockDim.x) {
                sm[off[r] + k] = src[l[r] + k];
                if (src2) sm2[off[r] + k] = src2[l[r] + k];
            }
    }
    // also when nothing was staged: s_red and sm are reused by the CTA's
    // next call only after every thread has passed this barrier
    __syncthreads();
    return ok;
}

constexpr int kMaskRow = 64;  // candidates per stencil row recorded in a hit mask

// What a density pass leaves for the relaxation of the same positions, per
// particle: the first slot of each stencil row (x, y, z) and how to walk
// (w): kRowsNone, no neighbours (out of the grid or beyond the bucket cap);
// kRowsMasked, walk the hit masks from those slots; kRowsFull, search the
// whole stencil again (a row longer than kMaskRow, or an overflowing bucket).
// kRowsMasked2: as kRowsMasked for rows of up to 2 kMaskRow candidates, the
// bits of candidates kMaskRow.. in Ctx::maskx (long-row masks).
constexpr int kRowsNone = 0, kRowsMasked = 1, kRowsFull = 2, kRowsMasked2 = 3;

// Visits the set bits of a 64-bit row mask in increasing order with one
// neighbour's data in flight: load(j) for slot base + t of the next bit is
// issued before visit(j, data) runs on the previous one, so the loads of a
// particle's neighbours overlap its arithmetic.  The visiting order is the
// bits' order.
template <class T, class Load, class Visit>
__device__ __forceinline__ void walk_mask(unsigned long long m, int base, int n, Load load,
                                          Visit visit)
{
    unsigned half[2] = {(unsigned)m, (unsigned)(m >> 32)};
    bool have = false;
    int jp = 0;
    T dp{};
#pragma unroll
    for (int hh = 0; hh < 2; ++hh) {
        unsigned b = half[hh];
        while (b) {
            const int j = base + 32 * hh + __ffs(b) - 1;
            b &= b - 1u;
            if (!in_bounds(j, n, kBadSlot)) continue;
            const T d = load(j);
            if (have) visit(jp, dp);
            jp = j;
            dp = d;
            have = true;
        }
    }
    if (have) visit(jp, dp);
}

// The neighbours (r2 <= h2, r2 exact as dist2_packed rounds it) of one
// stencil row of any length, in slot order: per chunk of 64 candidates a hit
// mask from the position filter, then walk_mask over the hits.  For rows too
// long for a stored mask; `self` (a slot or -1) is left out.
template <class T, class Pos, class Load, class Visit>
__device__ __forceinline__ void walk_row_hits(int a, int len, int self, int n, float2 mp, float h2,
                                              Pos pos_of, Load load, Visit visit)
{
    for (int c0 = 0; c0 < len; c0 += 64) {
        const int cl = min(len - c0, 64);
        const int n0 = min(cl, 32);
        unsigned lo = 0u, hi = 0u;
        for (int t = 0; t < n0; ++t) {
            float2 e;
            lo |= (unsigned)(dist2_packed(mp, pos_of(a + c0 + t), e) <= h2) << t;
        }
        for (int t = 32; t < cl; ++t) {
            float2 e;
            hi |= (unsigned)(dist2_packed(mp, pos_of(a + c0 + t), e) <= h2) << (t - 32);
        }
        unsigned long long m = ((unsigned long long)hi << 32) | lo;
        const int rel = self - (a + c0);
        if (rel >= 0 && rel < 64) m &= ~(1ull << rel);
        walk_mask<T>(m, a + c0, n, load, visit);
    }
}

}  // namespace sph
