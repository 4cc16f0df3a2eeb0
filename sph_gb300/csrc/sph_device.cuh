// sph_device.cuh -- device helpers shared by the libsph_cuda kernels.
#pragma once

#include "sph_internal.h"

namespace sph {

// hash_val (hash.c:35-47): key = floor(y/s) * size_x + floor(x/s), with the
// IEEE float division of the reference.  x == size_x * s aliases cell
// (0, gy+1) exactly as in the reference.  Keys outside [0, ncells) -- a
// negative or NaN coordinate, or y == size_y * s -- are undefined behaviour
// there; here they map to the "no cell" bucket `ncells`.
__device__ __forceinline__ unsigned cell_key(float x, float y, const Grid &g)
{
    const float fx = floorf(__fdiv_rn(x, g.spacing));
    const float fy = floorf(__fdiv_rn(y, g.spacing));
    if (!(fx >= 0.0f) || !(fy >= 0.0f) || fx > 1073741824.0f || fy > 1073741824.0f)
        return (unsigned)g.ncells;
    const long long k = (long long)(unsigned)fy * g.size_x + (long long)(unsigned)fx;
    return k < g.ncells ? (unsigned)k : (unsigned)g.ncells;
}

// checkVelocity, fluid.c:613-625
__device__ __forceinline__ float clamp5(float v)
{
    return v > 5.0f ? 5.0f : (v < -5.0f ? -5.0f : v);
}

// boundaryConditions, fluid.c:656-744.  Rounded step by step (no fused
// multiply-add) so the per-particle arithmetic equals the reference's.
__device__ __forceinline__ void boundary(float &x, float &y, const tunable_parameters &P,
                                         const Grid &g)
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
    if (x < g.min_x) x = g.min_x;
    else if (x > g.max_x) x = __fsub_rn(g.max_x, 0.001f);
    if (y < g.min_y) y = g.min_y;
    else if (y > g.max_y) y = __fsub_rn(g.max_y, 0.001f);
}

// r^2 rounded exactly as the reference computes it (two products, one sum,
// no contraction): the neighbour test r2 <= h2 must agree bit for bit.
__device__ __forceinline__ float dist2(float dx, float dy)
{
    return __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
}

// Visits the candidate slots of the 3x3 cell stencil around `key` in sorted
// order.  Without bucket overflow, the three cells of a stencil row are
// contiguous in the sorted arrays, so each row is one range
// [start[row+x0], start[row+x1+1]).  With overflow (`capped`), each cell is
// cut to its first max_bucket members in id order, as hash.c:160-165 keeps
// only the first max_bucket_size particles of a bucket.
template <class F>
__device__ __forceinline__ void for_each_candidate(unsigned key, const int *__restrict__ start,
                                                   const Grid &g, bool capped, F &&f)
{
    const int gy = (int)(key / (unsigned)g.size_x);
    const int gx = (int)key - gy * g.size_x;
    const int x0 = gx > 0 ? gx - 1 : 0;
    const int x1 = gx + 1 < g.size_x ? gx + 1 : g.size_x - 1;
    const int y0 = gy > 0 ? gy - 1 : 0;
    const int y1 = gy + 1 < g.size_y ? gy + 1 : g.size_y - 1;
    for (int y = y0; y <= y1; ++y) {
        const int row = y * g.size_x;
        if (!capped) {
            const int a = __ldg(start + row + x0), b = __ldg(start + row + x1 + 1);
            for (int j = a; j < b; ++j) f(j);
        } else {
            for (int x = x0; x <= x1; ++x) {
                const int a = __ldg(start + row + x);
                const int e = __ldg(start + row + x + 1);
                const int b = e - a > g.max_bucket ? a + g.max_bucket : e;
                for (int j = a; j < b; ++j) f(j);
            }
        }
    }
}

// A particle takes part in the neighbour search if its key is in the grid
// and, when some cell overflowed, it is among its cell's first max_bucket.
__device__ __forceinline__ bool searchable(unsigned key, int slot, const int *__restrict__ start,
                                           const Grid &g, bool capped)
{
    if (key >= (unsigned)g.ncells) return false;
    return !capped || slot - __ldg(start + key) < g.max_bucket;
}

// The three stencil rows of a cell (slot 0: gy-1, 1: gy, 2: gy+1), each the
// contiguous range [a[r], a[r] + len[r]) of sorted slots (empty outside the
// grid).  Valid when no cell overflowed its bucket cap.
__device__ __forceinline__ void stencil_rows(unsigned key, const int *__restrict__ start,
                                             const Grid &g, int (&a)[3], int (&len)[3])
{
    const int gy = (int)(key / (unsigned)g.size_x);
    const int gx = (int)key - gy * g.size_x;
    const int x0 = gx > 0 ? gx - 1 : 0;
    const int x1 = gx + 1 < g.size_x ? gx + 1 : g.size_x - 1;
#pragma unroll
    for (int r = 0; r < 3; ++r) {
        const int y = gy + r - 1;
        if (y < 0 || y >= g.size_y) {
            a[r] = 0;
            len[r] = 0;
        } else {
            const int row = y * g.size_x;
            a[r] = __ldg(start + row + x0);
            len[r] = __ldg(start + row + x1 + 1) - a[r];
        }
    }
}

constexpr int kMaskRow = 64;  // candidates per stencil row recorded in a hit mask

}  // namespace sph
