// sph_init.cu -- on-device scene initialisation (sph_cuda_init_lattice).
//
// The synthetic scenes' lattice blocks are generated on the GPU with the same
// counter-based generator (splitmix64) and the same IEEE double arithmetic
// as the host generator, so a device-initialised scene is bit-identical to
// the host-built one (the reference builds its fluid on the host with
// constructFluidVolume / initParticles, geometry.c:29-67, fluid.c:747-768).
#include <vector>

#include "sph_internal.h"

namespace sph {

struct LatticeDev {
    int n, cols, first;  // particles, per row, first particle index of the block
    int pad;
    double x0, y0, spacing, jitter;
    unsigned long long seed, counter0;
};

__device__ __forceinline__ double splitmix_uniform(unsigned long long seed, unsigned long long c)
{
    unsigned long long z = seed + (c + 1ull) * 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z = z ^ (z >> 31);
    return __dmul_rn((double)(z >> 11), 1.0 / 9007199254740992.0);
}

// One thread per particle; block b of the list covers [first, first + n).
__global__ void k_init_lattice(const LatticeDev *__restrict__ blocks, int nblocks, int n,
                               float2 *__restrict__ pos, float2 *__restrict__ vel,
                               float2 *__restrict__ prev, float4 *__restrict__ xr)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int lo = 0, hi = nblocks - 1;
    while (lo < hi) {  // last block with first <= i
        const int mid = (lo + hi + 1) >> 1;
        if (blocks[mid].first <= i) lo = mid; else hi = mid - 1;
    }
    const LatticeDev b = blocks[lo];
    const long long k = i - b.first;
    const long long row = k / b.cols, col = k - row * b.cols;
    const double u0 = splitmix_uniform(b.seed, b.counter0 + 2ull * (unsigned long long)k);
    const double u1 = splitmix_uniform(b.seed, b.counter0 + 2ull * (unsigned long long)k + 1ull);
    const double jx = __dmul_rn(__dadd_rn(__dmul_rn(u0, 2.0), -1.0), b.jitter);
    const double jy = __dmul_rn(__dadd_rn(__dmul_rn(u1, 2.0), -1.0), b.jitter);
    const double x = __dadd_rn(__dadd_rn(b.x0, __dmul_rn((double)col, b.spacing)), jx);
    const double y = __dadd_rn(__dadd_rn(b.y0, __dmul_rn((double)row, b.spacing)), jy);
    const float fx = __double2float_rn(x), fy = __double2float_rn(y);
    pos[i] = make_float2(fx, fy);
    vel[i] = make_float2(0.0f, 0.0f);
    prev[i] = make_float2(fx, fy);
    xr[i] = make_float4(fx, fy, 0.0f, 0.0f);
}

}  // namespace sph

using namespace sph;

extern "C" int sph_cuda_init_lattice(sph_cuda_t *h, const sph_lattice_block *blocks, int nblocks)
{
    if (!h || (!blocks && nblocks > 0) || nblocks < 0) {
        set_error("sph_cuda_init_lattice: bad arguments");
        return SPH_ERR_INVALID;
    }
    std::vector<LatticeDev> dev(nblocks);
    long long total = 0;
    for (int b = 0; b < nblocks; ++b) {
        const sph_lattice_block &s = blocks[b];
        if (s.n < 0 || s.cols <= 0 || !(s.spacing > 0.0) || !(s.jitter >= 0.0)) {
            set_error("lattice block %d: n %d, cols %d, spacing %g, jitter %g", b, s.n, s.cols,
                      s.spacing, s.jitter);
            return SPH_ERR_INVALID;
        }
        if (h->nscenes > 1 && (nblocks != h->nscenes || s.n != h->scenes[b].n)) {
            set_error("an ensemble of %d scenes takes one block per scene with the scene's count "
                      "(block %d has %d)", h->nscenes, b, s.n);
            return SPH_ERR_INVALID;
        }
        dev[b] = LatticeDev{s.n, s.cols, (int)total, 0, s.x0, s.y0, s.spacing, s.jitter, s.seed,
                            s.counter0};
        total += s.n;
    }
    if (total > h->capacity) {
        set_error("%lld particles above the handle's capacity %d", total, h->capacity);
        return SPH_ERR_INVALID;
    }
    const int n = (int)total;
    int rc = cuda_fail(cudaStreamSynchronize(h->stream), "sync");
    if (rc) return rc;
    if (h->nscenes == 1 && h->scenes[0].n != n) {
        h->scenes[0].n = n;
        rc = cuda_fail(cudaMemcpyAsync(&h->d_scenes[0].n, &h->scenes[0].n, sizeof(int),
                                       cudaMemcpyHostToDevice, h->stream), "scene count");
        if (!rc) {
            const int off[2] = {0, n};
            rc = cuda_fail(cudaMemcpyAsync(h->d_p_off, off, sizeof(off), cudaMemcpyHostToDevice,
                                           h->stream), "slot offsets");
        }
        if (!rc) rc = cuda_fail(cudaStreamSynchronize(h->stream), "sync");
        if (rc) return rc;
    }
    h->n = n;
    if (n > 0) {
        rc = ensure_scratch(h, dev.size() * sizeof(LatticeDev) + 16);
        if (rc) return rc;
        LatticeDev *d = (LatticeDev *)h->d_scratch;
        rc = cuda_fail(cudaMemcpyAsync(d, dev.data(), dev.size() * sizeof(LatticeDev),
                                       cudaMemcpyHostToDevice, h->stream), "blocks");
        if (rc) return rc;
        k_init_lattice<<<(n + kBlock - 1) / kBlock, kBlock, 0, h->stream>>>(
            d, nblocks, n, h->pos_b, h->vel_b, h->prev_c, h->xr_c);
        rc = cuda_fail(cudaGetLastError(), "init lattice");
        if (rc) return rc;
    }
    rc = cuda_fail(cudaMemsetAsync(h->d_state, 0, sizeof(DevState), h->stream), "state");
    if (!rc) rc = upload_soa_device(h, n);
    if (!rc) rc = cuda_fail(cudaStreamSynchronize(h->stream), "sync");
    return rc;
}
