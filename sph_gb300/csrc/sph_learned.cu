// sph_learned.cu -- learned relaxation (include/sph_learned.h).
//
//   k_messages   after the plain density pass: a walk of its hit masks that
//                aggregates the neighbour messages (offsets, velocities,
//                densities and near densities) -> 32-wide BF16 feature rows
//                and neighbour counts
//   k_mlp        fused 2-layer width-128 GELU MLP on the tcgen05 tensor cores:
//                one CTA per SM of four 256-thread pipelines, weights
//                resident in shared memory, FP32 accumulators in tensor memory
//   (k_relax_learned then applies the network's displacement and lists the
//    particles that take the plain relaxation for k_relax_fallback)
//
// Training: a generic tcgen05 GEMM (strided BF16 operands staged in shared
// memory, FP32 accumulation), bias/activation kernels, Adam on FP32 master
// weights; sample collection and the calibration of the error output.
#include <algorithm>
#include <cstddef>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_bf16.h>

#include "sph_device.cuh"
#include "sph_learned.h"
#include "sph_tc.cuh"


namespace sph {

int launch_probe(sph_cuda *h, int which, void *scratch, float2 *out);
size_t probe_scratch_bytes(int n);
int ensure_scratch(sph_cuda *h, size_t bytes);

namespace ml {

constexpr int IN = SPH_LEARNED_IN, HID = SPH_LEARNED_HIDDEN, OUT = SPH_LEARNED_OUT;
constexpr int MAXNB = SPH_LEARNED_MAX_NEIGHBORS;

// Flat parameter layout: W1 [HID x IN], b1, W2 [HID x HID], b2, W3 [OUT x HID], b3.
constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + HID * IN;
constexpr int OFF_W2 = OFF_B1 + HID;
constexpr int OFF_B2 = OFF_W2 + HID * HID;
constexpr int OFF_W3 = OFF_B2 + HID;
constexpr int OFF_B3 = OFF_W3 + OUT * HID;
constexpr int NPARAM = OFF_B3 + OUT;

// Outputs used: 0, 1 displacement / s; 2 predicted density error in % of rho0.

// Derivative of the activation 2 GELU (tanh form).
__device__ __forceinline__ float act_grad(float x)
{
    float t;
    const float u = 0.7978845608f * (x + 0.044715f * x * x * x);
    asm("tanh.approx.f32 %0, %1;" : "=f"(t) : "f"(u));
    return (1.0f + t) + x * (1.0f - t * t) * 0.7978845608f * (1.0f + 0.134145f * x * x);
}

// Output scale of a scene: s = h dt^2 (k + k_near + k_spring).
__device__ __forceinline__ float out_scale(const Scene *__restrict__ S)
{
    const float dt = __ldg(&S->P.time_step), h = __ldg(&S->P.smoothing_radius);
    return h * dt * dt * (__ldg(&S->P.k) + __ldg(&S->P.k_near) + __ldg(&S->P.k_spring));
}

// ---------------------------------------------------------------------------
// message pass
// ---------------------------------------------------------------------------

// A neighbour's record for the message walk: (x, y, rho, rho_near) and its
// previous position.
struct NbRec {
    float4 q;
    float2 qp;
};

// The particle's feature row, from the plain density pass's records (its
// (x, y, rho, rho_near), hit masks and stencil-row record, all in C order):
// messages of the neighbours j with r/h < 1 (self excluded),
// u = unit offset towards the neighbour, w = 1 - r/h,
// dv = (v_j - v_i) dt / h with v = (x - x_prev) / dt:
//   V1 = sum w u, V2 = sum w^2 u, M = sum w, T = sum w u u^T, D = sum w dv,
//   R1 = sum w (rho_j - rest) u, R2 = sum w^2 rho_near_j u
// (the neighbours' densities and near densities, as the relaxation's pair
// term uses them, fluid.c:588-608), with the particle's rho, rho_near,
// neighbour count (r2 <= h2), its scene's stiffness ratios a_k, a_n, a_s
// (k, k_near, k_spring over their sum) and the "own" terms of the
// relaxation formula a_k (rho - rest) V1, a_n rho_near V2, a_s V1.  A
// particle with a coincident neighbour (r2 <= 2e-12, where the reference
// nudges) or in an overflowing bucket gets count 65535: it always takes the
// plain relaxation.  Block 0 resets the step's fallback-list counters.
template <bool LM>
__global__ void __maxnreg__(48)
k_messages(Ctx c, const float4 *__restrict__ xr, const ulonglong2 *__restrict__ mask01,
           const unsigned long long *__restrict__ mask2, const int4 *__restrict__ rows,
           const float2 *__restrict__ prev, const int *__restrict__ start,
           const unsigned *__restrict__ occ_in, __nv_bfloat16 *__restrict__ feat,
           unsigned short *__restrict__ nbcount, unsigned *__restrict__ fb_count)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i == 0 && fb_count) {  // both fallback counters of the step (fb_count, fb_long)
        fb_count[0] = 0u;
        fb_count[1] = 0u;
    }
    if (i >= c.n) return;
    // the particle's streams, requested together
    const float4 me = xr[i];
    const int4 rw = __ldg(rows + i);
    const ulonglong2 m01 = __ldg(mask01 + i);
    const unsigned long long m2 = __ldg(mask2 + i);
    const float2 pp = prev[i];
    const Scene *S = c.scenes + scene_of(c, i);
    const float hh = __ldg(&S->P.smoothing_radius);
    const float h2 = __fmul_rn(hh, hh);
    const float h_recip = __fdiv_rn(1.0f, hh);
    const float dt = __ldg(&S->P.time_step);
    const float inv_dt = 1.0f / dt;
    const float vscale = dt * h_recip;
    const float rest = __ldg(&S->P.rest_density);
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    const float2 p = make_float2(me.x, me.y);
    const float vix = (p.x - pp.x) * inv_dt, viy = (p.y - pp.y) * inv_dt;
    const float2 mp = make_float2(-p.x, -p.y);
    float2 V1 = make_float2(0.0f, 0.0f), V2 = V1, Tdiag = V1, Dsum = V1, R1 = V1, R2 = V1;
    float Ms = 0.0f, Txy = 0.0f;
    int count = 0;
    bool degenerate = capped;
    // one neighbour (r2 <= h2 known, never the particle itself)
    auto visit = [&](int, const NbRec &d) {
        float2 e;  // q - p
        const float r2 = dist2_packed(mp, make_float2(d.q.x, d.q.y), e);
        const float rinv = rsqrtf(r2);
        const float ratio = r2 * rinv * h_recip;
        ++count;
        degenerate |= r2 <= 2e-12f;
        if (ratio < 1.0f) {
            const float omr = 1.0f - ratio;
            const float omr2 = omr * omr;
            // message sums in packed FP32x2 arithmetic
            const float2 u = __fmul2_rn(e, make_float2(rinv, rinv));
            const float2 w2 = make_float2(omr, omr);
            const float2 wu = __fmul2_rn(w2, u);
            V1 = __fadd2_rn(V1, wu);
            V2 = __ffma2_rn(make_float2(omr2, omr2), u, V2);
            Ms += omr;
            Tdiag = __ffma2_rn(wu, u, Tdiag);
            Txy += wu.x * u.y;
            const float pr = d.q.z - rest, prn = omr2 * d.q.w;
            R1 = __ffma2_rn(make_float2(pr, pr), wu, R1);
            R2 = __ffma2_rn(make_float2(prn, prn), u, R2);
            // sum w (x_j - x_prev_j); the velocities follow at the end
            Dsum = __ffma2_rn(w2, __fadd2_rn(make_float2(d.q.x, d.q.y),
                                             make_float2(-d.qp.x, -d.qp.y)), Dsum);
        }
    };
    auto load = [&](int j) {
        NbRec d;
        d.q = __ldg(xr + j);
        d.qp = __ldg(prev + j);
        return d;
    };
    if (!capped && rw.w == kRowsMasked) {
        const int ra[3] = {rw.x, rw.y, rw.z};
        const unsigned long long mm[3] = {m01.x, m01.y, m2};
#pragma unroll
        for (int r = 0; r < 3; ++r) walk_mask<NbRec>(mm[r], ra[r], c.n, load, visit);
    } else if (LM && !capped && rw.w == kRowsMasked2) {
        // long-row masks: each row's two masks in slot order
        const int ra[3] = {rw.x, rw.y, rw.z};
        const unsigned long long mm[3] = {m01.x, m01.y, m2};
        const unsigned long long *mx = c.maskx + 3 * (size_t)i;
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            walk_mask<NbRec>(mm[r], ra[r], c.n, load, visit);
            walk_mask<NbRec>(__ldg(mx + r), ra[r] + kMaskRow, c.n, load, visit);
        }
    } else if (!capped && rw.w == kRowsFull) {
        // a stencil row longer than a hit mask: the whole stencil, in slot
        // order
        const SG g = load_grid(S);
        const unsigned key = cell_key(p.x, p.y, g);
        for_each_candidate(key, start, g, false, c.max_bucket, c.n, [&](int j) {
            if (j == i) return;
            const NbRec d = load(j);
            float2 e;
            if (dist2_packed(mp, make_float2(d.q.x, d.q.y), e) > h2) return;
            visit(j, d);
        });
    }
    nbcount[i] = degenerate ? (unsigned short)65535 : (unsigned short)(count < 65534 ? count : 65534);
    const float a = me.z, b = me.w;
    const float V1x = V1.x, V1y = V1.y, V2x = V2.x, V2y = V2.y;
    const float Txx = Tdiag.x, Tyy = Tdiag.y;
    // sum w (v_j - v_i) = (sum w (x_j - x_prev_j)) / dt - v_i sum w
    const float Dx = Dsum.x * inv_dt - vix * Ms, Dy = Dsum.y * inv_dt - viy * Ms;

    const float k = __ldg(&S->P.k), kn = __ldg(&S->P.k_near), ks = __ldg(&S->P.k_spring);
    const float ksum = k + kn + ks;
    const float ak = k / ksum, an = kn / ksum, as = ks / ksum;
    const float ds = vscale * 2.5f;
    float f[IN];
    f[0] = a * 0.25f;
    f[1] = b * 0.5f;
    f[2] = V1x * 0.25f;
    f[3] = V1y * 0.25f;
    f[4] = V2x * 0.5f;
    f[5] = V2y * 0.5f;
    f[6] = Ms * 0.125f;
    f[7] = (float)min(count, MAXNB) * (1.0f / MAXNB);
    f[8] = Dx * ds;
    f[9] = Dy * ds;
    f[10] = Txx * 0.25f;
    f[11] = Txy * 0.25f;
    f[12] = Tyy * 0.25f;
    f[13] = ak;
    f[14] = an;
    f[15] = as;
    f[16] = rest * 0.25f;
    f[17] = ak * (a - rest) * V1x * 0.25f;
    f[18] = ak * (a - rest) * V1y * 0.25f;
    f[19] = an * b * V2x * 0.5f;
    f[20] = an * b * V2y * 0.5f;
    f[21] = as * V1x * 0.5f;
    f[22] = as * V1y * 0.5f;
    f[23] = ak * R1.x * 0.25f;
    f[24] = ak * R1.y * 0.25f;
    f[25] = an * R2.x * 0.5f;
    f[26] = an * R2.y * 0.5f;
#pragma unroll
    for (int e = 27; e < IN - 1; ++e) f[e] = 0.0f;
    f[IN - 1] = 1.0f;  // constant input: the first layer's bias
    uint4 *row = reinterpret_cast<uint4 *>(feat + (size_t)i * IN);
#pragma unroll
    for (int q = 0; q < IN / 8; ++q) {
        uint4 v;
        asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(v.x) : "f"(f[8 * q + 1]), "f"(f[8 * q + 0]));
        asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(v.y) : "f"(f[8 * q + 3]), "f"(f[8 * q + 2]));
        asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(v.z) : "f"(f[8 * q + 5]), "f"(f[8 * q + 4]));
        asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(v.w) : "f"(f[8 * q + 7]), "f"(f[8 * q + 6]));
        row[q] = v;
    }
}

// ---------------------------------------------------------------------------
// fused MLP inference (tcgen05)
// ---------------------------------------------------------------------------

// Inference layout.  The first layer's bias is folded into the weight of
// the constant feature 31 (= 1); the second layer's bias enters as one more
// K = 16 MMA of a ones column against the bias column; the activation is
// 2 GELU (the factor 2 is absorbed by the weights that follow it, in
// training and inference alike).
struct alignas(128) MlpWeights {
    unsigned char w1[HID * IN * 2];    // W1, column 31 + b1
    unsigned char w2[HID * HID * 2];   // W2
    unsigned char w2b[HID * 16 * 2];   // column 0 = b2 (BF16), the rest 0
    unsigned char w3[OUT * HID * 2];   // W3
    unsigned char ones[128 * 16 * 2];  // column 0 = 1, the rest 0
    float b3[OUT];
    uint32_t taddr;
};

struct alignas(128) MlpPipe {
    unsigned char x[128 * IN * 2];
    unsigned char hbuf[128 * HID * 2];
    uint64_t mbar;
};

// One CTA per SM of four independent pipelines of 256 threads (8 warps);
// pipeline p owns TMEM columns [128 p, 128 p + 128) (all three layers of a
// tile accumulate there in turn), its own operand tiles, mbarrier and named
// barrier.  The pipelines share the weights; their tensor-core work and
// epilogues interleave.
constexpr int kPipes = 4;
constexpr int kPipeThreads = 256;
constexpr int kMlpThreads = kPipes * kPipeThreads;
constexpr uint32_t kTmemCols = 128 * kPipes;

struct MlpSmem {
    MlpWeights w;
    MlpPipe pipe[kPipes];
};
// operand tiles start on 128-byte boundaries (descriptors and 16-byte stores)
static_assert(offsetof(MlpWeights, w2) % 128 == 0 && offsetof(MlpWeights, w2b) % 128 == 0 &&
                  offsetof(MlpWeights, w3) % 128 == 0 && offsetof(MlpWeights, ones) % 128 == 0,
              "weight tiles aligned");
static_assert(offsetof(MlpSmem, pipe) % 128 == 0 && sizeof(MlpPipe) % 128 == 0 &&
                  offsetof(MlpPipe, hbuf) % 128 == 0,
              "pipeline tiles aligned");
static_assert(sizeof(MlpSmem) + 1024 <= 227 * 1024, "fits the shared memory of one CTA");

__device__ __forceinline__ void stage_weights(MlpWeights &s, const __nv_bfloat16 *__restrict__ w,
                                              const float *__restrict__ wf)
{
    const int t = threadIdx.x;
    for (int e = t; e < HID * IN; e += blockDim.x) {
        const int r = e / IN, k = e % IN;
        const __nv_bfloat16 v =
            k == IN - 1 ? __float2bfloat16(wf[OFF_W1 + e] + wf[OFF_B1 + r]) : w[OFF_W1 + e];
        *reinterpret_cast<__nv_bfloat16 *>(s.w1 + tc::kmajor_offset(r, k, IN)) = v;
    }
    for (int e = t; e < HID * HID; e += blockDim.x) {
        const int r = e / HID, k = e % HID;
        *reinterpret_cast<__nv_bfloat16 *>(s.w2 + tc::kmajor_offset(r, k, HID)) = w[OFF_W2 + e];
    }
    for (int e = t; e < HID * 16; e += blockDim.x) {
        const int r = e / 16, k = e % 16;
        *reinterpret_cast<__nv_bfloat16 *>(s.w2b + tc::kmajor_offset(r, k, 16)) =
            __float2bfloat16(k == 0 ? wf[OFF_B2 + r] : 0.0f);
        *reinterpret_cast<__nv_bfloat16 *>(s.ones + tc::kmajor_offset(r, k, 16)) =
            __float2bfloat16(k == 0 ? 1.0f : 0.0f);
    }
    for (int e = t; e < OUT * HID; e += blockDim.x) {
        const int r = e / HID, k = e % HID;
        *reinterpret_cast<__nv_bfloat16 *>(s.w3 + tc::kmajor_offset(r, k, HID)) = w[OFF_W3 + e];
    }
    for (int e = t; e < OUT; e += blockDim.x) s.b3[e] = wf[OFF_B3 + e];
}

// Epilogue of a hidden layer in a pipeline: warp w (0..7 within it) takes
// TMEM lanes 32 (w % 4) .. + 31 (one row per thread) and columns
// 64 (w / 4) .. + 63 of the pipeline's accumulator; activation in BF16 into
// the K-major activation tile (16-byte stores).
__device__ __forceinline__ void hidden_epilogue(unsigned char *hbuf, uint32_t tacc, int tp)
{
    const int w = tp >> 5;
    const int row = 32 * (w & 3) + (tp & 31);
    const int c0 = 64 * (w >> 2);
    const uint32_t lane = (uint32_t)(32 * (w & 3)) << 16;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
        const int c = c0 + 32 * h;
        float v[32];
        tc::tmem_ld32(tacc + lane + (uint32_t)c, v);
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            uint4 o;
            o.x = tc::act_bf16x2(v[8 * q + 0], v[8 * q + 1]);
            o.y = tc::act_bf16x2(v[8 * q + 2], v[8 * q + 3]);
            o.z = tc::act_bf16x2(v[8 * q + 4], v[8 * q + 5]);
            o.w = tc::act_bf16x2(v[8 * q + 6], v[8 * q + 7]);
            *reinterpret_cast<uint4 *>(hbuf + tc::kmajor_offset(row, c + 8 * q, HID)) = o;
        }
    }
}

// Half a feature row (16 BF16 = 32 bytes) of row tile*128 + (tp >> 1).
__device__ __forceinline__ void load_feat(const __nv_bfloat16 *__restrict__ feat, int n, int tile,
                                          int tp, uint4 &a, uint4 &b)
{
    const int gi = tile * 128 + (tp >> 1);
    if (gi < n) {
        const uint4 *src = reinterpret_cast<const uint4 *>(feat + (size_t)gi * IN) + 2 * (tp & 1);
        a = __ldcs(src);
        b = __ldcs(src + 1);
    } else {
        a = make_uint4(0, 0, 0, 0);
        b = a;
    }
}

__device__ __forceinline__ void store_feat(unsigned char *x, int tp, const uint4 &a, const uint4 &b)
{
    const int r = tp >> 1, k = 16 * (tp & 1);
    *reinterpret_cast<uint4 *>(x + tc::kmajor_offset(r, k, IN)) = a;
    *reinterpret_cast<uint4 *>(x + tc::kmajor_offset(r, k + 8, IN)) = b;
}

// out[i] = (y0, y1, y2, 0) for n feature rows; tiles of 128 rows, pipeline
// p of CTA b takes tiles (b kPipes + p) + k gridDim.x kPipes.  The next
// tile's features are fetched while the current one runs.
__global__ void __launch_bounds__(kMlpThreads, 1)
k_mlp(int n, const __nv_bfloat16 *__restrict__ feat, const __nv_bfloat16 *__restrict__ wbf,
      const float *__restrict__ wf, float4 *__restrict__ out, unsigned *__restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    MlpSmem &S = *reinterpret_cast<MlpSmem *>(smem_raw);
    const int t = threadIdx.x;
    const int p = t / kPipeThreads, tp = t % kPipeThreads, w = tp >> 5;
    MlpPipe &P = S.pipe[p];
    const int bar = 1 + p;
    if (t < 32) {
        tc::tmem_alloc(&S.w.taddr, kTmemCols);
        tc::tmem_relinquish();
    }
    if (tp == 0) {
        tc::mbar_init(&P.mbar, 1);
        tc::mbar_fence_init();
    }
    stage_weights(S.w, wbf, wf);
    const int ntiles = (n + 127) / 128;
    const int stride = gridDim.x * kPipes;
    int tile = blockIdx.x * kPipes + p;
    {
        uint4 a, b;
        load_feat(feat, n, tile, tp, a, b);
        store_feat(P.x, tp, a, b);
    }
    tc::fence_async_smem();
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tacc = S.w.taddr + (uint32_t)(128 * p);
    const uint32_t sx = tc::smem_u32(P.x), sh = tc::smem_u32(P.hbuf);
    uint32_t phase = 0;
    bool ok = true;
    // `ok` stays uniform across the pipeline (every barrier after a wait is
    // a vote), so a wait that gives up ends its loop in all its threads.
    for (; tile < ntiles; tile += stride) {
        // layer 1: x (128 x 32) . W1'^T
        if (tp == 0) {
            tc::mma_tile(tacc, sx, tc::smem_u32(S.w.w1), HID, IN, false);
            tc::mma_commit(&P.mbar);
        }
        // the next tile's features, loaded now and stored at the end of this
        // tile: their DRAM latency hides behind the whole tile, not behind
        // layer 1 alone (6% off the kernel)
        uint4 na, nb;
        load_feat(feat, n, tile + stride, tp, na, nb);
        bool done = tc::mbar_wait(&P.mbar, phase);
        phase ^= 1u;
        tc::fence_after_sync();
        hidden_epilogue(P.hbuf, tacc, tp);
        tc::fence_async_smem();
        tc::fence_before_sync();
        ok = tc::named_sync_and(bar, kPipeThreads, done);
        tc::fence_after_sync();
        if (!ok) break;
        // layer 2: h1 (128 x 128) . W2^T + 1 . b2^T
        if (tp == 0) {
            tc::mma_tile(tacc, sh, tc::smem_u32(S.w.w2), HID, HID, false);
            tc::mma_tile(tacc, tc::smem_u32(S.w.ones), tc::smem_u32(S.w.w2b), HID, 16, true);
            tc::mma_commit(&P.mbar);
        }
        done = tc::mbar_wait(&P.mbar, phase);
        phase ^= 1u;
        tc::fence_before_sync();
        ok = tc::named_sync_and(bar, kPipeThreads, done);  // hbuf consumed before it is rewritten
        tc::fence_after_sync();
        if (!ok) break;
        hidden_epilogue(P.hbuf, tacc, tp);
        tc::fence_async_smem();
        tc::fence_before_sync();
        tc::named_sync(bar, kPipeThreads);
        tc::fence_after_sync();
        // layer 3: h2 (128 x 128) . W3^T -> columns [0, 16)
        if (tp == 0) {
            tc::mma_tile(tacc, sh, tc::smem_u32(S.w.w3), OUT, HID, false);
            tc::mma_commit(&P.mbar);
        }
        done = tc::mbar_wait(&P.mbar, phase);
        phase ^= 1u;
        tc::fence_after_sync();
        if (w < 4) {
            float v[16];
            tc::tmem_ld16(tacc + ((uint32_t)(32 * w) << 16), v);
            const int gi = tile * 128 + 32 * w + (tp & 31);
            if (gi < n && done)
                __stcs(out + gi, make_float4(v[0] + S.w.b3[0], v[1] + S.w.b3[1], v[2] + S.w.b3[2], 0.0f));
        }
        store_feat(P.x, tp, na, nb);  // layer 1 consumed x long ago
        tc::fence_async_smem();
        tc::fence_before_sync();
        ok = tc::named_sync_and(bar, kPipeThreads, done);  // read before layer 1 reuses it
        tc::fence_after_sync();
        if (!ok) break;
    }
    if (!ok && tp == 0) atomicAdd(err, 1u);
    tc::fence_before_sync();
    __syncthreads();
    if (t < 32) tc::tmem_dealloc(S.w.taddr, kTmemCols);
}

// ---------------------------------------------------------------------------
// generic tcgen05 GEMM for training
// ---------------------------------------------------------------------------

// C[m][n] (ldc) = sum_k A(m, k) B(n, k), A(m, k) = A[m * sam + k * sak],
// B(n, k) = B[n * sbn + k * sbk] (BF16), FP32 result; M, N, K any sizes
// (zero padded to the 128 x BN x 64 tiles).  One 128-thread CTA per tile.
constexpr int kGemmK = 64;

struct GemmSmem {
    unsigned char a[128 * kGemmK * 2];
    unsigned char b[128 * kGemmK * 2];
    uint64_t mbar;
    uint32_t taddr;
};

__global__ void __launch_bounds__(128, 1)
k_gemm(int M, int N, int K, const __nv_bfloat16 *__restrict__ A, long long sam, long long sak,
       const __nv_bfloat16 *__restrict__ B, long long sbn, long long sbk, float *__restrict__ C,
       long long ldc, int BN, unsigned *__restrict__ err)
{
    extern __shared__ __align__(1024) unsigned char smem_raw[];
    GemmSmem &s = *reinterpret_cast<GemmSmem *>(smem_raw);
    const int t = threadIdx.x, w = t >> 5;
    const int m0 = blockIdx.x * 128, n0 = blockIdx.y * BN;
    if (w == 0) {
        tc::tmem_alloc(&s.taddr, 128);
        tc::tmem_relinquish();
    }
    if (t == 0) {
        tc::mbar_init(&s.mbar, 1);
        tc::mbar_fence_init();
    }
    tc::fence_before_sync();
    __syncthreads();
    tc::fence_after_sync();
    const uint32_t tm = s.taddr;
    uint32_t phase = 0;
    bool ok = true;
    const __nv_bfloat16 zero = __float2bfloat16(0.0f);
    for (int k0 = 0; k0 < K; k0 += kGemmK) {
        for (int e = t; e < 128 * kGemmK; e += 128) {
            const int r = e / kGemmK, k = e % kGemmK;
            const int gm = m0 + r, gk = k0 + k;
            *reinterpret_cast<__nv_bfloat16 *>(s.a + tc::kmajor_offset(r, k, kGemmK)) =
                (gm < M && gk < K) ? A[gm * sam + gk * sak] : zero;
            if (r < BN) {
                const int gn = n0 + r;
                *reinterpret_cast<__nv_bfloat16 *>(s.b + tc::kmajor_offset(r, k, kGemmK)) =
                    (gn < N && gk < K) ? B[gn * sbn + gk * sbk] : zero;
            }
        }
        tc::fence_async_smem();
        tc::fence_before_sync();
        __syncthreads();
        tc::fence_after_sync();
        if (t == 0) {
            tc::mma_tile(tm, tc::smem_u32(s.a), tc::smem_u32(s.b), BN, kGemmK, k0 > 0);
            tc::mma_commit(&s.mbar);
        }
        const bool done = tc::mbar_wait(&s.mbar, phase);
        phase ^= 1u;
        tc::fence_before_sync();
        ok = __syncthreads_and(done) != 0;  // uniform: the smem tiles are free again
        tc::fence_after_sync();
        if (!ok) break;
    }
    if (ok) {
        const int row = 32 * (w & 3) + (t & 31);
        const uint32_t lane = (uint32_t)(32 * (w & 3)) << 16;
        for (int c = 0; c < BN; c += 16) {
            float v[16];
            tc::tmem_ld16(tm + lane + (uint32_t)c, v);
            const int gm = m0 + row;
            if (gm < M)
                for (int e = 0; e < 16; ++e) {
                    const int gn = n0 + c + e;
                    if (gn < N) C[gm * ldc + gn] = v[e];
                }
        }
    } else if (t == 0) {
        atomicAdd(err, 1u);
    }
    tc::fence_before_sync();
    __syncthreads();
    if (w == 0) tc::tmem_dealloc(tm, 128);
}

// ---------------------------------------------------------------------------
// elementwise training kernels
// ---------------------------------------------------------------------------

// Z (rows x cols, FP32 pre-activation without bias) -> Zb = Z + bf16(b)
// (kept), H = act(Zb) = 2 GELU(Zb) in BF16, computed as the inference kernel
// computes it (which adds the bias in BF16 through the tensor cores).  One
// thread per pair of columns (cols even).
__global__ void k_bias_act(int rows, int cols, float *__restrict__ Z, const float *__restrict__ b,
                           __nv_bfloat16 *__restrict__ H)
{
    const long long e = 2 * ((long long)blockIdx.x * blockDim.x + threadIdx.x);
    if (e >= (long long)rows * cols) return;
    const int c = (int)(e % cols);
    const float z0 = Z[e] + __bfloat162float(__float2bfloat16(b[c]));
    const float z1 = Z[e + 1] + __bfloat162float(__float2bfloat16(b[c + 1]));
    Z[e] = z0;
    Z[e + 1] = z1;
    *reinterpret_cast<uint32_t *>(H + e) = tc::act_bf16x2(z0, z1);
}

// Y += b3; dY = mask * 2 (Y - T) / rows (BF16); the squared error is added to *loss.
__global__ void k_out_grad(int rows, float *__restrict__ Y, const float *__restrict__ b3,
                           const float4 *__restrict__ T, int cmask, __nv_bfloat16 *__restrict__ dY,
                           double *__restrict__ loss)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    double l = 0.0;
    if (r < rows) {
        const float4 tt = T[r];
        const float tv[4] = {tt.x, tt.y, tt.z, tt.w};
        for (int c = 0; c < OUT; ++c) {
            const float y = Y[r * OUT + c] + b3[c];
            Y[r * OUT + c] = y;
            float g = 0.0f;
            if (c < 3 && ((cmask >> c) & 1)) {
                const float d = y - tv[c];
                l += (double)d * d;
                g = 2.0f * d / (float)rows;
            }
            dY[r * OUT + c] = __float2bfloat16(g);
        }
    }
    // block reduction of the loss
    __shared__ double sh[32];
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if ((threadIdx.x & 31) == 0) sh[threadIdx.x >> 5] = l;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
        atomicAdd(loss, s);
    }
}

// dZ = dH * act'(Zb) (BF16 out).
__global__ void k_act_back(int rows, int cols, const float *__restrict__ dH,
                            const float *__restrict__ Zb, __nv_bfloat16 *__restrict__ dZ)
{
    const long long e = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= (long long)rows * cols) return;
    dZ[e] = __float2bfloat16(dH[e] * act_grad(Zb[e]));
}

// Column sums of a BF16 matrix (bias gradients), one thread per column.
__global__ void k_colsum(int rows, int cols, const __nv_bfloat16 *__restrict__ D,
                         float *__restrict__ out)
{
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= cols) return;
    float s = 0.0f;
    for (int r = 0; r < rows; ++r) s += __bfloat162float(D[(size_t)r * cols + c]);
    out[c] = s;
}

// Adam on the FP32 master weights (where `mask` is set), then BF16 copies.
__global__ void k_adam(int n, float *__restrict__ w, const float *__restrict__ g,
                       float *__restrict__ m, float *__restrict__ v, const unsigned char *mask,
                       float lr, float b1t, float b2t, __nv_bfloat16 *__restrict__ wbf)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e >= n) return;
    if (!mask || mask[e]) {
        const float gg = g[e];
        const float mm = 0.9f * m[e] + 0.1f * gg;
        const float vv = 0.999f * v[e] + 0.001f * gg * gg;
        m[e] = mm;
        v[e] = vv;
        w[e] -= lr * (mm / (1.0f - b1t)) / (sqrtf(vv / (1.0f - b2t)) + 1e-8f);
    }
    wbf[e] = __float2bfloat16(w[e]);
}

// Gathers a batch of rows of the sample set.
__global__ void k_gather_rows(int rows, const int *__restrict__ idx,
                              const __nv_bfloat16 *__restrict__ X, const float4 *__restrict__ T,
                              __nv_bfloat16 *__restrict__ Xb, float4 *__restrict__ Tb)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const int s = idx[r];
    const uint4 *src = reinterpret_cast<const uint4 *>(X + (size_t)s * IN);
    uint4 *dst = reinterpret_cast<uint4 *>(Xb + (size_t)r * IN);
#pragma unroll
    for (int q = 0; q < IN / 8; ++q) dst[q] = src[q];
    Tb[r] = T[s];
}

__global__ void k_f32_to_bf16(int n, const float *__restrict__ in, __nv_bfloat16 *__restrict__ out)
{
    const int e = blockIdx.x * blockDim.x + threadIdx.x;
    if (e < n) out[e] = __float2bfloat16(in[e]);
}

// ---------------------------------------------------------------------------
// sample collection and calibration
// ---------------------------------------------------------------------------

// Appends the rows of sorted slots sel[0..rows): features and targets
// (plain displacement / s, error 0).
__global__ void k_append(Ctx c, int rows, const int *__restrict__ sel,
                         const __nv_bfloat16 *__restrict__ feat, const float2 *__restrict__ disp,
                         __nv_bfloat16 *__restrict__ X, float4 *__restrict__ T,
                         int *__restrict__ slot)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const int i = sel[r];
    const float s = out_scale(c.scenes + scene_of(c, i));
    const uint4 *src = reinterpret_cast<const uint4 *>(feat + (size_t)i * IN);
    uint4 *dst = reinterpret_cast<uint4 *>(X + (size_t)r * IN);
#pragma unroll
    for (int q = 0; q < IN / 8; ++q) dst[q] = src[q];
    const float2 d = disp[i];
    T[r] = make_float4(d.x / s, d.y / s, 0.0f, 1.0f);
    slot[r] = i;
}

// Density at displaced positions pos + disp (sorted order) over the stencil
// of the particle's undisplaced cell: the density each particle ends the
// relaxation with under a displacement field.
__global__ void k_density_displaced(Ctx c, const float2 *__restrict__ pos,
                                    const float2 *__restrict__ disp, const int *__restrict__ start,
                                    const unsigned *__restrict__ occ_in, float *__restrict__ rho)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const Scene *S = c.scenes + scene_of(c, i);
    const SG g = load_grid(S);
    const float hh = __ldg(&S->P.smoothing_radius), h2 = hh * hh, h_recip = 1.0f / hh;
    const bool capped = *occ_in > (unsigned)c.max_bucket;
    const float2 p0 = pos[i], dp = disp[i];
    const float px = p0.x + dp.x, py = p0.y + dp.y;
    const unsigned key = cell_key(p0.x, p0.y, g);
    float a = 0.0f;
    if (searchable(key, i, start, g, capped, c.max_bucket)) {
        for_each_candidate(key, start, g, capped, c.max_bucket, c.n, [&](int j) {
            if (j == i) return;
            const float2 q = pos[j], dq = disp[j];
            const float r2 = dist2(px - (q.x + dq.x), py - (q.y + dq.y));
            if (r2 > h2) return;
            const float ratio = (r2 > 0.0f ? r2 * rsqrtf(r2) : 0.0f) * h_recip;
            if (ratio < 1.0f) a += (1.0f - ratio) * (1.0f - ratio);
        });
    }
    rho[i] = a;
}

// Network displacement (sorted order) from its outputs.
__global__ void k_net_disp(Ctx c, const float4 *__restrict__ y, float2 *__restrict__ disp)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.n) return;
    const float s = out_scale(c.scenes + scene_of(c, i));
    const float4 v = y[i];
    disp[i] = make_float2(v.x * s, v.y * s);
}

// Error targets of rows [0, rows): |rho_net - rho_plain| in percent of the
// rest density, clipped at 10.
__global__ void k_err_targets(Ctx c, const float *__restrict__ rho_net,
                              const float *__restrict__ rho_plain, const int *__restrict__ slot,
                              int rows, float4 *__restrict__ T)
{
    const int r = blockIdx.x * blockDim.x + threadIdx.x;
    if (r >= rows) return;
    const int i = slot[r];
    const float rest = __ldg(&c.scenes[scene_of(c, i)].P.rest_density);
    const float e = fabsf(rho_net[i] - rho_plain[i]) / rest * 100.0f;
    float4 t = T[r];
    t.z = fminf(e, 10.0f);
    T[r] = t;
}

// Self-test of the bounded tensor-core wait: waits on an mbarrier that no
// operation arrives at; the wait gives up after its poll limit and the
// kernel records that (*gave_up = 1) instead of hanging.
__global__ void k_wait_selftest(unsigned *__restrict__ gave_up)
{
    __shared__ uint64_t mbar;
    if (threadIdx.x == 0) {
        tc::mbar_init(&mbar, 1);
        tc::mbar_fence_init();
    }
    __syncthreads();
    const bool done = tc::mbar_wait(&mbar, 0);
    if (threadIdx.x == 0) *gave_up = done ? 0u : 1u;
}

}  // namespace ml

// The learned-relaxation model.
struct LearnedModel {
    float *w = nullptr;         // FP32 master weights (device)
    float *g = nullptr, *m = nullptr, *v = nullptr;
    __nv_bfloat16 *wbf = nullptr;
    int adam_t = 0;
    // samples
    __nv_bfloat16 *X = nullptr;
    float4 *T = nullptr;
    int *slot = nullptr;  // sorted slot of each sample of the last collection (calibration)
    int nsamples = 0, cap = 0;
    unsigned calls = 0;
    unsigned *d_err = nullptr;
    cudaStream_t stream = nullptr;
    unsigned long long seed = 0;
};

}  // namespace sph

struct sph_learned : sph::LearnedModel {};

namespace sph {
namespace {

#define LTRY(expr)                          \
    do {                                    \
        const int _rc = (expr);             \
        if (_rc != SPH_OK) return _rc;      \
    } while (0)
#define LCUDA(call) LTRY(cuda_fail((call), #call))

inline int nblk(long long n, int bs = 256) { return (int)((n + bs - 1) / bs); }

size_t mlp_smem() { return sizeof(ml::MlpSmem) + 1024; }
// At least 60 KB, so that at most three GEMM CTAs (3 x 128 TMEM columns)
// share an SM.
size_t gemm_smem() { return std::max(sizeof(ml::GemmSmem) + 1024, (size_t)60 * 1024); }

int configure_kernels()
{
    static bool done = false;
    if (done) return SPH_OK;
    LCUDA(cudaFuncSetAttribute(ml::k_mlp, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_smem()));
    LCUDA(cudaFuncSetAttribute(ml::k_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gemm_smem()));
    done = true;
    return SPH_OK;
}

// Generic GEMM launch: C = A . B^T with strided operands.
int gemm(cudaStream_t st, int M, int N, int K, const __nv_bfloat16 *A, long long sam, long long sak,
         const __nv_bfloat16 *B, long long sbn, long long sbk, float *C, long long ldc, unsigned *err)
{
    const int BN = N >= 128 ? 128 : (N <= 16 ? 16 : (N <= 32 ? 32 : (N <= 64 ? 64 : 128)));
    dim3 grid((M + 127) / 128, (N + BN - 1) / BN);
    ml::k_gemm<<<grid, 128, gemm_smem(), st>>>(M, N, K, A, sam, sak, B, sbn, sbk, C, ldc, BN, err);
    return cuda_fail(cudaGetLastError(), "gemm launch");
}

int check_err(LearnedModel *l)
{
    unsigned e = 0;
    LCUDA(cudaMemcpyAsync(&e, l->d_err, sizeof(e), cudaMemcpyDeviceToHost, l->stream));
    LCUDA(cudaStreamSynchronize(l->stream));
    if (e) {
        set_error("tensor-core wait gave up %u times (mbarrier not completed)", e);
        return SPH_ERR_CUDA;
    }
    return SPH_OK;
}

int num_sms()
{
    int dev = 0, sms = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    return sms > 0 ? sms : 1;
}

// Training buffers for one batch size.
struct TrainBufs {
    int B = 0;
    __nv_bfloat16 *Xb = nullptr, *H1 = nullptr, *H2 = nullptr, *dY = nullptr, *dZ2 = nullptr,
                  *dZ1 = nullptr;
    float4 *Tb = nullptr;
    float *Z1 = nullptr, *Z2 = nullptr, *Y = nullptr, *dH2 = nullptr, *dH1 = nullptr;
    int *idx = nullptr;
    double *loss = nullptr;
    unsigned char *mask = nullptr;
    std::vector<void *> all;
    template <class T>
    int alloc(T **p, size_t n)
    {
        if (cudaMalloc((void **)p, n * sizeof(T)) != cudaSuccess) {
            set_error("cudaMalloc for training buffers failed");
            return SPH_ERR_ALLOC;
        }
        all.push_back(*p);
        return SPH_OK;
    }
    ~TrainBufs()
    {
        for (void *p : all) cudaFree(p);
    }
};

int make_bufs(TrainBufs &b, int B)
{
    using namespace ml;
    b.B = B;
    LTRY(b.alloc(&b.Xb, (size_t)B * IN));
    LTRY(b.alloc(&b.Tb, (size_t)B));
    LTRY(b.alloc(&b.Z1, (size_t)B * HID));
    LTRY(b.alloc(&b.H1, (size_t)B * HID));
    LTRY(b.alloc(&b.Z2, (size_t)B * HID));
    LTRY(b.alloc(&b.H2, (size_t)B * HID));
    LTRY(b.alloc(&b.Y, (size_t)B * OUT));
    LTRY(b.alloc(&b.dY, (size_t)B * OUT));
    LTRY(b.alloc(&b.dH2, (size_t)B * HID));
    LTRY(b.alloc(&b.dZ2, (size_t)B * HID));
    LTRY(b.alloc(&b.dH1, (size_t)B * HID));
    LTRY(b.alloc(&b.dZ1, (size_t)B * HID));
    LTRY(b.alloc(&b.idx, (size_t)B));
    LTRY(b.alloc(&b.loss, (size_t)nblk(B) + 1));
    LTRY(b.alloc(&b.mask, (size_t)NPARAM));
    return SPH_OK;
}

// One forward + backward + Adam step on the batch in b.Xb / b.Tb.
// cmask: outputs in the loss (bit 0, 1 displacement, bit 2 error);
// trunk = false trains the output layer only.
int train_batch(LearnedModel *l, TrainBufs &b, int cmask, bool trunk, float lr)
{
    using namespace ml;
    cudaStream_t st = l->stream;
    const int B = b.B;
    const __nv_bfloat16 *W1 = l->wbf + OFF_W1, *W2 = l->wbf + OFF_W2, *W3 = l->wbf + OFF_W3;
    // forward
    LTRY(gemm(st, B, HID, IN, b.Xb, IN, 1, W1, IN, 1, b.Z1, HID, l->d_err));
    k_bias_act<<<nblk((long long)B * HID / 2), 256, 0, st>>>(B, HID, b.Z1, l->w + OFF_B1, b.H1);
    LTRY(gemm(st, B, HID, HID, b.H1, HID, 1, W2, HID, 1, b.Z2, HID, l->d_err));
    k_bias_act<<<nblk((long long)B * HID / 2), 256, 0, st>>>(B, HID, b.Z2, l->w + OFF_B2, b.H2);
    LTRY(gemm(st, B, OUT, HID, b.H2, HID, 1, W3, HID, 1, b.Y, OUT, l->d_err));
    k_out_grad<<<nblk(B), 256, 0, st>>>(B, b.Y, l->w + OFF_B3, b.Tb, cmask, b.dY, b.loss);
    // backward: output layer
    LCUDA(cudaMemsetAsync(l->g, 0, NPARAM * sizeof(float), st));
    // dW3[o][h] = sum_b dY[b][o] H2[b][h]
    LTRY(gemm(st, OUT, HID, B, b.dY, 1, OUT, b.H2, 1, HID, l->g + OFF_W3, HID, l->d_err));
    k_colsum<<<1, OUT, 0, st>>>(B, OUT, b.dY, l->g + OFF_B3);
    if (trunk) {
        // dH2[b][h] = sum_o dY[b][o] W3[o][h]
        LTRY(gemm(st, B, HID, OUT, b.dY, OUT, 1, W3, 1, HID, b.dH2, HID, l->d_err));
        k_act_back<<<nblk((long long)B * HID), 256, 0, st>>>(B, HID, b.dH2, b.Z2, b.dZ2);
        LTRY(gemm(st, HID, HID, B, b.dZ2, 1, HID, b.H1, 1, HID, l->g + OFF_W2, HID, l->d_err));
        k_colsum<<<1, HID, 0, st>>>(B, HID, b.dZ2, l->g + OFF_B2);
        LTRY(gemm(st, B, HID, HID, b.dZ2, HID, 1, W2, 1, HID, b.dH1, HID, l->d_err));
        k_act_back<<<nblk((long long)B * HID), 256, 0, st>>>(B, HID, b.dH1, b.Z1, b.dZ1);
        LTRY(gemm(st, HID, IN, B, b.dZ1, 1, HID, b.Xb, 1, IN, l->g + OFF_W1, IN, l->d_err));
        // b1 stays zero: the first layer's bias is the weight of the constant feature 31
    }
    ++l->adam_t;
    const float b1t = powf(0.9f, (float)l->adam_t), b2t = powf(0.999f, (float)l->adam_t);
    k_adam<<<nblk(NPARAM), 256, 0, st>>>(NPARAM, l->w, l->g, l->m, l->v, trunk ? nullptr : b.mask,
                                         lr, b1t, b2t, l->wbf);
    return cuda_fail(cudaGetLastError(), "training step");
}

// Trains on samples [first, first + nsamples) for `epochs` shuffled passes.
int train_loop(LearnedModel *l, int first, int nsamples, int epochs, int batch, float lr,
               int cmask, bool trunk, float *loss)
{
    using namespace ml;
    if (nsamples < 128) {
        set_error("%d training samples: at least 128 are needed", nsamples);
        return SPH_ERR_STATE;
    }
    batch = std::max(128, std::min(batch, nsamples) / 128 * 128);
    const int per_epoch = nsamples / batch;
    TrainBufs b;
    LTRY(make_bufs(b, batch));
    int *d_order = nullptr;
    LTRY(b.alloc(&d_order, (size_t)per_epoch * batch));
    if (!trunk) {
        std::vector<unsigned char> mask(NPARAM, 0);
        for (int o = 0; o < OUT; ++o)
            if ((cmask >> o) & 1) {
                for (int h = 0; h < HID; ++h) mask[OFF_W3 + o * HID + h] = 1;
                mask[OFF_B3 + o] = 1;
            }
        LCUDA(cudaMemcpyAsync(b.mask, mask.data(), NPARAM, cudaMemcpyHostToDevice, l->stream));
        LCUDA(cudaStreamSynchronize(l->stream));
    }
    std::vector<int> order(nsamples);
    for (int i = 0; i < nsamples; ++i) order[i] = first + i;
    unsigned long long rng = l->seed * 0x9E3779B97F4A7C15ull + 17ull + (unsigned long long)l->adam_t;
    auto next = [&]() {
        rng += 0x9E3779B97F4A7C15ull;
        unsigned long long z = rng;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    };
    double last = 0.0;
    for (int ep = 0; ep < epochs; ++ep) {
        for (int i = nsamples - 1; i > 0; --i) std::swap(order[i], order[(int)(next() % (i + 1))]);
        LCUDA(cudaMemcpyAsync(d_order, order.data(), (size_t)per_epoch * batch * sizeof(int),
                              cudaMemcpyHostToDevice, l->stream));
        LCUDA(cudaMemsetAsync(b.loss, 0, sizeof(double), l->stream));
        for (int it = 0; it < per_epoch; ++it) {
            ml::k_gather_rows<<<nblk(batch), 256, 0, l->stream>>>(
                batch, d_order + (size_t)it * batch, l->X, l->T, b.Xb, b.Tb);
            LTRY(train_batch(l, b, cmask, trunk, lr));
        }
        double acc = 0.0;
        LCUDA(cudaMemcpyAsync(&acc, b.loss, sizeof(double), cudaMemcpyDeviceToHost, l->stream));
        LCUDA(cudaStreamSynchronize(l->stream));
        last = acc / ((double)per_epoch * batch);
    }
    LTRY(check_err(l));
    if (loss) *loss = (float)last;
    return SPH_OK;
}

// Message pass on the handle's C order into (feat, nbc), from the density
// records and hit masks the density pass has just left in the handle's
// C-order arrays.
int launch_messages(sph_cuda *h, __nv_bfloat16 *feat, unsigned short *nbc)
{
    if (h->n == 0) return SPH_OK;
    (h->long_masks ? ml::k_messages<true> : ml::k_messages<false>)<<<nblk(h->n), kBlock, 0,
                                                                      h->stream>>>(
        make_ctx(h), h->xr_c, h->mask01_c, h->mask2_c, h->rows_c, h->prev_c, h->start_c,
        &h->d_state->build_max_occ[SLOT_PREDICTED], feat, nbc, &h->d_state->fb_count);
    return cuda_fail(cudaGetLastError(), "messages");
}

int run_mlp(cudaStream_t st, LearnedModel *l, int n, const __nv_bfloat16 *feat, float4 *out,
            int sms)
{
    if (n == 0) return SPH_OK;
    LTRY(configure_kernels());
    const int ntiles = (n + 127) / 128;
    const int grid = std::min((ntiles + ml::kPipes - 1) / ml::kPipes, sms > 0 ? sms : num_sms());
    ml::k_mlp<<<grid, ml::kMlpThreads, mlp_smem(), st>>>(n, feat, l->wbf, l->w, out, l->d_err);
    return cuda_fail(cudaGetLastError(), "mlp launch");
}

// The per-particle buffers of a learned step (allocated once per handle).
int ensure_learned_buffers(sph_cuda *h)
{
    if (h->feat_c) return SPH_OK;
    const size_t N = (size_t)h->capacity + 1;
    LCUDA(cudaMalloc(&h->feat_c, N * ml::IN * sizeof(__nv_bfloat16)));
    LCUDA(cudaMalloc(&h->nbc_c, N * sizeof(unsigned short)));
    LCUDA(cudaMalloc(&h->net_c, N * sizeof(float4)));
    LCUDA(cudaMalloc(&h->fb_list, N * sizeof(int)));
    return SPH_OK;
}

// The predicted state of h's next step with its features and, with `l`,
// the network's outputs in h->net_c.  Leaves the A state as it is.
int predicted_features(sph_cuda *h, LearnedModel *l)
{
    LTRY(ensure_learned_buffers(h));
    LTRY(enqueue_predicted_state(h));  // ends with the density pass
    LTRY(launch_messages(h, (__nv_bfloat16 *)h->feat_c, h->nbc_c));
    if (l) {
        LCUDA(cudaStreamSynchronize(l->stream));  // weights written on the model's stream
        LTRY(run_mlp(h->stream, l, h->n, (const __nv_bfloat16 *)h->feat_c, h->net_c, h->num_sms));
    }
    return SPH_OK;
}

}  // namespace

// Learned passes of a step (called by enqueue_step when a model is
// attached): the features (the plain density pass, then the message pass)
// on the C order, then the network.  With `events`, events[0] is recorded
// after the features and events[1] after the network.
int launch_learned_passes(sph_cuda *h, cudaEvent_t *events)
{
    LearnedModel *l = h->learned;
    LTRY(launch_density_pass(h));
    LTRY(launch_messages(h, (__nv_bfloat16 *)h->feat_c, h->nbc_c));
    if (events) cudaEventRecord(events[0], h->stream);
    LTRY(run_mlp(h->stream, l, h->n, (const __nv_bfloat16 *)h->feat_c, h->net_c, h->num_sms));
    if (events) cudaEventRecord(events[1], h->stream);
    return SPH_OK;
}

unsigned bounds_flags_learned() { return read_bounds_flag(); }

void free_learned_buffers(sph_cuda *h)
{
    if (h->feat_c) cudaFree(h->feat_c);
    if (h->nbc_c) cudaFree(h->nbc_c);
    if (h->net_c) cudaFree(h->net_c);
    if (h->fb_list) cudaFree(h->fb_list);
    h->fb_list = nullptr;
    h->feat_c = nullptr;
    h->nbc_c = nullptr;
    h->net_c = nullptr;
    h->learned = nullptr;
}

}  // namespace sph

using namespace sph;

extern "C" {

int sph_learned_num_params(void) { return ml::NPARAM; }

int sph_learned_wait_selftest(int *gave_up)
{
    if (!gave_up) {
        set_error("null argument");
        return SPH_ERR_INVALID;
    }
    unsigned *d = nullptr;
    LCUDA(cudaMalloc(&d, sizeof(unsigned)));
    int rc = cuda_fail(cudaMemset(d, 0xFF, sizeof(unsigned)), "memset");
    if (!rc) {
        ml::k_wait_selftest<<<1, 32>>>(d);
        rc = cuda_fail(cudaGetLastError(), "selftest launch");
    }
    unsigned h = 0xFFFFFFFFu;
    if (!rc) rc = cuda_fail(cudaMemcpy(&h, d, sizeof(h), cudaMemcpyDeviceToHost), "selftest");
    cudaFree(d);
    if (!rc) *gave_up = (int)h;
    return rc;
}

int sph_learned_create(sph_learned_t **out, int max_samples, unsigned long long seed)
{
    if (!out || max_samples < 0) {
        set_error("sph_learned_create: bad arguments");
        return SPH_ERR_INVALID;
    }
    *out = nullptr;
    sph_learned *l = new (std::nothrow) sph_learned();
    if (!l) return SPH_ERR_ALLOC;
    l->seed = seed;
    l->cap = max_samples;
    auto fail = [&](int rc) {
        sph_learned_destroy(l);
        return rc;
    };
    int rc = configure_kernels();
    if (rc) return fail(rc);
    if ((rc = cuda_fail(cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking), "stream")) ||
        (rc = cuda_fail(cudaMalloc(&l->w, ml::NPARAM * sizeof(float)), "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&l->g, ml::NPARAM * sizeof(float)), "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&l->m, ml::NPARAM * sizeof(float)), "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&l->v, ml::NPARAM * sizeof(float)), "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&l->wbf, ml::NPARAM * sizeof(__nv_bfloat16)), "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&l->d_err, sizeof(unsigned)), "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&l->X, ((size_t)max_samples + 1) * ml::IN * sizeof(__nv_bfloat16)),
                        "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&l->T, ((size_t)max_samples + 1) * sizeof(float4)), "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&l->slot, ((size_t)max_samples + 1) * sizeof(int)), "cudaMalloc")))
        return fail(rc);
    // Glorot-uniform weights from a seeded splitmix64 stream, zero biases
    std::vector<float> w(ml::NPARAM, 0.0f);
    unsigned long long z0 = seed;
    auto uni = [&]() {
        z0 += 0x9E3779B97F4A7C15ull;
        unsigned long long z = z0;
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        return (double)(z >> 11) * (1.0 / 9007199254740992.0);
    };
    auto fill = [&](int off, int rows, int cols) {
        const double lim = std::sqrt(6.0 / (rows + cols));
        for (int e = 0; e < rows * cols; ++e) w[off + e] = (float)((uni() * 2.0 - 1.0) * lim);
    };
    fill(ml::OFF_W1, ml::HID, ml::IN);
    fill(ml::OFF_W2, ml::HID, ml::HID);
    fill(ml::OFF_W3, ml::OUT, ml::HID);
    rc = sph_learned_set_params(l, w.data());
    if (rc) return fail(rc);
    *out = l;
    return SPH_OK;
}

int sph_learned_destroy(sph_learned_t *l)
{
    if (!l) return SPH_OK;
    if (l->stream) cudaStreamSynchronize(l->stream);
    void *ptrs[] = {l->w, l->g, l->m, l->v, l->wbf, l->d_err, l->X, l->T, l->slot};
    for (void *p : ptrs)
        if (p) cudaFree(p);
    if (l->stream) cudaStreamDestroy(l->stream);
    delete l;
    return SPH_OK;
}

int sph_learned_get_params(sph_learned_t *l, float *out)
{
    if (!l || !out) {
        set_error("null argument");
        return SPH_ERR_INVALID;
    }
    LCUDA(cudaMemcpy(out, l->w, ml::NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    return SPH_OK;
}

int sph_learned_set_params(sph_learned_t *l, const float *in)
{
    if (!l || !in) {
        set_error("null argument");
        return SPH_ERR_INVALID;
    }
    LCUDA(cudaMemcpyAsync(l->w, in, ml::NPARAM * sizeof(float), cudaMemcpyHostToDevice, l->stream));
    LCUDA(cudaMemsetAsync(l->m, 0, ml::NPARAM * sizeof(float), l->stream));
    LCUDA(cudaMemsetAsync(l->v, 0, ml::NPARAM * sizeof(float), l->stream));
    LCUDA(cudaMemsetAsync(l->d_err, 0, sizeof(unsigned), l->stream));
    ml::k_f32_to_bf16<<<nblk(ml::NPARAM), 256, 0, l->stream>>>(ml::NPARAM, l->w, l->wbf);
    LCUDA(cudaStreamSynchronize(l->stream));
    l->adam_t = 0;
    return SPH_OK;
}

int sph_learned_gemm_check(const float *A, const float *B, float *C, int M, int N, int K)
{
    if (!A || !B || !C || M <= 0 || N <= 0 || K <= 0) {
        set_error("gemm_check: bad arguments");
        return SPH_ERR_INVALID;
    }
    LTRY(configure_kernels());
    cudaStream_t st = nullptr;
    LCUDA(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking));
    std::vector<__nv_bfloat16> a((size_t)M * K), b((size_t)N * K);
    for (size_t e = 0; e < a.size(); ++e) a[e] = __float2bfloat16(A[e]);
    for (size_t e = 0; e < b.size(); ++e) b[e] = __float2bfloat16(B[e]);
    __nv_bfloat16 *da = nullptr, *db = nullptr;
    float *dc = nullptr;
    unsigned *derr = nullptr;
    int rc = SPH_OK;
    if ((rc = cuda_fail(cudaMalloc(&da, a.size() * 2), "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&db, b.size() * 2), "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&dc, (size_t)M * N * 4), "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&derr, 4), "cudaMalloc"))) {
    } else {
        cudaMemcpyAsync(da, a.data(), a.size() * 2, cudaMemcpyHostToDevice, st);
        cudaMemcpyAsync(db, b.data(), b.size() * 2, cudaMemcpyHostToDevice, st);
        cudaMemsetAsync(derr, 0, 4, st);
        rc = gemm(st, M, N, K, da, K, 1, db, K, 1, dc, N, derr);
        unsigned e = 0;
        if (rc == SPH_OK) {
            cudaMemcpyAsync(C, dc, (size_t)M * N * 4, cudaMemcpyDeviceToHost, st);
            cudaMemcpyAsync(&e, derr, 4, cudaMemcpyDeviceToHost, st);
            rc = cuda_fail(cudaStreamSynchronize(st), "gemm sync");
        }
        if (rc == SPH_OK && e) {
            set_error("tensor-core wait gave up");
            rc = SPH_ERR_CUDA;
        }
    }
    cudaFree(da);
    cudaFree(db);
    cudaFree(dc);
    cudaFree(derr);
    cudaStreamDestroy(st);
    return rc;
}

int sph_learned_forward(sph_learned_t *l, const float *features, int n, float *out)
{
    if (!l || (n > 0 && (!features || !out)) || n < 0) {
        set_error("forward: bad arguments");
        return SPH_ERR_INVALID;
    }
    if (n == 0) return SPH_OK;
    std::vector<__nv_bfloat16> x((size_t)n * ml::IN);
    for (size_t e = 0; e < x.size(); ++e) x[e] = __float2bfloat16(features[e]);
    __nv_bfloat16 *dx = nullptr;
    float4 *dy = nullptr;
    int rc = SPH_OK;
    if ((rc = cuda_fail(cudaMalloc(&dx, x.size() * 2), "cudaMalloc")) ||
        (rc = cuda_fail(cudaMalloc(&dy, (size_t)n * sizeof(float4)), "cudaMalloc"))) {
        cudaFree(dx);
        return rc;
    }
    cudaMemcpyAsync(dx, x.data(), x.size() * 2, cudaMemcpyHostToDevice, l->stream);
    cudaMemsetAsync(l->d_err, 0, 4, l->stream);
    rc = run_mlp(l->stream, l, n, dx, dy, 0);
    std::vector<float4> y(n);
    if (rc == SPH_OK) {
        cudaMemcpyAsync(y.data(), dy, (size_t)n * sizeof(float4), cudaMemcpyDeviceToHost, l->stream);
        rc = check_err(l);
    }
    if (rc == SPH_OK)
        for (int i = 0; i < n; ++i) {
            for (int o = 0; o < ml::OUT; ++o) out[(size_t)i * ml::OUT + o] = 0.0f;
            out[(size_t)i * ml::OUT + 0] = y[i].x;
            out[(size_t)i * ml::OUT + 1] = y[i].y;
            out[(size_t)i * ml::OUT + 2] = y[i].z;
        }
    cudaFree(dx);
    cudaFree(dy);
    return rc;
}

int sph_learned_features(sph_cuda_t *h, float *features, int *counts)
{
    if (!h || !features) {
        set_error("features: null argument");
        return SPH_ERR_INVALID;
    }
    const int n = h->n;
    if (n == 0) return SPH_OK;
    LTRY(predicted_features(h, nullptr));
    std::vector<__nv_bfloat16> f((size_t)n * ml::IN);
    std::vector<unsigned short> cnt(n);
    std::vector<int> ids(n);
    LCUDA(cudaMemcpyAsync(f.data(), h->feat_c, f.size() * 2, cudaMemcpyDeviceToHost, h->stream));
    LCUDA(cudaMemcpyAsync(cnt.data(), h->nbc_c, (size_t)n * 2, cudaMemcpyDeviceToHost, h->stream));
    LCUDA(cudaMemcpyAsync(ids.data(), h->id_c, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream));
    LCUDA(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < n; ++i) {
        const int id = ids[i];
        for (int e = 0; e < ml::IN; ++e)
            features[(size_t)id * ml::IN + e] = __bfloat162float(f[(size_t)i * ml::IN + e]);
        if (counts) counts[id] = cnt[i] == 65535 ? -1 : (int)cnt[i];
    }
    return SPH_OK;
}

namespace {

// splitmix64 finaliser: the sample selection hash.
unsigned long long mix64(unsigned long long z)
{
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// Samples of h's predicted state: features and plain displacements of the
// selected particles appended at l->nsamples.  fraction >= 1 takes every
// eligible particle.  Returns the number appended in *added.
int collect_samples(LearnedModel *l, sph_cuda *h, float fraction, int *added)
{
    *added = 0;
    const int n = h->n;
    if (n == 0) return SPH_OK;
    LTRY(predicted_features(h, nullptr));
    // plain displacement (C order) through the learned relaxation with every
    // particle forced to fall back
    const size_t db = (((size_t)n * 8) + 255) & ~(size_t)255;
    LTRY(ensure_scratch(h, db + ((size_t)n + 1) * 4 + 256));
    float2 *disp = (float2 *)h->d_scratch;
    int *sel_d = (int *)((char *)h->d_scratch + db);
    const float thr = h->learned_thr;
    sph::LearnedModel *keep = h->learned;
    h->learned_thr = -1.0f;
    int rc = launch_learned_relax(h, disp);
    h->learned_thr = thr;
    h->learned = keep;
    LTRY(rc);
    std::vector<unsigned short> cnt(n);
    std::vector<int> ids(n);
    LCUDA(cudaMemcpyAsync(cnt.data(), h->nbc_c, (size_t)n * 2, cudaMemcpyDeviceToHost, h->stream));
    LCUDA(cudaMemcpyAsync(ids.data(), h->id_c, (size_t)n * 4, cudaMemcpyDeviceToHost, h->stream));
    LCUDA(cudaStreamSynchronize(h->stream));
    const unsigned long long salt = mix64(l->seed ^ (0xA5A5A5A5ull + l->calls));
    const double frac = std::min(1.0, std::max(0.0, (double)fraction));
    std::vector<int> sel;
    sel.reserve(std::min(n, std::max(0, l->cap - l->nsamples)));
    for (int i = 0; i < n && l->nsamples + (int)sel.size() < l->cap; ++i) {
        if (cnt[i] > ml::MAXNB) continue;
        if (frac < 1.0 &&
            (double)(mix64(salt ^ (unsigned long long)ids[i]) >> 11) * (1.0 / 9007199254740992.0) >= frac)
            continue;
        sel.push_back(i);
    }
    const int rows = (int)sel.size();
    if (rows > 0) {
        LCUDA(cudaMemcpyAsync(sel_d, sel.data(), (size_t)rows * 4, cudaMemcpyHostToDevice, h->stream));
        ml::k_append<<<nblk(rows), kBlock, 0, h->stream>>>(
            make_ctx(h), rows, sel_d, (const __nv_bfloat16 *)h->feat_c, disp,
            l->X + (size_t)l->nsamples * ml::IN, l->T + l->nsamples, l->slot + l->nsamples);
        LCUDA(cudaGetLastError());
        LCUDA(cudaStreamSynchronize(h->stream));
    }
    l->nsamples += rows;
    ++l->calls;
    *added = rows;
    return SPH_OK;
}

}  // namespace

int sph_learned_collect(sph_learned_t *l, sph_cuda_t *h, float fraction, int *added)
{
    if (!l || !h) {
        set_error("collect: null argument");
        return SPH_ERR_INVALID;
    }
    int got = 0;
    LTRY(collect_samples(l, h, fraction, &got));
    if (added) *added = got;
    return SPH_OK;
}

int sph_learned_num_samples(sph_learned_t *l)
{
    return l ? l->nsamples : 0;
}

int sph_learned_clear_samples(sph_learned_t *l)
{
    if (!l) {
        set_error("null model");
        return SPH_ERR_INVALID;
    }
    l->nsamples = 0;
    return SPH_OK;
}

int sph_learned_train(sph_learned_t *l, int epochs, int batch, float lr, float *loss)
{
    if (!l || epochs <= 0 || batch <= 0 || !(lr > 0.0f)) {
        set_error("train: bad arguments");
        return SPH_ERR_INVALID;
    }
    return train_loop(l, 0, l->nsamples, epochs, batch, lr, 0x3, true, loss);
}

int sph_learned_calibrate(sph_learned_t *l, sph_cuda_t *h, int epochs, float lr, float *loss)
{
    if (!l || !h || epochs <= 0 || !(lr > 0.0f)) {
        set_error("calibrate: bad arguments");
        return SPH_ERR_INVALID;
    }
    const int n = h->n;
    if (n == 0) return SPH_OK;
    // every eligible particle of the predicted state, appended after the
    // training samples (dropped again afterwards)
    const int base = l->nsamples;
    int rows = 0;
    LTRY(collect_samples(l, h, 1.0f, &rows));
    int rc = SPH_OK;
    float2 *dnet = nullptr, *dplain = nullptr;
    float *rn = nullptr, *rp = nullptr;
    do {
        if ((rc = cuda_fail(cudaMalloc(&dnet, (size_t)n * 8), "cudaMalloc")) ||
            (rc = cuda_fail(cudaMalloc(&dplain, (size_t)n * 8), "cudaMalloc")) ||
            (rc = cuda_fail(cudaMalloc(&rn, (size_t)n * 4), "cudaMalloc")) ||
            (rc = cuda_fail(cudaMalloc(&rp, (size_t)n * 4), "cudaMalloc")))
            break;
        // plain displacement: everyone falls back
        const float thr = h->learned_thr;
        h->learned_thr = -1.0f;
        rc = launch_learned_relax(h, dplain);
        h->learned_thr = thr;
        if (rc) break;
        // network displacement of the same state
        if ((rc = cuda_fail(cudaMemsetAsync(l->d_err, 0, 4, h->stream), "memset")) ||
            (rc = cuda_fail(cudaStreamSynchronize(l->stream), "sync")))
            break;
        if ((rc = run_mlp(h->stream, l, n, (const __nv_bfloat16 *)h->feat_c, h->net_c, h->num_sms)))
            break;
        const Ctx c = make_ctx(h);
        const unsigned *occ = &h->d_state->build_max_occ[SLOT_PREDICTED];
        ml::k_net_disp<<<nblk(n), kBlock, 0, h->stream>>>(c, h->net_c, dnet);
        ml::k_density_displaced<<<nblk(n), kBlock, 0, h->stream>>>(c, h->pos_c, dnet, h->start_c,
                                                                   occ, rn);
        ml::k_density_displaced<<<nblk(n), kBlock, 0, h->stream>>>(c, h->pos_c, dplain,
                                                                   h->start_c, occ, rp);
        if (rows > 0)
            ml::k_err_targets<<<nblk(rows), kBlock, 0, h->stream>>>(c, rn, rp, l->slot + base, rows,
                                                                    l->T + base);
        rc = cuda_fail(cudaStreamSynchronize(h->stream), "calibrate");
        if (rc == SPH_OK) rc = check_err(l);
    } while (false);
    cudaFree(dnet);
    cudaFree(dplain);
    cudaFree(rn);
    cudaFree(rp);
    if (rc == SPH_OK) rc = train_loop(l, base, rows, epochs, 4096, lr, 0x4, false, loss);
    l->nsamples = base;
    return rc;
}

int sph_cuda_set_learned(sph_cuda_t *h, sph_learned_t *l, float threshold)
{
    if (!h) {
        set_error("null handle");
        return SPH_ERR_INVALID;
    }
    LCUDA(cudaStreamSynchronize(h->stream));
    if (l) {
        LTRY(configure_kernels());
        LTRY(ensure_learned_buffers(h));
        // the weights are written on the model's stream and read on the handle's
        LCUDA(cudaStreamSynchronize(l->stream));
    }
    h->learned = l;
    h->learned_thr = threshold;
    const unsigned long long zero[2] = {0ull, 0ull};
    LCUDA(cudaMemcpy(&h->d_state->learned_steps, zero, sizeof(zero), cudaMemcpyHostToDevice));
    // the step graph changes
    if (h->exec) cudaGraphExecDestroy(h->exec);
    if (h->graph) cudaGraphDestroy(h->graph);
    h->exec = nullptr;
    h->graph = nullptr;
    h->graph_n = -1;
    return SPH_OK;
}

int sph_cuda_learned_counts(sph_cuda_t *h, unsigned long long *learned, unsigned long long *fallback)
{
    if (!h || !learned || !fallback) {
        set_error("null argument");
        return SPH_ERR_INVALID;
    }
    unsigned long long v[2];
    LCUDA(cudaMemcpyAsync(v, &h->d_state->learned_steps, sizeof(v), cudaMemcpyDeviceToHost,
                          h->stream));
    LCUDA(cudaStreamSynchronize(h->stream));
    if (h->learned) {
        // a tensor-core wait that gave up inside a step leaves its tiles'
        // outputs unwritten: report it here rather than hide it
        unsigned e = 0;
        LCUDA(cudaMemcpy(&e, h->learned->d_err, sizeof(e), cudaMemcpyDeviceToHost));
        if (e) {
            set_error("the network kernel's tensor-core wait gave up %u times: results of "
                      "the learned steps are not valid", e);
            return SPH_ERR_CUDA;
        }
    }
    const unsigned long long total = v[0] * (unsigned long long)h->n;
    *fallback = v[1];
    *learned = total >= v[1] ? total - v[1] : 0ull;
    return SPH_OK;
}

}  // extern "C"
