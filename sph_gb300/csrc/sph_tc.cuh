// sph_tc.cuh -- 5th-generation tensor core (tcgen05) building blocks, sm_100+.
//
// A CTA of 128 threads (one warpgroup) owns a 128-lane tile of tensor memory
// (TMEM).  Operands are staged in shared memory in the canonical K-major,
// no-swizzle layout: 8-row x 16-byte "core matrices" stored contiguously
// (128 bytes each), core matrices of one 8-row group consecutive along K.
// One thread issues tcgen05.mma (D[128 x N] += A[128 x 16] . B[N x 16]^T,
// BF16 inputs, FP32 accumulation in TMEM) and commits them to an mbarrier;
// the warpgroup waits on it (bounded) and reads D back with tcgen05.ld.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

namespace sph {
namespace tc {

constexpr int kCoreBytes = 128;   // one 8 x 16-byte core matrix
constexpr uint32_t kSpinLimit = 1u << 24;

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// Byte offset of element (r, k) of a K-major operand tile with `kdim`
// columns, in the no-swizzle core-matrix layout.
__device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int kdim)
{
    return (uint32_t)((r >> 3) * (kdim >> 3) * kCoreBytes + (k >> 3) * kCoreBytes + (r & 7) * 16 +
                      (k & 7) * 2);
}

// Shared-memory matrix descriptor (tcgen05): start address, leading- and
// stride-dimension byte offsets (16-byte units), descriptor version 1,
// no swizzle.  For the layout above: LBO = distance between the two core
// matrices along K that one instruction consumes, SBO = distance between
// 8-row groups.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // version
    return d;                // base offset 0, layout type 0 (no swizzle)
}

// Instruction descriptor for kind::f16 with BF16 A/B, FP32 D, both operands
// K-major, shape M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4)                        // D format: F32
           | (1u << 7)                      // A format: BF16
           | (1u << 10)                     // B format: BF16
           | ((uint32_t)(N >> 3) << 17)     // N / 8
           | ((uint32_t)(M >> 4) << 24);    // M / 16
}

__device__ __forceinline__ void tmem_alloc(uint32_t *dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(dst_smem)), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;"
                 :: "r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync()
{
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}

__device__ __forceinline__ void fence_after_sync()
{
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Makes generic-proxy writes to shared memory visible to the tensor core.
__device__ __forceinline__ void fence_async_smem()
{
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :: "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate) : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(mbar)), "r"(count)
                 : "memory");
}

__device__ __forceinline__ void mbar_fence_init()
{
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns()
{
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Waits for phase `parity` of the mbarrier to complete; gives up after
// kWaitNs nanoseconds of the GPU's global timer (or kSpinLimit polls) and
// returns false (the caller records an error).
constexpr uint64_t kWaitNs = 1000000000ull;  // 1 s: any tensor-core step takes microseconds
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity)
{
    const uint32_t a = smem_u32(mbar);
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t it = 0; it < kSpinLimit; ++it) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done) : "r"(a), "r"(parity) : "memory");
        if (done) return true;
        if (globaltimer_ns() - t0 > kWaitNs) return false;
    }
    return false;
}

// 32 lanes x 16 consecutive FP32 columns: thread t of warp w receives row
// 32 (w % 4) + t, columns [col, col + 16) of the accumulator.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 lanes x 32 consecutive FP32 columns (as tmem_ld16, twice as wide).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// The network's activation of two values in packed BF16 arithmetic:
// 2 GELU(x) = x (1 + tanh(x (c0 + c1 x^2))), c0 = sqrt(2/pi), c1 = 0.044715 c0,
// x = bf16(a), bf16(b) (GELU in its tanh form, scaled by 2: the next layer's
// weights absorb the factor).  Returns the packed pair (a in the low half).
__device__ __forceinline__ uint32_t act_bf16x2(float a, float b)
{
    uint32_t x, x2, t, u, th, y;
    asm("cvt.rn.bf16x2.f32 %0, %1, %2;" : "=r"(x) : "f"(b), "f"(a));
    const uint32_t c0 = 0x3F4C3F4Cu;    // bf16(0.7978846) x 2
    const uint32_t c1 = 0x3D123D12u;    // bf16(0.0356774) x 2
    const uint32_t zero = 0x80008000u;  // -0, the additive identity of fma
    asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(x2) : "r"(x), "r"(x), "r"(zero));
    asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(t) : "r"(x2), "r"(c1), "r"(c0));
    asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(u) : "r"(x), "r"(t), "r"(zero));
    asm("tanh.approx.bf16x2 %0, %1;" : "=r"(th) : "r"(u));
    asm("fma.rn.bf16x2 %0, %1, %2, %3;" : "=r"(y) : "r"(x), "r"(th), "r"(x));
    return y;
}

// Named barrier over `count` threads (ids 1..15; 0 is __syncthreads).
__device__ __forceinline__ void named_sync(int id, int count)
{
    asm volatile("bar.sync %0, %1;" :: "r"(id), "r"(count) : "memory");
}

// Named barrier that also ANDs a predicate over the participating threads.
__device__ __forceinline__ bool named_sync_and(int id, int count, bool v)
{
    uint32_t r;
    asm volatile(
        "{\n\t.reg .pred p, q;\n\t"
        "setp.ne.u32 p, %1, 0;\n\t"
        "bar.red.and.pred q, %2, %3, p;\n\t"
        "selp.u32 %0, 1, 0, q;\n\t}"
        : "=r"(r) : "r"((uint32_t)v), "r"(id), "r"(count) : "memory");
    return r != 0;
}

// D[128 x N] (+)= A[128 x K] . B[N x K]^T for operands staged in the
// K-major layout at smem_a / smem_b (K a multiple of 16).  Issued by one
// thread; the caller commits.
__device__ __forceinline__ void mma_tile(uint32_t tmem_d, uint32_t smem_a, uint32_t smem_b, int N,
                                         int K, bool accumulate_first)
{
    const uint32_t idesc = idesc_bf16(128, N);
    const uint32_t sbo = (uint32_t)(K >> 3) * kCoreBytes;
    for (int k = 0; k < K; k += 16) {
        const uint32_t koff = (uint32_t)(k >> 3) * kCoreBytes;
        const uint64_t ad = smem_desc(smem_a + koff, kCoreBytes, sbo);
        const uint64_t bd = smem_desc(smem_b + koff, kCoreBytes, sbo);
        mma_bf16(tmem_d, ad, bd, idesc, (k > 0 || accumulate_first) ? 1u : 0u);
    }
}

}  // namespace tc
}  // namespace sph
