// tc.cuh - 5th-generation tensor-core (tcgen05) building blocks for the split-BF16 density step.
//
// Operands live in shared memory in the K-major, no-swizzle canonical layout: the matrix is cut into core
// matrices of 8 rows x 8 bf16 (16 bytes) stored as contiguous 128-byte blocks, row-block-major:
//     byte(r, c) = ((r / 8) * (Kp / 8) + c / 8) * 128 + (r % 8) * 16 + (c % 8) * 2
// so along K consecutive core matrices are 128 bytes apart (leading-dimension byte offset) and along M/N
// consecutive 8-row groups are Kp * 16 bytes apart (stride-dimension byte offset).  One elected thread
// issues tcgen05.mma (M = 128, K = 16 per instruction, BF16 inputs, FP32 accumulator in tensor memory);
// completion is tracked by tcgen05.commit on an mbarrier whose waits are bounded (an error flag is set
// instead of spinning forever); the accumulator is read back with tcgen05.ld (32 lanes x 32 bits).
#pragma once
#include <cstdint>
#include <cuda_bf16.h>

#include "common.cuh"

#define TC_M 128

__device__ __forceinline__ uint32_t tc_smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// Byte offset of element (r, c) in the canonical layout of a matrix with Kp columns (Kp % 16 == 0).
__device__ __forceinline__ uint32_t tc_offset(int r, int c, int Kp)
{
    return (uint32_t)((((r >> 3) * (Kp >> 3) + (c >> 3)) << 7) + ((r & 7) << 4) + ((c & 7) << 1));
}

// Shared-memory matrix descriptor (tcgen05): start address, leading / stride byte offsets (all >> 4),
// the fixed 0b001 at bits 46-48, base offset 0, relative LBO, no swizzle.
__device__ __forceinline__ uint64_t tc_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo & 0x3FFFFu) >> 4) << 16) |
           ((uint64_t)((sbo & 0x3FFFFu) >> 4) << 32) | ((uint64_t)1 << 46);
}

// Instruction descriptor, kind::f16: FP32 accumulator (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1),
// both K-major (bits 15, 16 = 0), N >> 3 at bits 17-22, M >> 4 at bits 24-28.
__device__ __forceinline__ uint32_t tc_idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(uint32_t d_tmem, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate)
{
    asm volatile("{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\ttcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
                 :: "r"(d_tmem), "l"(a), "l"(b), "r"(idesc), "r"(accumulate) : "memory");
}

__device__ __forceinline__ void tc_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" :: "r"(bar) : "memory");
}

__device__ __forceinline__ void tc_alloc(uint32_t dst_smem, uint32_t ncols)   // whole warp
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" :: "r"(dst_smem), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t ncols)   // whole warp
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_proxy() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(bar), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// Bounded wait for the mbarrier phase with the given parity; false when the limit ran out.
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, int max_iter)
{
    for (int it = 0; it < max_iter; it++) {
        uint32_t done;
        asm volatile("{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
                     : "=r"(done) : "r"(bar), "r"(parity) : "memory");
        if (done) return true;
    }
    return false;
}

// 16 consecutive 32-bit accumulator columns of this thread's tensor-memory lane.
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                   "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int k = 0; k < 16; k++) v[k] = __uint_as_float(r[k]);
}

// Issue D[0:128, 0:Nn] (+)= A[m0 : m0+128, 0:Kp] * B[n0 : n0+Nn, 0:Kp]^T, K-major operands in the canonical
// layout (A and B may be the same array), one instruction per 16-deep K chunk.  One thread only.
__device__ __forceinline__ void tc_product(uint32_t d_tmem, uint32_t a_base, int m0, uint32_t b_base, int Nn, int Kp, bool accumulate,
                                           int n0 = 0)
{
    const uint32_t idesc = tc_idesc_bf16(TC_M, Nn), sbo = (uint32_t)Kp * 16u;
    for (int k0 = 0; k0 < Kp; k0 += 16) {
        const uint64_t a = tc_desc(a_base + tc_offset(m0, k0, Kp), 128u, sbo);
        const uint64_t b = tc_desc(b_base + tc_offset(n0, k0, Kp), 128u, sbo);
        tc_mma(d_tmem, a, b, idesc, (accumulate || k0 > 0) ? 1u : 0u);
    }
}

// BF16 split of x into hi + mid + lo (round to nearest at each level).
__device__ __forceinline__ void bf16_split3(float x, __nv_bfloat16 &h, __nv_bfloat16 &m, __nv_bfloat16 &l)
{
    h = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(h);
    m = __float2bfloat16_rn(r1);
    l = __float2bfloat16_rn(r1 - __bfloat162float(m));
}
