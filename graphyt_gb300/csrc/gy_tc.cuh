// gy_tc.cuh -- 5th-generation tensor core (tcgen05) building blocks for sm_103a: BF16
// operands in shared memory, FP32 accumulators in tensor memory (TMEM).
//
// Operand layout: K-major without swizzle.  A tile of R rows x K bf16 columns is stored as
// 8-row x 16-byte "core matrices" (8 x 8 bf16, 128 contiguous bytes, row r at +16 r); the
// core matrix of row block rb and column block kb sits at rb * SBO + kb * LBO.  Here
// LBO = 128 (column blocks adjacent) and SBO = (K / 8) * 128, so element (r, k) lives at
//   (r / 8) * SBO + (k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2   bytes.
// One tcgen05.mma of kind::f16 consumes 16 columns of K (two column blocks); the next
// 16 columns start 256 bytes further.
//
// Waits on mbarriers are bounded: after GY_TC_SPIN_LIMIT polls the wait gives up, reports
// it through a status word and returns false, so a kernel never hangs on a lost arrival.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "gy_common.cuh"

namespace gy {

#ifndef GY_TC_SPIN_LIMIT
#define GY_TC_SPIN_LIMIT (1u << 22)  // polls of an mbarrier (32 ns apart) before a wait gives up
#endif

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) in a K-major no-swizzle tile with K columns
__host__ __device__ __forceinline__ uint32_t tc_off(int r, int k, int K)
{
    return (uint32_t)((r >> 3) * (K >> 3) * 128 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2);
}

// shared-memory matrix descriptor: start address, leading (K) and stride (row block) byte
// offsets, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1 << 46;  // version
    return d;                // base offset 0, layout type 0 (no swizzle)
}

// instruction descriptor of kind::f16: BF16 A and B (both K-major), FP32 D, M x N
__host__ __device__ __forceinline__ uint32_t tc_idesc_bf16(int M, int N)
{
    uint32_t d = 0;
    d |= 1u << 4;                       // D format F32
    d |= 1u << 7;                       // A format BF16
    d |= 1u << 10;                      // B format BF16
    d |= (uint32_t)(N >> 3) << 17;      // N / 8
    d |= (uint32_t)(M >> 4) << 24;      // M / 16
    return d;
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread
__device__ __forceinline__ void tc_mma(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, bool accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n"
        :
        : "r"(tmem_d), "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
}

// arrive on the mbarrier once every tcgen05 operation this thread issued has completed
__device__ __forceinline__ void tc_commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_u32(mbar)) : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_u32(mbar)), "r"(count) : "memory");
}

// Wait for the phase with the given parity to complete; false if the wait gave up.  The
// poll is the non-blocking test_wait with a short sleep between polls, so the bound on the
// wait is the poll count times the sleep (a fraction of a second).
__device__ __forceinline__ bool mbar_wait(uint64_t *mbar, uint32_t parity)
{
    const uint32_t a = smem_u32(mbar);
    for (uint32_t it = 0; it < GY_TC_SPIN_LIMIT; it++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
        __nanosleep(32);
    }
    return false;
}

// the global nanosecond timer
__device__ __forceinline__ unsigned long long clock_now_ns()
{
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// make this thread's generic-proxy shared-memory writes visible to the tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// TMEM allocation by one full warp: ncols (a power of two >= 32) columns, base address
// written to *dst (shared memory)
__device__ __forceinline__ void tmem_alloc(uint32_t *dst, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_u32(dst)), "r"(ncols) : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols) : "memory");
}

// 16 consecutive FP32 columns of this thread's TMEM lane (warp w reads lanes 32w..32w+31)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float v[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// TMEM address of lane (row) `lane0` and column `col` relative to the allocation base
__device__ __forceinline__ uint32_t tmem_at(uint32_t base, int lane0, int col)
{
    return base + ((uint32_t)lane0 << 16) + (uint32_t)col;
}

}  // namespace gy
