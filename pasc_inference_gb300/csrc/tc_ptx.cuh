// tc_ptx.cuh -- inline-PTX helpers for the 5th-generation tensor cores (tcgen05) and tiled
// TMA tensor copies on sm_103a: tensor-memory allocation, UMMA shared-memory and instruction
// descriptors, the single-CTA BF16 MMA with FP32 accumulation in tensor memory, its commit to
// an mbarrier, and 32-lane tensor-memory loads.  mbarrier helpers come from sweep_tma.cuh.
#pragma once

#include <cuda.h>

#include "sweep_tma.cuh"

namespace pasc {

// tma_load_2d: sweep_tma.cuh

// ---- tensor memory -------------------------------------------------------------------
// Allocation by one full warp; the column base is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(unsigned int *slot, unsigned int ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)), "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish()
{
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(unsigned int taddr, unsigned int ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---- UMMA descriptors -----------------------------------------------------------------
// Shared-memory matrix descriptor for a K-major operand in the 128-byte swizzle layout: rows
// of 128 bytes (64 BF16), 8-row groups 1024 bytes apart (stride byte offset), atom base
// 1024-byte aligned; the K-steps of 16 elements inside an atom advance the start address by
// 32 bytes.  Fields: start >> 4 [0,14), leading byte offset >> 4 [16,30) (unused for this
// layout), stride byte offset >> 4 [32,46), version 1 [46,48), swizzle mode 2 = 128B [61,64).
__device__ __forceinline__ unsigned long long umma_desc_sw128(unsigned int saddr)
{
    unsigned long long d = (unsigned long long)((saddr >> 4) & 0x3FFFu);
    d |= 1ull << 16;
    d |= (unsigned long long)(1024 >> 4) << 32;
    d |= 1ull << 46;
    d |= 2ull << 61;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator [4,6) = 1, A BF16 [7,10) = 1,
// B BF16 [10,13) = 1, both K-major (bits 15, 16 = 0), N >> 3 at [17,23), M >> 4 at [24,29).
template <int M, int N>
__host__ __device__ constexpr unsigned int umma_idesc_bf16_f32()
{
    static_assert(M == 64 || M == 128, "M");
    static_assert(N % 16 == 0 && N >= 16 && N <= 256, "N");
    return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned int)(N >> 3) << 17) | ((unsigned int)(M >> 4) << 24);
}

// D[tmem] (+)= A[smem] * B[smem]^T, issued by one thread.
__device__ __forceinline__ void umma_bf16(unsigned int d_tmem, unsigned long long adesc, unsigned long long bdesc,
                                          unsigned int idesc, unsigned int accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// The mbarrier receives one arrival when all MMAs issued so far by this thread complete.
__device__ __forceinline__ void umma_commit(unsigned long long *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_addr(bar))
                 : "memory");
}

// 32 consecutive FP32 columns of this warp's 32 tensor-memory lanes (lane = thread).  The
// wait is tied to the destination registers so that no use is scheduled before it.
__device__ __forceinline__ void tmem_load_32cols(unsigned int taddr, float (&v)[32])
{
    unsigned int r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7]),
                   "+r"(r[8]), "+r"(r[9]), "+r"(r[10]), "+r"(r[11]), "+r"(r[12]), "+r"(r[13]), "+r"(r[14]),
                   "+r"(r[15]), "+r"(r[16]), "+r"(r[17]), "+r"(r[18]), "+r"(r[19]), "+r"(r[20]), "+r"(r[21]),
                   "+r"(r[22]), "+r"(r[23]), "+r"(r[24]), "+r"(r[25]), "+r"(r[26]), "+r"(r[27]), "+r"(r[28]),
                   "+r"(r[29]), "+r"(r[30]), "+r"(r[31])
                 :
                 : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace pasc
