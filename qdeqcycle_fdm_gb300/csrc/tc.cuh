// tc.cuh -- 5th-generation tensor-core (tcgen05) primitives for sm_103a:
// tensor-memory allocation, shared-memory matrix descriptors, the BF16 MMA
// with FP32 accumulation in tensor memory, its completion tracking on an
// mbarrier, and the tensor-memory -> register load of the epilogue.
//
// Conventions (PTX ISA, tcgen05 family):
//   * one warp allocates and frees the accumulator columns; the address it
//     receives is lane 0 / column base of a 128-lane x ncols region;
//   * a single thread issues tcgen05.mma; tcgen05.commit makes an mbarrier
//     arrive once every MMA that thread issued before it has completed;
//   * for an M = 128 accumulator, row m of D is tensor-memory lane m and
//     column n is column base + n; warp w of the CTA may read lanes
//     32*(w%4) .. 32*(w%4)+31.
// Operands are K-major tiles in shared memory written by TMA with the
// matching swizzle: rows of SW bytes (32, 64 or 128), eight-row groups of
// 8*SW bytes, tile bases 1024-byte aligned (an MMA may start on any row).
#pragma once

#include <stdint.h>

#include "tma.cuh"

namespace qd {

// ---- tensor memory ---------------------------------------------------------
// ncols: a power of two >= 32.  Executed by all 32 threads of one warp.
__device__ __forceinline__ void tmem_alloc(uint32_t *smem_dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(smem_dst)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_free(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// ---- descriptors -----------------------------------------------------------
// Swizzle of a K-major operand tile by its row width in bytes.
__host__ __device__ constexpr uint32_t sw_layout_type(int row_bytes) {
    return row_bytes == 128 ? 2u : (row_bytes == 64 ? 4u : 6u);   // 128B, 64B, 32B
}

// Shared-memory matrix descriptor: start address, leading-dimension offset
// (unused for swizzled K-major tiles, set to 16 B), stride between 8-row
// groups (8 * row_bytes), descriptor version 1, base offset 0, swizzle
// layout.  The MMA applies the swizzle to the absolute shared-memory
// address, as the TMA does when it writes a 1024-byte-aligned tile, so a
// start on any row of the tile (or 32 bytes into a row, for the K steps)
// reads the rows as written.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, int row_bytes) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(16u >> 4) << 16;
    d |= (uint64_t)((8u * (uint32_t)row_bytes) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)sw_layout_type(row_bytes) << 61;
    return d;
}

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 D, both
// operands K-major, M = 128, N = n (a multiple of 16, 16..256).
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int n) {
    return (1u << 4)                          // D format: F32
           | (1u << 7)                        // A format: BF16
           | (1u << 10)                       // B format: BF16
           | ((uint32_t)(n >> 3) << 17)       // N >> 3
           | ((uint32_t)(128 >> 4) << 24);    // M >> 4
}

// ---- MMA -------------------------------------------------------------------
// D[tmem] (+)= A[smem] * B[smem]^T, one 128 x N x 16 step; accumulate = 0
// overwrites D.
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// the mbarrier arrives once all previously issued MMAs of this thread finish
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_u32(bar))
                 : "memory");
}

// ---- epilogue --------------------------------------------------------------
// the load without the wait: issue several, then tmem_ld_wait() on each
// group of destination registers
__device__ __forceinline__ void tmem_ld8_issue(uint32_t taddr, uint32_t r[8]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(taddr)
        : "memory");
}
// Wait for this thread's outstanding tensor-memory loads.  The destination
// registers pass through the instruction as operands, so no use of them can
// be scheduled before it (the first call waits, repeated ones are free).
__device__ __forceinline__ void tmem_ld_wait(uint32_t r[8]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0]), "+r"(r[1]), "+r"(r[2]), "+r"(r[3]), "+r"(r[4]), "+r"(r[5]), "+r"(r[6]), "+r"(r[7])
                 :
                 : "memory");
}

// 8 consecutive FP32 columns of this thread's lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float v[8]) {
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(taddr)
        : "memory");
    tmem_ld_wait(r);
#pragma unroll
    for (int i = 0; i < 8; i++) v[i] = __uint_as_float(r[i]);
}

// ---- plain mbarrier arrive (for barriers a thread, not a copy, completes) --
__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

}  // namespace qd
