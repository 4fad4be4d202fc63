// tma.cuh -- Tensor Memory Accelerator staging for the multigrid tiles.
//
// One thread of a CTA issues a 2-D cp.async.bulk.tensor load per array of the
// tile (u, f, the face moduli) against one mbarrier; every thread then waits
// on the barrier.  Rules this code keeps (the TMA faults otherwise):
//   * the innermost (x) start coordinate times the element size is a
//     multiple of 16 bytes: callers round x down to a multiple of
//     16 / sizeof(T) elements;
//   * box widths times the element size are multiples of 16 bytes, boxes are
//     at most 256 per dimension, row strides are multiples of 16 bytes (the
//     level pitch is a multiple of 32 elements), destinations are 128-byte
//     aligned;
//   * only loads start at out-of-range coordinates (rows past the grid read
//     as zeros); nothing is stored through the TMA.
// The wait is bounded: if the transfer does not complete the kernel records
// the failure in a status word and returns, instead of spinning forever.
#pragma once

#include <cuda.h>
#include <stdint.h>

namespace qd {

static constexpr unsigned TMA_WAIT_LIMIT = 1u << 22;   // try_wait rounds before giving up

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// true once the phase with this parity has completed; false after `limit`
// polls
__device__ __forceinline__ bool mbar_wait_limit(uint64_t *bar, unsigned parity, unsigned limit) {
    const uint32_t a = smem_u32(bar);
    for (unsigned i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// the wait every staging pipeline uses: TMA_WAIT_LIMIT polls
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, unsigned parity) {
    return mbar_wait_limit(bar, parity, TMA_WAIT_LIMIT);
}

// 2-D tile load: box at (x, y) of the tensor into shared memory
__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, int x, int y,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// 3-D tile load: box at (x, y, z)
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, int x, int y, int z,
                                            uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
        " [%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"((uint64_t)map), "r"(x), "r"(y), "r"(z), "r"(smem_u32(bar))
        : "memory");
}

// host: build a 2-D tiled tensor map (rows of `width` elements, `pitch`
// elements apart, `height` rows) with a box of box_w x box_h elements
int make_tensor_map_2d(CUtensorMap *map, const void *base, bool fp64, int width, int height,
                       int pitch, int box_w, int box_h);
// general form: dtype a CUtensorMapDataType, esz its bytes, swizzle a
// CUtensorMapSwizzle (the box row must fit the swizzle span)
int encode_tiled_2d(CUtensorMap *map, const void *base, int dtype, int esz, long width, long height,
                    long pitch_bytes, int box_w, int box_h, int swizzle);
// unswizzled 3-D map: d0 innermost; strides of dimensions 1 and 2 in bytes
int encode_tiled_3d(CUtensorMap *map, const void *base, int dtype, int esz, long d0, long d1, long d2,
                    long stride1_bytes, long stride2_bytes, int box0, int box1, int box2, int swizzle);

}  // namespace qd
