// Tensor-memory-accelerator (TMA) copies and shared-memory mbarriers for sm_103a,
// written as inline PTX, and the host-side encoding of the tensor maps they read.
//
// Every wait here is bounded: a wait that runs out returns false and the caller sets
// the plan's error flag and goes on, so a kernel never spins forever.
#pragma once

#include <cuda.h>   // CUtensorMap and its enums (the encoder is fetched at run time)
#include "kore_common.cuh"

// Iteration limit of an mbarrier wait (each try_wait may itself suspend for a short,
// hardware-chosen time): seconds at most, far above any legitimate wait.
#define KORE_MBAR_SPIN_LIMIT (1u << 24)

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// make the initialised barriers visible to the async (TMA) proxy
__device__ __forceinline__ void mbar_fence_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// one arrival plus `bytes` of expected transaction (the TMA copy completes them)
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Wait until the phase of parity `parity` has completed; false when the wait ran out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
    for (uint32_t i = 0; i < KORE_MBAR_SPIN_LIMIT; ++i)
        if (mbar_try_wait(bar, parity)) return true;
    return false;
}

// 4-D tiled tensor copy global -> shared, completing on `bar`.  c0 is the innermost
// coordinate; c0 * element size must be a multiple of 16 bytes.
__device__ __forceinline__ void tma_load_4d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2,
                                            int c3) {
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4, %5}], [%6];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
        : "memory");
}

// 3-D tiled tensor copy global -> shared, completing on `bar`.
__device__ __forceinline__ void tma_load_3d(void *dst, const CUtensorMap *map, uint64_t *bar, int c0, int c1, int c2) {
    asm volatile(
        "cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3, %4}], [%5];" ::"r"(smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tma_prefetch_desc(const CUtensorMap *map) {
    asm volatile("prefetch.tensormap [%0];" ::"l"(reinterpret_cast<uint64_t>(map)) : "memory");
}

// Named barrier over the first `nthreads` threads of the block (id 1..15; id 0 is
// __syncthreads).
__device__ __forceinline__ void named_sync(int id, int nthreads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(nthreads) : "memory");
}

// ----------------------------------------------------------------------------- host
// Encodes a 4-D tiled tensor map over a column-major stack of square blocks:
//   dim 0: 2 S reals of one column (a complex entry is two reals), contiguous
//   dim 1: S columns of a block            (stride S complex entries)
//   dim 2: nblk blocks of one shift        (stride S*S complex entries)
//   dim 3: nshift shifts                   (stride shift_stride complex entries)
// with a box of box_rows complex rows x box_cols columns of one block.  Reads past a
// block's rows or columns return zeros.  real_bytes is 4 (complex64) or 8 (complex128).
int kore_encode_block_map(CUtensorMap *map, const void *base, int real_bytes, int S, int64_t nblk, int nshift,
                          int64_t shift_stride, int box_rows, int box_cols);

// 3-D float32 tensor map (dims innermost first, strides in bytes of dims 1 and 2) with
// an optional 128-byte swizzle (box[0] * 4 must then be 128 or less).
int kore_encode_f32_3d(CUtensorMap *map, const void *base, const uint64_t dims[3], const uint64_t strides[2],
                       const uint32_t box[3], int swizzle128);
