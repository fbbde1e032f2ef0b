// Fifth-generation tensor core helpers (tcgen05, sm_100 family): tensor
// memory allocation, shared-memory matrix descriptors for the 128-byte
// swizzled K-major layout, the TF32 MMA with an FP32 accumulator in tensor
// memory, its completion on an mbarrier, and the tensor-memory load.
//
// Layout used by every operand here (K-major, 128-byte swizzle): a matrix of
// R rows and K 32-bit elements is stored as K / 32 column blocks, each R / 8
// atoms of 8 rows x 128 bytes (1024 bytes, 1024-byte aligned); inside an
// atom, row r's 16-byte chunk c sits at chunk position c ^ r.  One MMA step
// covers 8 elements of K (32 bytes): its descriptor starts at the column
// block plus 32 bytes per step, with the atoms of consecutive 8-row groups
// 1024 bytes apart (stride byte offset).
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace mrl {
namespace tc {

// byte offset of element (row, k) of a K-major 128-byte-swizzled operand
// with `rows` rows (a multiple of 8) from its 1024-byte-aligned base
__host__ __device__ __forceinline__ uint32_t sw128_offset(int row, int k, int rows) {
    const uint32_t kb = (uint32_t)k >> 5, kc = ((uint32_t)k >> 2) & 7u, kw = (uint32_t)k & 3u;
    const uint32_t r8 = (uint32_t)row & 7u;
    return kb * (uint32_t)rows * 128u + ((uint32_t)row >> 3) * 1024u + r8 * 128u + ((kc ^ r8) << 4) + (kw << 2);
}

// shared-memory matrix descriptor: start address, stride byte offset 1024
// (8-row groups), leading byte offset unused by swizzled K-major layouts
// (encoded 1), descriptor version 1 (bit 46), 128-byte swizzle (mode 2)
__device__ __forceinline__ uint64_t sw128_desc(uint32_t saddr) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1u << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)2u << 61;
    return d;
}

// instruction descriptor of kind::tf32: FP32 accumulator, TF32 A and B,
// both K-major, no negation, shape M x N
__host__ __device__ constexpr uint32_t idesc_tf32(int M, int N) {
    return (1u << 4)                     // D format: F32
           | (2u << 7) | (2u << 10)      // A, B format: TF32
           | ((uint32_t)(N >> 3) << 17)  // N / 8
           | ((uint32_t)(M >> 4) << 24); // M / 16
}

// tensor memory: `ncols` columns (a power of two >= 32) for this CTA; the
// whole warp executes it; the base address is written to *slot (shared)
__device__ __forceinline__ void tmem_alloc(uint32_t *slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// D[tmem] (+)= A x B^T, A: M x K and B: N x K from shared memory (one K = 8 step)
__device__ __forceinline__ void mma_tf32(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         bool accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"((uint32_t)accumulate)
        : "memory");
}

// arrive once on the mbarrier when every MMA this thread issued has completed
__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     (uint32_t)__cvta_generic_to_shared(bar))
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// make this thread's generic-proxy shared-memory writes visible to the
// tensor core (async proxy)
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// 32 lanes x 32 columns of 32-bit values: thread t of the warp gets lane
// (taddr's lane + t), columns taddr's column .. +31
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    // the load and its wait in one statement: no use of r can be scheduled
    // between them
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// 32 lanes x 8 columns
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float (&v)[8]) {
    uint32_t r[8];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace mrl
