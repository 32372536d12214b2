// tc5_device.cuh -- inline PTX for the fifth-generation tensor cores
// (tcgen05): tensor-memory allocation, single-thread MMA issue with operands
// in shared memory, completion through an mbarrier, and tensor-memory loads.
//
// Operand layout used throughout: K-major, 128-byte swizzle.  A matrix of R
// rows and 64 half-precision K values per row is R x 128 bytes; 8 rows form
// a 1024-byte atom (base 1024-byte aligned) in which row r's 16-byte chunk c
// is stored at chunk c ^ (r % 8).  Element (r, k) is at byte
//   (r / 8) * 1024 + (r % 8) * 128 + (((k / 8) ^ (r % 8)) * 16) + (k % 8) * 2.
// Wider K is a sequence of such 64-wide blocks (R * 128 bytes apart).  One
// MMA consumes K = 16 (32 bytes of each row); the next K step starts 32 bytes
// further into the row.  Accumulators are FP32 in tensor memory: row i of an
// M = 128 result is TMEM lane i, column j its column j.
#pragma once
#include <cuda_fp16.h>
#include <stdint.h>

#include "tma_device.cuh"

namespace glsfft {

// Shared-memory matrix descriptor (K-major, 128-byte swizzle): start address
// >> 4 in bits 0-13, leading-dimension byte offset (unused for this layout;
// 16) in 16-29, stride-dimension byte offset (1024: the next 8-row atom) in
// 32-45, the fixed value 0b001 in 46-48, base offset 0, swizzle mode 2 in
// 61-63.
__device__ __forceinline__ uint64_t umma_desc_sw128(unsigned smem_addr) {
    uint64_t d = (uint64_t)((smem_addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)(16u >> 4) << 16;
    d |= (uint64_t)(1024u >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor of kind::f16: FP32 accumulator (bits 4-5 = 1),
// A and B FP16 (formats 0), both K-major, N >> 3 in bits 17-22, M >> 4 in
// bits 24-28.
__host__ __device__ constexpr uint32_t umma_idesc_f16(int m, int n) {
    return (1u << 4) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

// Tensor-memory allocation: warp-collective; the base address lands in
// *slot (shared memory).  ncols is a power of two >= 32.
template <int NCOLS>
__device__ __forceinline__ void tmem_alloc(unsigned *slot) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(slot)),
                 "n"(NCOLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
template <int NCOLS>
__device__ __forceinline__ void tmem_dealloc(unsigned taddr) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "n"(NCOLS)
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// generic-proxy shared-memory writes made visible to the tensor core
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D (tmem) = A * B^T (+ D when accumulate), A and B from shared memory.
__device__ __forceinline__ void umma_f16(unsigned d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, unsigned accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrive on the mbarrier once every MMA this thread issued before has completed
__device__ __forceinline__ void umma_commit(unsigned long long *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

// Four groups of 8 consecutive FP32 columns of this thread's lane (warp w
// reads lanes 32 * (w % 4) ..; each address carries the lane in bits 16-31),
// and the wait for them inside the same asm statement, so no use of the
// values can be scheduled before the data has arrived.
__device__ __forceinline__ void tmem_ld_4x8(unsigned t0, unsigned t1, unsigned t2, unsigned t3,
                                            float (&v)[32]) {
    unsigned r[32];
    asm volatile(
        "{\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%32];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%8,%9,%10,%11,%12,%13,%14,%15}, [%33];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%16,%17,%18,%19,%20,%21,%22,%23}, [%34];\n\t"
        "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%24,%25,%26,%27,%28,%29,%30,%31}, [%35];\n\t"
        "tcgen05.wait::ld.sync.aligned;\n\t}"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(t0), "r"(t1), "r"(t2), "r"(t3)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// byte offset of element (r, k) in a K-major 128-byte-swizzled block of
// 64-wide rows
__host__ __device__ constexpr unsigned sw128_offset(unsigned r, unsigned k) {
    return (r / 8) * 1024 + (r % 8) * 128 + (((k / 8) ^ (r % 8)) * 16) + (k % 8) * 2;
}

}  // namespace glsfft
