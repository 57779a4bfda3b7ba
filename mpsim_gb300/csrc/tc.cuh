// Blackwell (sm_103a) tensor-core building blocks: tcgen05 MMA with TMEM
// accumulators, shared-memory matrix descriptors, TMA bulk copies and the
// split of FP32 values into three bf16 pieces.
//
// Split precision.  x = x0 + x1 + x2 with each piece a bf16 (8 significant
// bits): x0 = bf16(x), x1 = bf16(x - x0), x2 = bf16(x - x0 - x1); both
// subtractions are exact in FP32 and the three pieces carry x to about 2^-26
// relative.  A product a b is formed from the six piece products of order
// <= 2 (a0b0, a0b1, a1b0, a0b2, a1b1, a2b0): every dropped term is below
// 2^-26 |a||b|, so a GEMM made of six bf16 MMAs with FP32 accumulation in TMEM
// is as accurate as an FP32 SIMT GEMM.  bf16 keeps FP32's exponent range, so
// no operand scaling is needed.
//
// Complex products run as real GEMMs on an embedding: a complex m x k times
// k x n product is a real m x 2k times 2k x 2n product whose A rows are the
// interleaved (re, im) rows of A and whose B columns come in pairs
// (conj(b), i conj(b)) -- see tcgemm.cu.
//
// Shared-memory tiles use the 128-byte swizzle (the canonical UMMA layout
// SWIZZLE_128B): a tile is a stack of 1024-byte atoms, each 8 rows of 128
// bytes, and the 16-byte chunk c of row r of an atom is stored at chunk
// c ^ (r & 7).  The same bytes read as a K-major operand (rows = M or N,
// 64 bf16 of K per row) or as an MN-major operand (rows = K, 64 bf16 of M or
// N per row).
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "common.cuh"

namespace mps {
namespace tc {

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

// ---------------------------------------------------------------------------
// bf16 split.
struct Split3 {
    __nv_bfloat16 p0, p1, p2;
};
__device__ __forceinline__ Split3 split3(float x) {
    Split3 s;
    s.p0 = __float2bfloat16_rn(x);
    const float r1 = x - __bfloat162float(s.p0);
    s.p1 = __float2bfloat16_rn(r1);
    const float r2 = r1 - __bfloat162float(s.p1);
    s.p2 = __float2bfloat16_rn(r2);
    return s;
}

// Byte offset of element k (bf16) of row r in a SW128 tile whose rows are
// 128 bytes (64 bf16) and whose 8-row atoms are consecutive (1024 bytes).
__device__ __forceinline__ uint32_t sw128_off(int r, int k) {
    const uint32_t o = (uint32_t)r * 128u + (uint32_t)k * 2u;
    return o ^ (((uint32_t)r & 7u) << 4);
}

// ---------------------------------------------------------------------------
// Descriptors.
//
// Shared-memory matrix descriptor (64 bits): start address >> 4 in [0,14),
// leading-dimension byte offset >> 4 in [16,30), stride-dimension byte
// offset >> 4 in [32,46), descriptor version 1 in [46,48), base offset 0 in
// [49,52), layout type in [61,64) (2 = SWIZZLE_128B).
// K-major SW128: SBO = byte distance between consecutive 8-row groups (1024
// for densely stacked atoms); LBO is not used.  MN-major SW128: LBO = byte
// distance between consecutive 64-element groups along M/N, SBO = byte
// distance between consecutive 8-row groups along K.
__device__ __forceinline__ uint64_t sdesc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
    d |= (uint64_t)1u << 46;
    d |= (uint64_t)2u << 61;
    return d;
}

// The descriptor of the operand byte_off bytes further (a multiple of 16):
// the start address field is linear and, for shared memory below 256 KB,
// never carries out of its 14 bits.
__device__ __forceinline__ uint64_t sdesc_add(uint64_t d, uint32_t byte_off) {
    return d + (uint64_t)(byte_off >> 4);
}

// Instruction descriptor of tcgen05.mma.kind::f16 with bf16 A and B and an
// FP32 accumulator: D format F32 (1) at [4,6), A format BF16 (1) at [7,10),
// B format BF16 (1) at [10,13), A / B MN-major flags at bits 15 / 16,
// N >> 3 at [17,23), M >> 4 at [24,29).
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, bool a_mn, bool b_mn) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((a_mn ? 1u : 0u) << 15) |
           ((b_mn ? 1u : 0u) << 16) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// ---------------------------------------------------------------------------
// TMEM.  Allocation and release are warp-wide (.sync.aligned): one whole
// warp calls them.  The allocated base address is written to *dst (shared).
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                     smem_u32(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols)
                 : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Makes this thread's generic-proxy shared-memory writes visible to the
// async proxy (the tensor core and TMA read shared memory through it).
__device__ __forceinline__ void fence_async_smem() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// D (TMEM) = A B (+ D when acc != 0); A and B in shared memory.
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                         uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}

// The mbarrier receives one arrival when every MMA this thread issued so far
// has completed (and its shared-memory reads are done).
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

// 32 consecutive 32-bit TMEM columns of this thread's lane (32x32b shape:
// warp w of a warpgroup reads lanes 32 (w % 4) .. 32 (w % 4) + 31).
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float* v) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

// The same for 16 columns.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ---------------------------------------------------------------------------
// 16-byte asynchronous global -> shared copy (L2 only); bytes beyond
// src_bytes (0 or 16) are filled with zeros.  Both addresses 16-byte aligned.
__device__ __forceinline__ void cp_async16(void* sdst, const void* gsrc, uint32_t src_bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(sdst)), "l"(gsrc),
                 "r"(src_bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
    asm volatile("cp.async.commit_group;" ::: "memory");
}
// Waits for all of this thread's cp.async groups.
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_group 0;" ::: "memory");
}

// ---------------------------------------------------------------------------
// mbarrier phase wait with an iteration limit; returns false when it ran out.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, unsigned parity, int limit) {
    for (int it = 0; it < limit; ++it)
        if (mbar_try_wait(bar, parity, 20000u)) return true;
    return false;
}

// Sets the expected transaction bytes of this phase and arrives (one arrival).
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile(
        "{\n\t.reg .b64 st;\n\t"
        "mbarrier.arrive.expect_tx.shared::cta.b64 st, [%0], %1;\n\t}" ::"r"(smem_u32(bar)),
        "r"(bytes)
        : "memory");
}

// TMA 1D bulk copy global -> shared (16-byte aligned addresses, size a multiple
// of 16), completing on the mbarrier's transaction count.
__device__ __forceinline__ void bulk_g2s(void* sdst, const void* gsrc, uint32_t bytes,
                                         uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
            "r"(smem_u32(sdst)),
        "l"(gsrc), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// TMA tiled 2D load through a tensor map (cuTensorMapEncodeTiled), completing
// on the mbarrier's transaction count.  c0 is the innermost coordinate.
__device__ __forceinline__ void tma_load_2d(void* sdst, const void* tmap, int c0, int c1,
                                            uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes "
        "[%0], [%1, {%2, %3}], [%4];" ::"r"(smem_u32(sdst)),
        "l"(tmap), "r"(c0), "r"(c1), "r"(smem_u32(bar))
        : "memory");
}

}  // namespace tc
}  // namespace mps
