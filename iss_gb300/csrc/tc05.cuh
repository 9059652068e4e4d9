// Blackwell (sm_103a) tensor-core building blocks in inline PTX: tensor
// memory (TMEM) allocation, tcgen05.mma with operands in shared memory,
// completion through an mbarrier, and TMEM -> register loads.
//
// Operand layout in shared memory: the canonical K-major layout without
// swizzling.  A tile of R rows (M or N) by K bf16 columns is a grid of "core
// matrices" of 8 rows x 8 columns (8 rows of 16 bytes, 128 bytes each);
// core matrix (r / 8, k / 8) starts at byte ((r / 8) * (K / 8) + k / 8) * 128,
// so the leading-dimension byte offset (next core matrix along K) is 128 and
// the stride-dimension byte offset (next 8-row group) is K / 8 * 128.
//
// Every wait on an mbarrier is bounded (wall clock, from %globaltimer): a
// wait that runs out sets an error flag and returns false, the caller stops
// issuing work and frees its TMEM.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace iss {
namespace tc05 {

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) of a K-major tile with K columns (K % 8 == 0)
__host__ __device__ __forceinline__ uint32_t kmajor_offset(int r, int k, int K) {
    return static_cast<uint32_t>((((r >> 3) * (K >> 3) + (k >> 3)) << 7) + ((r & 7) << 4) +
                                 ((k & 7) << 1));
}

// shared-memory matrix descriptor (tcgen05 format): start address, leading-
// and stride-dimension byte offsets (all >> 4), version 1, no swizzling
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = static_cast<uint64_t>((saddr & 0x3FFFFu) >> 4);
    d |= static_cast<uint64_t>((lbo & 0x3FFFFu) >> 4) << 16;
    d |= static_cast<uint64_t>((sbo & 0x3FFFFu) >> 4) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    return d;
}

// descriptor of the 16-column K slice `ks` of a K-major tile at saddr
__device__ __forceinline__ uint64_t kslice_desc(uint32_t saddr, int K, int ks) {
    return smem_desc(saddr + static_cast<uint32_t>(ks) * 256u, 128u,
                     static_cast<uint32_t>(K >> 3) << 7);
}

// instruction descriptor of kind::f16: bf16 A and B, both K-major, FP32 accumulator
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
           (static_cast<uint32_t>(M >> 4) << 24);
}

// ---- TMEM allocation (one full warp executes these) ----------------------
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;"
                 :: "r"(smem_addr(dst)), "r"(ncols) : "memory");
}
__device__ __forceinline__ void tmem_relinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" :: "r"(taddr), "r"(ncols)
                 : "memory");
}

// ---- ordering ------------------------------------------------------------
// generic-proxy shared-memory writes become visible to the tensor core
__device__ __forceinline__ void fence_smem_to_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// ---- MMA -------------------------------------------------------------------
// D[tmem] (+)= A[smem] * B[smem]^T for one 16-deep K slice
__device__ __forceinline__ void mma_bf16(uint32_t d_tmem, uint64_t a_desc, uint64_t b_desc,
                                         uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}"
        :: "r"(d_tmem), "l"(a_desc), "l"(b_desc), "r"(idesc), "r"(accumulate) : "memory");
}
// the mbarrier receives one arrival when all MMAs issued so far have completed
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];"
                 :: "r"(smem_addr(bar)) : "memory");
}

// ---- mbarrier ----------------------------------------------------------------
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count)
                 : "memory");
}
__device__ __forceinline__ void mbar_inval(uint64_t* bar) {
    asm volatile("mbarrier.inval.shared::cta.b64 [%0];" :: "r"(smem_addr(bar)) : "memory");
}
__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
// waits for the phase with the given parity to complete; false after about
// limit_ns of wall-clock time (or 2^26 polls), with *err set to code
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int* err, int code,
                                          uint64_t limit_ns = 1000000000ull) {
    const uint32_t a = smem_addr(bar);
    const uint64_t t0 = global_ns();
    for (uint32_t it = 0; it < (1u << 26); it++) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok) : "r"(a), "r"(parity) : "memory");
        if (ok) return true;
        if ((it & 63u) == 63u && global_ns() - t0 > limit_ns) break;
    }
    if (err) atomicCAS(err, 0, code);
    return false;
}

// ---- TMEM -> registers -------------------------------------------------------
// 32 consecutive FP32 columns of this thread's lane (32x32b shape: warp w of
// the warpgroup reads lanes 32 (w % 4) .. +31); the load and its wait are one
// asm statement, so no use of the registers can move above the wait
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n\t"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]),
          "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]),
          "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

// the same load without its wait: two of them can be in flight before one
// tmem_wait_ld()
__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, uint32_t (&r)[32]) {
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
}
__device__ __forceinline__ void tmem_wait_ld() {
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

// TMEM address of (lane 32 * (warp % 4), column col)
__device__ __forceinline__ uint32_t tmem_lane_addr(uint32_t base, int warp, int col) {
    return base + (static_cast<uint32_t>((warp & 3) * 32) << 16) + static_cast<uint32_t>(col);
}

}  // namespace tc05
}  // namespace iss
