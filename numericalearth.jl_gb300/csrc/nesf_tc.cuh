// nesf_tc.cuh -- the 5th-generation tensor-core (tcgen05) pieces of the warm-start
// network: TMEM allocation, BF16 MMAs with FP32 accumulation into TMEM, their
// completion through an mbarrier, and TMEM loads. Inline PTX for sm_103a.
//
// Operand layout in shared memory ("blocked"): a matrix with R rows and C columns,
// the C direction contiguous, is stored as 8 x 8 BF16 core matrices of 128 bytes
// (8 rows of 16 bytes); core matrix (rg, cg) starts at (cg * R / 8 + rg) * 128.
// In a descriptor without swizzling the leading byte offset (LBO) is the stride
// between core matrices along K and the stride byte offset (SBO) the stride along
// M (or N), for K-major and MN-major operands alike (checked against host GEMMs by
// nesf_mlp_selftest). The same bytes serve as a K-major operand (columns = K) and
// as an MN-major one (columns = M or N), which is how the backward pass reuses the
// forward activations and weights; `blocked_lbo` / `blocked_sbo` give the two
// offsets and `blocked_kstep` the advance per K = 16 slice.
//
// Every wait on an mbarrier is bounded: after kSpinLimit polls the caller gets
// `false`, records an error and leaves.
#pragma once

#include <cstdint>
#include <cuda_bf16.h>

namespace nesf {
namespace tc {

constexpr int kSpinLimit = 1 << 22;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// ------------------------------------------------------------ descriptors
// Shared-memory matrix descriptor: start address, LBO and SBO (each >> 4), the
// sm_100 descriptor version (bits 46-47 = 1), no swizzle, base offset 0.
__host__ __device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((addr >> 4) & 0x3FFF);
    d |= (uint64_t)((lbo >> 4) & 0x3FFF) << 16;
    d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// Instruction descriptor of tcgen05.mma .kind::f16: D in FP32, A and B in BF16,
// a_major / b_major = 0 for K-major, 1 for MN-major, N and M in units of 8 and 16.
__host__ __device__ __forceinline__ uint32_t idesc_bf16(int M, int N, int a_mn_major, int b_mn_major) {
    uint32_t d = 0;
    d |= 1u << 4;                          // D format: F32
    d |= 1u << 7;                          // A format: BF16
    d |= 1u << 10;                         // B format: BF16
    d |= (uint32_t)(a_mn_major & 1) << 15;
    d |= (uint32_t)(b_mn_major & 1) << 16;
    d |= (uint32_t)((N >> 3) & 0x3F) << 17;
    d |= (uint32_t)((M >> 4) & 0x1F) << 24;
    return d;
}

// Descriptor offsets of an R-row blocked matrix whose columns are K (k_is_col) or
// whose rows are K.
__host__ __device__ __forceinline__ uint32_t blocked_lbo(int R, bool k_is_col) {
    return k_is_col ? (uint32_t)(R / 8 * 128) : 128u;
}
__host__ __device__ __forceinline__ uint32_t blocked_sbo(int R, bool k_is_col) {
    return k_is_col ? 128u : (uint32_t)(R / 8 * 128);
}
__host__ __device__ __forceinline__ uint32_t blocked_kstep(int R, bool k_is_col) {
    return k_is_col ? (uint32_t)(2 * (R / 8) * 128) : 256u;
}

// Byte offset of element (r, c) in the blocked layout of an R-row matrix.
__host__ __device__ __forceinline__ uint32_t blocked_offset(int r, int c, int R) {
    return (uint32_t)(((c >> 3) * (R >> 3) + (r >> 3)) * 128 + (r & 7) * 16 + (c & 7) * 2);
}

// ------------------------------------------------------------------ TMEM
// Allocate `ncols` TMEM columns (a power of two >= 32); the whole warp calls it.
// The base address is written to *slot (shared memory).
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_addr(slot)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void fence_after_sync() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Make generic-proxy shared-memory writes visible to the tensor core.
__device__ __forceinline__ void fence_smem_to_async() {
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// ------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

// Bounded wait for the phase with the given parity to complete: false after
// `limit` polls.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int limit = kSpinLimit) {
    uint32_t a = smem_addr(bar);
    for (int i = 0; i < limit; i++) {
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

// ------------------------------------------------------------------ MMA
// D[128 x N] (TMEM) (+)= A x B, one K = 16 slice; issued by one thread.
__device__ __forceinline__ void mma_bf16(uint32_t dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// Arrive on `bar` once every MMA issued so far by this thread has completed.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     smem_addr(bar))
                 : "memory");
}

// K-slices of one GEMM: the descriptors advance by a_step / b_step bytes per slice.
__device__ __forceinline__ void mma_chain(uint32_t dtmem, uint32_t a_addr, uint32_t a_lbo, uint32_t a_sbo,
                                          uint32_t a_step, uint32_t b_addr, uint32_t b_lbo, uint32_t b_sbo,
                                          uint32_t b_step, uint32_t idesc, int ksteps, bool accumulate) {
    for (int k = 0; k < ksteps; k++) {
        uint64_t ad = smem_desc(a_addr + k * a_step, a_lbo, a_sbo);
        uint64_t bd = smem_desc(b_addr + k * b_step, b_lbo, b_sbo);
        mma_bf16(dtmem, ad, bd, idesc, (accumulate || k > 0) ? 1u : 0u);
    }
}

// ------------------------------------------------------------ TMEM loads
// Thread t of warp w (w = warp index within the 4-warp group) receives row
// 32 w + t, columns [col, col + 16) of the 128-lane accumulator at `taddr`.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// TMEM address of lane 32 w, column `col`, from the allocation base.
__device__ __forceinline__ uint32_t tmem_at(uint32_t base, int warp, int col) {
    return base + ((uint32_t)(32 * warp) << 16) + (uint32_t)col;
}

}  // namespace tc
}  // namespace nesf
