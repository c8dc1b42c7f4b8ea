// tc.cuh -- thin inline-PTX wrappers for the Blackwell tensor-core path used by the
// guiding network: mbarriers, tensor memory (TMEM) allocation, tcgen05.mma with
// shared-memory operand descriptors, tcgen05.commit and tcgen05.ld.
//
// Operand layout used throughout: bf16 matrices in shared memory in the canonical
// K-major layout without swizzling -- "core matrices" of 8 rows x 8 elements (8 x 16
// bytes, rows 16 bytes apart, 128 contiguous bytes), tiled [rows/8][K/8]:
//   byte offset of element (r, k) = ((r / 8) * (K / 8) + k / 8) * 128 + (r % 8) * 16 + (k % 8) * 2
// so core matrices adjacent along K are 128 bytes apart (leading byte offset) and those
// adjacent along rows are K/8 * 128 bytes apart (stride byte offset).  One
// tcgen05.mma of kind::f16 consumes K = 16, i.e. two core matrices along K.
//
// The same tile read as the transpose (an MN-major operand, instruction-descriptor
// transpose bits): its rows become the MMA's K and its columns the MMA's M (or N).  For
// MN-major operands without swizzling the stride byte offset is the distance between
// core matrices along M (N) -- 128 bytes here -- and the leading byte offset the
// distance between core matrices along K -- cols/8 * 128 bytes here.
//
// Accumulator placement in tensor memory (cta_group::1): for M = 128, row r is lane r;
// for M = 64, rows 16w .. 16w + 15 are lanes 32w .. 32w + 15 (lanes 0-15 of each warp's
// quarter), columns 0 .. N-1 in both cases.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace spgpu {
namespace tc {

__device__ __forceinline__ uint32_t smemAddr(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of bf16 element (r, k) in a [rows][K] K-major canonical tile
__host__ __device__ __forceinline__ uint32_t kmajorOffset(uint32_t r, uint32_t k, uint32_t K) {
    return ((r >> 3) * (K >> 3) + (k >> 3)) * 128u + (r & 7u) * 16u + (k & 7u) * 2u;
}

// ---------------------------------------------------------------- mbarrier
__device__ __forceinline__ void mbarInit(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smemAddr(bar)), "r"(count) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");   // visible to the async proxy
}
__device__ __forceinline__ bool mbarTryWait(uint64_t *bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smemAddr(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}
// Bounded wait: false if the phase did not complete within maxTries polls.
__device__ __forceinline__ bool mbarWait(uint64_t *bar, uint32_t phase, uint32_t maxTries) {
    for (uint32_t i = 0; i < maxTries; i++)
        if (mbarTryWait(bar, phase)) return true;
    return false;
}

// ---------------------------------------------------------------- bulk copies (TMA)
// One thread: announce `bytes` of transfer on *bar (its arrival for this phase) ...
__device__ __forceinline__ void mbarExpectTx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smemAddr(bar)), "r"(bytes)
                 : "memory");
}
// ... and copy global -> shared with the tensor memory accelerator; the bytes complete
// on *bar.  dst, src 16-byte aligned, bytes a multiple of 16.
__device__ __forceinline__ void bulkLoad(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smemAddr(dst)),
        "l"(src), "r"(bytes), "r"(smemAddr(bar))
        : "memory");
}

// ---------------------------------------------------------------- TMEM
// Executed by one full warp.  The allocated column base is written to *dst (shared).
__device__ __forceinline__ void tmemAlloc(uint32_t *dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smemAddr(dst)),
                 "r"(ncols)
                 : "memory");
}
__device__ __forceinline__ void tmemRelinquish() {
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmemDealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

// ---------------------------------------------------------------- fences
__device__ __forceinline__ void fenceAsyncShared() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fenceBeforeSync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fenceAfterSync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// ---------------------------------------------------------------- descriptors
// Shared-memory matrix descriptor: start address, leading / stride byte offsets (all
// >> 4), descriptor version 1, no swizzling.
__device__ __forceinline__ uint64_t smemDesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return static_cast<uint64_t>((addr >> 4) & 0x3FFFu) | (static_cast<uint64_t>((lbo >> 4) & 0x3FFFu) << 16) |
           (static_cast<uint64_t>((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
// Instruction descriptor of kind::f16: D f32, A and B bf16, both K-major, M x N.
__host__ __device__ constexpr uint32_t instrDescBf16(uint32_t M, uint32_t N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((N >> 3) << 17) | ((M >> 4) << 24);
}

// instruction-descriptor bits: A (B) is read MN-major, i.e. transposed
constexpr uint32_t kTransposeA = 1u << 15;
constexpr uint32_t kTransposeB = 1u << 16;

// D[tmem] (+)= A * B, issued by a single thread
__device__ __forceinline__ void mmaBf16(uint32_t dTmem, uint64_t aDesc, uint64_t bDesc, uint32_t idesc,
                                        uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dTmem),
        "l"(aDesc), "l"(bDesc), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrive on *bar once all previously issued MMAs of this thread have completed
__device__ __forceinline__ void mmaCommit(uint64_t *bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smemAddr(bar))
                 : "memory");
}

// TMEM -> registers: this warp's 32 lanes, 16 consecutive 32-bit columns each
__device__ __forceinline__ void tmemLoad16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

}  // namespace tc
}  // namespace spgpu
