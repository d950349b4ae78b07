// Blackwell fifth-generation tensor-core primitives (tcgen05, sm_100a/sm_103a)
// as inline PTX: tensor-memory allocation, BF16 MMA with FP32 accumulators in
// tensor memory, commit to an mbarrier, tensor-memory loads and the fences
// that order them against ordinary thread synchronisation.
//
// Operand tiles live in shared memory in the canonical K-major layout without
// swizzle: the tile is cut into "core matrices" of 8 rows x 8 elements (16-bit
// elements, 8 rows x 16 bytes = 128 contiguous bytes).  This file stores the
// core matrices of a tile with R rows and K columns K-group outer:
//     byte offset of element (r, k) = ((k/8) * (R/8) + r/8) * 128 + (r%8) * 16 + (k%8) * 2
// so neighbouring row groups are 128 bytes apart (the descriptor's stride
// byte offset, SBO) and neighbouring K groups R*16 bytes apart (its leading
// byte offset, LBO).  One MMA consumes 16 elements of K, i.e. two K groups;
// step s of a K loop starts at byte s * R * 32 of the tile.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace tf {
namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// byte offset of element (r, k) in a tile of R rows (see above)
__host__ __device__ __forceinline__ uint32_t tile_off(int R, int r, int k) {
    return (uint32_t)((((k >> 3) * (R >> 3) + (r >> 3)) << 7) + ((r & 7) << 4) + ((k & 7) << 1));
}

// Shared-memory matrix descriptor: start address, LBO and SBO in units of 16
// bytes, descriptor version 1 (bits 46-47), relative LBO, no swizzle.
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
    uint64_t d = 0;
    d |= (uint64_t)((saddr & 0x3FFFFu) >> 4);
    d |= (uint64_t)((lbo & 0x3FFFFu) >> 4) << 16;
    d |= (uint64_t)((sbo & 0x3FFFFu) >> 4) << 32;
    d |= (uint64_t)1 << 46;
    return d;
}

// descriptor of K-step s (16 elements) of a tile with R rows at saddr
__device__ __forceinline__ uint64_t tile_desc(uint32_t saddr, int R, int s) {
    return smem_desc(saddr + (uint32_t)(s * R * 32), (uint32_t)(R * 16), 128u);
}

// Instruction descriptor of tcgen05.mma kind::f16: BF16 A and B (format 1),
// FP32 accumulator (format 1), both operands K-major, dense, N/8 at bit 17,
// M/16 at bit 24.
__host__ __device__ constexpr uint32_t idesc_bf16_f32(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// D[tmem] (+)= A * B^T for one K-step; issued by a single thread
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

// arrive on mbar when every MMA issued so far by this thread has completed
__device__ __forceinline__ void commit(uint64_t* mbar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
                 : "memory");
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

// Waits for the phase with the given parity to complete; gives up after
// `limit` polls (each poll may itself suspend for a bounded time) and returns
// false then.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, uint32_t limit) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t i = 0; i < limit; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}\n"
            : "=r"(done)
            : "r"(a), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// whole warp: allocate ncols tensor-memory columns, address written to *dst
__device__ __forceinline__ void tmem_alloc(uint32_t* dst, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst)), "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}

// whole warp
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}

__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// make this thread's ordinary shared-memory stores visible to the tensor cores
__device__ __forceinline__ void fence_smem_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Whole warp: 16 consecutive FP32 columns of the warp's 32 tensor-memory lanes;
// lane l of warp w (w = 0..3) receives row 32 w + l.  taddr must carry the
// warp's lane base (32 w) in bits 16..31.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr)
        : "memory");
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

}  // namespace umma
}  // namespace tf
