// letkf_umma.cuh -- Blackwell tensor-core building blocks (tcgen05 + TMEM) in
// inline PTX: TMEM allocation, shared-memory matrix descriptors for K-major
// 128-byte-swizzled 16-bit (BF16 or FP16) tiles, the MMA issue, commit to an
// mbarrier, bounded mbarrier waits, TMEM loads and stores.
//
// Tile convention (K-major, SWIZZLE_128B, 16-bit elements): a tile holds R rows
// (R a multiple of 8) of 64 elements (128 bytes) along K.  Row r, 16-byte chunk
// c (elements 8c..8c+7) lives at
//     base + (r / 8) * 1024 + (r % 8) * 128 + ((c ^ (r % 8)) * 16)
// with base 1024-byte aligned.  Consecutive 8-row groups are 1024 bytes apart
// (the descriptor's stride byte offset); one MMA consumes 16 elements of K, so
// the k-th step of a 64-wide tile starts 32*k bytes after the tile base.
#pragma once

#include <stdint.h>

#ifndef LG_MBAR_SPIN_LIMIT
#define LG_MBAR_SPIN_LIMIT (1u << 22)
#endif

__device__ __forceinline__ uint32_t lg_smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ uint32_t lg_sw128_offset(int r, int c)
{
    return (uint32_t)((r >> 3) * 1024 + (r & 7) * 128 + (((c ^ (r & 7)) & 7) << 4));
}

// Shared-memory matrix descriptor: start address, stride byte offset 1024
// (8-row groups), leading byte offset unused for swizzled K-major tiles,
// descriptor version 1, 128-byte swizzle.
__device__ __forceinline__ uint64_t lg_desc_sw128(uint32_t smem_addr)
{
    uint64_t d = 0;
    d |= (uint64_t)((smem_addr & 0x3FFFFu) >> 4);
    d |= (uint64_t)1 << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= (uint64_t)1 << 46;
    d |= (uint64_t)2 << 61;
    return d;
}

// Instruction descriptor of kind::f16 with BF16 A and B, FP32 accumulator,
// both operands K-major, M x N.
__host__ __device__ constexpr uint32_t lg_idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}

// The same with FP16 A and B (type fields 0).
__host__ __device__ constexpr uint32_t lg_idesc_f16(int M, int N)
{
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void lg_tmem_alloc(uint32_t dst_smem, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(dst_smem),
                 "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void lg_tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

__device__ __forceinline__ void lg_tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;"); }
__device__ __forceinline__ void lg_tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;"); }

// Make generic-proxy shared-memory writes visible to the tensor core.
__device__ __forceinline__ void lg_fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;"); }

__device__ __forceinline__ void lg_mbar_init(uint64_t *mbar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(lg_smem_u32(mbar)), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;");
}

// Wait for phase `parity` of the mbarrier, at most `limit` polls (the
// kernels pass LG_MBAR_SPIN_LIMIT unless a context set another limit; 0 gives
// up at once).  Returns false if the wait ran out.
__device__ __forceinline__ bool lg_mbar_wait(uint64_t *mbar, uint32_t parity, uint32_t limit = LG_MBAR_SPIN_LIMIT)
{
    const uint32_t addr = lg_smem_u32(mbar);
    for (uint32_t i = 0; i < limit; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n"
            " selp.u32 %0, 1, 0, P;\n}\n"
            : "=r"(done)
            : "r"(addr), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// D[tmem] (+)= A * B^T for one K step of 16 BF16 or FP16 elements (the
// instruction descriptor gives the type of both operands).
__device__ __forceinline__ void lg_umma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc,
                                             uint32_t idesc, uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// Arrive on the mbarrier when every previously issued MMA of this thread is done.
__device__ __forceinline__ void lg_umma_commit(uint64_t *mbar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
                     lg_smem_u32(mbar))
                 : "memory");
}

// Load 16 consecutive 32-bit columns of this thread's TMEM lane.
__device__ __forceinline__ void lg_tmem_ld16(uint32_t taddr, float *v)
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

// Load 16 consecutive 32-bit columns at each of two TMEM addresses of this
// thread's lane, with one wait (in the same statement, so nothing reads the
// registers before the loads are done).
__device__ __forceinline__ void lg_tmem_ld16x2(uint32_t ta, uint32_t tb, float *va, float *vb)
{
    uint32_t a[16], b[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%32];\n"
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%33];\n"
        "tcgen05.wait::ld.sync.aligned;"
        : "=r"(a[0]), "=r"(a[1]), "=r"(a[2]), "=r"(a[3]), "=r"(a[4]), "=r"(a[5]), "=r"(a[6]), "=r"(a[7]),
          "=r"(a[8]), "=r"(a[9]), "=r"(a[10]), "=r"(a[11]), "=r"(a[12]), "=r"(a[13]), "=r"(a[14]), "=r"(a[15]),
          "=r"(b[0]), "=r"(b[1]), "=r"(b[2]), "=r"(b[3]), "=r"(b[4]), "=r"(b[5]), "=r"(b[6]), "=r"(b[7]),
          "=r"(b[8]), "=r"(b[9]), "=r"(b[10]), "=r"(b[11]), "=r"(b[12]), "=r"(b[13]), "=r"(b[14]), "=r"(b[15])
        : "r"(ta), "r"(tb)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) {
        va[i] = __uint_as_float(a[i]);
        vb[i] = __uint_as_float(b[i]);
    }
}

// Store 16 consecutive 32-bit columns of this thread's TMEM lane and wait
// until the stores are done.
__device__ __forceinline__ void lg_tmem_st16(uint32_t taddr, const float *v)
{
    asm volatile(
        "tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16};"
        ::"r"(taddr), "r"(__float_as_uint(v[0])), "r"(__float_as_uint(v[1])), "r"(__float_as_uint(v[2])),
        "r"(__float_as_uint(v[3])), "r"(__float_as_uint(v[4])), "r"(__float_as_uint(v[5])),
        "r"(__float_as_uint(v[6])), "r"(__float_as_uint(v[7])), "r"(__float_as_uint(v[8])),
        "r"(__float_as_uint(v[9])), "r"(__float_as_uint(v[10])), "r"(__float_as_uint(v[11])),
        "r"(__float_as_uint(v[12])), "r"(__float_as_uint(v[13])), "r"(__float_as_uint(v[14])),
        "r"(__float_as_uint(v[15]))
        : "memory");
    asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory");
}
