// vg_umma.cuh -- 5th-generation tensor-core (tcgen05) building blocks for
// sm_100-family GPUs, written from the PTX ISA: TMEM allocation, shared-
// memory matrix descriptors, the BF16 x BF16 -> FP32 MMA, commit to an
// mbarrier, and TMEM -> register loads.
//
// Operand layout used throughout (K-major, 128-byte swizzle): a tile of R
// rows x Kt columns of bf16 is stored as Kt/64 blocks of [R rows x 128 B];
// inside a block, row r's 16-byte chunk c (8 elements) lives at
//     block + r*128 + ((c ^ (r & 7)) * 16),
// every block 1024-byte aligned.  Its descriptor: start address, stride
// byte offset 1024 (8-row groups), leading byte offset 16 (unused for this
// swizzle), version 1, swizzle mode 2 (128 B).  One MMA consumes K = 16
// (32 bytes): the k-th step inside a 64-column block advances the start
// address by 32 bytes.
#pragma once
#include <cuda_bf16.h>
#include <stdint.h>

namespace umma {

__device__ __forceinline__ uint32_t smem_u32(const void *p)
{
    return (uint32_t)__cvta_generic_to_shared(p);
}

// The 1024-byte aligned start of a dynamic shared-memory array, derived by
// pointer arithmetic on the array itself (not through an integer), so that
// the compiler keeps shared-space addressing (32-bit, LDS / STS) for every
// pointer into it.
__device__ __forceinline__ uint8_t *align1024(uint8_t *dsm)
{
    return dsm + ((1024u - (smem_u32(dsm) & 1023u)) & 1023u);
}

// byte offset of element (r, k) inside a K-major SW128 tile of R rows
__device__ __forceinline__ uint32_t sw128_offset(int R, int r, int k)
{
    const int blk = k >> 6, c = (k & 63) >> 3;
    return (uint32_t)(blk * R * 128 + r * 128 + ((c ^ (r & 7)) << 4) + ((k & 7) << 1));
}

__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(16u >> 4) << 16) |
           ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) | (2ull << 61);
}

// instruction descriptor: D f32, A/B bf16, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N)
{
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

// --- TMEM allocation (one full warp executes these) ---
__device__ __forceinline__ void tmem_alloc(uint32_t slot_saddr, uint32_t ncols)
{
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot_saddr), "r"(ncols));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
}

__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols)
{
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols));
}

// --- mbarrier ---
__device__ __forceinline__ void mbar_init(uint32_t bar, uint32_t count)
{
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count));
    asm volatile("fence.mbarrier_init.release.cluster;");
}

// Bounded wait for the phase with the given parity to complete.  Returns
// false when the bound ran out (the caller records an error and winds down).
__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity, uint32_t max_iter = 1u << 22)
{
    for (uint32_t i = 0; i < max_iter; i++) {
        uint32_t done;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
            " selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(done)
            : "r"(bar), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// --- fences ---
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// --- MMA (one thread issues) ---
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         uint32_t accumulate)
{
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate));
}

// arrive on the mbarrier once every MMA issued so far by this thread completed
__device__ __forceinline__ void mma_commit(uint32_t bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                 : "memory");
}

// D[128 x N] (+)= A[128 x Kt] * B[N x Kt]^T; A, B K-major SW128 tiles at saddr
// (1024-aligned), issued as Kt/16 MMAs.  N <= 256, N % 16 == 0.
__device__ __forceinline__ void gemm_128xN(uint32_t tmem_d, uint32_t a_saddr, uint32_t b_saddr, int N,
                                           int Kt, int rowsB, uint32_t accumulate)
{
    const uint32_t idesc = idesc_bf16(128, N);
    for (int k = 0; k < Kt; k += 16) {
        const uint32_t aoff = (uint32_t)((k >> 6) * 128 * 128 + ((k & 63) << 1));
        const uint32_t boff = (uint32_t)((k >> 6) * rowsB * 128 + ((k & 63) << 1));
        mma_bf16(tmem_d, sdesc_sw128(a_saddr + aoff), sdesc_sw128(b_saddr + boff), idesc,
                 (k > 0 || accumulate) ? 1u : 0u);
    }
}

// General form with either operand K-major or MN-major.  An MN-major operand
// X (MN x Kt) is the SW128 tile of its transpose: R rows of MN elements (R >=
// Kt, the first Kt used), i.e. what sw128_offset(R, k, mn) addresses; its
// descriptor steps 64-element MN blocks by LBO = R * 128 bytes and 8-row K
// groups by SBO = 1024 bytes, and a K step of 16 advances the start by 16
// rows (2048 bytes).  a_rows / b_rows: the K-major tile's row count (the
// stride of its 64-column blocks), or R of an MN-major tile (0: R = Kt).
__device__ __forceinline__ uint64_t sdesc_sw128_lbo(uint32_t saddr, uint32_t lbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)(1024u >> 4) << 32) | (1ull << 46) | (2ull << 61);
}

__device__ __forceinline__ void gemm_128xN_ex(uint32_t tmem_d, uint32_t a_saddr, int a_mn, int a_rows,
                                              uint32_t b_saddr, int b_mn, int b_rows, int N, int Kt,
                                              uint32_t accumulate)
{
    const uint32_t idesc = idesc_bf16(128, N) | ((uint32_t)(a_mn ? 1 : 0) << 15) | ((uint32_t)(b_mn ? 1 : 0) << 16);
    for (int k = 0; k < Kt; k += 16) {
        uint64_t ad, bd;
        if (a_mn) ad = sdesc_sw128_lbo(a_saddr + (uint32_t)k * 128u, (uint32_t)(a_rows > 0 ? a_rows : Kt) * 128u);
        else ad = sdesc_sw128(a_saddr + (uint32_t)((k >> 6) * a_rows * 128 + ((k & 63) << 1)));
        if (b_mn) bd = sdesc_sw128_lbo(b_saddr + (uint32_t)k * 128u, (uint32_t)(b_rows > 0 ? b_rows : Kt) * 128u);
        else bd = sdesc_sw128(b_saddr + (uint32_t)((k >> 6) * b_rows * 128 + ((k & 63) << 1)));
        mma_bf16(tmem_d, ad, bd, idesc, (k > 0 || accumulate) ? 1u : 0u);
    }
}

// --- TMEM -> registers: 32 lanes x 32 bit, 16 consecutive columns.  The load
// and its wait sit in one asm statement, so no instruction can read the
// destination registers before the asynchronous load completed.
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16])
{
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]),
          "=r"(r[15])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr)
        : "memory");
#pragma unroll
    for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ float tmem_ld1(uint32_t taddr)
{
    uint32_t r;
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];\n"
        "tcgen05.wait::ld.sync.aligned;\n"
        : "=r"(r)
        : "r"(taddr)
        : "memory");
    return __uint_as_float(r);
}

// --- bulk global -> shared copy completing on an mbarrier (TMA, non-tensor).
// Addresses 16-byte aligned, size a multiple of 16.
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes)
{
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar)
{
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// --- bulk shared -> global copy in a bulk async-group (one thread issues).
// The threads that wrote the source execute fence_async_smem() and a CTA
// barrier first.  bulk_wait_read() returns once every committed group has
// finished reading shared memory (the source may then be overwritten);
// bulk_wait_all() once the global writes are complete as well.
__device__ __forceinline__ void bulk_s2g(void *dst, uint32_t src, uint32_t bytes)
{
    asm volatile("cp.async.bulk.global.shared::cta.bulk_group [%0], [%1], %2;" ::"l"(dst), "r"(src), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

}  // namespace umma
