// Blackwell (sm_103a) primitives for the tensor-memory pass: mbarriers with
// bounded waits, tcgen05 tensor-memory allocation, loads/stores and MMAs,
// shared-memory matrix descriptors, and TMA tensor copies. Inline PTX only.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hqs {
namespace tc05 {

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// ------------------------------------------------------------------ mbarrier
__device__ __forceinline__ void mbar_init(uint64_t* m, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(m)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ bool mbar_try(uint64_t* m, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
        : "=r"(ok)
        : "r"(smem_u32(m)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void mbar_arrive(uint64_t* m) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(m)) : "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* m, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(m)), "r"(bytes) : "memory");
}

__device__ __forceinline__ uint64_t globaltimer_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wait for the phase with the given parity to complete. Bounded in time:
// after kWaitNs nanoseconds (far above any legitimate wait of the pass, which
// is one tile's copy or compute time, microseconds) it raises *abort and
// returns false; it also returns false as soon as another thread of the CTA
// has raised *abort. The caller then leaves its loop.
constexpr uint64_t kWaitNs = 2000000000ULL;
__device__ __forceinline__ bool mbar_wait(uint64_t* m, uint32_t parity, volatile int* abort) {
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t i = 0;; ++i) {
        if (mbar_try(m, parity)) return true;
        if ((i & 63u) == 63u) {
            if (*abort) return false;
            if (globaltimer_ns() - t0 > kWaitNs) {
                *abort = 1;
                return false;
            }
        }
    }
}
// The same wait without the abort flag (tear-down: copies or MMAs in flight).
__device__ __forceinline__ bool mbar_wait_quiet(uint64_t* m, uint32_t parity) {
    const uint64_t t0 = globaltimer_ns();
    for (uint32_t i = 0;; ++i) {
        if (mbar_try(m, parity)) return true;
        if ((i & 63u) == 63u && globaltimer_ns() - t0 > kWaitNs) return false;
    }
}

// ------------------------------------------------------------------ fences
__device__ __forceinline__ void fence_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
// generic-proxy shared-memory writes made visible to the async proxy (MMA
// operand reads, TMA stores)
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// named barrier over `count` threads
__device__ __forceinline__ void bar_sync(uint32_t id, uint32_t count) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(count) : "memory");
}

// ------------------------------------------------------------------ tensor memory
// allocate / free: executed by one whole warp
__device__ __forceinline__ void tmem_alloc(uint32_t* dst_smem, uint32_t ncols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(dst_smem)),
                 "r"(ncols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_dealloc(uint32_t taddr, uint32_t ncols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(ncols) : "memory");
}
// eight consecutive 32-bit columns of this thread's lane (32x32b shape: the
// warp's 32 lanes, warp w reaching lanes 32 (w % 4) .. 32 (w % 4) + 31)
__device__ __forceinline__ void tmem_ld8(uint32_t ta, uint32_t (&r)[8]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(ta));
}
__device__ __forceinline__ void tmem_ld_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld4(uint32_t ta, uint32_t (&r)[4]) {
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x4.b32 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(ta));
}
// tcgen05.wait::ld for loads whose registers are still to be used: the
// registers pass through the asm, so no use of them is scheduled before the
// wait (the loads of the next chunk may be in flight while the current one
// is processed)
__device__ __forceinline__ void tmem_ld_wait_regs(uint32_t (&r)[6][4]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0][0]), "+r"(r[0][1]), "+r"(r[0][2]), "+r"(r[0][3]), "+r"(r[1][0]), "+r"(r[1][1]),
                   "+r"(r[1][2]), "+r"(r[1][3]), "+r"(r[2][0]), "+r"(r[2][1]), "+r"(r[2][2]), "+r"(r[2][3]),
                   "+r"(r[3][0]), "+r"(r[3][1]), "+r"(r[3][2]), "+r"(r[3][3]), "+r"(r[4][0]), "+r"(r[4][1]),
                   "+r"(r[4][2]), "+r"(r[4][3]), "+r"(r[5][0]), "+r"(r[5][1]), "+r"(r[5][2]), "+r"(r[5][3])
                 :
                 : "memory");
}
__device__ __forceinline__ void tmem_ld_wait_regs(uint32_t (&r)[4][4]) {
    asm volatile("tcgen05.wait::ld.sync.aligned;"
                 : "+r"(r[0][0]), "+r"(r[0][1]), "+r"(r[0][2]), "+r"(r[0][3]), "+r"(r[1][0]), "+r"(r[1][1]),
                   "+r"(r[1][2]), "+r"(r[1][3]), "+r"(r[2][0]), "+r"(r[2][1]), "+r"(r[2][2]), "+r"(r[2][3]),
                   "+r"(r[3][0]), "+r"(r[3][1]), "+r"(r[3][2]), "+r"(r[3][3])
                 :
                 : "memory");
}
__device__ __forceinline__ void tmem_st8(uint32_t ta, const uint32_t (&r)[8]) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%2,%3,%4,%5,%6,%7,%8};" ::"r"(ta), "r"(r[0]),
                 "r"(r[1]), "r"(r[2]), "r"(r[3]), "r"(r[4]), "r"(r[5]), "r"(r[6]), "r"(r[7])
                 : "memory");
}
__device__ __forceinline__ void tmem_st4(uint32_t ta, uint32_t a, uint32_t b, uint32_t c, uint32_t d) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x4.b32 [%0], {%1,%2,%3,%4};" ::"r"(ta), "r"(a), "r"(b), "r"(c), "r"(d)
                 : "memory");
}
__device__ __forceinline__ void tmem_st_wait() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }

// ------------------------------------------------------------------ MMA
// Shared-memory matrix descriptor of a K-major operand stored with the
// 128-byte swizzle: rows of 64 fp16 (128 B), 8-row groups 1024 B apart, the
// 16-byte chunk c of row r stored at chunk c ^ (r % 8) (the atom must be
// 1024-byte aligned). A K16 step further along the row adds 32 B to the start.
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t saddr) {
    uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
    d |= (uint64_t)1 << 16;              // leading byte offset (unused with this swizzle)
    d |= (uint64_t)(1024 >> 4) << 32;    // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;              // descriptor version
    d |= (uint64_t)2 << 61;              // 128-byte swizzle
    return d;
}
// Instruction descriptor: fp16 A and B, both K-major, fp32 accumulators, M x N.
__host__ __device__ constexpr uint32_t idesc_f16(int M, int N) {
    return (1u << 4) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// D (tensor memory) (+)= A (tensor memory) * B (shared memory)^T
__device__ __forceinline__ void mma_ts(uint32_t d, uint32_t a, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], [%1], %2, %3, p; }" ::"r"(d),
        "r"(a), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
// D (tensor memory) (+)= A (shared memory) * B (shared memory)^T
__device__ __forceinline__ void mma_ss(uint32_t d, uint64_t adesc, uint64_t bdesc, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{ .reg .pred p; setp.ne.b32 p, %4, 0; tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p; }" ::"r"(d),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(acc)
        : "memory");
}
// arrive on the mbarrier once every MMA this thread issued so far has completed
__device__ __forceinline__ void mma_commit(uint64_t* m) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(m))
                 : "memory");
}

// ------------------------------------------------------------------ TMA
// Tensor copies of a box of a tensor map (rank 1..5, coordinates c[0..rank)).
__device__ __forceinline__ void tma_load(void* dst, const void* tmap, const int32_t (&c)[5], int rank, uint64_t* bar) {
    const uint32_t s = smem_u32(dst), b = smem_u32(bar);
    const uint64_t t = reinterpret_cast<uint64_t>(tmap);
    switch (rank) {
        case 1:
            asm volatile("cp.async.bulk.tensor.1d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2}], [%3];"
                         ::"r"(s), "l"(t), "r"(c[0]), "r"(b) : "memory");
            break;
        case 2:
            asm volatile("cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];"
                         ::"r"(s), "l"(t), "r"(c[0]), "r"(c[1]), "r"(b) : "memory");
            break;
        case 3:
            asm volatile("cp.async.bulk.tensor.3d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], [%5];"
                         ::"r"(s), "l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(b) : "memory");
            break;
        case 4:
            asm volatile("cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], [%6];"
                         ::"r"(s), "l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(b) : "memory");
            break;
        default:
            asm volatile("cp.async.bulk.tensor.5d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5, %6}], [%7];"
                         ::"r"(s), "l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4]), "r"(b) : "memory");
            break;
    }
}
__device__ __forceinline__ void tma_store(const void* tmap, const int32_t (&c)[5], int rank, const void* src) {
    const uint32_t s = smem_u32(src);
    const uint64_t t = reinterpret_cast<uint64_t>(tmap);
    switch (rank) {
        case 1:
            asm volatile("cp.async.bulk.tensor.1d.global.shared::cta.tile.bulk_group [%0, {%1}], [%2];"
                         ::"l"(t), "r"(c[0]), "r"(s) : "memory");
            break;
        case 2:
            asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.tile.bulk_group [%0, {%1, %2}], [%3];"
                         ::"l"(t), "r"(c[0]), "r"(c[1]), "r"(s) : "memory");
            break;
        case 3:
            asm volatile("cp.async.bulk.tensor.3d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3}], [%4];"
                         ::"l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(s) : "memory");
            break;
        case 4:
            asm volatile("cp.async.bulk.tensor.4d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4}], [%5];"
                         ::"l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(s) : "memory");
            break;
        default:
            asm volatile("cp.async.bulk.tensor.5d.global.shared::cta.tile.bulk_group [%0, {%1, %2, %3, %4, %5}], [%6];"
                         ::"l"(t), "r"(c[0]), "r"(c[1]), "r"(c[2]), "r"(c[3]), "r"(c[4]), "r"(s) : "memory");
            break;
    }
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// wait until the shared-memory sources of all committed stores have been read
__device__ __forceinline__ void bulk_wait_read0() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// wait until all committed stores have completed
__device__ __forceinline__ void bulk_wait0() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }

}  // namespace tc05
}  // namespace hqs
