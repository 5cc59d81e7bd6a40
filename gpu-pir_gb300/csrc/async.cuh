// Asynchronous-copy and barrier helpers shared by the multiply kernels:
// mbarriers, 1-D bulk TMA copies, and waits bounded in wall-clock time.
#pragma once
#include <stdint.h>

namespace sp {

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
    return (uint32_t)__cvta_generic_to_shared(p);
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_addr(bar)) : "memory");
}

// 1-D bulk copy global -> shared, completing `bytes` of the barrier's
// transaction count.  dst, src and bytes must be multiples of 16.
__device__ __forceinline__ void tma_bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
            smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ uint64_t global_ns() {
    uint64_t t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Wall-clock limit of every barrier wait in the multiply kernels.
constexpr uint64_t WAIT_LIMIT_NS = 1000000000ull;

// Wait for phase `parity` of `bar`.  Gives up (returns false) after
// limit_ns, setting *abort, or as soon as another thread has set *abort.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t parity, volatile int *abort,
                                                  uint64_t limit_ns = WAIT_LIMIT_NS) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t i = 1;; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 15) == 0) {
            if (*abort) return false;
            if (global_ns() - t0 > limit_ns) {
                *abort = 1;
                return false;
            }
        }
    }
}

// Same wait without a shared abort flag (single-role kernels).
__device__ __forceinline__ bool mbar_wait_timed(uint64_t *bar, uint32_t parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const uint64_t t0 = global_ns();
    for (uint32_t i = 1;; i++) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 15) == 0 && global_ns() - t0 > WAIT_LIMIT_NS) return false;
    }
}

__device__ __forceinline__ uint32_t mod_u64_barrett(uint64_t x, uint32_t p, uint64_t mu) {
    // mu = floor(2^64 / p); the quotient estimate is at most 2 below the truth
    uint64_t q = __umul64hi(x, mu);
    uint64_t r = x - q * p;
    r = r >= p ? r - p : r;
    r = r >= p ? r - p : r;
    return (uint32_t)r;
}

}  // namespace sp
