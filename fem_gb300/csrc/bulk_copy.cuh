// bulk_copy.cuh - global-to-shared bulk copies (cp.async.bulk, the TMA engine's untiled form)
// completing on shared-memory mbarriers, with bounded waits.
//
// A copy needs a 16-byte aligned source and destination and a size that is a multiple of 16.
// Every wait is bounded: it gives up after a time limit (device %globaltimer) or a number of
// polls, whichever comes first, records an error code in a device word that the host reads, and
// returns false instead of spinning on.
#pragma once

#include <cstdint>

namespace bulk {

constexpr unsigned long long kWaitNs = 2000000000ull;  // 2 s
constexpr long kWaitPolls = 1L << 26;

__device__ __forceinline__ unsigned long long device_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned smem_addr(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// a barrier that completes a phase on one arrival plus the expected bytes
__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(bar)) : "memory");
}

// makes barrier initialisations visible to the copy engine (after the inits, before the first copy)
__device__ __forceinline__ void fence_mbar_init() { asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory"); }

// orders this thread's earlier ordinary accesses to shared memory before later bulk copies' writes
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory"); }

// the one arrival of the barrier's current phase, announcing `bytes` to come
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_addr(bar)), "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, unsigned parity) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2;\n selp.b32 %0, 1, 0, P;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity)
        : "memory");
    return done != 0;
}

// one poll that lets the hardware suspend the thread until the phase completes or about
// `suspend_ns` have passed
__device__ __forceinline__ bool mbar_try_suspend(uint64_t* bar, unsigned parity, unsigned suspend_ns) {
    unsigned done;
    asm volatile(
        "{\n .reg .pred P;\n mbarrier.try_wait.parity.shared::cta.b64 P, [%1], %2, %3;\n selp.b32 %0, 1, 0, P;\n}\n"
        : "=r"(done)
        : "r"(smem_addr(bar)), "r"(parity), "r"(suspend_ns)
        : "memory");
    return done != 0;
}

// true once the phase of `parity` has completed.  After limit_ns (or kWaitPolls polls), or at once
// when *err is already set elsewhere, *err = code (if still 0) and false.  The error word and the
// clock are read every 64 polls: a read of global memory costs as much as the wait it interrupts.
// suspend_ns > 0: each poll may suspend the thread that long (fewer polls, fewer issued
// instructions while the copies are in flight).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, unsigned parity, int* err, int code,
                                          unsigned long long limit_ns = kWaitNs, unsigned suspend_ns = 0) {
    unsigned long long t0 = 0;
    for (long polls = 0;; polls++) {
        if (polls == 1) t0 = device_ns();
        if (suspend_ns ? mbar_try_suspend(bar, parity, suspend_ns) : mbar_try(bar, parity)) return true;
        if ((polls & 63) == 63 && (polls > kWaitPolls || *(volatile int*)err || device_ns() - t0 > limit_ns)) {
            atomicCAS(err, 0, code);
            return false;
        }
    }
}

// the same wait bounded by time only (not cut short by the error word): used after a failure to
// let copies still in flight land before the block exits
__device__ __forceinline__ void mbar_drain(uint64_t* bar, unsigned parity, unsigned long long limit_ns = kWaitNs) {
    const unsigned long long t0 = device_ns();
    while (!mbar_try(bar, parity) && device_ns() - t0 < limit_ns) {
    }
}

// an L2 policy for data read once (streamed matrices): evicted first, so that reused vectors stay
__device__ __forceinline__ uint64_t evict_first_policy() {
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;\n" : "=l"(p));
    return p;
}

// bytes from global `src` to shared `dst`, completing on `bar` (which must expect them)
__device__ __forceinline__ void copy(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                     smem_addr(dst)),
                 "l"(src), "r"(bytes), "r"(smem_addr(bar))
                 : "memory");
}

__device__ __forceinline__ void copy_hint(void* dst, const void* src, unsigned bytes, uint64_t* bar,
                                          uint64_t policy) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint [%0], [%1], %2, [%3], "
        "%4;\n" ::"r"(smem_addr(dst)),
        "l"(src), "r"(bytes), "r"(smem_addr(bar)), "l"(policy)
        : "memory");
}

}  // namespace bulk
