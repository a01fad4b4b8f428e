// Shared-memory mbarriers and asynchronous copies (sm_90+ PTX), shared by the
// pipelined kernels.  Every wait is bounded: it gives up after WAIT_CYCLES of
// SM clock (about two seconds) and returns false, so a kernel whose copies
// never land records an error and returns instead of hanging the GPU.
#pragma once

#include <stdint.h>
#include <cuda_runtime.h>

namespace tv3 {

constexpr long long WAIT_CYCLES = 4000000000LL;  // about 2 s at 2 GHz

// device error bits written to Ctl::err by pipelined kernels on a timeout
constexpr unsigned ERR_UMMA_TIMEOUT = 0x10u;
constexpr unsigned ERR_TILED_TIMEOUT = 0x20u;

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* b, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count) : "memory");
}
// make the initialised barriers visible to the async proxy (bulk copies)
__device__ __forceinline__ void mbar_fence_init() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
// one arrival that also announces `bytes` of asynchronous copies
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(b)), "r"(bytes) : "memory");
}
// one plain arrival (release: earlier shared-memory accesses of the thread are ordered before it)
__device__ __forceinline__ void mbar_arrive(uint64_t* b) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(b)) : "memory");
}
// bounded wait (`limit` cycles of SM clock) for the completion of phase
// `parity`; false on timeout.  Each try_wait may suspend the thread until the
// phase completes or about a microsecond passes (the suspend-time hint), so a
// waiting warp does not spin on the issue slots that the working warps of its
// SM need.
__device__ __forceinline__ bool mbar_wait(uint64_t* b, unsigned parity, long long limit = WAIT_CYCLES) {
    const unsigned a = smem_u32(b);
    const long long t0 = clock64();
    for (;;) {
        unsigned ok;
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}\n"
            : "=r"(ok)
            : "r"(a), "r"(parity), "r"(1000u)
            : "memory");
        if (ok) return true;
        if (clock64() - t0 > limit) return false;
    }
}

// bulk copy (TMA engine) of `bytes` from global to shared memory, completing
// on barrier `bar`; addresses 16-byte aligned, bytes a multiple of 16
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
        "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

// per-thread asynchronous copy of 4 or 8 bytes from global to shared memory
template <int BYTES>
__device__ __forceinline__ void cp_async(void* dst, const void* src) {
    static_assert(BYTES == 4 || BYTES == 8 || BYTES == 16, "cp.async size");
    asm volatile("cp.async.ca.shared.global [%0], [%1], %2;" ::"r"(smem_u32(dst)), "l"(src), "n"(BYTES) : "memory");
}
// arrive on `bar` once every earlier cp.async of this thread has landed (the
// barrier's expected count includes this arrival)
__device__ __forceinline__ void cp_async_arrive(uint64_t* b) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;" ::: "memory"); }
// close the thread's current group of cp.async copies
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
// wait until at most N of the thread's committed groups are still in flight
template <int N>
__device__ __forceinline__ void cp_async_wait_group() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// named barrier over `threads` threads (a multiple of 32) of the CTA
__device__ __forceinline__ void named_sync(int id, int threads) {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
}

}  // namespace tv3
