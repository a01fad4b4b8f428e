// Self-test of the bounded device waits (mbar.cuh).  One warp waits, with a
// caller-given limit, on an mbarrier phase that nothing completes: the wait
// must give up and report it, and the context must stay usable.  The kernel
// then completes the phase itself (one arrival), so the barrier ends in a
// finished state, and returns.  The wait is bounded by construction; nothing
// faults or hangs.  No counterpart in the reference (its kernels have no
// device-side waits).
#include <stdint.h>
#include "dbuf.h"
#include "mbar.cuh"
#include "ops.h"

namespace tv3 {

__global__ void k_wait_probe(long long limit, int* timed_out, long long* waited) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    const long long t0 = clock64();
    const bool ok = mbar_wait(&bar, 0, limit);
    const long long t1 = clock64();
    __syncthreads();
    if (threadIdx.x == 0) {
        *timed_out = ok ? 0 : 1;
        *waited = t1 - t0;
        mbar_arrive(&bar);  // the one expected arrival: phase 0 completes
    }
}

void selftest_bounded_wait(long long cycles, int* timed_out, long long* waited) {
    DBuf<long long> w(1);
    DBuf<int> t(1);
    k_wait_probe<<<1, 32>>>(cycles, t.p, w.p);
    TV3_CUDA(cudaGetLastError());
    TV3_CUDA(cudaDeviceSynchronize());
    TV3_CUDA(cudaMemcpy(timed_out, t.p, sizeof(int), cudaMemcpyDeviceToHost));
    TV3_CUDA(cudaMemcpy(waited, w.p, sizeof(long long), cudaMemcpyDeviceToHost));
}

}  // namespace tv3
