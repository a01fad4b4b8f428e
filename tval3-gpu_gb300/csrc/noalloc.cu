// Dense A^T*y that allocates no device memory.
//
// Who needs it: callers that must not allocate once they are running, e.g.
// an acquisition loop that reconstructs every frame under a fixed memory
// budget, or a host application that hands all device memory to its own
// pool allocator.  cudaMalloc can block the whole device, fail under memory
// pressure, and cannot be called while a stream is being captured, so such
// callers cannot create an operator handle (which owns its scratch) per
// call.  This variant takes the caller's device arrays and keeps its slab
// partial sums in one file-scope static device array instead.
//
// The kernels are the slab scheme of the dense operator's A^T*y (one column
// tile of 256 threads per block, each block sums a slab of rows, a second
// pass adds the slabs in a fixed order), with the slab count bounded so that
// slabs * cols fits the static scratch.
//
// Limits and rules:
//  - cols <= TVAL3_NOALLOC_SCRATCH_FLOATS (1,048,576); larger is rejected.
//  - a call on a stream that is not being captured looks up the scratch
//    address of the current device (cudaGetSymbolAddress with that device
//    current) and remembers it; a call on a stream under capture uses the
//    remembered address, so the first call on a device must come before any
//    capture, e.g. once during start-up.  Looking the address up again on
//    every uncaptured call keeps it right after a cudaDeviceReset (which
//    reloads the module); a graph captured before such a reset must not be
//    replayed after it.
//  - nothing in the scratch has to start at zero: the partial pass writes
//    every (slab, column) entry that the sum pass reads in the same call.
//  - the scratch is shared by all calls on a device: calls that overlap in
//    time (other streams, other host threads) race on it and must be ordered
//    by the caller.
#include <algorithm>
#include <mutex>
#include <string>
#include "ops.h"
#include "tval3/tval3_c.h"

namespace tv3 {

constexpr long NOALLOC_SCRATCH_FLOATS = 1L << 20;  // 4 MiB per device
constexpr int NOALLOC_MAX_DEVICES = 64;

static __device__ __align__(256) float g_noalloc_scratch[NOALLOC_SCRATCH_FLOATS];

namespace {

float* g_scratch_ptr[NOALLOC_MAX_DEVICES] = {};
std::mutex g_scratch_mu;

// Address of the static scratch on the current device: looked up when `s`
// is not capturing, remembered for calls made under capture.
float* scratch_for_current_device(cudaStream_t s) {
    int dev = 0;
    TV3_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES) throw Error{TVAL3_ERR_UNSUPPORTED, "device ordinal out of range"};
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    TV3_CUDA(cudaStreamIsCapturing(s, &cs));
    std::lock_guard<std::mutex> lk(g_scratch_mu);
    if (cs == cudaStreamCaptureStatusNone) {
        void* p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess || !p)
            throw Error{TVAL3_ERR_CUDA, std::string("cudaGetSymbolAddress of the static scratch failed: ") +
                                            cudaGetErrorString(e)};
        g_scratch_ptr[dev] = (float*)p;
    } else if (!g_scratch_ptr[dev]) {
        throw Error{TVAL3_ERR_ARG, "Argument error: the first no-allocation call on a device must come before any "
                                   "stream capture!"};
    }
    return g_scratch_ptr[dev];
}

__global__ void __launch_bounds__(256) k_rmatvec_part(long m, long n, long rows_per_slab, const float* __restrict__ A,
                                                      const float* __restrict__ y, float* __restrict__ part) {
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long slab = blockIdx.y;
    const long r0 = slab * rows_per_slab, r1 = min(m, r0 + rows_per_slab);
    if (c >= n) return;
    float s = 0.f;
    for (long r = r0; r < r1; ++r) s += A[r * n + c] * y[r];
    part[slab * n + c] = s;
}

__global__ void k_rmatvec_sum(long n, int slabs, const float* __restrict__ part, float* __restrict__ x) {
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int k = 0; k < slabs; ++k) s += part[(long)k * n + c];
        x[c] = s;
    }
}

}  // namespace

void dense_rmatvec_noalloc_f32(long rows, long cols, const float* A, const float* y, float* x, cudaStream_t s) {
    if (rows < 0 || cols < 0) throw Error{TVAL3_ERR_SHAPE, "Argument error: negative matrix size!"};
    if (cols > NOALLOC_SCRATCH_FLOATS)
        throw Error{TVAL3_ERR_SHAPE, "Argument error: cols = " + std::to_string(cols) +
                                         " exceeds the static scratch of " +
                                         std::to_string(NOALLOC_SCRATCH_FLOATS) + " floats!"};
    if (cols == 0) return;
    if ((!A && rows > 0) || (!y && rows > 0) || !x) throw Error{TVAL3_ERR_ARG, "Argument error: NULL device array!"};
    float* part = scratch_for_current_device(s);
    if (rows == 0) {
        TV3_CUDA(cudaMemsetAsync(x, 0, (size_t)cols * sizeof(float), s));
        return;
    }
    const long tiles = (cols + 255) / 256;
    long slabs = std::max<long>(1, (long)num_sms() * 8 / tiles);
    slabs = std::min<long>(slabs, NOALLOC_SCRATCH_FLOATS / cols);
    slabs = std::min<long>(slabs, rows);
    const long rows_per_slab = (rows + slabs - 1) / slabs;
    slabs = (rows + rows_per_slab - 1) / rows_per_slab;
    k_rmatvec_part<<<dim3((unsigned)tiles, (unsigned)slabs), 256, 0, s>>>(rows, cols, rows_per_slab, A, y, part);
    const long g = std::min<long>(tiles, (long)num_sms() * 8);
    k_rmatvec_sum<<<(unsigned)g, 256, 0, s>>>(cols, (int)slabs, part, x);
    TV3_CUDA(cudaGetLastError());
}

}  // namespace tv3
