// Shrinkage as a differentiable operator (autograd binding): the forward map
// W = shrink(v, t) and its hand-written adjoint over n voxels (the per-voxel
// math and its derivatives are in shrink3.cuh).  The adjoint returns
// gv = (dW/dv)^T gW per voxel and the per-voxel contributions
// gt_i = <dW/dt, gW>_i, which the caller sums.
#include "ops.h"
#include "shrink3.cuh"
#include "tval3_internal.cuh"

namespace tv3 {

template <class T>
__global__ void k_shrink_fwd(long n, const T* __restrict__ v, T t, int iso, T* __restrict__ W) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const T vv[3] = {v[i], v[n + i], v[2 * n + i]};
        T w[3];
        shrink3_fwd(vv, t, iso, w);
        W[i] = w[0];
        W[n + i] = w[1];
        W[2 * n + i] = w[2];
    }
}

template <class T>
__global__ void k_shrink_bwd(long n, const T* __restrict__ v, T t, int iso, const T* __restrict__ gW,
                             T* __restrict__ gv, T* __restrict__ gt) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const T vv[3] = {v[i], v[n + i], v[2 * n + i]};
        const T g[3] = {gW[i], gW[n + i], gW[2 * n + i]};
        T out[3];
        const T dt = shrink3_bwd(vv, t, iso, g, out);
        gv[i] = out[0];
        gv[n + i] = out[1];
        gv[2 * n + i] = out[2];
        if (gt) gt[i] = dt;
    }
}

template <class T>
void shrink_fwd(long n, const T* v, double t, int iso, T* W, cudaStream_t s) {
    long g = std::min<long>((n + 255) / 256, (long)num_sms() * 16);
    if (n > 0) k_shrink_fwd<T><<<(int)std::max<long>(g, 1), 256, 0, s>>>(n, v, (T)t, iso, W);
    TV3_CUDA(cudaGetLastError());
}

template <class T>
void shrink_bwd(long n, const T* v, double t, int iso, const T* gW, T* gv, T* gt, cudaStream_t s) {
    long g = std::min<long>((n + 255) / 256, (long)num_sms() * 16);
    if (n > 0) k_shrink_bwd<T><<<(int)std::max<long>(g, 1), 256, 0, s>>>(n, v, (T)t, iso, gW, gv, gt);
    TV3_CUDA(cudaGetLastError());
}

template void shrink_fwd<float>(long, const float*, double, int, float*, cudaStream_t);
template void shrink_fwd<double>(long, const double*, double, int, double*, cudaStream_t);
template void shrink_bwd<float>(long, const float*, double, int, const float*, float*, float*, cudaStream_t);
template void shrink_bwd<double>(long, const double*, double, int, const double*, double*, double*, cudaStream_t);

}  // namespace tv3
