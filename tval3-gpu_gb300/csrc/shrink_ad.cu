// Shrinkage as a differentiable operator (autograd binding): the forward map
// W = shrink(v, t) of shrinkage_kernel (3d/tval3_gpu_3d_kernels.cu:1249-1300,
// anisotropic) and of isotropic TV, and its hand-written adjoint.
//
// anisotropic, per component:  W_a = sign(v_a) max(|v_a| - t, 0)
//     dW_a/dv_a = [|v_a| > t],   dW_a/dt = -sign(v_a) [|v_a| > t]
// isotropic, per voxel (v in R^3):  W = v max(|v| - t, 0) / |v|
//     on |v| > t:  dW/dv = (1 - t/|v|) I + t v v^T / |v|^3,  dW/dt = -v / |v|
//     elsewhere 0 (the subgradient at the kink is taken as 0)
// The adjoint returns gv = (dW/dv)^T gW per voxel and the per-voxel
// contributions gt_i = <dW/dt, gW>_i, which the caller sums.
#include "ops.h"
#include "tval3_internal.cuh"

namespace tv3 {

template <class T>
__global__ void k_shrink_fwd(long n, const T* __restrict__ v, T t, int iso, T* __restrict__ W) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const T v0 = v[i], v1 = v[n + i], v2 = v[2 * n + i];
        if (!iso) {
            const T vv[3] = {v0, v1, v2};
            for (int a = 0; a < 3; ++a) {
                T m = fabs(vv[a]) - t;
                m = m > T(0) ? m : T(0);
                W[a * n + i] = vv[a] >= T(0) ? m : -m;
            }
        } else {
            const T nv = sqrt(v0 * v0 + v1 * v1 + v2 * v2);
            const T sc = nv > t ? (nv - t) / nv : T(0);
            W[i] = v0 * sc;
            W[n + i] = v1 * sc;
            W[2 * n + i] = v2 * sc;
        }
    }
}

template <class T>
__global__ void k_shrink_bwd(long n, const T* __restrict__ v, T t, int iso, const T* __restrict__ gW,
                             T* __restrict__ gv, T* __restrict__ gt) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const T vv[3] = {v[i], v[n + i], v[2 * n + i]};
        const T g[3] = {gW[i], gW[n + i], gW[2 * n + i]};
        T out[3] = {T(0), T(0), T(0)}, dt = T(0);
        if (!iso) {
            for (int a = 0; a < 3; ++a)
                if (fabs(vv[a]) > t) {
                    out[a] = g[a];
                    dt -= (vv[a] >= T(0) ? g[a] : -g[a]);
                }
        } else {
            const T nv = sqrt(vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2]);
            if (nv > t) {
                const T s = T(1) - t / nv;
                const T vg = vv[0] * g[0] + vv[1] * g[1] + vv[2] * g[2];
                const T c = t * vg / (nv * nv * nv);
                for (int a = 0; a < 3; ++a) out[a] = s * g[a] + c * vv[a];
                dt = -vg / nv;
            }
        }
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
