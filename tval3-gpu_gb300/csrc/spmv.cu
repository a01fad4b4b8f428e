// CSR sparse matrix-vector products for A*x (rows = rays) and A^T*y (the CSR
// of A^T, i.e. the reference's CSC arrays used "implicitly transposed",
// 3d/mat_vec_mul_sparse.h:1727-1745).  Replaces cusparseScsrmv
// (3d/blas_wrapper.h:241-289).
//
// One group of G lanes per row, grid-stride over rows; G = 32 for the long
// ray rows of A, smaller for the short voxel rows of A^T.  Matrix values and
// column indices are streamed with the evict-first policy; x is gathered
// through L1/L2 (it fits in L2 for every configuration of this library).
// Values may be FP32, FP64, BF16 or FP16; for the 16-bit formats a per-row
// FP32 scale of A is applied to the row sum (A*x) or to the gathered y (A^T*y),
// so A^T is the exact adjoint of the quantised A.
//
// Optional fused epilogues (solver only): lam3 = ||Au - b||^2 and
// lam5 = <delta, Au - b> (3d/tval3_gpu_3d_kernels.cu:876-919), ||Ad||^2 for the
// first-iteration step size (3d/tval3_gpu_3d.cpp:577-610), and g = A^T Au - Atb
// (3d/tval3_gpu_3d.cpp:565).
#include "tval3_internal.cuh"
#include "launch.h"

namespace tv3 {

template <class T, class V, int G, int EPI>
__global__ void __launch_bounds__(256) k_spmv(SpmvArgs<T, V> a) {
    count_launch(a.ctl);
    const int lane = threadIdx.x % G;
    const long grp = ((long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const long ngrp = ((long)gridDim.x * blockDim.x) / G;
    int sel = 0;
    if (a.by_parity) sel = a.ctl->parity;
    const T* __restrict__ x = a.x[sel];
    T* __restrict__ y = a.y[sel];
    const int* __restrict__ ptr = a.ptr;
    const int* __restrict__ ind = a.ind;
    const V* __restrict__ val = a.val;
    double acc0 = 0.0, acc1 = 0.0;
    // the group mask for the shuffles: G consecutive lanes
    const unsigned gmask = (G == 32) ? FULL : (((1u << G) - 1u) << ((threadIdx.x & 31) / G * G));
    for (long r = grp; r < a.rows; r += ngrp) {
        const int beg = __ldg(ptr + r), end = __ldg(ptr + r + 1);
        T s = T(0);
        int k = beg + lane;
        if (a.xscale) {
            const float* __restrict__ xs = a.xscale;
            for (; k < end; k += G) {
                int c = __ldcs(ind + k);
                s += (T)Acc<T, V>::load(val + k) * (x[c] * (T)__ldg(xs + c));
            }
        } else {
            for (; k + 3 * G < end; k += 4 * G) {
                int c0 = __ldcs(ind + k), c1 = __ldcs(ind + k + G), c2 = __ldcs(ind + k + 2 * G),
                    c3 = __ldcs(ind + k + 3 * G);
                T v0 = (T)Acc<T, V>::load(val + k), v1 = (T)Acc<T, V>::load(val + k + G),
                  v2 = (T)Acc<T, V>::load(val + k + 2 * G), v3 = (T)Acc<T, V>::load(val + k + 3 * G);
                T x0 = x[c0], x1 = x[c1], x2 = x[c2], x3 = x[c3];
                s += v0 * x0;
                s += v1 * x1;
                s += v2 * x2;
                s += v3 * x3;
            }
            for (; k < end; k += G) s += (T)Acc<T, V>::load(val + k) * x[__ldcs(ind + k)];
        }
#pragma unroll
        for (int o = G / 2; o; o >>= 1) s += __shfl_down_sync(gmask, s, o, G);
        if (lane == 0) {
            if (a.rscale) s *= (T)__ldg(a.rscale + r);
            if (EPI == SPMV_PLAIN) {
                y[r] = s;
            } else if (EPI == SPMV_SUB) {
                y[r] = s - a.sub[r];
            } else if (EPI == SPMV_LAM35) {
                y[r] = s;
                double t = (double)s - (double)a.b[r];
                acc0 += t * t;
                acc1 += (double)a.delta[r] * t;
            } else if (EPI == SPMV_NORM2) {
                acc0 += (double)s * (double)s;
            }
        }
    }
    if (EPI == SPMV_LAM35 || EPI == SPMV_NORM2) {
        double v[2] = {acc0, acc1}, tot[2];
        if (grid_reduce<2>(v, a.part, a.ticket, tot) && threadIdx.x == 0) {
            Ctl* c = a.ctl;
            if (EPI == SPMV_LAM35) {
                c->lam3 = tot[0];
                c->lam5 = tot[1];
            } else {
                // first inner iteration: tau = |<d,d> / (||Dd||^2 + mu/beta ||Ad||^2)|
                c->Add = tot[0];
                c->tau = fabs(c->dd / (c->dDd + c->muDbeta * c->Add));
            }
        }
    }
}

template <class T, class V, int EPI>
static void launch_g(const SpmvArgs<T, V>& a, int G, int grid, cudaStream_t s) {
    switch (G) {
        case 4: k_spmv<T, V, 4, EPI><<<grid, 256, 0, s>>>(a); break;
        case 8: k_spmv<T, V, 8, EPI><<<grid, 256, 0, s>>>(a); break;
        case 16: k_spmv<T, V, 16, EPI><<<grid, 256, 0, s>>>(a); break;
        default: k_spmv<T, V, 32, EPI><<<grid, 256, 0, s>>>(a); break;
    }
}

template <class T, class V>
void launch_spmv(const SpmvArgs<T, V>& a, int epi, int G, int grid, cudaStream_t s) {
    switch (epi) {
        case SPMV_SUB: launch_g<T, V, SPMV_SUB>(a, G, grid, s); break;
        case SPMV_LAM35: launch_g<T, V, SPMV_LAM35>(a, G, grid, s); break;
        case SPMV_NORM2: launch_g<T, V, SPMV_NORM2>(a, G, grid, s); break;
        default: launch_g<T, V, SPMV_PLAIN>(a, G, grid, s); break;
    }
}

template void launch_spmv<float, float>(const SpmvArgs<float, float>&, int, int, int, cudaStream_t);
template void launch_spmv<double, double>(const SpmvArgs<double, double>&, int, int, int, cudaStream_t);
template void launch_spmv<double, float>(const SpmvArgs<double, float>&, int, int, int, cudaStream_t);
template void launch_spmv<float, __nv_bfloat16>(const SpmvArgs<float, __nv_bfloat16>&, int, int, int, cudaStream_t);
template void launch_spmv<float, __half>(const SpmvArgs<float, __half>&, int, int, int, cudaStream_t);

}  // namespace tv3
