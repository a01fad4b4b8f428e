// CSR sparse matrix-vector products for A*x (rows = rays) and A^T*y (the CSR
// of A^T, i.e. the reference's CSC arrays used "implicitly transposed",
// 3d/mat_vec_mul_sparse.h:1727-1745).  Replaces cusparseScsrmv
// (3d/blas_wrapper.h:241-289).
//
// One group of G lanes per row, grid-stride over rows.  Every lane reads four
// consecutive nonzeros with one 16-byte load of column indices and one
// 16-byte (FP32), 32-byte (FP64) or 8-byte (BF16/FP16) load of values, from a
// 4-aligned base below the row start; elements outside [row start, row end)
// are masked.  The index and value arrays are allocated with SPMV_PAD
// elements of slack so these loads never leave the allocation.  Two such
// chunks are issued before their gathers, so each lane keeps 4 streaming
// loads and 8 gathers in flight.  Matrix streams use the evict-first policy;
// x is gathered through L1/L2 (it fits in L2 for every configuration).
// For 16-bit values a per-ray FP32 scale of A is applied to the row sum (A*x)
// or to the gathered y (A^T*y), so A^T is the exact adjoint of the quantised A.
//
// Optional fused epilogues (solver only): lam3 = ||Au - b||^2 and
// lam5 = <delta, Au - b> (3d/tval3_gpu_3d_kernels.cu:876-919), ||Ad||^2 for the
// first-iteration step size (3d/tval3_gpu_3d.cpp:577-610), and g = A^T Au - Atb
// (3d/tval3_gpu_3d.cpp:565).
#include <algorithm>
#include "tval3_internal.cuh"
#include "launch.h"

namespace tv3 {

// four consecutive values from a 16-byte aligned element index
template <class V> struct Vec4;
template <> struct Vec4<float> {
    __device__ static __forceinline__ void load(const float* p, float (&o)[4]) {
        float4 v = __ldcs(reinterpret_cast<const float4*>(p));
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    }
};
template <> struct Vec4<double> {
    __device__ static __forceinline__ void load(const double* p, double (&o)[4]) {
        double2 a = __ldcs(reinterpret_cast<const double2*>(p));
        double2 b = __ldcs(reinterpret_cast<const double2*>(p) + 1);
        o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
    }
};
template <> struct Vec4<__nv_bfloat16> {
    __device__ static __forceinline__ void load(const __nv_bfloat16* p, float (&o)[4]) {
        uint2 u = __ldcs(reinterpret_cast<const uint2*>(p));
        o[0] = __uint_as_float(u.x << 16); o[1] = __uint_as_float(u.x & 0xffff0000u);
        o[2] = __uint_as_float(u.y << 16); o[3] = __uint_as_float(u.y & 0xffff0000u);
    }
};
template <> struct Vec4<__half> {
    __device__ static __forceinline__ void load(const __half* p, float (&o)[4]) {
        uint2 u = __ldcs(reinterpret_cast<const uint2*>(p));
        __half2 a = *reinterpret_cast<__half2*>(&u.x), b = *reinterpret_cast<__half2*>(&u.y);
        float2 fa = __half22float2(a), fb = __half22float2(b);
        o[0] = fa.x; o[1] = fa.y; o[2] = fb.x; o[3] = fb.y;
    }
};
template <class V> struct VT { using type = float; };
template <> struct VT<double> { using type = double; };

// VEC = 1: every lane reads four consecutive nonzeros per chunk (16-byte
// loads), two chunks in flight, masked outside the row: for long rows.
// VEC = 0: lanes stride over single nonzeros (no masked work): for short rows,
// where most four-element slots of the VEC form would be empty.
template <class T, class V, int G, int EPI, int VEC>
__global__ void __launch_bounds__(256) k_spmv(SpmvArgs<T, V> a) {
    count_launch(a.ctl);
    using VV = typename VT<V>::type;
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
    const float* __restrict__ xs = a.xscale;
    double acc0 = 0.0, acc1 = 0.0;
    const unsigned gmask = (G == 32) ? FULL : (((1u << G) - 1u) << ((threadIdx.x & 31) / G * G));
    for (long r = grp; r < a.rows; r += ngrp) {
        const int beg = __ldg(ptr + r), end = __ldg(ptr + r + 1);
        RowAcc<T> acc;
        if (VEC) {
            for (int base = (beg & ~3) + 4 * lane; base < end; base += 8 * G) {
                const int base2 = base + 4 * G;
                int4 c0 = __ldcs(reinterpret_cast<const int4*>(ind + base));
                int4 c1 = __ldcs(reinterpret_cast<const int4*>(ind + base2));
                VV v0[4], v1[4];
                Vec4<V>::load(val + base, v0);
                Vec4<V>::load(val + base2, v1);
                const int cc[8] = {c0.x, c0.y, c0.z, c0.w, c1.x, c1.y, c1.z, c1.w};
                T xv[8];
                bool ok[8];
#pragma unroll
                for (int e = 0; e < 8; ++e) {
                    const int k = (e < 4 ? base : base2) + (e & 3);
                    ok[e] = (k >= beg && k < end);
                    xv[e] = ok[e] ? x[cc[e]] : T(0);
                    if (xs && ok[e]) xv[e] *= (T)__ldg(xs + cc[e]);
                }
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (ok[e]) madd(acc, v0[e], xv[e]);
#pragma unroll
                for (int e = 0; e < 4; ++e)
                    if (ok[4 + e]) madd(acc, v1[e], xv[4 + e]);
            }
        } else {
            int k = beg + lane;
            for (; k + G < end; k += 2 * G) {
                const int c0 = __ldcs(ind + k), c1 = __ldcs(ind + k + G);
                const VV v0 = (VV)Acc<VV, V>::load(val + k), v1 = (VV)Acc<VV, V>::load(val + k + G);
                T x0 = x[c0], x1 = x[c1];
                if (xs) {
                    x0 *= (T)__ldg(xs + c0);
                    x1 *= (T)__ldg(xs + c1);
                }
                madd(acc, v0, x0);
                madd(acc, v1, x1);
            }
            if (k < end) {
                const int c0 = __ldcs(ind + k);
                T x0 = x[c0];
                if (xs) x0 *= (T)__ldg(xs + c0);
                madd(acc, (VV)Acc<VV, V>::load(val + k), x0);
            }
        }
        T s = acc.value();
#pragma unroll
        for (int o = G / 2; o; o >>= 1) s += shfl_down(gmask, s, o, G);
        if (lane == 0) {
            if (a.rscale) s *= (T)__ldg(a.rscale + r);
            if (EPI == SPMV_PLAIN) {
                y[r] = s;
            } else if (EPI == SPMV_SUB) {
                y[r] = s - a.sub[r];
            } else if (EPI == SPMV_LAM35) {
                y[r] = s;
                double t = acc_d(to_acc(s) - to_acc(a.b[r]));
                acc0 += t * t;
                acc1 += acc_d(to_acc(a.delta[r])) * t;
            } else if (EPI == SPMV_NORM2) {
                const double sd = acc_d(to_acc(s));
                acc0 += sd * sd;
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
                lam35_post(c);
            } else {
                // first inner iteration: tau = |<d,d> / (||Dd||^2 + mu/beta ||Ad||^2)|
                c->Add = tot[0];
                c->tau = fabs(c->dd / (c->dDd + c->muDbeta * c->Add));
            }
        }
    }
}

// Multi-RHS form (L > 1 right-hand sides, the reference's csrmm with `layers`
// columns, 2d/mat_vec_mul.h:65-71): vectors are interleaved, element
// (row, layer) at row * L + layer, so the L values one nonzero gathers are
// contiguous.  One group of G lanes per row (G = L rounded up to a power of
// two, at most 32; layers beyond 32 in further passes); lane l accumulates
// layer l.  The row's indices and values are read once per pass for all its
// layers (broadcast loads).  Same epilogues as k_spmv, summed over layers.
template <class T, class V, int G, int EPI>
__global__ void __launch_bounds__(256) k_spmm(SpmvArgs<T, V> a) {
    count_launch(a.ctl);
    using VV = typename VT<V>::type;
    const long L = a.L;
    const int lane = threadIdx.x % G;
    const long grp = ((long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const long ngrp = ((long)gridDim.x * blockDim.x) / G;
    int sel = 0;
    if (a.by_parity) sel = a.ctl->parity;
    const T* __restrict__ x = a.x[sel];
    T* __restrict__ y = a.y[sel];
    const int* __restrict__ ind = a.ind;
    const V* __restrict__ val = a.val;
    const float* __restrict__ xs = a.xscale;
    double acc0 = 0.0, acc1 = 0.0;
    for (long r = grp; r < a.rows; r += ngrp) {
        const int beg = __ldg(a.ptr + r), end = __ldg(a.ptr + r + 1);
        for (long l0 = 0; l0 < L; l0 += G) {
            const long l = l0 + lane;
            const bool on = l < L;
            RowAcc<T> acc;
            int k = beg;
            for (; k + 1 < end; k += 2) {
                const int c0 = __ldg(ind + k), c1 = __ldg(ind + k + 1);
                const VV v0 = (VV)Acc<VV, V>::load(val + k), v1 = (VV)Acc<VV, V>::load(val + k + 1);
                if (on) {
                    T x0 = x[(long)c0 * L + l], x1 = x[(long)c1 * L + l];
                    if (xs) {
                        x0 *= (T)__ldg(xs + c0);
                        x1 *= (T)__ldg(xs + c1);
                    }
                    madd(acc, v0, x0);
                    madd(acc, v1, x1);
                }
            }
            if (k < end && on) {
                const int c0 = __ldg(ind + k);
                T x0 = x[(long)c0 * L + l];
                if (xs) x0 *= (T)__ldg(xs + c0);
                madd(acc, (VV)Acc<VV, V>::load(val + k), x0);
            }
            if (on) {
                T s = acc.value();
                if (a.rscale) s *= (T)__ldg(a.rscale + r);
                const long o = r * L + l;
                if (EPI == SPMV_PLAIN) {
                    y[o] = s;
                } else if (EPI == SPMV_SUB) {
                    y[o] = s - a.sub[o];
                } else if (EPI == SPMV_LAM35) {
                    y[o] = s;
                    double t = acc_d(to_acc(s) - to_acc(a.b[o]));
                    acc0 += t * t;
                    acc1 += acc_d(to_acc(a.delta[o])) * t;
                } else if (EPI == SPMV_NORM2) {
                    const double sd = acc_d(to_acc(s));
                    acc0 += sd * sd;
                }
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
                lam35_post(c);
            } else {
                c->Add = tot[0];
                c->tau = fabs(c->dd / (c->dDd + c->muDbeta * c->Add));
            }
        }
    }
}

template <class T, class V, int EPI>
static void launch_mm(const SpmvArgs<T, V>& a, cudaStream_t s) {
    int G = 1;
    while (G < a.L && G < 32) G <<= 1;
    long g = (a.rows * G + 255) / 256;
    const long cap = (long)num_sms() * 16;
    const int grid = (int)std::max<long>(1, std::min(g, cap));
    switch (G) {
        case 2: k_spmm<T, V, 2, EPI><<<grid, 256, 0, s>>>(a); break;
        case 4: k_spmm<T, V, 4, EPI><<<grid, 256, 0, s>>>(a); break;
        case 8: k_spmm<T, V, 8, EPI><<<grid, 256, 0, s>>>(a); break;
        case 16: k_spmm<T, V, 16, EPI><<<grid, 256, 0, s>>>(a); break;
        default: k_spmm<T, V, 32, EPI><<<grid, 256, 0, s>>>(a); break;
    }
}

// lanes: the group size G (4, 8, 16, 32), plus SPMV_SCALAR for the scalar-lane variant
template <class T, class V, int EPI, int VEC>
static void launch_v(const SpmvArgs<T, V>& a, int G, int grid, cudaStream_t s) {
    switch (G) {
        case 4: launch_k(k_spmv<T, V, 4, EPI, VEC>, dim3(grid), dim3(256), 0, s, a); break;
        case 8: launch_k(k_spmv<T, V, 8, EPI, VEC>, dim3(grid), dim3(256), 0, s, a); break;
        case 16: launch_k(k_spmv<T, V, 16, EPI, VEC>, dim3(grid), dim3(256), 0, s, a); break;
        default: launch_k(k_spmv<T, V, 32, EPI, VEC>, dim3(grid), dim3(256), 0, s, a); break;
    }
}

template <class T, class V, int EPI>
static void launch_g(const SpmvArgs<T, V>& a, int lanes, int grid, cudaStream_t s) {
    if (lanes & SPMV_SCALAR) launch_v<T, V, EPI, 0>(a, lanes & ~SPMV_SCALAR, grid, s);
    else launch_v<T, V, EPI, 1>(a, lanes, grid, s);
}

template <class T, class V>
void launch_spmv(const SpmvArgs<T, V>& a, int epi, int lanes, int grid, cudaStream_t s) {
    if (a.L > 1) {
        switch (epi) {
            case SPMV_SUB: launch_mm<T, V, SPMV_SUB>(a, s); break;
            case SPMV_LAM35: launch_mm<T, V, SPMV_LAM35>(a, s); break;
            case SPMV_NORM2: launch_mm<T, V, SPMV_NORM2>(a, s); break;
            default: launch_mm<T, V, SPMV_PLAIN>(a, s); break;
        }
        return;
    }
    switch (epi) {
        case SPMV_SUB: launch_g<T, V, SPMV_SUB>(a, lanes, grid, s); break;
        case SPMV_LAM35: launch_g<T, V, SPMV_LAM35>(a, lanes, grid, s); break;
        case SPMV_NORM2: launch_g<T, V, SPMV_NORM2>(a, lanes, grid, s); break;
        default: launch_g<T, V, SPMV_PLAIN>(a, lanes, grid, s); break;
    }
}

template void launch_spmv<float, float>(const SpmvArgs<float, float>&, int, int, int, cudaStream_t);
template void launch_spmv<double, double>(const SpmvArgs<double, double>&, int, int, int, cudaStream_t);
template void launch_spmv<double, float>(const SpmvArgs<double, float>&, int, int, int, cudaStream_t);
template void launch_spmv<df64, float>(const SpmvArgs<df64, float>&, int, int, int, cudaStream_t);
template void launch_spmv<float, __nv_bfloat16>(const SpmvArgs<float, __nv_bfloat16>&, int, int, int, cudaStream_t);
template void launch_spmv<float, __half>(const SpmvArgs<float, __half>&, int, int, int, cudaStream_t);
template void launch_spmv<df64, __nv_bfloat16>(const SpmvArgs<df64, __nv_bfloat16>&, int, int, int, cudaStream_t);
template void launch_spmv<df64, __half>(const SpmvArgs<df64, __half>&, int, int, int, cudaStream_t);

}  // namespace tv3
