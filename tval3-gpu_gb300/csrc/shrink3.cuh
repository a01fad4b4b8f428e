// Shrinkage of one voxel's difference vector v = (v_y, v_x, v_z) with
// threshold t, and its adjoint (shrinkage_kernel,
// 3d/tval3_gpu_3d_kernels.cu:1249-1300, anisotropic; isotropic TV added):
//
// anisotropic, per component:  W_a = sign(v_a) max(|v_a| - t, 0)
//     dW_a/dv_a = [|v_a| > t],   dW_a/dt = -sign(v_a) [|v_a| > t]
// isotropic, per voxel:  W = v max(|v| - t, 0) / |v|
//     on |v| > t:  dW/dv = (1 - t/|v|) I + t v v^T / |v|^3,  dW/dt = -v / |v|
//     elsewhere 0 (the subgradient at the kink is taken as 0)
#pragma once

#include <math.h>

namespace tv3 {

template <class T>
__device__ __forceinline__ void shrink3_fwd(const T v[3], T t, int iso, T W[3]) {
    if (!iso) {
        for (int a = 0; a < 3; ++a) {
            T m = fabs(v[a]) - t;
            m = m > T(0) ? m : T(0);
            W[a] = v[a] >= T(0) ? m : -m;
        }
    } else {
        const T nv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        const T sc = nv > t ? (nv - t) / nv : T(0);
        for (int a = 0; a < 3; ++a) W[a] = v[a] * sc;
    }
}

// gv = (dW/dv)^T gW; returns <dW/dt, gW>
template <class T>
__device__ __forceinline__ T shrink3_bwd(const T v[3], T t, int iso, const T gW[3], T gv[3]) {
    T dt = T(0);
    for (int a = 0; a < 3; ++a) gv[a] = T(0);
    if (!iso) {
        for (int a = 0; a < 3; ++a)
            if (fabs(v[a]) > t) {
                gv[a] = gW[a];
                dt -= (v[a] >= T(0) ? gW[a] : -gW[a]);
            }
    } else {
        const T nv = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
        if (nv > t) {
            const T s = T(1) - t / nv;
            const T vg = v[0] * gW[0] + v[1] * gW[1] + v[2] * gW[2];
            const T c = t * vg / (nv * nv * nv);
            for (int a = 0; a < 3; ++a) gv[a] = s * gW[a] + c * v[a];
            dt = -vg / nv;
        }
    }
    return dt;
}

}  // namespace tv3
