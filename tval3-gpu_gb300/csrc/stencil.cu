// Volume kernels of the TVAL3 loop: the periodic difference operator D and
// its adjoint, shrinkage, the step-size, gradient, backtracking and multiplier
// updates, each fused with the reductions the loop needs.  Every reducing
// kernel ends in a deterministic grid reduction whose last block updates the
// device control block (tval3_internal.cuh), so no value crosses to the host.
// The element type T is float, double or df64 (double-float on the FP32
// pipes); per-thread sums use acc_t<T>.
//
// Reference counterparts (3d/tval3_gpu_3d.cpp unless noted):
//   k_D_only / k_descend   D_gpu :271-314 (+ axpy and nonneg_kernel, :671-701;
//                          k_descend also lam2_4_kernel's sums at the new point)
//   armijo_decide          f and the Armijo test, min_u_gpu :848-858 (run by the A*U
//                          product's lam3/lam5 epilogue, tval3_internal.cuh)
//   k_Dd_norm              get_tau_gpu first iteration :583-600
//   k_gradient (BB step)   get_tau_kernel, 3d/tval3_gpu_3d_kernels.cu:1017-1067
//   k_g2                   V = DU - W, lam2_4_kernel, Dt_gpu (get_g_gpu :484-571)
//   k_shrink               shrinkage_kernel, 3d/tval3_gpu_3d_kernels.cu:1249-1300
//   k_gradient             get_gradient_gpu :896-919 and the RelChg test :1178-1200
//   k_bt_coef / k_bt_apply min_u_gpu Armijo branch :848-890 with update_g_gpu :706-818
//                          (g2 at the accepted point is not formed: update_W's
//                          g2 replaces it before anything reads it)
//   k_outer_relchg         :1204-1220
//   k_mlp                  update_mlp_gpu :1034-1083 and continuation :1222-1237
//   k_outer_grad           DtsAtd and get_gradient :1238-1249
#include <math.h>
#include <type_traits>
#include <algorithm>
#include <map>
#include <mutex>
#include "tval3_internal.cuh"
#include "launch.h"

namespace tv3 {

// Division of a voxel index by the invariant dimensions with one high
// multiply (Granlund & Montgomery, "Division by invariant integers using
// multiplication", 1994): q = (umulhi(i, M) + i) >> L with L = ceil(log2 d),
// M = floor(2^32 (2^L - d) / d) + 1; exact for i < 2^31.
struct FastDiv {
    unsigned d, M, L;
};
static FastDiv make_div(unsigned d) {
    FastDiv f;
    f.d = d;
    unsigned L = 0;
    while ((1ull << L) < d) ++L;
    f.L = L;
    f.M = (unsigned)((((1ull << L) - d) << 32) / d + 1);
    return f;
}
__device__ __forceinline__ unsigned fdiv(unsigned i, const FastDiv& f) {
    return (unsigned)(((unsigned long long)__umulhi(i, f.M) + i) >> f.L);
}

// Volume geometry of the vectors: element i = voxel * L + layer, voxel =
// y + x*p + z*p*q.  With L > 1 (layers sharing A) the differences stay inside
// each layer.
struct Geo {
    FastDiv p, q;
    int r;
    FastDiv l;  // layers (d = 1: one volume)
};

struct Nb {
    long yp, ym, xp, xm, zp, zm;
};

__device__ __forceinline__ Nb neighbours(const Geo& g, long i) {
    unsigned v = (unsigned)i;
    long u = 1;  // element stride of one voxel
    if (g.l.d > 1) {
        v = fdiv(v, g.l);
        u = g.l.d;
    }
    const unsigned t = fdiv(v, g.p);
    const int y = (int)(v - t * g.p.d);
    const unsigned zz = fdiv(t, g.q);
    const int x = (int)(t - zz * g.q.d);
    const int z = (int)zz;
    const long p = g.p.d, q = g.q.d, pq = p * q;
    Nb o;
    o.yp = (y + 1 < (int)p) ? i + u : i - y * u;
    o.ym = (y > 0) ? i - u : i + (p - 1) * u;
    o.xp = (x + 1 < (int)q) ? i + p * u : i - (long)x * p * u;
    o.xm = (x > 0) ? i - p * u : i + (q - 1) * p * u;
    o.zp = (z + 1 < g.r) ? i + pq * u : i - (long)z * pq * u;
    o.zm = (z > 0) ? i - pq * u : i + (long)(g.r - 1) * pq * u;
    return o;
}

#define GRID_STRIDE(i, N) for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < (N); i += (long)gridDim.x * blockDim.x)

// Two consecutive elements with one 16-byte (8-byte for float) load or store:
// the pass-per-vector kernels move 150 MB-sized sets where wide, streaming
// accesses reach ~1.5x the bandwidth of 8-byte ones.  Used when every vector
// offset is even (n even), so all pair addresses are aligned.
template <class T> struct Two { T a, b; };
__device__ __forceinline__ Two<float> ld2(const float* p) {
    const float2 v = *reinterpret_cast<const float2*>(p);
    return {v.x, v.y};
}
__device__ __forceinline__ Two<double> ld2(const double* p) {
    const double2 v = *reinterpret_cast<const double2*>(p);
    return {v.x, v.y};
}
__device__ __forceinline__ Two<df64> ld2(const df64* p) {
    const float4 v = *reinterpret_cast<const float4*>(p);
    return {df64(v.x, v.y), df64(v.z, v.w)};
}
__device__ __forceinline__ void st2(float* p, float a, float b) { *reinterpret_cast<float2*>(p) = make_float2(a, b); }
__device__ __forceinline__ void st2(double* p, double a, double b) { *reinterpret_cast<double2*>(p) = make_double2(a, b); }
__device__ __forceinline__ void st2(df64* p, df64 a, df64 b) {
    *reinterpret_cast<float4*>(p) = make_float4(a.hi, a.lo, b.hi, b.lo);
}
#define GRID_STRIDE_PAIRS(i, N) \
    for (long i = 2 * ((long)blockIdx.x * blockDim.x + threadIdx.x); i < (N); i += 2 * (long)gridDim.x * blockDim.x)

template <class T> __device__ __forceinline__ T proj(T v, int nonneg) { return (nonneg && v < T(0)) ? T(0) : v; }

// x / beta: division as in the reference for float and double; for df64 the
// caller passes 1/beta and multiplies (same value to ~1e-15, a tenth of the
// cost of a double-float division)
template <class T> __device__ __forceinline__ T div_beta(T x, T bt, T) { return x / bt; }
template <> __device__ __forceinline__ df64 div_beta<df64>(df64 x, df64, df64 ibt) { return x * ibt; }

// ---------------------------------------------------------------------------
// b scaling (scaleb_gpu :226-266): one block finds the entries of smallest and
// largest |b| (first occurrence on ties, as the reference's strict scan), the
// next kernel writes b*scl.
// ---------------------------------------------------------------------------
template <class E>
__global__ void __launch_bounds__(1024) k_scale_find(const E* __restrict__ b, long m, Ctl* ctl) {
    count_launch(ctl);
    double amin = INFINITY, amax = -1.0;
    long imin = -1, imax = -1;
    for (long i = threadIdx.x; i < m; i += blockDim.x) {
        double a = fabs((double)b[i]);
        if (a < amin) { amin = a; imin = i; }
        if (a > amax) { amax = a; imax = i; }
    }
    __shared__ double sa[2][1024];
    __shared__ long si[2][1024];
    sa[0][threadIdx.x] = amin; si[0][threadIdx.x] = imin;
    sa[1][threadIdx.x] = amax; si[1][threadIdx.x] = imax;
    __syncthreads();
    for (int o = blockDim.x / 2; o; o >>= 1) {
        if (threadIdx.x < o) {
            int j = threadIdx.x + o;
            double a0 = sa[0][j]; long i0 = si[0][j];
            if (i0 >= 0 && (si[0][threadIdx.x] < 0 || a0 < sa[0][threadIdx.x] ||
                            (a0 == sa[0][threadIdx.x] && i0 < si[0][threadIdx.x]))) {
                sa[0][threadIdx.x] = a0; si[0][threadIdx.x] = i0;
            }
            double a1 = sa[1][j]; long i1 = si[1][j];
            if (i1 >= 0 && (si[1][threadIdx.x] < 0 || a1 > sa[1][threadIdx.x] ||
                            (a1 == sa[1][threadIdx.x] && i1 < si[1][threadIdx.x]))) {
                sa[1][threadIdx.x] = a1; si[1][threadIdx.x] = i1;
            }
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) {
        double scl = 1.0;
        if (m > 0 && si[0][0] >= 0 && si[1][0] >= 0) {
            double dif = fabs((double)b[si[1][0]] - (double)b[si[0][0]]);
            // the reference divides by zero when dif == 0; a constant-|b| input keeps scl = 1
            if (dif > 0.0) {
                if (dif < 0.5) scl = 0.5 / dif;
                else if (dif > 1.5) scl = 1.5 / dif;
            }
        }
        ctl->scl = scl;
    }
}

// b_in is the caller's m x L column-major array; b is interleaved (ray * L + layer)
template <class T>
__global__ void k_scale_apply(const Ext<T>* __restrict__ b_in, T* __restrict__ b, long m, int L, Ctl* ctl) {
    count_launch(ctl);
    const double scl = ctl->scl;
    const Ext<T> s = (Ext<T>)scl;
    const long m1 = m / L;
    GRID_STRIDE(i, m) {
        const long src = (L == 1) ? i : (i % L) * m1 + i / L;
        b[i] = from_ext<T>((scl == 1.0) ? b_in[src] : b_in[src] * s);
    }
}

// ---------------------------------------------------------------------------
// D at start-up: DU[0] = D U[0]
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_D_only(SolverBufs<T> B, Geo g) {
    count_launch(B.ctl);
    const T* __restrict__ U = B.U[0];
    T* __restrict__ DU = B.DU[0];
    GRID_STRIDE(i, B.n) {
        Nb nb = neighbours(g, i);
        T u = U[i];
        DU[i] = U[nb.yp] - u;
        DU[B.n + i] = U[nb.xp] - u;
        DU[2 * B.n + i] = U[nb.zp] - u;
    }
}

// ---------------------------------------------------------------------------
// Shrinkage of one voxel (shrinkage_kernel, 3d/tval3_gpu_3d_kernels.cu:1249-1300,
// plus the isotropic form): u = DU - sigma/beta, W = shrink(u, 1/beta); adds
// the voxel's TV term to l1 and (DU - W)^2, sigma (DU - W) to l2, l4 (the
// sums update_W needs).  Used by k_shrink and, speculatively for the full
// step, by k_descend.
// ---------------------------------------------------------------------------
template <class T, class A>
__device__ __forceinline__ void shrink_voxel(T d0, T d1, T d2, T s0, T s1, T s2, T bt, T ib, int iso, T& w0, T& w1,
                                             T& w2, A& l1, ProdAcc<T>& l2, ProdAcc<T>& l4) {
    T u0 = d0 - div_beta(s0, bt, ib);
    T u1 = d1 - div_beta(s1, bt, ib);
    T u2 = d2 - div_beta(s2, bt, ib);
    if (!iso) {
        T t0 = fabs(u0) - ib, t1 = fabs(u1) - ib, t2 = fabs(u2) - ib;
        t0 = (t0 >= T(0)) ? t0 : T(0);
        t1 = (t1 >= T(0)) ? t1 : T(0);
        t2 = (t2 >= T(0)) ? t2 : T(0);
        w0 = (u0 >= T(0)) ? t0 : -t0;
        w1 = (u1 >= T(0)) ? t1 : -t1;
        w2 = (u2 >= T(0)) ? t2 : -t2;
        l1 += to_acc(t0) + to_acc(t1) + to_acc(t2);
    } else if constexpr (std::is_same<T, df64>::value) {
        // |u| and 1/|u| from one reciprocal square root: t = |u| - 1/beta and
        // t/|u| = 1 - (1/beta)(1/|u|), so no double-float division runs
        const df64 ss = sum_sq3(u0, u1, u2);
        T t = T(0), sc = T(0);
        if (ss.hi > 0.f) {
            const df64 y = rsqrt_df(ss);
            t = ss * y - ib;
            if (t > T(0)) sc = df64(1.f) - ib * y;
            else t = T(0);
        }
        w0 = u0 * sc;
        w1 = u1 * sc;
        w2 = u2 * sc;
        l1 += to_acc(t);
    } else {
        T nv = sqrt(u0 * u0 + u1 * u1 + u2 * u2);
        T t = nv - ib;
        t = (t > T(0)) ? t : T(0);
        T sc = (t > T(0)) ? t / nv : T(0);
        w0 = u0 * sc;
        w1 = u1 * sc;
        w2 = u2 * sc;
        l1 += to_acc(t);
    }
    const T v0 = d0 - w0, v1 = d1 - w1, v2 = d2 - w2;
    l2.add(v0, v0);
    l2.add(v1, v1);
    l2.add(v2, v2);
    l4.add(v0, s0);
    l4.add(v1, s1);
    l4.add(v2, s2);
}

// ---------------------------------------------------------------------------
// descent step fused with D: U = P(Up - tau d), DU = D U, and the two terms
// of the new point's Lagrangian that need DU: lam2 = ||DU - W||^2 and
// lam4 = <sigma, DU - W> (get_g_gpu's lam2_4 pass, :528-547, done here while
// DU is in registers instead of by a second pass over DU, W and sigma).  The
// same pass forms update_W's shrinkage of the full step into the free W slot
// with its lam1, lam2, lam4: most steps pass the Armijo test, which then
// commits it (armijo_decide) and no shrinkage pass runs.  U at the forward
// neighbours is recomputed from Up and d (same expression, so bit-identical
// to the stored value).  Normal mode reads the current slot, writes the other
// one and flips the parity (the previous values become Up, gp, g2p, Aup, DUp
// without copies, :831-833); restart mode reads the previous slot (U = Up,
// :878) and writes the current one.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256, 4) k_descend(SolverBufs<T> B, Geo g, int restart) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    using A = acc_t<T>;
    const int cur = ctl->parity, ws = ctl->wsel;
    const int src = restart ? 1 - cur : cur, dst = restart ? cur : 1 - cur;
    const T* __restrict__ Up = B.U[src];
    const T* __restrict__ d = B.d;
    T* __restrict__ U = B.U[dst];
    T* __restrict__ DU = B.DU[dst];
    const T* __restrict__ W = B.W[ws];
    T* __restrict__ Wn = B.W[1 - ws];  // speculative update_W of the full step
    const T* __restrict__ S = B.sig;
    const T mt = scal<T>(-ctl->tau);
    const T bt = scal<T>(ctl->beta), ib = scal<T>(1.0 / ctl->beta);
    const int nn = ctl->nonneg, iso = ctl->iso;
    const long n = B.n;
    ProdAcc<T> l2, l4, l2s, l4s;
    A l1s(0.f);
    if (g.l.d == 1 && (g.p.d % 2) == 0) {
        // voxel pairs (i, i+1) with y even: they share x and z, so their +x
        // and +z neighbours are pairs too and the +y neighbour of i is i+1
        GRID_STRIDE_PAIRS(i, n) {
            const Nb nb = neighbours(g, i);
            const Two<T> u0 = ld2(Up + i), d0 = ld2(d + i);
            const T uca = proj(u0.a + mt * d0.a, nn), ucb = proj(u0.b + mt * d0.b, nn);
            const unsigned ya = (unsigned)i - fdiv((unsigned)i, g.p) * g.p.d;  // even, <= p - 2
            const long yb = (ya + 2 < g.p.d) ? i + 2 : i + 2 - (long)g.p.d;     // +y neighbour of i+1
            const T uyb = proj(Up[yb] + mt * d[yb], nn);
            const Two<T> ux = ld2(Up + nb.xp), dx = ld2(d + nb.xp);
            const Two<T> uz = ld2(Up + nb.zp), dz = ld2(d + nb.zp);
            const T uxa = proj(ux.a + mt * dx.a, nn), uxb = proj(ux.b + mt * dx.b, nn);
            const T uza = proj(uz.a + mt * dz.a, nn), uzb = proj(uz.b + mt * dz.b, nn);
            const Two<T> dv[3] = {{ucb - uca, uyb - ucb}, {uxa - uca, uxb - ucb}, {uza - uca, uzb - ucb}};
            st2(U + i, uca, ucb);
            Two<T> sg[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                st2(DU + c * n + i, dv[c].a, dv[c].b);
                const Two<T> w = ld2(W + c * n + i);
                sg[c] = ld2(S + c * n + i);
                const T va = dv[c].a - w.a, vb = dv[c].b - w.b;
                l2.add(va, va);
                l2.add(vb, vb);
                l4.add(va, sg[c].a);
                l4.add(vb, sg[c].b);
            }
            T a0, a1, a2, b0, b1, b2;
            shrink_voxel(dv[0].a, dv[1].a, dv[2].a, sg[0].a, sg[1].a, sg[2].a, bt, ib, iso, a0, a1, a2, l1s, l2s, l4s);
            shrink_voxel(dv[0].b, dv[1].b, dv[2].b, sg[0].b, sg[1].b, sg[2].b, bt, ib, iso, b0, b1, b2, l1s, l2s, l4s);
            st2(Wn + i, a0, b0);
            st2(Wn + n + i, a1, b1);
            st2(Wn + 2 * n + i, a2, b2);
        }
    } else {
        GRID_STRIDE(i, n) {
            Nb nb = neighbours(g, i);
            T uc = proj(Up[i] + mt * d[i], nn);
            T uy = proj(Up[nb.yp] + mt * d[nb.yp], nn);
            T ux = proj(Up[nb.xp] + mt * d[nb.xp], nn);
            T uz = proj(Up[nb.zp] + mt * d[nb.zp], nn);
            const T dv[3] = {uy - uc, ux - uc, uz - uc};
            U[i] = uc;
            T sg[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                DU[c * n + i] = dv[c];
                sg[c] = S[c * n + i];
                const T v = dv[c] - W[c * n + i];
                l2.add(v, v);
                l4.add(v, sg[c]);
            }
            T w0, w1, w2;
            shrink_voxel(dv[0], dv[1], dv[2], sg[0], sg[1], sg[2], bt, ib, iso, w0, w1, w2, l1s, l2s, l4s);
            Wn[i] = w0;
            Wn[n + i] = w1;
            Wn[2 * n + i] = w2;
        }
    }
    double v[5] = {l2.value(), l4.value(), acc_d(l1s), l2s.value(), l4s.value()}, tot[5];
    if (grid_reduce<5>(v, B.part, B.ticket, tot) && threadIdx.x == 0) {
        ctl->lam2 = tot[0];
        ctl->lam4 = tot[1];
        ctl->lam1s = tot[2];
        ctl->lam2s = tot[3];
        ctl->lam4s = tot[4];
        if (!restart) ctl->parity = 1 - cur;
        // the A*U product that follows takes the Armijo decision in its
        // lam3/lam5 epilogue
        ctl->post_mode = restart ? EPI_G2_RESTART : EPI_G2_DESCEND;
        ctl->post_graph = B.use_graph;
        ctl->post_h_arm = B.h_arm;
    }
}

// ---------------------------------------------------------------------------
// first inner iteration: ||D d||^2 and <d,d>
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_Dd_norm(SolverBufs<T> B, Geo g) {
    count_launch(B.ctl);
    using A = acc_t<T>;
    const T* __restrict__ d = B.d;
    A s0(0.f), s1(0.f);
    GRID_STRIDE(i, B.n) {
        Nb nb = neighbours(g, i);
        T dc = d[i];
        A a = to_acc(d[nb.yp] - dc), b = to_acc(d[nb.xp] - dc), c = to_acc(d[nb.zp] - dc), e = to_acc(dc);
        s0 += a * a + b * b + c * c;
        s1 += e * e;
    }
    double v[2] = {acc_d(s0), acc_d(s1)}, tot[2];
    if (grid_reduce<2>(v, B.part, B.ticket, tot) && threadIdx.x == 0) {
        B.ctl->dDd = tot[0];
        B.ctl->dd = tot[1];
    }
}

// ---------------------------------------------------------------------------
// g2 = D^T (DU - W) with lam2 = ||DU - W||^2 and lam4 = <sigma, DU - W>
// (start-up get_g; after a descent lam2 and lam4 come from k_descend, and the
// g2 of the new point is replaced by update_W's before anything reads it).
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_g2(SolverBufs<T> B, Geo g) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    const int cur = ctl->parity;
    const long n = B.n;
    const T* __restrict__ DU = B.DU[cur];
    const T* __restrict__ W = B.W[ctl->wsel];
    const T* __restrict__ S = B.sig;
    T* __restrict__ g2 = B.g2[cur];
    ProdAcc<T> l2, l4;
    GRID_STRIDE(i, n) {
        T v0 = DU[i] - W[i], v1 = DU[n + i] - W[n + i], v2 = DU[2 * n + i] - W[2 * n + i];
        Nb nb = neighbours(g, i);
        T v0m = DU[nb.ym] - W[nb.ym];
        T v1m = DU[n + nb.xm] - W[n + nb.xm];
        T v2m = DU[2 * n + nb.zm] - W[2 * n + nb.zm];
        g2[i] = v0m - v0 + v1m - v1 + v2m - v2;
        l2.add(v0, v0);
        l2.add(v1, v1);
        l2.add(v2, v2);
        l4.add(v0, S[i]);
        l4.add(v1, S[n + i]);
        l4.add(v2, S[2 * n + i]);
    }
    double v[2] = {l2.value(), l4.value()}, tot[2];
    if (grid_reduce<2>(v, B.part, B.ticket, tot) && threadIdx.x == 0) {
        ctl->lam2 = tot[0];
        ctl->lam4 = tot[1];
        ctl->f = fval(ctl);
        ctl->armijo_fail = 0;
    }
}

// ---------------------------------------------------------------------------
// shrinkage: W = shrink(DU - sigma/beta, 1/beta), lam1 = TV(W), and the
// terms of update_W that need only the voxel itself: lam2 = ||DU - W||^2,
// lam4 = <sigma, DU - W>
// ---------------------------------------------------------------------------
template <class T, bool PAIRS>
__global__ void __launch_bounds__(256, 4) k_shrink(SolverBufs<T> B, int mode) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    using A = acc_t<T>;
    const int cur = ctl->parity, ws = ctl->wsel;
    const long n = B.n;
    const T* __restrict__ DU = B.DU[cur];
    const T* __restrict__ S = B.sig;
    T* __restrict__ W = B.W[1 - ws];  // the new W goes to the free slot
    const T bt = scal<T>(ctl->beta), ib = scal<T>(1.0 / ctl->beta);
    const int iso = ctl->iso;
    A l1(0.f);
    ProdAcc<T> l2, l4;
    if (PAIRS) {
        GRID_STRIDE_PAIRS(i, n) {
            const Two<T> d0 = ld2(DU + i), d1 = ld2(DU + n + i), d2 = ld2(DU + 2 * n + i);
            const Two<T> s0 = ld2(S + i), s1 = ld2(S + n + i), s2 = ld2(S + 2 * n + i);
            T a0, a1, a2, b0, b1, b2;
            shrink_voxel(d0.a, d1.a, d2.a, s0.a, s1.a, s2.a, bt, ib, iso, a0, a1, a2, l1, l2, l4);
            shrink_voxel(d0.b, d1.b, d2.b, s0.b, s1.b, s2.b, bt, ib, iso, b0, b1, b2, l1, l2, l4);
            st2(W + i, a0, b0);
            st2(W + n + i, a1, b1);
            st2(W + 2 * n + i, a2, b2);
        }
    } else {
        GRID_STRIDE(i, n) shrink_voxel(DU[i], DU[n + i], DU[2 * n + i], S[i], S[n + i], S[2 * n + i], bt, ib, iso, W[i],
                                       W[n + i], W[2 * n + i], l1, l2, l4);
    }
    double v[3] = {acc_d(l1), l2.value(), l4.value()}, tot[3];
    if (grid_reduce<3>(v, B.part, B.ticket, tot) && threadIdx.x == 0) {
        ctl->wsel = 1 - ws;
        if (mode == EPI_G2_UPDATE_W) {
            // update_W (:1016-1029): f takes the new lam1, lam2, lam4; then the
            // nonmonotone reference values (:1176-1177)
            ctl->f -= ctl->lam1 + ctl->beta / 2 * ctl->lam2 - ctl->lam4;
            ctl->lam1 = tot[0];
            ctl->lam2 = tot[1];
            ctl->lam4 = tot[2];
            ctl->f += ctl->lam1 + ctl->beta / 2 * ctl->lam2 - ctl->lam4;
            const double Qp = ctl->Q;
            ctl->Q = ctl->gam * Qp + 1.0;
            ctl->C = (ctl->gam * Qp * ctl->C + ctl->f) / ctl->Q;
        } else {
            ctl->lam1 = tot[0];  // start-up: k_g2 forms lam2, lam4 and f next
        }
    }
}

// ---------------------------------------------------------------------------
// d = mu/beta g + g2 + DtsAtd, with ||Up||, ||U - Up|| (RelChg) and <d,d>
// (mode 0: start-up, mode 1: inner iteration).  In an inner iteration the
// same pass forms the next iteration's Barzilai-Borwein step (get_tau_gpu,
// :612-664): ss = ||U - Up||^2 and sy = <U - Up, (g2 - g2p) + mu/beta (g - gp)>
// read exactly the vectors the next get_tau would (update_W changes only g2,
// which is final here), so tau is ready when the next iteration starts; a
// first iteration overwrites it with the exact step.
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_gradient(SolverBufs<T> B, int iter) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    using A = acc_t<T>;
    const int cur = ctl->parity, prv = 1 - cur;
    const T mdb = scal<T>(ctl->muDbeta);
    const A mdbA = scal<A>(ctl->muDbeta);
    const T *__restrict__ g = B.g[cur], *__restrict__ g2 = B.g2[cur], *__restrict__ dts = B.DtsAtd;
    const T *__restrict__ gp = B.g[prv], *__restrict__ g2p = B.g2[prv];
    const T *__restrict__ U = B.U[cur], *__restrict__ Up = B.U[prv];
    const Ext<T>* __restrict__ xs = static_cast<const Ext<T>*>(B.xstar);
    const double iscl = 1.0 / ctl->scl;
    T* __restrict__ d = B.d;
    ProdAcc<A> s0, s1, s2, s4;
    double s3 = 0.0;
    GRID_STRIDE(i, B.n) {
        const T gi = g[i], g2i = g2[i];
        T di = mdb * gi + g2i + dts[i];
        d[i] = di;
        const A ad = to_acc(di);
        s2.add(ad, ad);
        if (iter) {
            A u = to_acc(U[i]), up = to_acc(Up[i]);
            A du = u - up;
            s0.add(up, up);
            s1.add(du, du);
            A dg = to_acc(gi) - to_acc(gp[i]);
            A dg2 = to_acc(g2i) - to_acc(g2p[i]);
            s4.add(du, dg2 + mdbA * dg);
            if (xs) {
                double e = acc_d(u) * iscl - (double)xs[i];
                s3 += e * e;
            }
        }
    }
    double v[5] = {s0.value(), s1.value(), s2.value(), s3, s4.value()}, tot[5];
    if (grid_reduce<5>(v, B.part, B.ticket, tot) && threadIdx.x == 0) {
        ctl->dd = tot[2];
        if (!iter) {
            ctl->Q = 1.0;
            ctl->C = ctl->f;
        } else {
            ctl->tau = fabs(tot[1] / tot[4]);  // next iteration's BB step
            ctl->nrmup = sqrt(tot[0]);
            ctl->relchg = sqrt(tot[1]) / ctl->nrmup;
            if (B.trace && xs) B.trace[ctl->count_total] = sqrt(tot[3]);
            ctl->count_total += 1;
            ctl->inner_break = ((ctl->relchg < ctl->tol_inn) && !ctl->fst) || (ctl->count_total >= ctl->maxit);
            ctl->fst = 0;
            if (B.use_graph) cudaGraphSetConditional(B.h_inner, ctl->inner_break ? 0u : 1u);
        }
    }
}

// ---------------------------------------------------------------------------
// The end of an inner iteration in one pass: update_W's g2 = D^T (DU - W)
// (its lam2 and lam4 come from k_shrink) and get_gradient's d with the next
// step size and the stopping test (k_gradient, iter 1).  g2[i] is formed and
// used by the same thread, so the pass saves the store-and-reload of g2 and a
// launch.
// ---------------------------------------------------------------------------
template <class T>
__global__ void __launch_bounds__(256, 4) k_g2_gradient(SolverBufs<T> B, Geo geo) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    using A = acc_t<T>;
    const int cur = ctl->parity, prv = 1 - cur;
    const long n = B.n;
    const T* __restrict__ DU = B.DU[cur];
    const T* __restrict__ W = B.W[ctl->wsel];
    T* __restrict__ g2o = B.g2[cur];
    const T mdb = scal<T>(ctl->muDbeta);
    const A mdbA = scal<A>(ctl->muDbeta);
    const T *__restrict__ g = B.g[cur], *__restrict__ dts = B.DtsAtd;
    const T *__restrict__ gp = B.g[prv], *__restrict__ g2p = B.g2[prv];
    const T *__restrict__ U = B.U[cur], *__restrict__ Up = B.U[prv];
    const Ext<T>* __restrict__ xs = static_cast<const Ext<T>*>(B.xstar);
    const double iscl = 1.0 / ctl->scl;
    T* __restrict__ d = B.d;
    ProdAcc<A> s0, s1, s2, s4;
    double s3 = 0.0;
    // the gradient part of one voxel, given its g2
    auto grad = [&](long i, T g2i, T gi, T dtsi, T Ui, T Upi, T gpi, T g2pi, T& di) {
        di = mdb * gi + g2i + dtsi;
        const A ad = to_acc(di);
        s2.add(ad, ad);
        const A u = to_acc(Ui), up = to_acc(Upi);
        const A du = u - up;
        s0.add(up, up);
        s1.add(du, du);
        const A dg = to_acc(gi) - to_acc(gpi);
        const A dg2 = to_acc(g2i) - to_acc(g2pi);
        s4.add(du, dg2 + mdbA * dg);
        if (xs) {
            double e = acc_d(u) * iscl - (double)xs[i];
            s3 += e * e;
        }
    };
    if (geo.l.d == 1 && (geo.p.d % 2) == 0) {
        // voxel pairs (i, i+1) with y even: -x and -z neighbours are pairs, the
        // -y neighbour of i+1 is i
        GRID_STRIDE_PAIRS(i, n) {
            const Nb nb = neighbours(geo, i);
            Two<T> va[3];
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                const Two<T> du = ld2(DU + c * n + i), w = ld2(W + c * n + i);
                va[c] = {du.a - w.a, du.b - w.b};
            }
            const T v0m = DU[nb.ym] - W[nb.ym];
            const Two<T> dxm = ld2(DU + n + nb.xm), wxm = ld2(W + n + nb.xm);
            const Two<T> dzm = ld2(DU + 2 * n + nb.zm), wzm = ld2(W + 2 * n + nb.zm);
            const T g2a = v0m - va[0].a + (dxm.a - wxm.a) - va[1].a + (dzm.a - wzm.a) - va[2].a;
            const T g2b = va[0].a - va[0].b + (dxm.b - wxm.b) - va[1].b + (dzm.b - wzm.b) - va[2].b;
            st2(g2o + i, g2a, g2b);
            const Two<T> gi = ld2(g + i), dt = ld2(dts + i), u = ld2(U + i), up = ld2(Up + i);
            const Two<T> gpi = ld2(gp + i), g2pi = ld2(g2p + i);
            T da, db;
            grad(i, g2a, gi.a, dt.a, u.a, up.a, gpi.a, g2pi.a, da);
            grad(i + 1, g2b, gi.b, dt.b, u.b, up.b, gpi.b, g2pi.b, db);
            st2(d + i, da, db);
        }
    } else GRID_STRIDE(i, n) {
        const Nb nb = neighbours(geo, i);
        const T v0 = DU[i] - W[i], v1 = DU[n + i] - W[n + i], v2 = DU[2 * n + i] - W[2 * n + i];
        const T v0m = DU[nb.ym] - W[nb.ym];
        const T v1m = DU[n + nb.xm] - W[n + nb.xm];
        const T v2m = DU[2 * n + nb.zm] - W[2 * n + nb.zm];
        const T g2i = v0m - v0 + v1m - v1 + v2m - v2;
        g2o[i] = g2i;
        T di;
        grad(i, g2i, g[i], dts[i], U[i], Up[i], gp[i], g2p[i], di);
        d[i] = di;
    }
    double v[5] = {s0.value(), s1.value(), s2.value(), s3, s4.value()}, tot[5];
    if (grid_reduce<5>(v, B.part, B.ticket, tot) && threadIdx.x == 0) {
        // get_gradient, the next BB step and the inner stopping test
        ctl->dd = tot[2];
        ctl->tau = fabs(tot[1] / tot[4]);
        ctl->nrmup = sqrt(tot[0]);
        ctl->relchg = sqrt(tot[1]) / ctl->nrmup;
        if (B.trace && xs) B.trace[ctl->count_total] = sqrt(tot[3]);
        ctl->count_total += 1;
        const int natural = ((ctl->relchg < ctl->tol_inn) && !ctl->fst) || (ctl->count_total >= ctl->maxit);
        ctl->paused = !natural && (ctl->count_total >= ctl->pause_at);
        ctl->inner_break = natural || ctl->paused;
        ctl->fst = 0;
        if (B.use_graph) cudaGraphSetConditional(B.h_inner, ctl->inner_break ? 0u : 1u);
    }
}

// ---------------------------------------------------------------------------
// Backtracking in closed form.  update_g_gpu (:706-818) moves every quantity
// along X(a) = Xp + a (X1 - Xp) (X1 the rejected full step) and re-evaluates
// f(a) = lam1 + beta/2 lam2 + mu/2 lam3 - lam4 - lam5 for a = gamma, gamma^2,
// ... (at most five, :859-888).  Along that segment lam2 and lam3 are exact
// quadratics and lam4, lam5 exact linear functions of a, so one pass over
// V0 = DUp - W, dV = DU1 - DUp, r0 = Aup - b, dr = Au1 - Aup gives their ten
// coefficients; the epilogue then runs the whole Armijo loop on scalars and
// either accepts the first admissible a or asks for the restart (cnt == 5,
// :876-882).  k_bt_apply materialises the accepted point once.
// ---------------------------------------------------------------------------
// Three blocks per SM (80 registers): with the ten compensated accumulators
// and the pair loads, 64 registers spill 24 bytes in double-float.
template <class T>
__global__ void __launch_bounds__(256, 3) k_bt_coef(SolverBufs<T> B) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    using A = acc_t<T>;
    const int cur = ctl->parity, prv = 1 - cur;
    const long n = B.n, m = B.m;
    const T *__restrict__ DU = B.DU[cur], *__restrict__ DUp = B.DU[prv];
    const T *__restrict__ Au = B.Au[cur], *__restrict__ Aup = B.Au[prv];
    const T *__restrict__ W = B.W[ctl->wsel], *__restrict__ S = B.sig, *__restrict__ bb = B.b, *__restrict__ dl = B.delta;
    // compensated product sums (ProdAcc), as in the other reductions
    ProdAcc<A> a2, b2, c2, a4, b4, a3, b3, c3, a5, b5;
    const long N = n > m ? n : m;
    auto vox = [&](T dp, T w, T du, T sg) {
        const A v0 = to_acc(dp - w), dv = to_acc(du - dp), s = to_acc(sg);
        a2.add(v0, v0);
        b2.add(v0, dv);
        c2.add(dv, dv);
        a4.add(s, v0);
        b4.add(s, dv);
    };
    auto ray = [&](T ap, T b_, T au, T d_) {
        const A r0 = to_acc(ap) - to_acc(b_), dr = to_acc(au) - to_acc(ap), d = to_acc(d_);
        a3.add(r0, r0);
        b3.add(r0, dr);
        c3.add(dr, dr);
        a5.add(d, r0);
        b5.add(d, dr);
    };
    if (n % 2 == 0 && m % 2 == 0) {
        // two elements per 16-byte (8-byte for float) access
        GRID_STRIDE_PAIRS(i, N) {
            if (i < n) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const long k = c * n + i;
                    const Two<T> dp = ld2(DUp + k), w = ld2(W + k), du = ld2(DU + k), sg = ld2(S + k);
                    vox(dp.a, w.a, du.a, sg.a);
                    vox(dp.b, w.b, du.b, sg.b);
                }
            }
            if (i < m) {
                const Two<T> ap = ld2(Aup + i), b_ = ld2(bb + i), au = ld2(Au + i), d_ = ld2(dl + i);
                ray(ap.a, b_.a, au.a, d_.a);
                ray(ap.b, b_.b, au.b, d_.b);
            }
        }
    } else {
        GRID_STRIDE(i, N) {
            if (i < n) {
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    const long k = c * n + i;
                    vox(DUp[k], W[k], DU[k], S[k]);
                }
            }
            if (i < m) ray(Aup[i], bb[i], Au[i], dl[i]);
        }
    }
    double v[10] = {a2.value(), b2.value(), c2.value(), a4.value(), b4.value(),
                    a3.value(), b3.value(), c3.value(), a5.value(), b5.value()},
           tot[10];
    if (grid_reduce<10>(v, B.part, B.ticket, tot) && threadIdx.x == 0) {
        // alpha was already multiplied by gamma once by the Armijo epilogue of k_g2
        int cnt = 0;
        bool fail = true;
        while (fail && cnt < 5) {
            const double al = ctl->alpha;
            ctl->lam2 = tot[0] + 2.0 * al * tot[1] + al * al * tot[2];
            ctl->lam4 = tot[3] + al * tot[4];
            ctl->lam3 = tot[5] + 2.0 * al * tot[6] + al * al * tot[7];
            ctl->lam5 = tot[8] + al * tot[9];
            ctl->f = fval(ctl);
            ++cnt;
            armijo(ctl);
            fail = ctl->armijo_fail;
            if (fail && cnt < 5) ctl->alpha *= ctl->gamma;
        }
        ctl->cnt = cnt;
        ctl->backtracks += cnt;
        if (fail) ctl->gam *= ctl->rate_gam;  // restart follows (:876-882)
    }
}

// X = Xp + alpha (X1 - Xp) for U, g, g2, DU (n) and Au (m), in place in the
// current slot (the full-step values X1 are read before they are replaced)
template <class T>
__global__ void k_bt_apply(SolverBufs<T> B) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    if (ctl->armijo_fail) return;  // restart path: nothing to apply
    const int cur = ctl->parity, prv = 1 - cur;
    const long n = B.n, m = B.m;
    const T al = scal<T>(ctl->alpha);
    T *__restrict__ U = B.U[cur], *__restrict__ g = B.g[cur];
    T *__restrict__ DU = B.DU[cur], *__restrict__ Au = B.Au[cur];
    const T *__restrict__ Up = B.U[prv], *__restrict__ gp = B.g[prv];
    const T *__restrict__ DUp = B.DU[prv], *__restrict__ Aup = B.Au[prv];
    const long N = n > m ? n : m;
    GRID_STRIDE(i, N) {
        if (i < n) {
            T p = Up[i];
            U[i] = p + al * (U[i] - p);
            p = gp[i];
            g[i] = p + al * (g[i] - p);
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                p = DUp[c * n + i];
                DU[c * n + i] = p + al * (DU[c * n + i] - p);
            }
        }
        if (i < m) {
            T p = Aup[i];
            Au[i] = p + al * (Au[i] - p);
        }
    }
}

// ---------------------------------------------------------------------------
// outer loop: RelChgOut = ||U - rcdU|| / ||Up||, rcdU = U
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_outer_relchg(SolverBufs<T> B) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    using A = acc_t<T>;
    if (ctl->paused) {
        // stopped by the pause limit in the middle of an outer iteration: the
        // outer step is left for the resumed solve
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            ctl->done = 1;
            if (B.use_graph) cudaGraphSetConditional(B.h_mlp, 0u);
        }
        return;
    }
    const T* __restrict__ U = B.U[ctl->parity];
    T* __restrict__ R = B.rcdU;
    A s(0.f);
    GRID_STRIDE(i, B.n) {
        T u = U[i];
        A e = to_acc(u) - to_acc(R[i]);
        s += e * e;
        R[i] = u;
    }
    double v[1] = {acc_d(s)}, tot[1];
    if (grid_reduce<1>(v, B.part, B.ticket, tot) && threadIdx.x == 0) {
        ctl->count_outer += 1;
        ctl->relchgout = sqrt(tot[0]) / ctl->nrmup;
        ctl->done = (ctl->relchgout < ctl->tol);
        if (B.use_graph) cudaGraphSetConditional(B.h_mlp, ctl->done ? 0u : 1u);
    }
}

// copies one control flag into a graph conditional handle
__global__ void k_cond(Ctl* ctl, unsigned long long h, int src) {
    count_launch(ctl);
    unsigned v = 0;
    switch (src) {
        case COND_FST: v = ctl->fst ? 1u : 0u; break;
        case COND_RESTART: v = ctl->armijo_fail ? 1u : 0u; break;
        case COND_ONE: v = 1u; break;
        default: v = ctl->done ? 0u : 1u; break;
    }
    cudaGraphSetConditional(h, v);
}

void launch_cond(Ctl* ctl, unsigned long long handle, int src, cudaStream_t s) {
    k_cond<<<1, 1, 0, s>>>(ctl, handle, src);
}

// ---------------------------------------------------------------------------
// skip-A^T heuristic (get_g_gpu, 3d/tval3_gpu_3d.cpp:398-468): after A*U,
// ||Au - last_Au|| / ||Au|| and the reference's rule decide whether this
// get_g forms A^T Au (forced at start-up and at a restart; always during the
// first numInitIterations calls; then while the skip budget allows, or when
// Au moved more than maxRelativeChange).  A skipped call keeps the previous g
// (the reference also subtracts Atb from it once more, :562-565: a defect
// not reproduced).
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_skip_decide(SolverBufs<T> B, int force) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    const T* __restrict__ Au = B.Au[ctl->parity];
    const T* __restrict__ la = B.last_Au;
    double dn = 0.0, an = 0.0;
    GRID_STRIDE(i, B.m) {
        const double a = acc_d(to_acc(Au[i])), d = a - acc_d(to_acc(la[i]));
        dn += d * d;
        an += a * a;
    }
    double v[2] = {dn, an}, tot[2];
    if (grid_reduce<2>(v, B.part, B.ticket, tot) && threadIdx.x == 0) {
        const double rel = sqrt(tot[0]) / sqrt(tot[1]);
        ctl->rel_change = rel;
        int mult = 1;
        if (force) {
            ctl->cur_skip = 0.0;
        } else if (ctl->cur_init < ctl->num_init) {
            ctl->cur_init += 1;
            ctl->cur_skip = 0.0;
        } else if (ctl->cur_skip < 1.0) {
            ctl->cur_skip += ctl->skip_ratio;
        } else if (!(rel > ctl->max_rel_change)) {
            ctl->cur_skip -= 1.0;
            mult = 0;
        }
        ctl->do_mult = mult;
        if (mult) ctl->products_T += 1;
        if (B.use_graph) {
            cudaGraphSetConditional(B.h_mult, mult ? 1u : 0u);
            cudaGraphSetConditional(B.h_keep, mult ? 0u : 1u);
        }
    }
}

template <class T>
__global__ void k_skip_copy(SolverBufs<T> B, int which) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    const int cur = ctl->parity;
    if (which == 0) {
        const T* __restrict__ Au = B.Au[cur];
        T* __restrict__ la = B.last_Au;
        GRID_STRIDE(i, B.m) la[i] = Au[i];
    } else {
        const T* __restrict__ gp = B.g[1 - cur];
        T* __restrict__ g = B.g[cur];
        GRID_STRIDE(i, B.n) g[i] = gp[i];
    }
}

// ---------------------------------------------------------------------------
// multiplier update and continuation
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_mlp(SolverBufs<T> B) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    using A = acc_t<T>;
    const int cur = ctl->parity;
    const long n = B.n, m = B.m;
    const T bt = scal<T>(ctl->beta), mut = scal<T>(ctl->mu);
    const T *__restrict__ DU = B.DU[cur], *__restrict__ W = B.W[ctl->wsel], *__restrict__ Au = B.Au[cur], *__restrict__ bb = B.b;
    T *__restrict__ S = B.sig, *__restrict__ dl = B.delta;
    A l4(0.f), l5(0.f);
    const long N = n > m ? n : m;
    GRID_STRIDE(i, N) {
        if (i < n) {
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                T v = DU[a * n + i] - W[a * n + i];
                T s = S[a * n + i] - bt * v;
                S[a * n + i] = s;
                l4 += to_acc(s) * to_acc(v);
            }
        }
        if (i < m) {
            T aub = Au[i] - bb[i];
            T dv = dl[i] - mut * aub;
            dl[i] = dv;
            l5 += to_acc(dv) * to_acc(aub);
        }
    }
    double v[2] = {acc_d(l4), acc_d(l5)}, tot[2];
    if (grid_reduce<2>(v, B.part, B.ticket, tot) && threadIdx.x == 0) {
        ctl->f += ctl->lam4 + ctl->lam5;
        ctl->lam4 = tot[0];
        ctl->lam5 = tot[1];
        ctl->f -= ctl->lam4 + ctl->lam5;
        ctl->beta_prev = ctl->beta;
        ctl->beta *= ctl->rate_cnt;
        ctl->mu *= ctl->rate_cnt;
        if (ctl->beta > ctl->beta_max) ctl->beta = ctl->beta_max;
        if (ctl->mu > ctl->mu_max) ctl->mu = ctl->mu_max;
        ctl->muDbeta = ctl->mu / ctl->beta;
        ctl->f = fval(ctl);
    }
}

template <class T>
__global__ void k_outer_grad(SolverBufs<T> B) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    using A = acc_t<T>;
    const int cur = ctl->parity;
    const T ratio = scal<T>(ctl->beta_prev / ctl->beta);
    const T mdb = scal<T>(ctl->muDbeta);
    const T *__restrict__ g = B.g[cur], *__restrict__ g2 = B.g2[cur];
    T *__restrict__ d = B.d, *__restrict__ dts = B.DtsAtd;
    A s(0.f);
    GRID_STRIDE(i, B.n) {
        T t = ratio * d[i];
        dts[i] = t;
        T di = mdb * g[i] + g2[i] + t;
        d[i] = di;
        A a = to_acc(di);
        s += a * a;
    }
    double v[1] = {acc_d(s)}, tot[1];
    if (grid_reduce<1>(v, B.part, B.ticket, tot) && threadIdx.x == 0) {
        ctl->dd = tot[0];
        ctl->gam = ctl->gam0;
        ctl->Q = 1.0;
        ctl->C = ctl->f;
        ctl->fst = 1;
        ctl->done = !(ctl->count_outer < ctl->maxcnt && ctl->count_total < ctl->maxit);
    }
}

// ---------------------------------------------------------------------------
// U_out = U / scl (:1272-1277) and rel_error vs Ut (:1308-1324)
// ---------------------------------------------------------------------------
template <class T>
__global__ void k_finalize(SolverBufs<T> B, Ext<T>* __restrict__ out, const Ext<T>* __restrict__ Ut) {
    Ctl* ctl = B.ctl;
    count_launch(ctl);
    const T* __restrict__ U = B.U[ctl->parity];
    const double scl = ctl->scl;
    const T s = scal<T>(scl);
    double e = 0.0, t = 0.0;
    const long L = B.L, n1 = B.n / B.L;
    GRID_STRIDE(i, B.n) {
        // out and Ut are the caller's n x L column-major arrays
        const long o = (L == 1) ? i : (i % L) * n1 + i / L;
        Ext<T> u = to_ext<T>((scl == 1.0) ? U[i] : U[i] / s);
        out[o] = u;
        if (Ut) {
            double dv = (double)Ut[o] - (double)u;
            e += dv * dv;
            t += (double)Ut[o] * Ut[o];
        }
    }
    double v[2] = {e, t}, tot[2];
    if (grid_reduce<2>(v, B.part, B.ticket, tot) && threadIdx.x == 0)
        ctl->rel_error = Ut ? sqrt(tot[0]) / sqrt(tot[1]) : 0.0;
}

// standalone D and D^T (operator entry points)
template <class T>
__global__ void k_D_plain(Geo g, long n, const T* __restrict__ U, T* __restrict__ DU) {
    GRID_STRIDE(i, n) {
        Nb nb = neighbours(g, i);
        T u = U[i];
        DU[i] = U[nb.yp] - u;
        DU[n + i] = U[nb.xp] - u;
        DU[2 * n + i] = U[nb.zp] - u;
    }
}

template <class T>
__global__ void k_Dt_plain(Geo g, long n, const T* __restrict__ V, T* __restrict__ out) {
    GRID_STRIDE(i, n) {
        Nb nb = neighbours(g, i);
        out[i] = V[nb.ym] - V[i] + V[n + nb.xm] - V[n + i] + V[2 * n + nb.zm] - V[2 * n + i];
    }
}

// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
// SM count of the current device, looked up once per device
int num_sms() {
    constexpr int MAXDEV = 64;
    static int sms[MAXDEV] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= MAXDEV) dev = 0;
    if (!sms[dev]) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 1;
        sms[dev] = v;
    }
    return sms[dev];
}

// Blocks of a grid-stride reducing kernel (256 threads): `want` (about one per
// 1,024 elements, so that small solves leave room for others), but never
// more than can be resident at once.  A grid one wave larger than the GPU
// holds runs its last partial wave at a fraction of the occupancy (608 blocks
// of a kernel that fits 3 per SM took two full waves' time).
static int resident_grid(const void* kernel, int want) {
    static std::mutex mu;
    static std::map<const void*, int> cap;
    std::lock_guard<std::mutex> lk(mu);
    auto it = cap.find(kernel);
    if (it == cap.end()) {
        int nb = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&nb, kernel, 256, 0) != cudaSuccess || nb < 1) nb = 1;
        it = cap.emplace(kernel, nb * num_sms()).first;
    }
    return std::max(1, std::min(want, it->second));
}
template <class... P, class... A>
static void rlaunch(void (*kernel)(P...), int want, cudaStream_t s, A... args) {
    launch_k(kernel, dim3(resident_grid(reinterpret_cast<const void*>(kernel), want)), dim3(256), 0, s, args...);
}

static int ew_grid(long n) {
    long g = (n + 255) / 256;
    long cap = (long)num_sms() * 16;
    if (g > cap) g = cap;
    if (g < 1) g = 1;
    return (int)g;
}

static Geo geo_of(int p, int q, int r, int L = 1) {
    Geo g;
    g.p = make_div((unsigned)p);
    g.q = make_div((unsigned)q);
    g.r = r;
    g.l = make_div((unsigned)(L > 1 ? L : 1));
    return g;
}
template <class T> static Geo geo_of(const SolverBufs<T>& B) { return geo_of(B.p, B.q, B.r, B.L); }

template <class T> void launch_scale_b(const void* b_in, SolverBufs<T>& B, cudaStream_t s) {
    const Ext<T>* b = static_cast<const Ext<T>*>(b_in);
    k_scale_find<Ext<T>><<<1, 1024, 0, s>>>(b, B.m, B.ctl);
    k_scale_apply<T><<<ew_grid(B.m), 256, 0, s>>>(b, B.b, B.m, B.L, B.ctl);
}
template <class T> void launch_D_only(SolverBufs<T>& B, cudaStream_t s) {
    k_D_only<T><<<ew_grid(B.n), 256, 0, s>>>(B, geo_of(B));
}
template <class T> void launch_descend(SolverBufs<T>& B, int restart, cudaStream_t s) {
    rlaunch(k_descend<T>, B.grid, s, B, geo_of(B), restart);
}
template <class T> void launch_Dd_norm(SolverBufs<T>& B, cudaStream_t s) {
    rlaunch(k_Dd_norm<T>, B.grid, s, B, geo_of(B));
}
template <class T> void launch_g2(SolverBufs<T>& B, int mode, cudaStream_t s) {
    // after a descent the A*U epilogue took the Armijo decision (lam35_post)
    if (mode != EPI_G2_DESCEND && mode != EPI_G2_RESTART) rlaunch(k_g2<T>, B.grid, s, B, geo_of(B));
}
template <class T> void launch_shrink(SolverBufs<T>& B, int mode, cudaStream_t s) {
    if (B.n % 2 == 0) rlaunch(k_shrink<T, true>, B.grid, s, B, mode);
    else rlaunch(k_shrink<T, false>, B.grid, s, B, mode);
}
template <class T> void launch_g2_gradient(SolverBufs<T>& B, cudaStream_t s) {
    rlaunch(k_g2_gradient<T>, B.grid, s, B, geo_of(B));
}
template <class T> void launch_gradient(SolverBufs<T>& B, int mode, cudaStream_t s) {
    rlaunch(k_gradient<T>, B.grid, s, B, mode);
}
template <class T> void launch_bt_coef(SolverBufs<T>& B, cudaStream_t s) { rlaunch(k_bt_coef<T>, B.grid, s, B); }
template <class T> void launch_bt_apply(SolverBufs<T>& B, cudaStream_t s) {
    rlaunch(k_bt_apply<T>, B.grid, s, B);
}
template <class T> void launch_outer_relchg(SolverBufs<T>& B, cudaStream_t s) { rlaunch(k_outer_relchg<T>, B.grid, s, B); }
template <class T> void launch_mlp(SolverBufs<T>& B, cudaStream_t s) { rlaunch(k_mlp<T>, B.grid, s, B); }
template <class T> void launch_outer_grad(SolverBufs<T>& B, cudaStream_t s) { rlaunch(k_outer_grad<T>, B.grid, s, B); }
template <class T> void launch_skip_decide(SolverBufs<T>& B, int force, cudaStream_t s) {
    rlaunch(k_skip_decide<T>, B.grid, s, B, force);
}
template <class T> void launch_skip_copy(SolverBufs<T>& B, int which, cudaStream_t s) {
    k_skip_copy<T><<<ew_grid(which == 0 ? B.m : B.n), 256, 0, s>>>(B, which);
}
template <class T> void launch_finalize(SolverBufs<T>& B, void* U_out, const void* Ut, cudaStream_t s) {
    rlaunch(k_finalize<T>, B.grid, s, B, static_cast<Ext<T>*>(U_out), static_cast<const Ext<T>*>(Ut));
}
template <class T> void launch_D_plain(int p, int q, int r, const T* U, T* DU3, cudaStream_t s) {
    long n = (long)p * q * r;
    k_D_plain<T><<<ew_grid(n), 256, 0, s>>>(geo_of(p, q, r), n, U, DU3);
}
template <class T> void launch_Dt_plain(int p, int q, int r, const T* V3, T* out, cudaStream_t s) {
    long n = (long)p * q * r;
    k_Dt_plain<T><<<ew_grid(n), 256, 0, s>>>(geo_of(p, q, r), n, V3, out);
}

#define INST(T)                                                                     \
    template void launch_scale_b<T>(const void*, SolverBufs<T>&, cudaStream_t);     \
    template void launch_D_only<T>(SolverBufs<T>&, cudaStream_t);                   \
    template void launch_descend<T>(SolverBufs<T>&, int, cudaStream_t);             \
    template void launch_Dd_norm<T>(SolverBufs<T>&, cudaStream_t);                  \
    template void launch_g2<T>(SolverBufs<T>&, int, cudaStream_t);                  \
    template void launch_shrink<T>(SolverBufs<T>&, int, cudaStream_t);              \
    template void launch_gradient<T>(SolverBufs<T>&, int, cudaStream_t);            \
    template void launch_g2_gradient<T>(SolverBufs<T>&, cudaStream_t);              \
    template void launch_bt_coef<T>(SolverBufs<T>&, cudaStream_t);                  \
    template void launch_bt_apply<T>(SolverBufs<T>&, cudaStream_t);                 \
    template void launch_outer_relchg<T>(SolverBufs<T>&, cudaStream_t);             \
    template void launch_mlp<T>(SolverBufs<T>&, cudaStream_t);                      \
    template void launch_outer_grad<T>(SolverBufs<T>&, cudaStream_t);               \
    template void launch_skip_decide<T>(SolverBufs<T>&, int, cudaStream_t);                  \
    template void launch_skip_copy<T>(SolverBufs<T>&, int, cudaStream_t);                    \
    template void launch_finalize<T>(SolverBufs<T>&, void*, const void*, cudaStream_t);
INST(float)
INST(double)
INST(df64)
template void launch_D_plain<float>(int, int, int, const float*, float*, cudaStream_t);
template void launch_D_plain<double>(int, int, int, const double*, double*, cudaStream_t);
template void launch_Dt_plain<float>(int, int, int, const float*, float*, cudaStream_t);
template void launch_Dt_plain<double>(int, int, int, const double*, double*, cudaStream_t);

}  // namespace tv3
