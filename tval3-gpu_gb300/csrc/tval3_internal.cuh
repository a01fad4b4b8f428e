// Internal definitions shared by the sm_103a kernels and the host solver.
//
// Layout in HBM (column-major, y fastest, as in the reference's
// 3d/tval3_gpu_3d_kernels.cu:1501): voxel (y, x, z) of a p x q x r volume sits
// at y + p*(x + q*z).  The three components of D*U are stored as three
// consecutive n-vectors (component 0 along y, 1 along x, 2 along z; the
// reference calls them Uy, Ux, Uz).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

#include "df64.cuh"

namespace tv3 {

constexpr unsigned FULL = 0xffffffffu;

// ---------------------------------------------------------------------------
// Vector element types: float, double, or df64 (double-float, FP32 pipes).
// Per-thread accumulation of the loop's inner products uses acc_t<T>: double
// for float and double vectors, df64 for df64 vectors (so no FP64 arithmetic
// runs per element in the double-float mode); only the block partials become
// double.  Ext<T> is the caller-facing element type (double for df64).
// ---------------------------------------------------------------------------
__device__ __forceinline__ double to_acc(float v) { return (double)v; }
__device__ __forceinline__ double to_acc(double v) { return v; }
__device__ __forceinline__ df64 to_acc(df64 v) { return v; }
template <class T> using acc_t = decltype(to_acc(T()));
__device__ __forceinline__ double acc_d(double a) { return a; }
__device__ __forceinline__ double acc_d(df64 a) { return (double)a; }

template <class T> struct ExtT { using type = T; };
template <> struct ExtT<df64> { using type = double; };
template <class T> using Ext = typename ExtT<T>::type;

// conversions between the caller-facing and the internal element type
template <class T> __device__ __forceinline__ T from_ext(Ext<T> v) { return (T)v; }
template <> __device__ __forceinline__ df64 from_ext<df64>(double v) { return df64(v); }
template <class T> __device__ __forceinline__ Ext<T> to_ext(T v) { return (Ext<T>)v; }
template <> __device__ __forceinline__ double to_ext<df64>(df64 v) { return (double)v; }
// a double scalar from the control block as an element-type constant
template <class T> __device__ __forceinline__ T scal(double v) { return (T)v; }
template <> __device__ __forceinline__ df64 scal<df64>(double v) { return df64(v); }

// Row-sum accumulators of the SpMV: plain sums for float/double, and for
// df64 the compensated dot product "Dot2" (Ogita, Rump & Oishi, "Accurate sum
// and dot product", SIAM J. Sci. Comput. 2005): the high parts are summed
// with TwoSum and every rounding error (of the sums and of the exact TwoProd
// products) is collected in one FP32 term, normalised once at the end.  The
// result is as accurate as if accumulated in twice the working precision, at
// ~11 FP32 operations per nonzero instead of ~26 for a full df64 add.
template <class T> struct RowAcc {
    T s;
    __device__ __forceinline__ RowAcc() : s(T(0)) {}
    __device__ __forceinline__ T value() const { return s; }
};
template <> struct RowAcc<df64> {
    float s, c;
    __device__ __forceinline__ RowAcc() : s(0.f), c(0.f) {}
    __device__ __forceinline__ df64 value() const { return fast_two_sum(s, c); }
};
// a + b of two partial accumulations (b's terms after a's)
__device__ __forceinline__ void combine(RowAcc<float>& a, const RowAcc<float>& b) { a.s += b.s; }
__device__ __forceinline__ void combine(RowAcc<double>& a, const RowAcc<double>& b) { a.s += b.s; }
__device__ __forceinline__ void combine(RowAcc<df64>& a, const RowAcc<df64>& b) {
    const df64 t = two_sum(a.s, b.s);
    a.s = t.hi;
    a.c = __fadd_rn(a.c, __fadd_rn(b.c, t.lo));
}
// one more summand p (sums of partial results): for df64 the high parts are
// added with TwoSum and the low parts and rounding errors collected in the
// compensation term, as in madd
__device__ __forceinline__ void add(RowAcc<float>& a, float p) { a.s += p; }
__device__ __forceinline__ void add(RowAcc<double>& a, double p) { a.s += p; }
__device__ __forceinline__ void add(RowAcc<df64>& a, df64 p) {
    const df64 t = two_sum(a.s, p.hi);
    a.s = t.hi;
    a.c = __fadd_rn(a.c, __fadd_rn(t.lo, p.lo));
}
__device__ __forceinline__ void madd(RowAcc<float>& a, float v, float x) { a.s = fmaf(v, x, a.s); }
__device__ __forceinline__ void madd(RowAcc<double>& a, float v, double x) { a.s = fma((double)v, x, a.s); }
__device__ __forceinline__ void madd(RowAcc<double>& a, double v, double x) { a.s = fma(v, x, a.s); }
__device__ __forceinline__ void madd(RowAcc<df64>& a, float v, df64 x) {
    df64 p = two_prod(x.hi, v);                // exact product of the high part
    float pl = __fmaf_rn(x.lo, v, p.lo);       // + low part (error of order u^2)
    df64 t = two_sum(a.s, p.hi);
    a.s = t.hi;
    a.c = __fadd_rn(a.c, __fadd_rn(t.lo, pl));
}

// Sums of products a*b for the loop's reductions (lam2, lam4, ...): FP64 for
// float and double vectors; for double-float vectors the exact high product
// plus the cross terms, accumulated with a compensated (Dot2-style) float
// pair, which costs about half the instructions of full double-float
// arithmetic and keeps errors of order u^2 per term.
template <class T> struct ProdAcc {
    double s = 0.0;
    __device__ __forceinline__ void add(T a, T b) { s = fma((double)a, (double)b, s); }
    __device__ __forceinline__ double value() const { return s; }
};
template <> struct ProdAcc<df64> {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(df64 a, df64 b) {
        df64 p = two_prod(a.hi, b.hi);
        const float pl = __fmaf_rn(a.hi, b.lo, __fmaf_rn(a.lo, b.hi, p.lo));
        df64 t = two_sum(s, p.hi);
        s = t.hi;
        c = __fadd_rn(c, __fadd_rn(t.lo, pl));
    }
    __device__ __forceinline__ double value() const { return (double)s + (double)c; }
};

__device__ __forceinline__ float shfl_down(unsigned mask, float v, int o, int w) { return __shfl_down_sync(mask, v, o, w); }
__device__ __forceinline__ double shfl_down(unsigned mask, double v, int o, int w) { return __shfl_down_sync(mask, v, o, w); }
__device__ __forceinline__ df64 shfl_down(unsigned mask, df64 v, int o, int w) {
    return df64(__shfl_down_sync(mask, v.hi, o, w), __shfl_down_sync(mask, v.lo, o, w));
}

// ---------------------------------------------------------------------------
// Device-resident control block of one solve.  All scalars of the TVAL3 loop
// (penalties, Lagrangian terms, step sizes, nonmonotone reference values,
// counters and branch flags) live here, so the loop runs without host round
// trips; kernels read their scalar inputs from it and the last block of each
// reducing kernel writes the results back.  Mirrors tval3_data_gpu
// (3d/tval3_gpu_3d.cpp:86-199) plus the loop locals of :1089-1345.
// ---------------------------------------------------------------------------
struct Ctl {
    // options (constant during a solve)
    double mu_max, beta_max, rate_cnt, tol, tol_inn, c_arm, gamma, gam0, rate_gam;
    int maxcnt, maxit, nonneg, iso;
    // penalties
    double mu, beta, muDbeta, beta_prev;
    // Lagrangian and its terms
    double f, lam1, lam2, lam3, lam4, lam5;
    // line search
    double tau, alpha, c_armij, C, Q, gam, dd, dDd, Add;
    // stopping tests
    double nrmup, relchg, relchgout, scl, rel_error;
    // counters and flags
    int count_outer, count_total, fst, cnt;
    int armijo_fail;   // 1: the Armijo test failed for the current step
    int inner_break;   // 1: the inner loop ends after this iteration
    int done;          // 1: the solve is finished
    int parity;        // slot index of the "current" ping-pong buffers
    int backtracks, restarts;
    int err;           // device-side error word (0 = none)
    unsigned launches; // kernels of this solve that ran (each counts itself once)
    // skip-A^T heuristic (3d/tval3_gpu_3d.cpp:155-157, :398-468)
    double skip_ratio, max_rel_change, cur_skip, rel_change;
    unsigned num_init, cur_init;
    int do_mult;       // 1: this get_g forms A^T Au; 0: it keeps the current g
    int products_T;    // A^T products formed by get_g
    // pausing: the solve stops after pause_at total iterations without ending
    // the outer iteration, so a saved state resumes exactly
    int pause_at, paused;
    // W slot in use; the descent writes a speculative update_W result (W of
    // the full step, its lam1, lam2, lam4) into the other slot, committed by
    // the Armijo test when the full step is accepted
    int wsel;
    double lam1s, lam2s, lam4s;
    // The Armijo decision after a descent is taken by the one thread that
    // finishes the A*U product's lam3/lam5 epilogue (lam35_post below):
    // k_descend arms it (post_mode EPI_G2_DESCEND or EPI_G2_RESTART, with the
    // graph's IF handle), and taking it clears post_mode.
    int post_mode, post_graph;
    unsigned long long post_h_arm;
};

// Programmatic dependent launch: a kernel launched with programmatic stream
// serialization (launch_k) may have its blocks scheduled while the kernel
// before it drains; griddepcontrol.wait holds every thread until that kernel
// has completed and its memory writes are visible.  For a kernel launched
// without the attribute it returns at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Entry of every solver kernel, before its first global-memory access: the
// dependent-launch wait, then the kernel counts itself once (block 0, thread 0).
__device__ __forceinline__ void count_launch(Ctl* c) {
    pdl_wait();
    if (c && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&c->launches, 1u);
}

// Epilogue selectors of the reducing kernels.
enum Epi : int {
    EPI_NONE = 0,
    EPI_LAM35 = 1,        // A*U: lam3, lam5
    EPI_ADD = 2,          // A*d at the first inner iteration: ||Ad||^2 -> tau
    EPI_G2_INIT = 3,      // get_g at start-up: f
    EPI_G2_DESCEND = 4,   // get_g after a descent step: f and the Armijo test
    EPI_G2_RESTART = 5,   // get_g after the restart descent: f
    EPI_G2_UPDATE_W = 6,  // update_W: f, Q, C
};

// f = lam1 + beta/2 lam2 + mu/2 lam3 - lam4 - lam5 (the augmented Lagrangian)
__device__ __forceinline__ double fval(const Ctl* c) {
    return c->lam1 + c->beta / 2 * c->lam2 + c->mu / 2 * c->lam3 - c->lam4 - c->lam5;
}

__device__ __forceinline__ void armijo(Ctl* c) {
    // |f| > |C - alpha * c_armij| : step rejected (3d/tval3_gpu_3d.cpp:848, :855)
    const int fail = fabs(c->f) > fabs(c->C - c->alpha * c->c_armij);
    c->armijo_fail = fail;
}

// f and the nonmonotone Armijo test after a descent (min_u_gpu,
// 3d/tval3_gpu_3d.cpp:848-858); one thread, once lam1..lam5 of the new point
// are known.  After the restart descent only f is formed (:876-882).
__device__ inline void armijo_decide(Ctl* ctl, int mode, int use_graph, unsigned long long h_arm) {
    ctl->f = fval(ctl);
    if (mode == EPI_G2_DESCEND) {
        ctl->alpha = 1.0;
        ctl->cnt = 0;
        ctl->c_armij = ctl->dd * ctl->tau * ctl->c_arm * ctl->beta;
        armijo(ctl);
        if (ctl->armijo_fail) {
            ctl->alpha *= ctl->gamma;
        } else {
            // full step accepted: update_W is the descent's speculative one
            // (:1016-1029), then the nonmonotone reference values (:1176-1177)
            ctl->wsel = 1 - ctl->wsel;
            ctl->f -= ctl->lam1 + ctl->beta / 2 * ctl->lam2 - ctl->lam4;
            ctl->lam1 = ctl->lam1s;
            ctl->lam2 = ctl->lam2s;
            ctl->lam4 = ctl->lam4s;
            ctl->f += ctl->lam1 + ctl->beta / 2 * ctl->lam2 - ctl->lam4;
            const double Qp = ctl->Q;
            ctl->Q = ctl->gam * Qp + 1.0;
            ctl->C = (ctl->gam * Qp * ctl->C + ctl->f) / ctl->Q;
        }
        if (use_graph) cudaGraphSetConditional(h_arm, ctl->armijo_fail ? 1u : 0u);
    } else {
        ctl->armijo_fail = 0;
        ctl->restarts += 1;
    }
}

// Called by the thread that has just written lam3 and lam5 of an A*U
// product: takes the Armijo decision that the descent armed, if any.
__device__ __forceinline__ void lam35_post(Ctl* c) {
    const int mode = c->post_mode;
    if (mode) {
        c->post_mode = 0;
        armijo_decide(c, mode, c->post_graph, c->post_h_arm);
    }
}

// ---------------------------------------------------------------------------
// Value loads.  Matrix streams are read once per product: load them with the
// evict-first policy (__ldcs) so they do not push x out of L2.
// ---------------------------------------------------------------------------
template <class V> __device__ __forceinline__ float ldv_f(const V* p);
template <> __device__ __forceinline__ float ldv_f<float>(const float* p) { return __ldcs(p); }
template <> __device__ __forceinline__ float ldv_f<__nv_bfloat16>(const __nv_bfloat16* p) {
    unsigned short u = __ldcs(reinterpret_cast<const unsigned short*>(p));
    return __uint_as_float(((unsigned)u) << 16);
}
template <> __device__ __forceinline__ float ldv_f<__half>(const __half* p) {
    unsigned short u = __ldcs(reinterpret_cast<const unsigned short*>(p));
    return __half2float(__ushort_as_half(u));
}

template <class T, class V> struct Acc;
template <> struct Acc<float, float> {
    __device__ static __forceinline__ float load(const float* p) { return __ldcs(p); }
};
template <> struct Acc<double, double> {
    __device__ static __forceinline__ double load(const double* p) { return __ldcs(p); }
};
template <> struct Acc<float, __nv_bfloat16> {
    __device__ static __forceinline__ float load(const __nv_bfloat16* p) { return ldv_f(p); }
};
template <> struct Acc<float, __half> {
    __device__ static __forceinline__ float load(const __half* p) { return ldv_f(p); }
};
template <> struct Acc<double, float> {
    __device__ static __forceinline__ double load(const float* p) { return (double)__ldcs(p); }
};
template <> struct Acc<df64, float> {
    __device__ static __forceinline__ df64 load(const float* p) { return df64(__ldcs(p)); }
};

// ---------------------------------------------------------------------------
// Deterministic grid reduction.  Every block reduces NV doubles with warp
// shuffles, writes its partials to part[k*gridDim.x + block], and takes a
// ticket; the last block sums the partials in block order (so the result
// depends only on the grid size, never on scheduling), resets the ticket and
// returns true with the totals in tot[] (valid in all threads of that block).
// ---------------------------------------------------------------------------
template <int NV>
__device__ __forceinline__ bool grid_reduce(double (&v)[NV], double* part, unsigned* ticket, double (&tot)[NV]) {
    __shared__ double sh[NV][32];
    __shared__ int is_last;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double t = v[k];
#pragma unroll
        for (int o = 16; o; o >>= 1) t += __shfl_down_sync(FULL, t, o);
        if (lane == 0) sh[k][warp] = t;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int k = 0; k < NV; ++k) {
            double t = (lane < nw) ? sh[k][lane] : 0.0;
#pragma unroll
            for (int o = 16; o; o >>= 1) t += __shfl_down_sync(FULL, t, o);
            if (lane == 0) part[(size_t)k * gridDim.x + blockIdx.x] = t;
        }
    }
    if (threadIdx.x == 0) {
        __threadfence();
        unsigned t = atomicAdd(ticket, 1u);
        is_last = (t == gridDim.x - 1);
    }
    __syncthreads();
    if (!is_last) return false;
    __threadfence();
    // fixed-order sum of the partials: thread j adds blocks j, j+B, ...; then a
    // fixed shuffle tree.
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double t = 0.0;
        for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) t += __ldcg(part + (size_t)k * gridDim.x + b);
#pragma unroll
        for (int o = 16; o; o >>= 1) t += __shfl_down_sync(FULL, t, o);
        if (lane == 0) sh[k][warp] = t;
    }
    __syncthreads();
#pragma unroll
    for (int k = 0; k < NV; ++k) {
        double t = 0.0;
        for (int w = 0; w < nw; ++w) t += sh[k][w];
        tot[k] = t;
    }
    if (threadIdx.x == 0) *ticket = 0u;
    return true;
}

// Voxel coordinates from a linear index.
struct Vol {
    int p, q, r;  // dim_y (fastest), dim_x, dim_z
    long n;       // p*q*r
    long pq;
};

}  // namespace tv3
