// One differentiable inner step of the TVAL3 u-subproblem and its
// hand-written adjoint (the autograd path).  The step is the reference's
// inner iteration (3d/tval3_gpu_3d.cpp:823-1029) without the nonmonotone
// Armijo decision, which is discrete:
//
//   DU  = D U,  V = DU - sigma/beta,  W = shrink(V, 1/beta)
//   g2  = D^T (DU - W - sigma/beta)                       (get_g_gpu :484-571)
//   g   = A^T (A U - b - delta/mu)
//   d   = g2 + kappa g,  kappa = mu/beta                  (get_gradient :896-919)
//   tau = |<s,s> / <s,y>|,  s = U - Up,  y = g2 - g2p + kappa (g - gp)
//         (first step: |<d,d> / (||D d||^2 + kappa ||A d||^2)|, :583-600, 1017-1067)
//   Un  = max(U - tau d, 0)  (or U - tau d without the projection)
//
// Outputs Un, g, g2 (g and g2 are the next step's gp, g2p).  The adjoint
// takes the output adjoints and returns those of U, Up, gp, g2p, b and
// (mu, beta).  It recomputes the step's intermediates from the inputs (the
// step is its own checkpoint: a chain of steps keeps only U, g, g2 per step)
// and then runs the transposed chain: the projection mask, the BB quotient's
// derivative (d tau/d<s,s> = 1/|<s,y>|, d tau/d<s,y> = -tau/<s,y>), the
// transposed products A^T, A, D^T, D and the shrinkage subgradient
// (shrink3.cuh).  Every elementwise part and every reduction is a kernel of
// this file; the scalar sums are deterministic grid reductions in FP64.
#include <cuda_runtime.h>
#include <algorithm>
#include "dbuf.h"
#include "launch.h"
#include "ops.h"
#include "shrink3.cuh"
#include "tval3_internal.cuh"

namespace tv3 {

namespace {

// device scalars of one step
enum {
    S_A = 0,      // <s,s> (first step: <d,d>)
    S_C = 1,      // <s,y> (first step: ||Dd||^2 + kappa ||Ad||^2)
    S_TAU = 2,
    S_AD2 = 3,    // ||A d||^2 (first step)
    S_DD2 = 4,    // ||D d||^2 (first step)
    S_TAUB = 5,   // adjoint of tau
    S_KAPB = 6,   // adjoint of kappa
    S_BETAB = 7,  // adjoint of beta (shrinkage and sigma terms)
    S_MUB = 8,    // adjoint of mu (delta term)
    S_N = 16
};

constexpr int UB = 256;  // threads per block of every kernel here

struct UVol {
    int p, q, r;
    long n;
};

__device__ __forceinline__ void nb_plus(const UVol& g, long i, long& yp, long& xp, long& zp) {
    const long pq = (long)g.p * g.q;
    const int y = (int)(i % g.p);
    const long t = i / g.p;
    const int x = (int)(t % g.q), z = (int)(t / g.q);
    yp = (y + 1 < g.p) ? i + 1 : i - y;
    xp = (x + 1 < g.q) ? i + g.p : i - (long)x * g.p;
    zp = (z + 1 < g.r) ? i + pq : i - (long)z * pq;
}

__device__ __forceinline__ void nb_minus(const UVol& g, long i, long& ym, long& xm, long& zm) {
    const long pq = (long)g.p * g.q;
    const int y = (int)(i % g.p);
    const long t = i / g.p;
    const int x = (int)(t % g.q), z = (int)(t / g.q);
    ym = (y > 0) ? i - 1 : i + (g.p - 1);
    xm = (x > 0) ? i - g.p : i + (long)(g.q - 1) * g.p;
    zm = (z > 0) ? i - pq : i + (long)(g.r - 1) * pq;
}

#define U_STRIDE(i, N) for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < (N); i += (long)gridDim.x * blockDim.x)

template <class T>
__device__ __forceinline__ T opt(const T* p, long i) {
    return p ? p[i] : T(0);
}

// DU of voxel i and V = DU - sigma/beta
template <class T>
__device__ __forceinline__ void du_v(const UVol& g, const T* __restrict__ U, const T* __restrict__ sig, T ib, long i,
                                     T du[3], T v[3]) {
    long yp, xp, zp;
    nb_plus(g, i, yp, xp, zp);
    const T u = U[i];
    du[0] = U[yp] - u;
    du[1] = U[xp] - u;
    du[2] = U[zp] - u;
    for (int c = 0; c < 3; ++c) v[c] = du[c] - opt(sig, c * g.n + i) * ib;
}

// ---------------------------------------------------------------------------
// forward
// ---------------------------------------------------------------------------
// P = DU - shrink(V, 1/beta) - sigma/beta (3n), whose D^T is g2
template <class T>
__global__ void __launch_bounds__(UB) k_uf_p(UVol g, const T* __restrict__ U, const T* __restrict__ sig,
                                             const double* __restrict__ mub, int iso, T* __restrict__ P) {
    const T ib = (T)(1.0 / mub[1]);
    U_STRIDE(i, g.n) {
        T du[3], v[3], w[3];
        du_v(g, U, sig, ib, i, du, v);
        shrink3_fwd(v, ib, iso, w);
        for (int c = 0; c < 3; ++c) P[c * g.n + i] = du[c] - w[c] - opt(sig, c * g.n + i) * ib;
    }
}

// r = A U - b - delta/mu (in place on A U)
template <class T>
__global__ void __launch_bounds__(UB) k_uf_resid(long m, T* __restrict__ r, const T* __restrict__ b,
                                                 const T* __restrict__ delta, const double* __restrict__ mub) {
    const T imu = (T)(1.0 / mub[0]);
    U_STRIDE(i, m) r[i] = r[i] - b[i] - opt(delta, i) * imu;
}

// d = g2 + kappa g, and the BB quotient's sums <s,s>, <s,y> (the last block
// sets tau); first step: <d,d> only
template <class T, bool FIRST>
__global__ void __launch_bounds__(UB) k_uf_dir(long n, const T* __restrict__ U, const T* __restrict__ Up,
                                               const T* __restrict__ g, const T* __restrict__ g2,
                                               const T* __restrict__ gp, const T* __restrict__ g2p,
                                               const double* __restrict__ mub, T* __restrict__ d, double* part,
                                               unsigned* ticket, double* sc) {
    const T kap = (T)(mub[0] / mub[1]);
    double a = 0.0, c = 0.0;
    U_STRIDE(i, n) {
        const T di = g2[i] + kap * g[i];
        d[i] = di;
        if (FIRST) {
            a += (double)di * di;
        } else {
            const double s = (double)U[i] - (double)Up[i];
            const double y = ((double)g2[i] - (double)g2p[i]) + (double)kap * ((double)g[i] - (double)gp[i]);
            a += s * s;
            c += s * y;
        }
    }
    double v[2] = {a, c}, tot[2];
    if (grid_reduce<2>(v, part, ticket, tot) && threadIdx.x == 0) {
        sc[S_A] = tot[0];
        if (!FIRST) {
            sc[S_C] = tot[1];
            sc[S_TAU] = fabs(tot[0] / tot[1]);
        }
    }
}

// ||x||^2 into sc[slot]; with tau_mode the last block also forms the first
// step's c = ||Dd||^2 + kappa ||Ad||^2 and tau = |<d,d> / c|
template <class T>
__global__ void __launch_bounds__(UB) k_uf_norm(long len, const T* __restrict__ x, double* part, unsigned* ticket,
                                                double* sc, int slot, int tau_mode, const double* __restrict__ mub) {
    double a = 0.0;
    U_STRIDE(i, len) a += (double)x[i] * (double)x[i];
    double v[1] = {a}, tot[1];
    if (grid_reduce<1>(v, part, ticket, tot) && threadIdx.x == 0) {
        sc[slot] = tot[0];
        if (tau_mode) {
            const double c = sc[S_DD2] + mub[0] / mub[1] * sc[S_AD2];
            sc[S_C] = c;
            sc[S_TAU] = fabs(sc[S_A] / c);
        }
    }
}

template <class T>
__global__ void __launch_bounds__(UB) k_uf_update(long n, const T* __restrict__ U, const T* __restrict__ d,
                                                  const double* __restrict__ sc, int nonneg, T* __restrict__ Un) {
    const T tau = (T)sc[S_TAU];
    U_STRIDE(i, n) {
        const T z = U[i] - tau * d[i];
        Un[i] = (nonneg && z < T(0)) ? T(0) : z;
    }
}

// ---------------------------------------------------------------------------
// adjoint
// ---------------------------------------------------------------------------
// projection: Zb = gUn [U - tau d > 0]; tau_bar = -<Zb, d>; d_bar = -tau Zb;
// U_bar = Zb
template <class T>
__global__ void __launch_bounds__(UB) k_ub_proj(long n, const T* __restrict__ U, const T* __restrict__ d,
                                                const T* __restrict__ gUn, int nonneg, double* part, unsigned* ticket,
                                                double* sc, T* __restrict__ db, T* __restrict__ Ub) {
    const T tau = (T)sc[S_TAU];
    double tb = 0.0;
    U_STRIDE(i, n) {
        const T di = d[i];
        T z = gUn ? gUn[i] : T(0);
        if (nonneg && !(U[i] - tau * di > T(0))) z = T(0);
        tb -= (double)z * (double)di;
        db[i] = -tau * z;
        Ub[i] = z;
    }
    double v[1] = {tb}, tot[1];
    if (grid_reduce<1>(v, part, ticket, tot) && threadIdx.x == 0) sc[S_TAUB] = tot[0];
}

// BB quotient (not the first step): a_bar = tau_bar/|c|, c_bar = -tau_bar tau/c;
// s_bar = 2 a_bar s + c_bar y, y_bar = c_bar s; then the adjoints of U, Up,
// gp, g2p, and the totals G = gg + kappa (y_bar + d_bar), G2 = gg2 + y_bar +
// d_bar of g and g2; kappa_bar = <y_bar, g - gp> + <d_bar, g>
template <class T>
__global__ void __launch_bounds__(UB) k_ub_bb(long n, const T* __restrict__ U, const T* __restrict__ Up,
                                              const T* __restrict__ g, const T* __restrict__ g2,
                                              const T* __restrict__ gp, const T* __restrict__ g2p,
                                              const T* __restrict__ gg, const T* __restrict__ gg2,
                                              const T* __restrict__ db, const double* __restrict__ mub, double* part,
                                              unsigned* ticket, double* sc, T* __restrict__ Ub, T* __restrict__ gUp,
                                              T* __restrict__ ggp, T* __restrict__ gg2p, T* __restrict__ G,
                                              T* __restrict__ G2) {
    const double kapd = mub[0] / mub[1];
    const T kap = (T)kapd;
    const double tb = sc[S_TAUB], c = sc[S_C], tau = sc[S_TAU];
    const T ab = (T)(tb / fabs(c)), cb = (T)(-tb * tau / c);
    double kb = 0.0;
    U_STRIDE(i, n) {
        const T s = U[i] - Up[i];
        const T dgi = g[i] - gp[i];
        const T y = (g2[i] - g2p[i]) + kap * dgi;
        const T sb = T(2) * ab * s + cb * y;
        const T yb = cb * s;
        const T dbi = db[i];
        Ub[i] += sb;
        if (gUp) gUp[i] = -sb;
        if (ggp) ggp[i] = -kap * yb;
        if (gg2p) gg2p[i] = -yb;
        G[i] = opt(gg, i) + kap * (yb + dbi);
        G2[i] = opt(gg2, i) + yb + dbi;
        kb += (double)yb * (double)dgi + (double)dbi * (double)g[i];
    }
    double v[1] = {kb}, tot[1];
    if (grid_reduce<1>(v, part, ticket, tot) && threadIdx.x == 0) sc[S_KAPB] = tot[0];
}

// first step: tau = |<d,d>| / c with c = ||Dd||^2 + kappa ||Ad||^2:
// d_bar += 2 a_bar d + 2 c_bar (D^T D d + kappa A^T A d); kappa_bar =
// c_bar ||Ad||^2 + <d_bar, g>; G, G2 as above without the y terms
template <class T>
__global__ void __launch_bounds__(UB) k_ub_first(long n, const T* __restrict__ d, const T* __restrict__ g,
                                                 const T* __restrict__ gg, const T* __restrict__ gg2,
                                                 const T* __restrict__ db, const T* __restrict__ DtDd,
                                                 const T* __restrict__ AtAd, const double* __restrict__ mub,
                                                 double* part, unsigned* ticket, double* sc, T* __restrict__ G,
                                                 T* __restrict__ G2) {
    const double kapd = mub[0] / mub[1];
    const T kap = (T)kapd;
    const double tb = sc[S_TAUB], c = sc[S_C], tau = sc[S_TAU];
    const T ab = (T)(tb / fabs(c));
    const double cbd = -tb * tau / c;
    const T cb = (T)cbd;
    double kb = 0.0;
    U_STRIDE(i, n) {
        const T dbt = db[i] + T(2) * ab * d[i] + T(2) * cb * (DtDd[i] + kap * AtAd[i]);
        G[i] = opt(gg, i) + kap * dbt;
        G2[i] = opt(gg2, i) + dbt;
        kb += (double)dbt * (double)g[i];
    }
    double v[1] = {kb}, tot[1];
    if (grid_reduce<1>(v, part, ticket, tot) && threadIdx.x == 0) sc[S_KAPB] = tot[0] + cbd * sc[S_AD2];
}

// shrinkage and sigma terms: with Pb = D G2 (the adjoint of P), W_bar = -Pb,
// V_bar = (dW/dV)^T W_bar, DU_bar = Pb + V_bar (in place of Pb);
// beta_bar = (<Pb + V_bar, sigma> - sum t_bar) / beta^2
template <class T>
__global__ void __launch_bounds__(UB) k_ub_shrink(UVol g, const T* __restrict__ U, const T* __restrict__ sig,
                                                  const double* __restrict__ mub, int iso, T* __restrict__ Pb,
                                                  double* part, unsigned* ticket, double* sc) {
    const double beta = mub[1];
    const T ib = (T)(1.0 / beta);
    double bs = 0.0, tbs = 0.0;
    U_STRIDE(i, g.n) {
        T du[3], v[3], wb[3], vb[3], pb[3];
        du_v(g, U, sig, ib, i, du, v);
        for (int c = 0; c < 3; ++c) {
            pb[c] = Pb[c * g.n + i];
            wb[c] = -pb[c];
        }
        tbs += (double)shrink3_bwd(v, ib, iso, wb, vb);
        for (int c = 0; c < 3; ++c) {
            const T dub = pb[c] + vb[c];
            Pb[c * g.n + i] = dub;
            bs += (double)dub * (double)opt(sig, c * g.n + i);
        }
    }
    double vv[2] = {bs, tbs}, tot[2];
    if (grid_reduce<2>(vv, part, ticket, tot) && threadIdx.x == 0) sc[S_BETAB] = (tot[0] - tot[1]) / (beta * beta);
}

// b_bar = -r_bar; mu_bar (delta term) = <r_bar, delta> / mu^2
template <class T>
__global__ void __launch_bounds__(UB) k_ub_resid(long m, const T* __restrict__ rb, const T* __restrict__ delta,
                                                 const double* __restrict__ mub, double* part, unsigned* ticket,
                                                 double* sc, T* __restrict__ gb) {
    double a = 0.0;
    U_STRIDE(i, m) {
        if (gb) gb[i] = -rb[i];
        if (delta) a += (double)rb[i] * (double)delta[i];
    }
    double v[1] = {a}, tot[1];
    if (grid_reduce<1>(v, part, ticket, tot) && threadIdx.x == 0) sc[S_MUB] = tot[0] / (mub[0] * mub[0]);
}

// U_bar += D^T DU_bar + A^T r_bar
template <class T>
__global__ void __launch_bounds__(UB) k_ub_final(UVol g, const T* __restrict__ DUb, const T* __restrict__ AtRb,
                                                 T* __restrict__ Ub) {
    U_STRIDE(i, g.n) {
        long ym, xm, zm;
        nb_minus(g, i, ym, xm, zm);
        const long n = g.n;
        const T dt = DUb[ym] - DUb[i] + DUb[n + xm] - DUb[n + i] + DUb[2 * n + zm] - DUb[2 * n + i];
        Ub[i] += dt + AtRb[i];
    }
}

// (mu_bar, beta_bar) from kappa = mu/beta and the direct terms
__global__ void k_ub_scalars(const double* __restrict__ sc, const double* __restrict__ mub, double* __restrict__ gmub) {
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        const double mu = mub[0], beta = mub[1], kb = sc[S_KAPB];
        gmub[0] = sc[S_MUB] + kb / beta;
        gmub[1] = sc[S_BETAB] - kb * mu / (beta * beta);
    }
}

int ugrid(long n) {
    const long g = (n + UB - 1) / UB;
    return (int)std::max<long>(1, std::min<long>(g, (long)num_sms() * 4));
}

// stream-ordered scratch of one call
template <class T>
struct SBuf {
    T* p = nullptr;
    cudaStream_t s;
    SBuf(size_t n, cudaStream_t s_) : s(s_) {
        tmp_pool_init();
        TV3_CUDA(cudaMallocAsync((void**)&p, std::max<size_t>(n, 1) * sizeof(T), s));
    }
    ~SBuf() {
        if (p) cudaFreeAsync(p, s);
    }
    SBuf(const SBuf&) = delete;
    SBuf& operator=(const SBuf&) = delete;
};

template <class T>
void product(const LinOp<T>* op, int trans, const T* x, T* y, cudaStream_t s) {
    op->apply(trans, plain_io<T>(x, y), SPMV_PLAIN, s);
}

// the step's forward intermediates: g2, g, d and the scalars (first step also Dd, Ad)
template <class T>
struct Fwd {
    SBuf<T> P, r, g, g2, d, Dd, Ad;
    SBuf<double> part, sc;
    SBuf<unsigned> ticket;
    Fwd(long n, long m, bool first, cudaStream_t s)
        : P(3 * n, s), r(m, s), g(n, s), g2(n, s), d(n, s), Dd(first ? 3 * n : 1, s), Ad(first ? m : 1, s),
          part(4 * 4096, s), sc(S_N, s), ticket(1, s) {
        TV3_CUDA(cudaMemsetAsync(ticket.p, 0, sizeof(unsigned), s));
        TV3_CUDA(cudaMemsetAsync(sc.p, 0, S_N * sizeof(double), s));
    }
};

template <class T>
void run_forward(const LinOp<T>* op, const UVol& v, bool first, int iso, const double* mub, const T* U, const T* Up,
                 const T* gp, const T* g2p, const T* b, const T* sig, const T* delta, Fwd<T>& f, T* g_out, T* g2_out,
                 cudaStream_t s) {
    const long n = v.n, m = op->m;
    T* g = g_out ? g_out : f.g.p;
    T* g2 = g2_out ? g2_out : f.g2.p;
    k_uf_p<T><<<ugrid(n), UB, 0, s>>>(v, U, sig, mub, iso, f.P.p);
    launch_Dt_plain<T>(v.p, v.q, v.r, f.P.p, g2, s);
    product(op, 0, U, f.r.p, s);
    k_uf_resid<T><<<ugrid(m), UB, 0, s>>>(m, f.r.p, b, delta, mub);
    product(op, 1, f.r.p, g, s);
    if (first) {
        k_uf_dir<T, true><<<ugrid(n), UB, 0, s>>>(n, U, Up, g, g2, gp, g2p, mub, f.d.p, f.part.p, f.ticket.p, f.sc.p);
        launch_D_plain<T>(v.p, v.q, v.r, f.d.p, f.Dd.p, s);
        k_uf_norm<T><<<ugrid(3 * n), UB, 0, s>>>(3 * n, f.Dd.p, f.part.p, f.ticket.p, f.sc.p, S_DD2, 0, mub);
        product(op, 0, f.d.p, f.Ad.p, s);
        k_uf_norm<T><<<ugrid(m), UB, 0, s>>>(m, f.Ad.p, f.part.p, f.ticket.p, f.sc.p, S_AD2, 1, mub);
    } else {
        k_uf_dir<T, false><<<ugrid(n), UB, 0, s>>>(n, U, Up, g, g2, gp, g2p, mub, f.d.p, f.part.p, f.ticket.p,
                                                     f.sc.p);
    }
    TV3_CUDA(cudaGetLastError());
}

}  // namespace

template <class T>
void unroll_step(const LinOp<T>* op, int p, int q, int r, int first, int iso, int nonneg, const double* mub,
                 const T* U, const T* Up, const T* gp, const T* g2p, const T* b, const T* sig, const T* delta, T* Un,
                 T* g, T* g2, cudaStream_t s) {
    const UVol v{p, q, r, (long)p * q * r};
    Fwd<T> f(v.n, op->m, first != 0, s);
    run_forward(op, v, first != 0, iso, mub, U, Up, gp, g2p, b, sig, delta, f, g, g2, s);
    k_uf_update<T><<<ugrid(v.n), UB, 0, s>>>(v.n, U, f.d.p, f.sc.p, nonneg, Un);
    TV3_CUDA(cudaGetLastError());
}

template <class T>
void unroll_step_adjoint(const LinOp<T>* op, int p, int q, int r, int first, int iso, int nonneg, const double* mub,
                         const T* U, const T* Up, const T* gp, const T* g2p, const T* b, const T* sig, const T* delta,
                         const T* gUn, const T* gg, const T* gg2, T* gU, T* gUp, T* ggp, T* gg2p, T* gb, double* gmub,
                         cudaStream_t s) {
    const UVol v{p, q, r, (long)p * q * r};
    const long n = v.n, m = op->m;
    Fwd<T> f(n, m, first != 0, s);
    run_forward<T>(op, v, first != 0, iso, mub, U, Up, gp, g2p, b, sig, delta, f, nullptr, nullptr, s);
    SBuf<T> db(n, s), G(n, s), G2(n, s), tA(n, s), tB(n, s);
    k_ub_proj<T><<<ugrid(n), UB, 0, s>>>(n, U, f.d.p, gUn, nonneg, f.part.p, f.ticket.p, f.sc.p, db.p, gU);
    if (first) {
        launch_Dt_plain<T>(p, q, r, f.Dd.p, tA.p, s);  // D^T D d
        product(op, 1, f.Ad.p, tB.p, s);                // A^T A d
        k_ub_first<T><<<ugrid(n), UB, 0, s>>>(n, f.d.p, f.g.p, gg, gg2, db.p, tA.p, tB.p, mub, f.part.p, f.ticket.p,
                                              f.sc.p, G.p, G2.p);
    } else {
        k_ub_bb<T><<<ugrid(n), UB, 0, s>>>(n, U, Up, f.g.p, f.g2.p, gp, g2p, gg, gg2, db.p, mub, f.part.p,
                                           f.ticket.p, f.sc.p, gU, gUp, ggp, gg2p, G.p, G2.p);
    }
    // g2 = D^T P: P_bar = D G2 (into P's buffer), then the shrinkage adjoint
    launch_D_plain<T>(p, q, r, G2.p, f.P.p, s);
    k_ub_shrink<T><<<ugrid(n), UB, 0, s>>>(v, U, sig, mub, iso, f.P.p, f.part.p, f.ticket.p, f.sc.p);
    // g = A^T r: r_bar = A G, U_bar += A^T r_bar, b_bar = -r_bar
    product(op, 0, G.p, f.r.p, s);
    k_ub_resid<T><<<ugrid(m), UB, 0, s>>>(m, f.r.p, delta, mub, f.part.p, f.ticket.p, f.sc.p, gb);
    product(op, 1, f.r.p, tB.p, s);
    k_ub_final<T><<<ugrid(n), UB, 0, s>>>(v, f.P.p, tB.p, gU);
    if (gmub) k_ub_scalars<<<1, 32, 0, s>>>(f.sc.p, mub, gmub);
    TV3_CUDA(cudaGetLastError());
}

#define TV3_UNROLL(T)                                                                                                 \
    template void unroll_step<T>(const LinOp<T>*, int, int, int, int, int, int, const double*, const T*, const T*,    \
                                 const T*, const T*, const T*, const T*, const T*, T*, T*, T*, cudaStream_t);         \
    template void unroll_step_adjoint<T>(const LinOp<T>*, int, int, int, int, int, int, const double*, const T*,      \
                                         const T*, const T*, const T*, const T*, const T*, const T*, const T*,         \
                                         const T*, const T*, T*, T*, T*, T*, T*, double*, cudaStream_t);
TV3_UNROLL(float)
TV3_UNROLL(double)

}  // namespace tv3
