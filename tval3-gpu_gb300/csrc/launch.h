// Host-side launch interface of the kernels (internal to the library).
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <stdint.h>

namespace tv3 {

struct Ctl;

void throw_cuda(cudaError_t e, const char* what);

// Launch with programmatic stream serialization: inside a stream (and in a
// captured graph) the kernel's blocks may be scheduled while the previous
// kernel drains, hiding most of the launch gap.  The kernel must call
// pdl_wait() (count_launch does) before touching memory the previous kernel
// writes.
template <class... P, class... A>
void launch_k(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A... args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = block;
    cfg.dynamicSmemBytes = smem;
    cfg.stream = s;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    const cudaError_t e = cudaLaunchKernelEx(&cfg, kernel, args...);
    if (e != cudaSuccess) throw_cuda(e, "cudaLaunchKernelEx");
}

enum SpmvEpi : int { SPMV_PLAIN = 0, SPMV_SUB = 1, SPMV_LAM35 = 2, SPMV_NORM2 = 3 };

// Slack (elements) behind the index and value arrays of a CSR operator: the
// SpMV reads four-element chunks from a 4-aligned base, at most 4*G + 3
// elements past the last nonzero (G <= 32).  The slack is zero-filled.
constexpr long SPMV_PAD = 256;

// flag in the lanes-per-row argument of launch_spmv: single-nonzero lanes
// (short rows) instead of four-element chunks (long rows)
constexpr int SPMV_SCALAR = 64;

// Arguments of one CSR product y = M x (M is A or the CSR of A^T).  x and y
// are ping-pong pairs: with by_parity set, the kernel uses slot ctl->parity.
template <class T, class V>
struct SpmvArgs {
    long rows;
    const int* ptr;
    const int* ind;
    const V* val;
    const float* rscale;  // per-row scale applied to the row sum (A*x), or null
    const float* xscale;  // per-entry scale of the gathered x (A^T*y), or null
    const T* x[2];
    T* y[2];
    int by_parity;
    const T* sub;    // SPMV_SUB: y = Mx - sub
    const T* b;      // SPMV_LAM35
    const T* delta;  // SPMV_LAM35
    Ctl* ctl;
    double* part;
    unsigned* ticket;
    int L;           // > 1: multi-RHS, vectors interleaved (element (row, layer) at row * L + layer)
};

template <class T, class V>
void launch_spmv(const SpmvArgs<T, V>& a, int epi, int G, int grid, cudaStream_t s);

// Buffers of one solve (see solver.cu).  Slot arrays are ping-pong pairs
// indexed by ctl->parity ("current") and 1 - parity ("previous").
template <class T>
struct SolverBufs {
    int p, q, r;   // dim_y (fastest), dim_x, dim_z
    int L;         // layers sharing A (>= 1); vectors interleaved, layer fastest
    long n, m;     // vector lengths: voxels * L and rays * L
    T* U[2];
    T* g[2];
    T* g2[2];
    T* Au[2];
    T* DU[2];      // 3n each
    T* d;
    T* DtsAtd;
    T* Atb;
    T* W[2];       // 3n each; slot ctl->wsel is current, the other takes the next W
    T* sig;        // 3n
    T* b;          // m, scaled
    T* delta;      // m
    T* rcdU;
    const void* xstar;  // optional reference solution (unscaled, caller type) for the relerr trace
    double* trace;      // optional per-iteration error norm vs xstar
    int use_dtsatd;
    Ctl* ctl;
    double* part;
    unsigned* ticket;
    int grid;         // grid of the reducing kernels
    // CUDA graph conditional handles (whole-solve graph only): the epilogues
    // that decide a branch set the matching handle when use_graph is set.
    int use_graph;
    unsigned long long h_inner;  // WHILE: continue the inner loop
    unsigned long long h_arm;    // IF: Armijo test failed after the descent
    unsigned long long h_mlp;    // IF: outer loop continues (multiplier update)
    // skip-A^T heuristic (skip_ratio != 0 only): A*U of the last A^T product,
    // and the IF handles of "multiply" and "keep g"
    T* last_Au;
    unsigned long long h_mult, h_keep;
};

// Flags that the tiny condition kernel copies from the control block into a
// conditional handle.
enum CondSrc : int { COND_FST = 0, COND_RESTART = 1, COND_ONE = 2, COND_NOT_DONE = 3 };
void launch_cond(Ctl* ctl, unsigned long long handle, int src, cudaStream_t s);

// stencil.cu
// b_in, U_out and Ut are caller-facing arrays: float for float vectors,
// double for double and double-float vectors.
template <class T> void launch_scale_b(const void* b_in, SolverBufs<T>& B, cudaStream_t s);
template <class T> void launch_D_only(SolverBufs<T>& B, cudaStream_t s);
template <class T> void launch_descend(SolverBufs<T>& B, int restart, cudaStream_t s);
template <class T> void launch_Dd_norm(SolverBufs<T>& B, cudaStream_t s);
template <class T> void launch_g2(SolverBufs<T>& B, int mode, cudaStream_t s);
template <class T> void launch_shrink(SolverBufs<T>& B, int mode, cudaStream_t s);
template <class T> void launch_g2_gradient(SolverBufs<T>& B, cudaStream_t s);  // g2 (update_W) + gradient, fused
template <class T> void launch_gradient(SolverBufs<T>& B, int mode, cudaStream_t s);
template <class T> void launch_bt_coef(SolverBufs<T>& B, cudaStream_t s);
template <class T> void launch_bt_apply(SolverBufs<T>& B, cudaStream_t s);
template <class T> void launch_outer_relchg(SolverBufs<T>& B, cudaStream_t s);
template <class T> void launch_mlp(SolverBufs<T>& B, cudaStream_t s);
template <class T> void launch_outer_grad(SolverBufs<T>& B, cudaStream_t s);
// skip-A^T decision after A*U (force: start-up and restart calls) and the
// copies of its two branches (0: last_Au = Au, 1: g = the previous g)
template <class T> void launch_skip_decide(SolverBufs<T>& B, int force, cudaStream_t s);
template <class T> void launch_skip_copy(SolverBufs<T>& B, int which, cudaStream_t s);
template <class T> void launch_finalize(SolverBufs<T>& B, void* U_out, const void* Ut, cudaStream_t s);

// Standalone operators (tval3_D / tval3_Dt entry points).
template <class T> void launch_D_plain(int p, int q, int r, const T* U, T* DU3, cudaStream_t s);
template <class T> void launch_Dt_plain(int p, int q, int r, const T* V3, T* out, cudaStream_t s);

int num_sms();

}  // namespace tv3
