// Linear operators A (rays x voxels) behind the mat_vec_mul interface
// (3d/mat_vec_mul_sparse.h:1703, 3d/mat_vec_mul_dense.h:37,
// 3d/mat_vec_mul_dynamic.h:683, 3d/mat_vec_mul.h:733).  Internal to the
// library; the C ABI wraps them in tval3_op handles.
#pragma once

#include <cuda_runtime.h>
#include <chrono>
#include <memory>
#include <string>
#include "launch.h"
#include "tval3_internal.cuh"

namespace tv3 {

// Seconds spent in the parts of the last host entry call on this thread:
// [0] matrix upload, [1] input validation, [2] operator layout (copies,
// transposes, quantisation, ray-matrix build), [3] tile layouts and kernel
// choice, [4] graph capture and instantiation, [5] the host-to-device copies
// alone (inside [0]).  Entry points reset it; a PhaseTimer adds the wall time
// of its scope.
inline thread_local double sub_phase[6] = {0, 0, 0, 0, 0, 0};
struct PhaseTimer {
    int k;
    std::chrono::steady_clock::time_point t0;
    explicit PhaseTimer(int k_) : k(k_), t0(std::chrono::steady_clock::now()) {}
    ~PhaseTimer() {
        sub_phase[k] += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    }
};

template <class T> struct LinOp;
// column-major k-column product through one interleaved multi-RHS apply (ops.cu)
template <class T>
void apply_interleaved(const LinOp<T>& op, int trans, int k, const T* X, T* Y, cudaStream_t s);

// I/O of one product inside the solver.  x and y are ping-pong pairs selected
// by ctl->parity when by_parity is set; epilogues as in SpmvEpi.
template <class T>
struct MatIO {
    const T* x[2];
    T* y[2];
    int by_parity;
    const T* sub;
    const T* b;
    const T* delta;
    Ctl* ctl;
    double* part;
    unsigned* ticket;
    int L;  // > 1: L right-hand sides, interleaved (element (row, layer) at row * L + layer)
};

template <class T>
MatIO<T> plain_io(const T* x, T* y) {
    MatIO<T> io{};
    io.x[0] = io.x[1] = x;
    io.y[0] = io.y[1] = y;
    return io;
}

// Error raised inside the library; converted to a status at the C ABI.
struct Error {
    int status;
    std::string msg;
};

void throw_cuda(cudaError_t e, const char* what);
#define TV3_CUDA(call)                                           \
    do {                                                         \
        cudaError_t e_ = (call);                                 \
        if (e_ != cudaSuccess) ::tv3::throw_cuda(e_, #call);     \
    } while (0)

template <class T>
struct LinOp {
    long m = 0, n = 0, nnz = 0;
    int kind = 0;  // 0 CSR, 1 dense, 2 on-the-fly geometry
    virtual ~LinOp() {}
    // trans 0: y[rows m] = A x ; trans 1: y[rows n] = A^T x
    virtual void apply(int trans, const MatIO<T>& io, int epi, cudaStream_t s) const = 0;
    // allocate what products with L interleaved right-hand sides need (called
    // before any product, outside stream capture)
    virtual void prepare(int L) const { (void)L; }
    // the volume the columns form (dim_y fastest, dim_x, dim_z): lets stored
    // operators regroup A^T by voxel tiles (tiled.cu); called outside capture
    virtual void set_volume(int p, int q, int r) const {
        (void)p;
        (void)q;
        (void)r;
    }
    // settle what the chosen kernels still need before use, e.g. the lane
    // timing of a CSR product the build-time contest did not need (called by
    // a solver after set_volume, outside capture)
    virtual void ready() const {}
    // true when apply() takes L > 1 interleaved right-hand sides
    virtual bool multi_rhs() const { return false; }
    // kernel of A*x (trans 0) or A^T*y (trans 1): 0 = CSR kernels, 1 =
    // tile-staged (when built); the build-time timing picks one, the caller
    // may pin it.  Returns false when the variant is not available.
    virtual bool set_variant(int trans, int variant) const {
        (void)trans;
        return variant == 0;
    }
    virtual int variant(int trans) const {
        (void)trans;
        return 0;
    }
    // multi-RHS products: columns of length n (trans 0: X n x k -> Y m x k),
    // column-major; operators with multi_rhs() run one interleaved product
    virtual void apply_multi(int trans, int k, const T* X, T* Y, cudaStream_t s) const {
        const long lx = trans ? m : n, ly = trans ? n : m;
        if (k > 1 && multi_rhs()) {
            apply_interleaved(*this, trans, k, X, Y, s);
            return;
        }
        for (int j = 0; j < k; ++j) apply(trans, plain_io<T>(X + j * lx, Y + j * ly), SPMV_PLAIN, s);
    }
    // export the stored matrix as FP32 CSR (stored operators only)
    virtual void export_csr(int*, int*, float*, int*, int*, float*) const {
        throw Error{7, "operator has no stored CSR"};
    }
    // the stored values and per-row scales as the products apply them: entry
    // (r, c) = val * row_scale[r] exactly (16-bit storage: the 16-bit values
    // widened to FP32; other storage: the FP32 values and scales of one)
    virtual void export_scaled(float*, float*, float*) const { throw Error{7, "operator has no stored CSR"}; }
    // operators whose kernels have bounded device waits (the tensor-core
    // products) record a timeout of a product made outside a solve in an
    // error word of their own: this waits for the stream, returns the word
    // (0 = none) and clears it.  Operators without such waits return 0 at once.
    virtual int take_error(cudaStream_t s) const {
        (void)s;
        return 0;
    }
};

// A*x from one operator, A^T*y from another: the reference's sparse_geom_mm
// (on-the-fly ray traversal for A*x, stored sparse matrix for A^T*y,
// 3d/mat_vec_mul.h:733-756).
template <class T>
struct SplitOp : LinOp<T> {
    std::unique_ptr<LinOp<T>> nop, top;
    SplitOp(std::unique_ptr<LinOp<T>> a, std::unique_ptr<LinOp<T>> b) : nop(std::move(a)), top(std::move(b)) {
        this->m = nop->m;
        this->n = nop->n;
        this->nnz = top->nnz;
        this->kind = 3;
    }
    void apply(int trans, const MatIO<T>& io, int epi, cudaStream_t s) const override {
        (trans ? top : nop)->apply(trans, io, epi, s);
    }
    void prepare(int L) const override {
        nop->prepare(L);
        top->prepare(L);
    }
    void set_volume(int p, int q, int r) const override { top->set_volume(p, q, r); }
    void ready() const override {
        nop->ready();
        top->ready();
    }
    bool set_variant(int trans, int v) const override { return (trans ? top : nop)->set_variant(trans, v); }
    int take_error(cudaStream_t s) const override { return nop->take_error(s) | top->take_error(s); }
    int variant(int trans) const override { return (trans ? top : nop)->variant(trans); }
};

// CSR operator: A and the CSR of A^T on the device.
template <class T>
LinOp<T>* make_csr_op_device(long rows, long cols, long nnz, const int* d_ptr, const int* d_ind, const T* d_val,
                             const int* d_tptr, const int* d_tind, const T* d_tval, int precision,
                             cudaStream_t s);

// FP32 stored values, FP64 vectors (precision TVAL3_PREC_FP32_F64VEC).
LinOp<double>* make_csr_op_f64vec(long rows, long cols, long nnz, const int* d_ptr, const int* d_ind,
                                  const float* d_val, const int* d_tptr, const int* d_tind, const float* d_tval,
                                  cudaStream_t s, bool tune = true);

// Double-float products over the arrays of an FP32-value / FP64-vector CSR
// operator (precision TVAL3_PREC_FP32_DF64); the view does not own the arrays.
LinOp<df64>* make_df64_view(const LinOp<double>* base);

// Mixed precision (TVAL3_PREC_BF16_DF64 = 6, TVAL3_PREC_FP16_DF64 = 7): the
// FP32 device CSR quantised to 16-bit values with a per-ray FP32 scale,
// products and vectors in double-float.  The transpose is built when d_tptr
// is null.
LinOp<df64>* make_csr_op_df64q(long rows, long cols, long nnz, const int* d_ptr, const int* d_ind,
                               const float* d_val, const int* d_tptr, const int* d_tind, const float* d_tval,
                               int precision, cudaStream_t s);
void convert_to_df64(const double* in, void* out, long n, cudaStream_t s);
void convert_from_df64(const void* in, double* out, long n, cudaStream_t s);

// Bounded-wait self-test (selftest.cu): one warp waits `cycles` of SM clock
// on an mbarrier phase that nothing completes.
void selftest_bounded_wait(long long cycles, int* timed_out, long long* waited);

// Differentiable shrinkage (shrink_ad.cu): W = shrink(v, t) and its adjoint.
template <class T> void shrink_fwd(long n, const T* v, double t, int iso, T* W, cudaStream_t s);
template <class T>
void shrink_bwd(long n, const T* v, double t, int iso, const T* gW, T* gv, T* gt, cudaStream_t s);

// One differentiable TVAL3 inner step and its adjoint (unroll.cu).
template <class T>
void unroll_step(const LinOp<T>* op, int p, int q, int r, int first, int iso, int nonneg, const double* mub,
                 const T* U, const T* Up, const T* gp, const T* g2p, const T* b, const T* sig, const T* delta, T* Un,
                 T* g, T* g2, cudaStream_t s);
template <class T>
void unroll_step_adjoint(const LinOp<T>* op, int p, int q, int r, int first, int iso, int nonneg, const double* mub,
                         const T* U, const T* Up, const T* gp, const T* g2p, const T* b, const T* sig, const T* delta,
                         const T* gUn, const T* gg, const T* gg2, T* gU, T* gUp, T* ggp, T* gg2p, T* gb, double* gmub,
                         cudaStream_t s);

// Ray-geometry operators (ray.cu).
struct RayList;  // compacted ray list and geometry on the device
template <class T>
LinOp<T>* make_geometry_op(const void* geometry_host, int mode, int precision, cudaStream_t s);

// Dense operator (dense.cu).
template <class T>
LinOp<T>* make_dense_op(long rows, long cols, const void* h_data, int row_major, int val_type, int precision,
                        cudaStream_t s);

// Device CSR transpose: (ptr, ind, val) of rows x cols -> CSR of A^T with rows
// ascending inside every column (the reference's CSC order).
template <class V>
void csr_transpose_device(long rows, long cols, long nnz, const int* ptr, const int* ind, const V* val, int* tptr,
                          int* tind, V* tval, cudaStream_t s);

}  // namespace tv3
