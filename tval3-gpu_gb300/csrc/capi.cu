// C ABI (include/tval3/tval3_c.h).  Every entry point validates its
// arguments like the reference's check_params_1/2 (3d/tval3_gpu_3d.cpp:
// 1351-1380), converts internal errors to a status code plus a thread-local
// message (the reference throws tval3_gpu_exception, :1439-1445), and runs on
// the caller's current device.
#include <atomic>
#include <chrono>
#include <cmath>
#include <thread>
#include <cstring>
#include <memory>
#include <new>
#include <string>
#include <type_traits>
#include <vector>
#include "solver.h"
#include "tval3/tval3_c.h"

using namespace tv3;

struct tval3_op_s {
    int dbl = 0;  // caller-facing vector type double?
    int precision = 0;
    LinOp<float>* f = nullptr;
    LinOp<double>* d = nullptr;
    // double-float products: a view of d (TVAL3_PREC_FP32_DF64), or an
    // operator of its own with 16-bit storage and d null (BF16_DF64, FP16_DF64)
    LinOp<df64>* q = nullptr;
    long long device_bytes = 0;  // device memory its creation kept
    ~tval3_op_s() {
        delete q;
        delete f;
        delete d;
    }
    // shape and stored arrays: the owning operator of whichever kind
    long rows() const { return d ? d->m : (q ? q->m : f->m); }
    long cols() const { return d ? d->n : (q ? q->n : f->n); }
    long nnz() const { return d ? d->nnz : (q ? q->nnz : f->nnz); }
    template <class F>
    void with_store(F fn) const {
        if (d) fn(*d);
        else if (q) fn(*q);
        else fn(*f);
    }
};

struct tval3_batch_s {
    Batch<float>* f = nullptr;
    Batch<double>* d = nullptr;
    Batch<df64>* q = nullptr;
    ~tval3_batch_s() {
        delete f;
        delete d;
        delete q;
    }
};

struct tval3_solver_s {
    int dbl = 0;
    Solver<float>* f = nullptr;
    Solver<double>* d = nullptr;
    Solver<df64>* q = nullptr;
    ~tval3_solver_s() {
        delete f;
        delete d;
        delete q;
    }
};

namespace {

// Upload of a caller's host array (timed as its own phase).  cudaMemcpy from
// pageable memory runs at the link's rate on Grace systems (~190 GB/s for
// 440 MB); a device copy kernel reading the array through the host's page
// tables was as fast in steady state but now and then took 15-50 ms for the
// same 440 MB, when the translations had to be walked again.
void h2d(void* dst, const void* src, size_t bytes) {
    if (!bytes) return;
    PhaseTimer pc(5);
    TV3_CUDA(cudaMemcpy(dst, src, bytes, cudaMemcpyHostToDevice));
}

thread_local std::string g_err;
// seconds of the phases of this thread's last reference entry-point call:
// operator (input checks, upload, transpose / quantisation, ray-matrix build),
// set-up (b upload, solver workspace, tile-staged layouts and kernel choice),
// solve (graph capture on first use, then the solve), download of U
thread_local double g_phase[4] = {0, 0, 0, 0};
// start of a host entry call: clears the phase records
std::chrono::steady_clock::time_point entry_clock() {
    for (double& v : sub_phase) v = 0.0;
    for (double& v : g_phase) v = 0.0;
    return std::chrono::steady_clock::now();
}

tval3_status fail(int st, const std::string& msg) {
    g_err = msg;
    return (tval3_status)st;
}

template <class F>
tval3_status guard(F f) {
    try {
        g_err.clear();
        f();
        return TVAL3_OK;
    } catch (const Error& e) {
        return fail(e.status, e.msg);
    } catch (const std::bad_alloc&) {
        return fail(TVAL3_ERR_NOMEM, "host allocation failed");
    } catch (const std::exception& e) {
        return fail(TVAL3_ERR_ARG, std::string("Internal error: ") + e.what());
    }
}

[[noreturn]] void arg_error(int st, const std::string& msg) { throw Error{st, msg}; }

template <class T>
struct HostVec {
    T* p = nullptr;
};

// true when pred(k) holds for every k in [0, n); large ranges are split over
// the host's cores (input validation of 10^7-10^8 nonzeros)
template <class F>
bool all_of_range(long n, F pred) {
    const long chunk = 1L << 20;
    if (n <= 4 * chunk) {
        for (long k = 0; k < n; ++k)
            if (!pred(k)) return false;
        return true;
    }
    const unsigned hw = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    std::atomic<bool> ok{true};
    std::vector<std::thread> th;
    for (unsigned t = 0; t < hw; ++t)
        th.emplace_back([&, t] {
            for (long k = (long)t * chunk; k < n && ok.load(std::memory_order_relaxed); k += (long)hw * chunk) {
                const long e = std::min(n, k + chunk);
                for (long j = k; j < e; ++j)
                    if (!pred(j)) {
                        ok = false;
                        return;
                    }
            }
        });
    for (auto& x : th) x.join();
    return ok;
}

// Matrices above this many nonzeros are scanned on the device (one pass over
// the uploaded arrays) instead of by host threads; smaller ones, and values
// narrowed from FP64 to FP32 on the way up, are scanned on the host.
constexpr long DEVICE_CHECK_NNZ = 1L << 22;

void check_sparse(const tval3_sparse_host* A, bool host_scan = true) {
    if (!A) arg_error(TVAL3_ERR_ARG, "Argument error: A is NULL!");
    if (A->rows < 0 || A->cols < 0 || A->nnz < 0) arg_error(TVAL3_ERR_SHAPE, "Argument error: negative matrix size!");
    if (A->format < 1 || A->format > 3) arg_error(TVAL3_ERR_ARG, "Argument error: unknown sparse format!");
    if (A->val_type != TVAL3_PREC_FP32 && A->val_type != TVAL3_PREC_FP64)
        arg_error(TVAL3_ERR_ARG, "Argument error: sparse values must be FP32 or FP64!");
    auto chk = [&](const int* ptr, const int* ind, const void* val, long rows, long cols, const char* what) {
        if (!ptr || (A->nnz > 0 && (!ind || !val)))
            arg_error(TVAL3_ERR_ARG, std::string("Argument error: missing ") + what + " arrays!");
        if (ptr[0] != 0 || ptr[rows] != A->nnz)
            arg_error(TVAL3_ERR_SHAPE, std::string("Argument error: inconsistent ") + what + " pointer array!");
        if (!host_scan) return;
        if (!all_of_range(rows, [&](long r) { return ptr[r + 1] >= ptr[r]; }))
            arg_error(TVAL3_ERR_SHAPE, std::string("Argument error: decreasing ") + what + " pointers!");
        if (!all_of_range(A->nnz, [&](long k) { return ind[k] >= 0 && ind[k] < cols; }))
            arg_error(TVAL3_ERR_SHAPE, std::string("Argument error: ") + what + " index out of range!");
        bool fin;
        if (A->val_type == TVAL3_PREC_FP32) {
            const float* v = (const float*)val;
            fin = all_of_range(A->nnz, [&](long k) { return std::isfinite(v[k]); });
        } else {
            const double* v = (const double*)val;
            fin = all_of_range(A->nnz, [&](long k) { return std::isfinite(v[k]); });
        }
        if (!fin) arg_error(TVAL3_ERR_NONFINITE, "Argument error: non-finite matrix value!");
    };
    if (A->format & TVAL3_SPARSE_CSR) chk(A->csr_ptr, A->csr_ind, A->csr_val, A->rows, A->cols, "CSR");
    if (A->format & TVAL3_SPARSE_CSC) chk(A->csc_ptr, A->csc_ind, A->csc_val, A->cols, A->rows, "CSC");
}

// One pass over a device CSR (or CSC) triple: bit 0 decreasing pointers,
// bit 1 an index outside [0, cols), bit 2 a non-finite value.
template <class V>
__global__ void k_validate_sparse(const int* __restrict__ ptr, long rows, const int* __restrict__ ind,
                                  const V* __restrict__ val, long nnz, long cols, unsigned* __restrict__ flags) {
    unsigned f = 0u;
    const long N = rows > nnz ? rows : nnz;
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
        if (i < rows && ptr[i + 1] < ptr[i]) f |= 1u;
        if (i < nnz) {
            const int c = ind[i];
            if (c < 0 || c >= cols) f |= 2u;
            if (!isfinite(val[i])) f |= 4u;
        }
    }
    f = __reduce_or_sync(0xffffffffu, f);
    if (f && (threadIdx.x & 31) == 0) atomicOr(flags, f);
}

// the checks of check_sparse's host scan, on uploaded arrays, with the same
// errors in the same order
template <class V>
void validate_device(const int* ptr, long rows, const int* ind, const V* val, long nnz, long cols, const char* what) {
    DBuf<unsigned> flags(1);
    TV3_CUDA(cudaMemset(flags.p, 0, sizeof(unsigned)));
    const long N = std::max(rows, nnz);
    const long grid = std::max<long>(1, std::min<long>((N + 255) / 256, (long)num_sms() * 16));
    k_validate_sparse<V><<<(unsigned)grid, 256>>>(ptr, rows, ind, val, nnz, cols, flags.p);
    TV3_CUDA(cudaGetLastError());
    unsigned f = 0;
    TV3_CUDA(cudaMemcpy(&f, flags.p, sizeof(unsigned), cudaMemcpyDeviceToHost));
    if (f & 1u) arg_error(TVAL3_ERR_SHAPE, std::string("Argument error: decreasing ") + what + " pointers!");
    if (f & 2u) arg_error(TVAL3_ERR_SHAPE, std::string("Argument error: ") + what + " index out of range!");
    if (f & 4u) arg_error(TVAL3_ERR_NONFINITE, "Argument error: non-finite matrix value!");
}

template <class T>
void to_device(DBuf<T>& d, const void* h, long n, int src_type) {
    d.alloc(std::max<long>(n, 1));
    if (n <= 0) return;
    bool src_double = (src_type == TVAL3_PREC_FP64);
    if (src_double == (sizeof(T) == 8)) {
        h2d(d.p, h, n * sizeof(T));
    } else {
        std::vector<T> tmp(n);
        if (src_double)
            for (long i = 0; i < n; ++i) tmp[i] = (T)((const double*)h)[i];
        else
            for (long i = 0; i < n; ++i) tmp[i] = (T)((const float*)h)[i];
        TV3_CUDA(cudaMemcpy(d.p, tmp.data(), n * sizeof(T), cudaMemcpyHostToDevice));
    }
}

// FP32 device copies of a host sparse matrix (FP64 values are narrowed on the
// host), with the CSR of A built on the device when only the CSC was given
struct F32Csr {
    DBuf<int> ptr, ind, tptr, tind;
    DBuf<float> val, tval;
};

void upload_f32(const tval3_sparse_host* A, bool dev_check, F32Csr& c) {
    const long m = A->rows, n = A->cols, nnz = A->nnz;
    std::unique_ptr<PhaseTimer> up(new PhaseTimer(0));
    if (A->format & TVAL3_SPARSE_CSR) {
        c.ptr.alloc(m + 1);
        c.ind.alloc(std::max<long>(nnz, 1));
        h2d(c.ptr.p, A->csr_ptr, (m + 1) * sizeof(int));
        h2d(c.ind.p, A->csr_ind, nnz * sizeof(int));
        to_device(c.val, A->csr_val, nnz, A->val_type);
    }
    if (A->format & TVAL3_SPARSE_CSC) {
        c.tptr.alloc(n + 1);
        c.tind.alloc(std::max<long>(nnz, 1));
        h2d(c.tptr.p, A->csc_ptr, (n + 1) * sizeof(int));
        h2d(c.tind.p, A->csc_ind, nnz * sizeof(int));
        to_device(c.tval, A->csc_val, nnz, A->val_type);
    }
    up.reset();
    PhaseTimer pv(1);
    if (dev_check) {
        if (A->format & TVAL3_SPARSE_CSR) validate_device<float>(c.ptr.p, m, c.ind.p, c.val.p, nnz, n, "CSR");
        if (A->format & TVAL3_SPARSE_CSC) validate_device<float>(c.tptr.p, n, c.tind.p, c.tval.p, nnz, m, "CSC");
    }
    if (!(A->format & TVAL3_SPARSE_CSR)) {
        c.ptr.alloc(m + 1);
        c.ind.alloc(std::max<long>(nnz, 1));
        c.val.alloc(std::max<long>(nnz, 1));
        csr_transpose_device<float>(n, m, nnz, c.tptr.p, c.tind.p, c.tval.p, c.ptr.p, c.ind.p, c.val.p, 0);
    }
}

// mixed-precision operator (TVAL3_PREC_BF16_DF64 / FP16_DF64) from a host
// sparse matrix: FP32 values uploaded, then quantised on the device
LinOp<df64>* sparse_op_mixed(const tval3_sparse_host* A, int precision) {
    if (!A) arg_error(TVAL3_ERR_ARG, "Argument error: A is NULL!");
    const bool dev_check = A->nnz > DEVICE_CHECK_NNZ && A->val_type == TVAL3_PREC_FP32;
    check_sparse(A, !dev_check);
    F32Csr c;
    upload_f32(A, dev_check, c);
    PhaseTimer pl(2);
    return make_csr_op_df64q(A->rows, A->cols, A->nnz, c.ptr.p, c.ind.p, c.val.p, c.tptr.p,
                             c.tptr.p ? c.tind.p : nullptr, c.tptr.p ? c.tval.p : nullptr, precision, 0);
}

bool is_mixed(int precision) { return precision == TVAL3_PREC_BF16_DF64 || precision == TVAL3_PREC_FP16_DF64; }

// device operator from a host sparse matrix.  FP32 values under FP64 vectors
// (TVAL3_PREC_FP32_F64VEC) go up as FP32 and stay FP32.  tune = false skips
// the lane timing (an operator that only backs a double-float view).
template <class T>
LinOp<T>* sparse_op(const tval3_sparse_host* A, int precision, bool tune = true) {
    if (!A) arg_error(TVAL3_ERR_ARG, "Argument error: A is NULL!");
    const bool narrowed = std::is_same<T, float>::value && A->val_type == TVAL3_PREC_FP64;
    const bool dev_check = A->nnz > DEVICE_CHECK_NNZ && !narrowed;
    check_sparse(A, !dev_check);
    const long m = A->rows, n = A->cols, nnz = A->nnz;
    if constexpr (std::is_same<T, double>::value) {
        if (precision == TVAL3_PREC_FP32_F64VEC && A->val_type == TVAL3_PREC_FP32) {
            F32Csr c;
            upload_f32(A, dev_check, c);
            PhaseTimer pl(2);
            return make_csr_op_f64vec(m, n, nnz, c.ptr.p, c.ind.p, c.val.p, c.tptr.p, c.tptr.p ? c.tind.p : nullptr,
                                      c.tptr.p ? c.tval.p : nullptr, 0, tune);
        }
    }
    DBuf<int> ptr, ind, tptr, tind;
    DBuf<T> val, tval;
    cudaStream_t s = 0;
    std::unique_ptr<PhaseTimer> up(new PhaseTimer(0));
    if (A->format & TVAL3_SPARSE_CSR) {
        ptr.alloc(m + 1);
        ind.alloc(std::max<long>(nnz, 1));
        h2d(ptr.p, A->csr_ptr, (m + 1) * sizeof(int));
        h2d(ind.p, A->csr_ind, nnz * sizeof(int));
        to_device(val, A->csr_val, nnz, A->val_type);
    }
    if (A->format & TVAL3_SPARSE_CSC) {
        tptr.alloc(n + 1);
        tind.alloc(std::max<long>(nnz, 1));
        h2d(tptr.p, A->csc_ptr, (n + 1) * sizeof(int));
        h2d(tind.p, A->csc_ind, nnz * sizeof(int));
        to_device(tval, A->csc_val, nnz, A->val_type);
    }
    up.reset();
    if (dev_check) {
        PhaseTimer pv(1);
        if (A->format & TVAL3_SPARSE_CSR) validate_device<T>(ptr.p, m, ind.p, val.p, nnz, n, "CSR");
        if (A->format & TVAL3_SPARSE_CSC) validate_device<T>(tptr.p, n, tind.p, tval.p, nnz, m, "CSC");
    }
    PhaseTimer pl(2);
    if (!(A->format & TVAL3_SPARSE_CSR)) {
        // only CSC given: its transpose is the CSR of A
        ptr.alloc(m + 1);
        ind.alloc(std::max<long>(nnz, 1));
        val.alloc(std::max<long>(nnz, 1));
        csr_transpose_device<T>(n, m, nnz, tptr.p, tind.p, tval.p, ptr.p, ind.p, val.p, s);
    }
    return make_csr_op_device<T>(m, n, nnz, ptr.p, ind.p, val.p, tptr.p ? tptr.p : nullptr,
                                 tptr.p ? tind.p : nullptr, tptr.p ? tval.p : nullptr, precision, s);
}

void check_opts(const tval3_options* o) {
    if (!o) arg_error(TVAL3_ERR_ARG, "Argument error: opts is NULL!");
    if (!(o->skipMulRatio >= 0.0) || !std::isfinite(o->skipMulRatio) || std::isnan(o->maxRelativeChange))
        arg_error(TVAL3_ERR_ARG, "Argument error: skipMulRatio must be finite and >= 0!");
    if (!(o->beta > 0) || !(o->mu > 0) || !(o->beta0 > 0) || !(o->mu0 > 0))
        arg_error(TVAL3_ERR_ARG, "Argument error: mu, mu0, beta, beta0 must be positive!");
}

// calls f on whichever solver the handle holds (float, double or double-float)
template <class F>
void with_solver(tval3_solver s, F f) {
    if (s->q) f(*s->q);
    else if (s->d) f(*s->d);
    else f(*s->f);
}

template <class T>
void check_vec(const T* v, long n, const char* what) {
    for (long i = 0; i < n; ++i)
        if (!std::isfinite((double)v[i])) arg_error(TVAL3_ERR_NONFINITE, std::string("Argument error: non-finite ") + what + "!");
}

// the common body of the reference entry points: host U/b/Ut, operator built
template <class T>
void solve_host(LinOp<T>* op, Ext<T>* U, int dim_y, int dim_x, int dim_z, const Ext<T>* b, int b_len,
                const tval3_options* opts, const Ext<T>* Ut, int Ut_len, tval3_info* info,
                std::chrono::steady_clock::time_point t0, int layers = 1) {
    using E = Ext<T>;
    std::unique_ptr<LinOp<T>> hold(op);
    using clk = std::chrono::steady_clock;
    const auto ta = clk::now();
    const long n = (long)dim_y * dim_x * dim_z * layers;
    DBuf<E> db, dU, dUt;
    db.alloc(std::max<long>(b_len, 1));
    dU.alloc(std::max<long>(n, 1));
    h2d(db.p, b, b_len * sizeof(E));
    const bool use_ut = Ut && Ut_len == n && n > 0;
    if (use_ut) {
        dUt.alloc(n);
        h2d(dUt.p, Ut, n * sizeof(E));
    }
    Solver<T> s(op, dim_y, dim_x, dim_z, *opts, layers);
    s.mode = 1;  // the whole solve as one graph launch
    TV3_CUDA(cudaDeviceSynchronize());
    const auto tb = clk::now();
    tval3_info inf{};
    s.solve(db.p, dU.p, use_ut ? dUt.p : nullptr, &inf, 0);
    const auto tc = clk::now();
    TV3_CUDA(cudaMemcpy(U, dU.p, n * sizeof(E), cudaMemcpyDeviceToHost));
    const auto td = clk::now();
    auto sec = [](clk::time_point a, clk::time_point b) { return std::chrono::duration<double>(b - a).count(); };
    g_phase[0] = sec(t0, ta);
    g_phase[1] = sec(ta, tb);
    g_phase[2] = sec(tb, tc);
    g_phase[3] = sec(tc, td);
    inf.outer_secs = sec(t0, td);
    if (info) *info = inf;
}

template <class T>
void check_problem(const T* U, int dim_y, int dim_x, int dim_z, long A_rows, long A_cols, const T* b, int b_len,
                   const T* Ut, int Ut_len) {
    if (!U || dim_y <= 0 || dim_x <= 0 || dim_z <= 0) arg_error(TVAL3_ERR_ARG, "Argument error: U must be a non-empty volume!");
    const long n = (long)dim_y * dim_x * dim_z;
    if (Ut && Ut_len > 0 && Ut_len != n) arg_error(TVAL3_ERR_SHAPE, "Argument error: U and Ut must have the same size!");
    if (n != A_cols) arg_error(TVAL3_ERR_SHAPE, "Argument error: the length of U must be equal to A.dim_x!");
    if (b_len != A_rows) arg_error(TVAL3_ERR_SHAPE, "Argument error: b.len must be equal to A.dim_y!");
    if (b_len > 0 && !b) arg_error(TVAL3_ERR_ARG, "Argument error: b is NULL!");
    check_vec(b, b_len, "measurement b");
}

// The 2D entries' form (2d/tval3.cu:1406-1426): layers = b.len / A.rows
// columns of b share A; U holds A.cols * layers values (U and Ut column-major,
// one image per column).  Returns the number of layers.
template <class T>
int check_problem_2d(const T* U, int rows, int cols, long A_rows, long A_cols, const T* b, int b_len, const T* Ut,
                     int Ut_len) {
    if (!U || rows <= 0 || cols <= 0) arg_error(TVAL3_ERR_ARG, "Argument error: U must be a non-empty image!");
    const long n = (long)rows * cols;
    if (n != A_cols) arg_error(TVAL3_ERR_SHAPE, "Argument error: the length of U must be equal to A.cols * layers!");
    if (A_rows == 0 && b_len == 0) return 1;
    if (A_rows <= 0 || b_len <= 0 || b_len % A_rows != 0)
        arg_error(TVAL3_ERR_SHAPE, "Argument error: b.len must be equal to A.rows * layers!");
    const int layers = (int)(b_len / A_rows);
    if (Ut && Ut_len > 0 && Ut_len != n * layers)
        arg_error(TVAL3_ERR_SHAPE, "Argument error: U and Ut must have the same size!");
    if (!b) arg_error(TVAL3_ERR_ARG, "Argument error: b is NULL!");
    check_vec(b, b_len, "measurement b");
    return layers;
}

// a product that timed out in a bounded device wait is an error of the call
void check_product(tval3_op op, cudaStream_t s) {
    int e = 0;
    if (op->q) e = op->q->take_error(s);
    else if (op->d) e = op->d->take_error(s);
    else e = op->f->take_error(s);
    if (e) arg_error(TVAL3_ERR_TIMEOUT, "a bounded device wait of the product ran out (error bits " +
                                            std::to_string(e) + "); the output is incomplete");
}

// the operator of a handle whose products take vectors of type T
template <class T>
const LinOp<T>* vec_op(tval3_op op);
template <>
const LinOp<float>* vec_op<float>(tval3_op op) {
    if (!op || !op->f) arg_error(TVAL3_ERR_ARG, "Argument error: the _f32 step needs an FP32-vector operator!");
    return op->f;
}
template <>
const LinOp<double>* vec_op<double>(tval3_op op) {
    if (!op || !op->d || op->q) arg_error(TVAL3_ERR_ARG, "Argument error: the _f64 step needs an FP64-vector operator!");
    return op->d;
}

template <class T>
void unroll_checks(tval3_op op, int p, int q, int r, int first, const double* mub, const T* U, const T* Up,
                   const T* gp, const T* g2p, const T* b) {
    const LinOp<T>* A = vec_op<T>(op);
    if (p <= 0 || q <= 0 || r <= 0 || (long)p * q * r != A->n)
        arg_error(TVAL3_ERR_SHAPE, "Argument error: the volume must have A.cols voxels!");
    if (!mub || !U || !b || (!first && (!Up || !gp || !g2p)))
        arg_error(TVAL3_ERR_ARG, "Argument error: NULL input of the unrolled step!");
}

template <class T>
void unroll_fwd_entry(tval3_op op, int p, int q, int r, int first, int iso, int nonneg, const double* mub, const T* U,
                      const T* Up, const T* gp, const T* g2p, const T* b, const T* sig, const T* delta, T* Un, T* g,
                      T* g2, void* stream) {
    unroll_checks<T>(op, p, q, r, first, mub, U, Up, gp, g2p, b);
    if (!Un || !g || !g2) arg_error(TVAL3_ERR_ARG, "Argument error: NULL output of the unrolled step!");
    const LinOp<T>* A = vec_op<T>(op);
    unroll_step<T>(A, p, q, r, first, iso, nonneg, mub, U, Up, gp, g2p, b, sig, delta, Un, g, g2, (cudaStream_t)stream);
    check_product(op, (cudaStream_t)stream);
}

template <class T>
void unroll_bwd_entry(tval3_op op, int p, int q, int r, int first, int iso, int nonneg, const double* mub, const T* U,
                      const T* Up, const T* gp, const T* g2p, const T* b, const T* sig, const T* delta, const T* gUn,
                      const T* gg, const T* gg2, T* gU, T* gUp, T* ggp, T* gg2p, T* gb, double* gmub, void* stream) {
    unroll_checks<T>(op, p, q, r, first, mub, U, Up, gp, g2p, b);
    if (!gU) arg_error(TVAL3_ERR_ARG, "Argument error: NULL adjoint of U!");
    const LinOp<T>* A = vec_op<T>(op);
    unroll_step_adjoint<T>(A, p, q, r, first, iso, nonneg, mub, U, Up, gp, g2p, b, sig, delta, gUn, gg, gg2, gU,
                           first ? nullptr : gUp, first ? nullptr : ggp, first ? nullptr : gg2p, gb, gmub,
                           (cudaStream_t)stream);
    check_product(op, (cudaStream_t)stream);
}

}  // namespace

namespace tv3 {
// noalloc.cu: dense A^T*y with its slab partials in a static device array
void dense_rmatvec_noalloc_f32(long rows, long cols, const float* A, const float* y, float* x, cudaStream_t s);
}  // namespace tv3

extern "C" {

void tval3_options_default(tval3_options* o) {
    if (!o) return;
    std::memset(o, 0, sizeof(*o));
    o->mu = 256.0; o->mu0 = 256.0; o->beta = 32.0; o->beta0 = 32.0; o->rate_cnt = 2.0;
    o->tol = 1e-6; o->tol_inn = 1e-3; o->maxcnt = 10; o->maxit = 1025; o->c = 1e-5;
    o->gamma = 0.6; o->gam = 0.9995; o->rate_gam = 0.9; o->isreal = 1; o->nonneg = 1;
    o->numInitIterations = 0; o->skipMulRatio = 0.0; o->maxRelativeChange = 0.0;
    o->tv_type = TVAL3_TV_ANISO;
    o->precision = -1;
}

const char* tval3_last_error_message(void) { return g_err.c_str(); }

tval3_status tval3_last_call_phases(double* secs, int n) {
    return guard([&] {
        if (!secs || n < 0) arg_error(TVAL3_ERR_ARG, "Argument error: NULL phase array!");
        for (int i = 0; i < n && i < 4; ++i) secs[i] = g_phase[i];
        for (int i = 4; i < n && i < 10; ++i) secs[i] = sub_phase[i - 4];
    });
}
const char* tval3_version(void) { return "tval3-gb300 0.1 (sm_103a)"; }

tval3_status tval3_gpu_3d_sparse_f32(float* U, int dim_y, int dim_x, int dim_z, const tval3_sparse_host* A,
                                     const float* b, int b_len, const tval3_options* opts, const float* Ut,
                                     int Ut_len, int, int, int, const int*, tval3_info* info) {
    return guard([&] {
        auto t0 = entry_clock();
        check_opts(opts);
        if (!A) arg_error(TVAL3_ERR_ARG, "Argument error: A is NULL!");
        check_problem(U, dim_y, dim_x, dim_z, A->rows, A->cols, b, b_len, Ut, Ut_len);
        solve_host<float>(sparse_op<float>(A, TVAL3_PREC_FP32), U, dim_y, dim_x, dim_z, b, b_len, opts, Ut, Ut_len,
                          info, t0);
    });
}

tval3_status tval3_gpu_3d_sparse_f64(double* U, int dim_y, int dim_x, int dim_z, const tval3_sparse_host* A,
                                     const double* b, int b_len, const tval3_options* opts, const double* Ut,
                                     int Ut_len, int, int, int, const int*, tval3_info* info) {
    return guard([&] {
        auto t0 = entry_clock();
        check_opts(opts);
        if (!A) arg_error(TVAL3_ERR_ARG, "Argument error: A is NULL!");
        check_problem(U, dim_y, dim_x, dim_z, A->rows, A->cols, b, b_len, Ut, Ut_len);
        // FP32 matrix values keep their storage (FP64 vectors and reductions)
        const int prec = (A->val_type == TVAL3_PREC_FP32) ? TVAL3_PREC_FP32_F64VEC : TVAL3_PREC_FP64;
        if (prec == TVAL3_PREC_FP32_F64VEC && opts->precision == TVAL3_PREC_FP32_DF64) {
            // double-float solve over the FP32 matrix; FP64 at the interface
            std::unique_ptr<LinOp<double>> base(sparse_op<double>(A, prec, false));
            solve_host<df64>(make_df64_view(base.get()), U, dim_y, dim_x, dim_z, b, b_len, opts, Ut, Ut_len, info,
                             t0);
            return;
        }
        if (is_mixed(opts->precision)) {
            // 16-bit matrix with per-ray scales, double-float solve
            solve_host<df64>(sparse_op_mixed(A, opts->precision), U, dim_y, dim_x, dim_z, b, b_len, opts, Ut, Ut_len,
                             info, t0);
            return;
        }
        solve_host<double>(sparse_op<double>(A, prec), U, dim_y, dim_x, dim_z, b, b_len, opts, Ut, Ut_len, info, t0);
    });
}

tval3_status tval3_gpu_sparse(float* U, int rows, int cols, const tval3_sparse_host* A, const float* b, int b_len,
                              const tval3_options* opts, const float* Ut, int Ut_len, int, tval3_info* info) {
    return guard([&] {
        auto t0 = entry_clock();
        check_opts(opts);
        if (!A) arg_error(TVAL3_ERR_ARG, "Argument error: A is NULL!");
        const int layers = check_problem_2d(U, rows, cols, A->rows, A->cols, b, b_len, Ut, Ut_len);
        solve_host<float>(sparse_op<float>(A, TVAL3_PREC_FP32), U, rows, cols, 1, b, b_len, opts, Ut, Ut_len, info,
                          t0, layers);
    });
}

tval3_status tval3_gpu_3d_dense_f32(float* U, int dim_y, int dim_x, int dim_z, const tval3_dense_host* A,
                                    const float* b, int b_len, const tval3_options* opts, const float* Ut,
                                    int Ut_len, int, int, int, const int*, tval3_info* info) {
    return guard([&] {
        auto t0 = entry_clock();
        check_opts(opts);
        if (!A || !A->data || A->rows < 0 || A->cols < 0) arg_error(TVAL3_ERR_ARG, "Argument error: bad dense matrix!");
        check_problem(U, dim_y, dim_x, dim_z, A->rows, A->cols, b, b_len, Ut, Ut_len);
        solve_host<float>(make_dense_op<float>(A->rows, A->cols, A->data, A->row_major, A->val_type, TVAL3_PREC_FP32, 0),
                          U, dim_y, dim_x, dim_z, b, b_len, opts, Ut, Ut_len, info, t0);
    });
}

tval3_status tval3_gpu_3d_dense_f64(double* U, int dim_y, int dim_x, int dim_z, const tval3_dense_host* A,
                                    const double* b, int b_len, const tval3_options* opts, const double* Ut,
                                    int Ut_len, int, int, int, const int*, tval3_info* info) {
    return guard([&] {
        auto t0 = entry_clock();
        check_opts(opts);
        if (!A || !A->data || A->rows < 0 || A->cols < 0) arg_error(TVAL3_ERR_ARG, "Argument error: bad dense matrix!");
        check_problem(U, dim_y, dim_x, dim_z, A->rows, A->cols, b, b_len, Ut, Ut_len);
        solve_host<double>(make_dense_op<double>(A->rows, A->cols, A->data, A->row_major, A->val_type, TVAL3_PREC_FP64, 0),
                           U, dim_y, dim_x, dim_z, b, b_len, opts, Ut, Ut_len, info, t0);
    });
}

tval3_status tval3_gpu_dense(float* U, int rows, int cols, const tval3_dense_host* A, const float* b, int b_len,
                             const tval3_options* opts, const float* Ut, int Ut_len, int, tval3_info* info) {
    return guard([&] {
        auto t0 = entry_clock();
        check_opts(opts);
        if (!A || !A->data || A->rows < 0 || A->cols < 0) arg_error(TVAL3_ERR_ARG, "Argument error: bad dense matrix!");
        const int layers = check_problem_2d(U, rows, cols, A->rows, A->cols, b, b_len, Ut, Ut_len);
        const int prec = (opts->precision == TVAL3_PREC_BF16) ? TVAL3_PREC_BF16 : TVAL3_PREC_FP32;
        solve_host<float>(make_dense_op<float>(A->rows, A->cols, A->data, A->row_major, A->val_type, prec, 0), U,
                          rows, cols, 1, b, b_len, opts, Ut, Ut_len, info, t0, layers);
    });
}

tval3_status tval3_gpu_3d_geometry_f32(float* U, int dim_y, int dim_x, int dim_z, const tval3_geometry_host* A,
                                       const float* b, int b_len, const tval3_options* opts, const float* Ut,
                                       int Ut_len, int, int, int, const int*, tval3_info* info) {
    return guard([&] {
        auto t0 = entry_clock();
        check_opts(opts);
        if (!A) arg_error(TVAL3_ERR_ARG, "Argument error: A is NULL!");
        if (A->rv_y != dim_y || A->rv_x != dim_x || A->rv_z != dim_z)
            arg_error(TVAL3_ERR_SHAPE, "Argument error: the volume of U must equal the geometry's rv_y x rv_x x rv_z!");
        // the reference evaluates this overload on the fly (geom_mm_multGPU): no matrix is stored, for
        // Bresenham and Siddon rays alike
        LinOp<float>* op = make_geometry_op<float>(A, 1, TVAL3_PREC_FP32, 0);
        try {
            check_problem(U, dim_y, dim_x, dim_z, op->m, op->n, b, b_len, Ut, Ut_len);
        } catch (...) {
            delete op;
            throw;
        }
        solve_host<float>(op, U, dim_y, dim_x, dim_z, b, b_len, opts, Ut, Ut_len, info, t0);
    });
}

tval3_status tval3_gpu_3d_geometry_sparse_f32(float* U, int dim_y, int dim_x, int dim_z,
                                              const tval3_geometry_host* A_geo, const tval3_sparse_host* A_mat,
                                              const float* b, int b_len, const tval3_options* opts, const float* Ut,
                                              int Ut_len, int, int, int, const int*, tval3_info* info) {
    return guard([&] {
        auto t0 = entry_clock();
        check_opts(opts);
        if (!A_geo || !A_mat) arg_error(TVAL3_ERR_ARG, "Argument error: A is NULL!");
        check_problem(U, dim_y, dim_x, dim_z, A_mat->rows, A_mat->cols, b, b_len, Ut, Ut_len);
        std::unique_ptr<LinOp<float>> geo(make_geometry_op<float>(A_geo, 1, TVAL3_PREC_FP32, 0));
        std::unique_ptr<LinOp<float>> mat(sparse_op<float>(A_mat, TVAL3_PREC_FP32));
        if (geo->m != mat->m || geo->n != mat->n)
            arg_error(TVAL3_ERR_SHAPE, "Argument error: geometry and sparse matrix disagree in shape!");
        solve_host<float>(new SplitOp<float>(std::move(geo), std::move(mat)), U, dim_y, dim_x, dim_z, b, b_len, opts,
                          Ut, Ut_len, info, t0);
    });
}

tval3_status tval3_gpu_3d_geometry_f64(double* U, int dim_y, int dim_x, int dim_z, const tval3_geometry_host* A,
                                       const double* b, int b_len, const tval3_options* opts, const double* Ut,
                                       int Ut_len, int, int, int, const int*, tval3_info* info) {
    return guard([&] {
        auto t0 = entry_clock();
        check_opts(opts);
        if (!A) arg_error(TVAL3_ERR_ARG, "Argument error: A is NULL!");
        if (A->rv_y != dim_y || A->rv_x != dim_x || A->rv_z != dim_z)
            arg_error(TVAL3_ERR_SHAPE, "Argument error: the volume of U must equal the geometry's rv_y x rv_x x rv_z!");
        // the ray matrix is built on the device and stored (FP32 path lengths);
        // the solve runs in FP64, double-float, or double-float over a 16-bit
        // copy of the matrix, as opts->precision asks
        const int pr = opts->precision;
        if (pr == TVAL3_PREC_FP32_DF64 || is_mixed(pr)) {
            std::unique_ptr<LinOp<double>> base;
            LinOp<df64>* op = nullptr;
            if (pr == TVAL3_PREC_FP32_DF64) {
                base.reset(make_geometry_op<double>(A, 0, TVAL3_PREC_FP32_DF64, 0));
                op = make_df64_view(base.get());
            } else {
                op = make_geometry_op<df64>(A, 0, pr, 0);
            }
            try {
                check_problem(U, dim_y, dim_x, dim_z, op->m, op->n, b, b_len, Ut, Ut_len);
            } catch (...) {
                delete op;
                throw;
            }
            solve_host<df64>(op, U, dim_y, dim_x, dim_z, b, b_len, opts, Ut, Ut_len, info, t0);
            return;
        }
        LinOp<double>* op = make_geometry_op<double>(A, 0, TVAL3_PREC_FP32_F64VEC, 0);
        try {
            check_problem(U, dim_y, dim_x, dim_z, op->m, op->n, b, b_len, Ut, Ut_len);
        } catch (...) {
            delete op;
            throw;
        }
        solve_host<double>(op, U, dim_y, dim_x, dim_z, b, b_len, opts, Ut, Ut_len, info, t0);
    });
}

tval3_status tval3_gpu_3d_geometry_sparse_f64(double* U, int dim_y, int dim_x, int dim_z,
                                              const tval3_geometry_host* A_geo, const tval3_sparse_host* A_mat,
                                              const double* b, int b_len, const tval3_options* opts,
                                              const double* Ut, int Ut_len, int, int, int, const int*,
                                              tval3_info* info) {
    return guard([&] {
        auto t0 = entry_clock();
        check_opts(opts);
        if (!A_geo || !A_mat) arg_error(TVAL3_ERR_ARG, "Argument error: A is NULL!");
        if (A_geo->rv_y != dim_y || A_geo->rv_x != dim_x || A_geo->rv_z != dim_z)
            arg_error(TVAL3_ERR_SHAPE, "Argument error: the volume of U must equal the geometry's rv_y x rv_x x rv_z!");
        check_problem(U, dim_y, dim_x, dim_z, A_mat->rows, A_mat->cols, b, b_len, Ut, Ut_len);
        // A*x from the geometry's ray matrix (built on the device), A^T*y from
        // the given sparse matrix, both with FP64 vectors
        std::unique_ptr<LinOp<double>> geo(make_geometry_op<double>(A_geo, 0, TVAL3_PREC_FP32_F64VEC, 0));
        const int prec = (A_mat->val_type == TVAL3_PREC_FP32) ? TVAL3_PREC_FP32_F64VEC : TVAL3_PREC_FP64;
        std::unique_ptr<LinOp<double>> mat(sparse_op<double>(A_mat, prec));
        if (geo->m != mat->m || geo->n != mat->n)
            arg_error(TVAL3_ERR_SHAPE, "Argument error: geometry and sparse matrix disagree in shape!");
        solve_host<double>(new SplitOp<double>(std::move(geo), std::move(mat)), U, dim_y, dim_x, dim_z, b, b_len,
                           opts, Ut, Ut_len, info, t0);
    });
}

// ---------------------------------------------------------------------------
// operators
// ---------------------------------------------------------------------------
tval3_status tval3_op_create_sparse(tval3_op* op, const tval3_sparse_host* A, int precision) {
    return guard([&] {
        if (!op) arg_error(TVAL3_ERR_ARG, "Argument error: op is NULL!");
        if (precision < 0 || precision > 7) arg_error(TVAL3_ERR_ARG, "Argument error: unknown precision!");
        const long long b0 = dbuf_live_bytes;
        auto* h = new tval3_op_s();
        try {
            h->precision = precision;
            if (is_mixed(precision)) {
                h->dbl = 1;
                h->q = sparse_op_mixed(A, precision);
            } else if (precision == TVAL3_PREC_FP32_DF64) {
                h->dbl = 1;
                h->d = sparse_op<double>(A, TVAL3_PREC_FP32_F64VEC, false);
                h->q = make_df64_view(h->d);
            } else if (precision == TVAL3_PREC_FP64 || precision == TVAL3_PREC_FP32_F64VEC) {
                h->dbl = 1;
                h->d = sparse_op<double>(A, precision);
            } else {
                h->f = sparse_op<float>(A, precision);
            }
        } catch (...) {
            delete h;
            throw;
        }
        h->device_bytes = dbuf_live_bytes - b0;
        *op = h;
    });
}

tval3_status tval3_op_create_sparse_device(tval3_op* op, int rows, int cols, int nnz, const int* d_ptr,
                                           const int* d_ind, const float* d_val, int precision, void* stream) {
    return guard([&] {
        if (!op) arg_error(TVAL3_ERR_ARG, "Argument error: op is NULL!");
        if (rows < 0 || cols < 0 || nnz < 0 || !d_ptr) arg_error(TVAL3_ERR_ARG, "Argument error: bad device CSR!");
        if (precision == TVAL3_PREC_FP64 || precision < 0 || precision > 3)
            arg_error(TVAL3_ERR_UNSUPPORTED, "device CSR input takes FP32 values (FP32/BF16/FP16 storage)");
        const long long b0 = dbuf_live_bytes;
        auto* h = new tval3_op_s();
        try {
            h->precision = precision;
            h->f = make_csr_op_device<float>(rows, cols, nnz, d_ptr, d_ind, d_val, nullptr, nullptr, nullptr, precision,
                                             (cudaStream_t)stream);
        } catch (...) {
            delete h;
            throw;
        }
        h->device_bytes = dbuf_live_bytes - b0;
        *op = h;
    });
}

tval3_status tval3_op_create_geometry(tval3_op* op, const tval3_geometry_host* G, int mode, int precision) {
    return guard([&] {
        if (!op) arg_error(TVAL3_ERR_ARG, "Argument error: op is NULL!");
        if (mode < 0 || mode > 1) arg_error(TVAL3_ERR_ARG, "Argument error: unknown geometry mode!");
        if (precision == TVAL3_PREC_FP64 || precision < 0 || precision > 7)
            arg_error(TVAL3_ERR_UNSUPPORTED, "geometry operators store FP32/BF16/FP16 values");
        if (mode == 1 && precision != TVAL3_PREC_FP32)
            arg_error(TVAL3_ERR_UNSUPPORTED, "on-the-fly traversal stores nothing; use FP32");
        const long long b0 = dbuf_live_bytes;
        auto* h = new tval3_op_s();
        try {
            h->precision = precision;
            if (is_mixed(precision)) {
                h->dbl = 1;
                h->q = make_geometry_op<df64>(G, mode, precision, 0);
            } else if (precision == TVAL3_PREC_FP32_F64VEC || precision == TVAL3_PREC_FP32_DF64) {
                h->dbl = 1;
                h->d = make_geometry_op<double>(G, mode, precision, 0);
                if (precision == TVAL3_PREC_FP32_DF64) h->q = make_df64_view(h->d);
            } else {
                h->f = make_geometry_op<float>(G, mode, precision, 0);
            }
            // the geometry fixes the volume: regroup A^T by voxel tiles now
            if (G && mode == 0) {
                if (h->q) h->q->set_volume(G->rv_y, G->rv_x, G->rv_z);
                else if (h->d) h->d->set_volume(G->rv_y, G->rv_x, G->rv_z);
                else h->f->set_volume(G->rv_y, G->rv_x, G->rv_z);
            }
        } catch (...) {
            delete h;
            throw;
        }
        h->device_bytes = dbuf_live_bytes - b0;
        *op = h;
    });
}

tval3_status tval3_op_create_dense(tval3_op* op, const tval3_dense_host* A, int precision) {
    return guard([&] {
        if (!op || !A || !A->data || A->rows < 0 || A->cols < 0) arg_error(TVAL3_ERR_ARG, "Argument error: bad dense matrix!");
        if (precision == TVAL3_PREC_FP16 || precision < 0 || precision > 3)
            arg_error(TVAL3_ERR_UNSUPPORTED, "dense storage: FP32, FP64 or BF16");
        const long long b0 = dbuf_live_bytes;
        auto* h = new tval3_op_s();
        try {
            h->precision = precision;
            if (precision == TVAL3_PREC_FP64) {
                h->dbl = 1;
                h->d = make_dense_op<double>(A->rows, A->cols, A->data, A->row_major, A->val_type, precision, 0);
            } else {
                h->f = make_dense_op<float>(A->rows, A->cols, A->data, A->row_major, A->val_type, precision, 0);
            }
        } catch (...) {
            delete h;
            throw;
        }
        h->device_bytes = dbuf_live_bytes - b0;
        *op = h;
    });
}

tval3_status tval3_op_destroy(tval3_op op) {
    return guard([&] { delete op; });
}

tval3_status tval3_op_shape(tval3_op op, int* rows, int* cols, int64_t* nnz) {
    return guard([&] {
        if (!op) arg_error(TVAL3_ERR_ARG, "Argument error: op is NULL!");
        if (rows) *rows = (int)op->rows();
        if (cols) *cols = (int)op->cols();
        if (nnz) *nnz = op->nnz();
    });
}

tval3_status tval3_selftest_bounded_wait(int64_t cycles, int* timed_out, int64_t* waited_cycles) {
    return guard([&] {
        if (!timed_out || !waited_cycles) arg_error(TVAL3_ERR_ARG, "Argument error: timed_out or waited_cycles is NULL!");
        if (cycles < 0 || cycles > 4000000000LL) arg_error(TVAL3_ERR_ARG, "Argument error: cycles outside [0, 4e9]!");
        long long w = 0;
        selftest_bounded_wait((long long)cycles, timed_out, &w);
        *waited_cycles = (int64_t)w;
    });
}

tval3_status tval3_op_device_bytes(tval3_op op, int64_t* bytes) {
    return guard([&] {
        if (!op || !bytes) arg_error(TVAL3_ERR_ARG, "Argument error: op or bytes is NULL!");
        *bytes = op->device_bytes;
    });
}

tval3_status tval3_op_export_csr(tval3_op op, int* ptr, int* ind, float* val, int* tptr, int* tind, float* tval) {
    return guard([&] {
        if (!op) arg_error(TVAL3_ERR_ARG, "Argument error: op is NULL!");
        op->with_store([&](auto& A) { A.export_csr(ptr, ind, val, tptr, tind, tval); });
    });
}

tval3_status tval3_op_export_csr_scaled(tval3_op op, int* ptr, int* ind, float* val, float* row_scale, int* tptr,
                                        int* tind, float* tval) {
    return guard([&] {
        if (!op) arg_error(TVAL3_ERR_ARG, "Argument error: op is NULL!");
        op->with_store([&](auto& A) {
            A.export_csr(ptr, ind, nullptr, tptr, tind, nullptr);
            A.export_scaled(val, row_scale, tval);
        });
    });
}

// a bounded device wait of a standalone product that ran out (the product's
// output is incomplete)

tval3_status tval3_mat_vec_mul(tval3_op op, int trans, const void* x, void* y, void* stream) {
    return guard([&] {
        if (!op || !x || !y) arg_error(TVAL3_ERR_ARG, "Argument error: NULL operator or vector!");
        cudaStream_t s = (cudaStream_t)stream;
        if (op->q) op->q->apply(trans ? 1 : 0, plain_io<df64>((const df64*)x, (df64*)y), SPMV_PLAIN, s);
        else if (op->dbl) op->d->apply(trans ? 1 : 0, plain_io<double>((const double*)x, (double*)y), SPMV_PLAIN, s);
        else op->f->apply(trans ? 1 : 0, plain_io<float>((const float*)x, (float*)y), SPMV_PLAIN, s);
        check_product(op, s);
    });
}

tval3_status tval3_mat_mat_mul(tval3_op op, int trans, int nrhs, const void* X, void* Y, void* stream) {
    return guard([&] {
        if (!op || !X || !Y || nrhs < 0) arg_error(TVAL3_ERR_ARG, "Argument error: bad multi-RHS product!");
        cudaStream_t s = (cudaStream_t)stream;
        if (op->q) op->q->apply_multi(trans ? 1 : 0, nrhs, (const df64*)X, (df64*)Y, s);
        else if (op->dbl) op->d->apply_multi(trans ? 1 : 0, nrhs, (const double*)X, (double*)Y, s);
        else op->f->apply_multi(trans ? 1 : 0, nrhs, (const float*)X, (float*)Y, s);
        check_product(op, s);
    });
}

tval3_status tval3_op_set_variant(tval3_op op, int trans, int variant) {
    return guard([&] {
        if (!op) arg_error(TVAL3_ERR_ARG, "Argument error: op is NULL!");
        bool ok = op->q ? op->q->set_variant(trans ? 1 : 0, variant)
                        : (op->dbl ? op->d->set_variant(trans ? 1 : 0, variant) : op->f->set_variant(trans ? 1 : 0, variant));
        if (!ok) arg_error(TVAL3_ERR_UNSUPPORTED, "product variant not available for this operator");
    });
}

tval3_status tval3_op_get_variant(tval3_op op, int trans, int* variant) {
    return guard([&] {
        if (!op || !variant) arg_error(TVAL3_ERR_ARG, "Argument error: NULL argument!");
        *variant = op->q ? op->q->variant(trans ? 1 : 0)
                         : (op->dbl ? op->d->variant(trans ? 1 : 0) : op->f->variant(trans ? 1 : 0));
    });
}

tval3_status tval3_mat_mat_mul_interleaved(tval3_op op, int trans, int nrhs, const void* X, void* Y, void* stream) {
    return guard([&] {
        if (!op || !X || !Y || nrhs < 1) arg_error(TVAL3_ERR_ARG, "Argument error: bad multi-RHS product!");
        cudaStream_t s = (cudaStream_t)stream;
        auto run = [&](auto* A, auto* x, auto* y) {
            using T = std::remove_const_t<std::remove_pointer_t<decltype(x)>>;
            if (nrhs > 1 && !A->multi_rhs())
                arg_error(TVAL3_ERR_UNSUPPORTED, "operator has no interleaved multi-RHS product");
            A->prepare(nrhs);
            MatIO<T> io = plain_io<T>(x, y);
            io.L = nrhs;
            A->apply(trans ? 1 : 0, io, SPMV_PLAIN, s);
        };
        if (op->q) run(op->q, (const df64*)X, (df64*)Y);
        else if (op->dbl) run(op->d, (const double*)X, (double*)Y);
        else run(op->f, (const float*)X, (float*)Y);
        check_product(op, s);
    });
}

tval3_status tval3_shrink_f32(int64_t n, const float* v, double t, int iso, float* W, void* stream) {
    return guard([&] {
        if (n < 0 || (n > 0 && (!v || !W))) arg_error(TVAL3_ERR_ARG, "Argument error: bad shrinkage arrays!");
        shrink_fwd<float>((long)n, v, t, iso, W, (cudaStream_t)stream);
    });
}
tval3_status tval3_shrink_f64(int64_t n, const double* v, double t, int iso, double* W, void* stream) {
    return guard([&] {
        if (n < 0 || (n > 0 && (!v || !W))) arg_error(TVAL3_ERR_ARG, "Argument error: bad shrinkage arrays!");
        shrink_fwd<double>((long)n, v, t, iso, W, (cudaStream_t)stream);
    });
}
tval3_status tval3_shrink_adjoint_f32(int64_t n, const float* v, double t, int iso, const float* gW, float* gv,
                                      float* gt, void* stream) {
    return guard([&] {
        if (n < 0 || (n > 0 && (!v || !gW || !gv))) arg_error(TVAL3_ERR_ARG, "Argument error: bad shrinkage arrays!");
        shrink_bwd<float>((long)n, v, t, iso, gW, gv, gt, (cudaStream_t)stream);
    });
}
tval3_status tval3_shrink_adjoint_f64(int64_t n, const double* v, double t, int iso, const double* gW, double* gv,
                                      double* gt, void* stream) {
    return guard([&] {
        if (n < 0 || (n > 0 && (!v || !gW || !gv))) arg_error(TVAL3_ERR_ARG, "Argument error: bad shrinkage arrays!");
        shrink_bwd<double>((long)n, v, t, iso, gW, gv, gt, (cudaStream_t)stream);
    });
}

tval3_status tval3_unroll_step_f32(tval3_op op, int p, int q, int r, int first, int iso, int nonneg,
                                   const double* mub, const float* U, const float* Up, const float* gp,
                                   const float* g2p, const float* b, const float* sig, const float* delta, float* Un,
                                   float* g, float* g2, void* stream) {
    return guard([&] {
        unroll_fwd_entry<float>(op, p, q, r, first, iso, nonneg, mub, U, Up, gp, g2p, b, sig, delta, Un, g, g2,
                                stream);
    });
}
tval3_status tval3_unroll_step_f64(tval3_op op, int p, int q, int r, int first, int iso, int nonneg,
                                   const double* mub, const double* U, const double* Up, const double* gp,
                                   const double* g2p, const double* b, const double* sig, const double* delta,
                                   double* Un, double* g, double* g2, void* stream) {
    return guard([&] {
        unroll_fwd_entry<double>(op, p, q, r, first, iso, nonneg, mub, U, Up, gp, g2p, b, sig, delta, Un, g, g2,
                                 stream);
    });
}
tval3_status tval3_unroll_step_adjoint_f32(tval3_op op, int p, int q, int r, int first, int iso, int nonneg,
                                           const double* mub, const float* U, const float* Up, const float* gp,
                                           const float* g2p, const float* b, const float* sig, const float* delta,
                                           const float* gUn, const float* gg, const float* gg2, float* gU,
                                           float* gUp, float* ggp, float* gg2p, float* gb, double* gmub,
                                           void* stream) {
    return guard([&] {
        unroll_bwd_entry<float>(op, p, q, r, first, iso, nonneg, mub, U, Up, gp, g2p, b, sig, delta, gUn, gg, gg2,
                                gU, gUp, ggp, gg2p, gb, gmub, stream);
    });
}
tval3_status tval3_unroll_step_adjoint_f64(tval3_op op, int p, int q, int r, int first, int iso, int nonneg,
                                           const double* mub, const double* U, const double* Up, const double* gp,
                                           const double* g2p, const double* b, const double* sig,
                                           const double* delta, const double* gUn, const double* gg,
                                           const double* gg2, double* gU, double* gUp, double* ggp, double* gg2p,
                                           double* gb, double* gmub, void* stream) {
    return guard([&] {
        unroll_bwd_entry<double>(op, p, q, r, first, iso, nonneg, mub, U, Up, gp, g2p, b, sig, delta, gUn, gg, gg2,
                                 gU, gUp, ggp, gg2p, gb, gmub, stream);
    });
}

tval3_status tval3_df64_from_f64(const double* d_in, void* d_pairs, int64_t n, void* stream) {
    return guard([&] {
        if (n < 0 || (n > 0 && (!d_in || !d_pairs))) arg_error(TVAL3_ERR_ARG, "Argument error: bad conversion!");
        convert_to_df64(d_in, d_pairs, (long)n, (cudaStream_t)stream);
    });
}

tval3_status tval3_df64_to_f64(const void* d_pairs, double* d_out, int64_t n, void* stream) {
    return guard([&] {
        if (n < 0 || (n > 0 && (!d_pairs || !d_out))) arg_error(TVAL3_ERR_ARG, "Argument error: bad conversion!");
        convert_from_df64(d_pairs, d_out, (long)n, (cudaStream_t)stream);
    });
}

// ---------------------------------------------------------------------------
// device-resident solver
// ---------------------------------------------------------------------------
tval3_status tval3_solver_create(tval3_solver* s, tval3_op A, int dim_y, int dim_x, int dim_z,
                                 const tval3_options* opts) {
    return guard([&] {
        if (!s || !A) arg_error(TVAL3_ERR_ARG, "Argument error: NULL solver or operator!");
        check_opts(opts);
        const long n = (long)dim_y * dim_x * dim_z;
        const long cols = A->cols();
        if (dim_y <= 0 || dim_x <= 0 || dim_z <= 0 || n != cols)
            arg_error(TVAL3_ERR_SHAPE, "Argument error: the length of U must be equal to A.dim_x!");
        auto* h = new tval3_solver_s();
        try {
            h->dbl = A->dbl;
            if (A->q) h->q = new Solver<df64>(A->q, dim_y, dim_x, dim_z, *opts);
            else if (A->dbl) h->d = new Solver<double>(A->d, dim_y, dim_x, dim_z, *opts);
            else h->f = new Solver<float>(A->f, dim_y, dim_x, dim_z, *opts);
        } catch (...) {
            delete h;
            throw;
        }
        *s = h;
    });
}

tval3_status tval3_solver_create_layers(tval3_solver* s, tval3_op A, int dim_y, int dim_x, int dim_z, int layers,
                                        const tval3_options* opts) {
    return guard([&] {
        if (!s || !A) arg_error(TVAL3_ERR_ARG, "Argument error: NULL solver or operator!");
        if (layers < 1) arg_error(TVAL3_ERR_ARG, "Argument error: layers must be positive!");
        check_opts(opts);
        const long n = (long)dim_y * dim_x * dim_z;
        const long cols = A->cols();
        if (dim_y <= 0 || dim_x <= 0 || dim_z <= 0 || n != cols)
            arg_error(TVAL3_ERR_SHAPE, "Argument error: the length of U must be equal to A.dim_x!");
        auto* h = new tval3_solver_s();
        try {
            h->dbl = A->dbl;
            if (A->q) h->q = new Solver<df64>(A->q, dim_y, dim_x, dim_z, *opts, layers);
            else if (A->dbl) h->d = new Solver<double>(A->d, dim_y, dim_x, dim_z, *opts, layers);
            else h->f = new Solver<float>(A->f, dim_y, dim_x, dim_z, *opts, layers);
        } catch (...) {
            delete h;
            throw;
        }
        *s = h;
    });
}

tval3_status tval3_solver_set_mode(tval3_solver s, int mode) {
    return guard([&] {
        if (!s || mode < 0 || mode > 1) arg_error(TVAL3_ERR_ARG, "Argument error: bad solver mode!");
        with_solver(s, [&](auto& v) { v.mode = mode; });
    });
}

tval3_status tval3_solver_solve(tval3_solver s, const void* d_b, void* d_U, const void* d_Ut, tval3_info* info,
                                void* stream) {
    return guard([&] {
        if (!s || !d_b || !d_U) arg_error(TVAL3_ERR_ARG, "Argument error: NULL solver or vector!");
        with_solver(s, [&](auto& v) { v.solve(d_b, d_U, d_Ut, info, (cudaStream_t)stream); });
    });
}

tval3_status tval3_solver_set_pause(tval3_solver s, int iterations) {
    return guard([&] {
        if (!s || iterations < 0) arg_error(TVAL3_ERR_ARG, "Argument error: bad pause!");
        with_solver(s, [&](auto& v) {
            v.pause_at = iterations;
            // the limit is a graph parameter: rebuild on the next solve
            if (v.gexec) cudaGraphExecDestroy(v.gexec);
            v.gexec = nullptr;
            if (v.rexec) cudaGraphExecDestroy(v.rexec);
            v.rexec = nullptr;
        });
    });
}

tval3_status tval3_solver_state_size(tval3_solver s, size_t* bytes) {
    return guard([&] {
        if (!s || !bytes) arg_error(TVAL3_ERR_ARG, "Argument error: NULL argument!");
        with_solver(s, [&](auto& v) { *bytes = v.state_bytes(); });
    });
}

tval3_status tval3_solver_save_state(tval3_solver s, void* host_state, void* stream) {
    return guard([&] {
        if (!s || !host_state) arg_error(TVAL3_ERR_ARG, "Argument error: NULL argument!");
        with_solver(s, [&](auto& v) { v.save_state(host_state, (cudaStream_t)stream); });
    });
}

tval3_status tval3_solver_resume(tval3_solver s, const void* host_state, void* d_U, const void* d_Ut,
                                 tval3_info* info, void* stream) {
    return guard([&] {
        if (!s || !host_state || !d_U) arg_error(TVAL3_ERR_ARG, "Argument error: NULL argument!");
        with_solver(s, [&](auto& v) { v.resume(host_state, d_U, d_Ut, info, (cudaStream_t)stream); });
    });
}

tval3_status tval3_solver_set_trace(tval3_solver s, const void* d_xstar) {
    return guard([&] {
        if (!s) arg_error(TVAL3_ERR_ARG, "Argument error: NULL solver!");
        with_solver(s, [&](auto& v) {
            if (d_xstar && v.L > 1) arg_error(TVAL3_ERR_UNSUPPORTED, "error trace of a multi-layer solver");
            v.xstar = d_xstar;
            if (v.gexec) cudaGraphExecDestroy(v.gexec);
            v.gexec = nullptr;
        });
    });
}

tval3_status tval3_solver_trace(tval3_solver s, double* host_err, int len) {
    return guard([&] {
        if (!s || !host_err) arg_error(TVAL3_ERR_ARG, "Argument error: NULL solver or buffer!");
        with_solver(s, [&](auto& v) { v.read_trace(host_err, len); });
    });
}

tval3_status tval3_solver_destroy(tval3_solver s) {
    return guard([&] { delete s; });
}

// ---------------------------------------------------------------------------
// stencils
// ---------------------------------------------------------------------------
tval3_status tval3_D_f32(int dim_y, int dim_x, int dim_z, const float* U, float* DU, void* stream) {
    return guard([&] {
        if (dim_y <= 0 || dim_x <= 0 || dim_z <= 0 || !U || !DU) arg_error(TVAL3_ERR_ARG, "Argument error: bad volume!");
        launch_D_plain<float>(dim_y, dim_x, dim_z, U, DU, (cudaStream_t)stream);
        TV3_CUDA(cudaGetLastError());
    });
}
tval3_status tval3_Dt_f32(int dim_y, int dim_x, int dim_z, const float* V, float* out, void* stream) {
    return guard([&] {
        if (dim_y <= 0 || dim_x <= 0 || dim_z <= 0 || !V || !out) arg_error(TVAL3_ERR_ARG, "Argument error: bad volume!");
        launch_Dt_plain<float>(dim_y, dim_x, dim_z, V, out, (cudaStream_t)stream);
        TV3_CUDA(cudaGetLastError());
    });
}
tval3_status tval3_D_f64(int dim_y, int dim_x, int dim_z, const double* U, double* DU, void* stream) {
    return guard([&] {
        if (dim_y <= 0 || dim_x <= 0 || dim_z <= 0 || !U || !DU) arg_error(TVAL3_ERR_ARG, "Argument error: bad volume!");
        launch_D_plain<double>(dim_y, dim_x, dim_z, U, DU, (cudaStream_t)stream);
        TV3_CUDA(cudaGetLastError());
    });
}
tval3_status tval3_Dt_f64(int dim_y, int dim_x, int dim_z, const double* V, double* out, void* stream) {
    return guard([&] {
        if (dim_y <= 0 || dim_x <= 0 || dim_z <= 0 || !V || !out) arg_error(TVAL3_ERR_ARG, "Argument error: bad volume!");
        launch_Dt_plain<double>(dim_y, dim_x, dim_z, V, out, (cudaStream_t)stream);
        TV3_CUDA(cudaGetLastError());
    });
}

tval3_status tval3_batch_create(tval3_batch* batch, const tval3_op* ops, const int* dims, int count,
                                const tval3_options* opts) {
    return guard([&] {
        if (!batch || !ops || !dims || count <= 0) arg_error(TVAL3_ERR_ARG, "Argument error: empty batch!");
        check_opts(opts);
        // 0: float vectors, 1: double, 2: double-float
        auto kind = [](tval3_op op) { return op->q ? 2 : (op->dbl ? 1 : 0); };
        for (int i = 0; i < count; ++i) {
            if (!ops[i]) arg_error(TVAL3_ERR_ARG, "Argument error: NULL operator in batch!");
            if (kind(ops[i]) != kind(ops[0]))
                arg_error(TVAL3_ERR_ARG, "Argument error: all operators of a batch must have the same vector type!");
            const int* d = dims + 3 * (long)i;
            const long n = (long)d[0] * d[1] * d[2];
            const long cols = ops[i]->cols();
            if (d[0] <= 0 || d[1] <= 0 || d[2] <= 0 || n != cols)
                arg_error(TVAL3_ERR_SHAPE, "Argument error: the length of U must be equal to A.dim_x!");
        }
        auto* h = new tval3_batch_s();
        try {
            auto fill = [&](auto*& bt, auto get) {
                using BT = std::remove_reference_t<decltype(*bt)>;
                using ST = std::remove_pointer_t<typename decltype(BT::s)::value_type>;
                bt = new BT();
                for (int i = 0; i < count; ++i) {
                    const int* d = dims + 3 * (long)i;
                    bt->s.push_back(nullptr);
                    bt->s.back() = new ST(get(ops[i]), d[0], d[1], d[2], *opts);
                }
            };
            if (kind(ops[0]) == 2) fill(h->q, [](tval3_op op) { return op->q; });
            else if (kind(ops[0]) == 1) fill(h->d, [](tval3_op op) { return op->d; });
            else fill(h->f, [](tval3_op op) { return op->f; });
        } catch (...) {
            delete h;
            throw;
        }
        *batch = h;
    });
}

tval3_status tval3_batch_solve(tval3_batch batch, const void* const* d_b, void* const* d_U, const void* const* d_Ut,
                               tval3_info* infos, void* stream) {
    return guard([&] {
        if (!batch || !d_b || !d_U) arg_error(TVAL3_ERR_ARG, "Argument error: NULL batch or vector list!");
        const size_t k = batch->q ? batch->q->s.size() : (batch->d ? batch->d->s.size() : batch->f->s.size());
        for (size_t i = 0; i < k; ++i)
            if (!d_b[i] || !d_U[i]) arg_error(TVAL3_ERR_ARG, "Argument error: NULL vector in batch!");
        std::vector<const void*> ut(k, nullptr);
        if (d_Ut) ut.assign(d_Ut, d_Ut + k);
        cudaStream_t st = (cudaStream_t)stream;
        if (batch->q) batch->q->solve(d_b, d_U, ut.data(), infos, st);
        else if (batch->d) batch->d->solve(d_b, d_U, ut.data(), infos, st);
        else batch->f->solve(d_b, d_U, ut.data(), infos, st);
    });
}

tval3_status tval3_batch_tuned_grid(tval3_batch batch, int64_t* elems_per_block) {
    return guard([&] {
        if (!batch || !elems_per_block) arg_error(TVAL3_ERR_ARG, "Argument error: batch or output is NULL!");
        *elems_per_block = batch->q ? batch->q->grid_elems : (batch->d ? batch->d->grid_elems : batch->f->grid_elems);
    });
}

tval3_status tval3_batch_destroy(tval3_batch batch) {
    return guard([&] { delete batch; });
}

tval3_status tval3_gpu_batched(const tval3_slice_host* slices, int count, const tval3_options* opts,
                               tval3_info* infos) {
    return guard([&] {
        auto t0 = entry_clock();
        if (!slices || count <= 0) arg_error(TVAL3_ERR_ARG, "Argument error: empty batch!");
        check_opts(opts);
        for (int i = 0; i < count; ++i) {
            const tval3_slice_host& sl = slices[i];
            if (!sl.A) arg_error(TVAL3_ERR_ARG, "Argument error: A is NULL!");
            check_sparse(sl.A, false);  // O(nnz) checks run in sparse_op
            check_problem(sl.U, sl.rows, sl.cols, 1, sl.A->rows, sl.A->cols, sl.b, sl.b_len, sl.Ut, sl.Ut_len);
        }
        std::vector<std::unique_ptr<LinOp<float>>> ops;
        std::vector<DBuf<float>> db(count), dU(count), dUt(count);
        std::vector<const void*> pb(count), put(count, nullptr);
        std::vector<void*> pU(count);
        Batch<float> bt;
        for (int i = 0; i < count; ++i) {
            const tval3_slice_host& sl = slices[i];
            const long n = (long)sl.rows * sl.cols;
            ops.emplace_back(sparse_op<float>(sl.A, TVAL3_PREC_FP32));
            db[i].alloc(std::max(sl.b_len, 1));
            dU[i].alloc(std::max<long>(n, 1));
            if (sl.b_len) TV3_CUDA(cudaMemcpy(db[i].p, sl.b, sl.b_len * sizeof(float), cudaMemcpyHostToDevice));
            if (sl.Ut && sl.Ut_len == n) {
                dUt[i].alloc(n);
                TV3_CUDA(cudaMemcpy(dUt[i].p, sl.Ut, n * sizeof(float), cudaMemcpyHostToDevice));
                put[i] = dUt[i].p;
            }
            pb[i] = db[i].p;
            pU[i] = dU[i].p;
            bt.s.push_back(new Solver<float>(ops.back().get(), sl.rows, sl.cols, 1, *opts));
        }
        std::vector<tval3_info> inf(count);
        bt.solve(pb.data(), pU.data(), put.data(), inf.data(), 0);
        for (int i = 0; i < count; ++i) {
            const tval3_slice_host& sl = slices[i];
            TV3_CUDA(cudaMemcpy(sl.U, dU[i].p, (size_t)sl.rows * sl.cols * sizeof(float), cudaMemcpyDeviceToHost));
        }
        const double secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
        for (int i = 0; i < count; ++i) {
            inf[i].outer_secs = secs;
            if (infos) infos[i] = inf[i];
        }
    });
}

tval3_status tval3_dense_rmatvec_f32_noalloc(int rows, int cols, const float* d_A, const float* d_y, float* d_x,
                                             void* stream) {
    return guard([&] { dense_rmatvec_noalloc_f32(rows, cols, d_A, d_y, d_x, (cudaStream_t)stream); });
}

}  // extern "C"
