// tval3.hpp -- header-only C++ shim restoring the reference's interface
// (modk/tval3-gpu) on top of the C ABI in tval3_c.h.
//
//   tval3_gpu_3d(U, A, b, opts, Ut, pagelocked, mainGPU, numGPUs, gpuArray)
//       3d/tval3_gpu_3d.cpp:23-69 (sparse, dense, geometry, geometry+sparse;
//       float and double: all eight overloads)
//   tval3_gpu(U, A, b, opts, Ut, pagelocked)        2d/tval3_gpu.h:9-19
//   mat_host / sparse_mat_host / geometry_host      2d/container_host.h:25-127,
//                                                   3d/container_device.h:103-172
//   tval3_options / tval3_info                      2d/tval3_types.h:7-43
//   tval3_gpu_exception, illegal_mat_gpu_assignment, cuda_exception
//                                                   2d/tval3_types.h:45-49,
//                                                   2d/container_host.h:18-22,
//                                                   2d/handle_error.h:14-41
//   tval3::op::mat_vec_mul(trans, x, y, stream)     the mat_vec_mul interface
//
// Status codes from the C ABI are rethrown as the reference's exception
// types: argument and shape errors as tval3_gpu_exception, CUDA errors as
// "Internal error: ..." tval3_gpu_exception (3d/tval3_gpu_3d.cpp:1439-1445).
#ifndef TVAL3_HPP_
#define TVAL3_HPP_

#include <stddef.h>
#include <stdint.h>

#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

// The C ABI lives in namespace tval3c so that its plain structs do not clash
// with the reference's class templates tval3_options<T> / tval3_info<T>
// (the functions keep their C linkage).
namespace tval3c {
#include "tval3_c.h"
}

enum T_alloc { allocated_in_constructor, preallocated_buffer };
enum T_mat_format { mat_col_major, mat_row_major };
enum T_sparse_mat_format { sparse_mat_csc, sparse_mat_csr, sparse_mat_both };

class illegal_mat_gpu_assignment : public std::runtime_error {
   public:
    explicit illegal_mat_gpu_assignment(const std::string& m) : std::runtime_error(m) {}
};
class tval3_gpu_exception : public std::runtime_error {
   public:
    explicit tval3_gpu_exception(const std::string& m) : std::runtime_error(m) {}
};
class cuda_exception : public std::runtime_error {
   public:
    explicit cuda_exception(const std::string& m) : std::runtime_error(m) {}
};

namespace tval3 {
inline void check(tval3c::tval3_status st) {
    if (st == tval3c::TVAL3_OK) return;
    std::string msg = tval3c::tval3_last_error_message();
    if (st == tval3c::TVAL3_ERR_CUDA || st == tval3c::TVAL3_ERR_NOMEM || st == tval3c::TVAL3_ERR_TIMEOUT)
        throw tval3_gpu_exception("Internal error: " + msg);
    throw tval3_gpu_exception(msg);
}
}  // namespace tval3

template <class Type>
struct tval3_options {
    Type mu, mu0, beta, beta0, rate_cnt, tol, tol_inn;
    int maxcnt, maxit;
    Type c, gamma, gam, rate_gam;
    bool isreal, nonneg;
    unsigned int numInitIterations;
    Type skipMulRatio, maxRelativeChange;
    tval3c::tval3_tv tv_type;
    tval3_options()
        : mu(256), mu0(256), beta(32), beta0(32), rate_cnt(2), tol(1e-6), tol_inn(1e-3), maxcnt(10), maxit(1025),
          c(1e-5), gamma(0.6), gam(0.9995), rate_gam(0.9), isreal(true), nonneg(true), numInitIterations(0),
          skipMulRatio(0), maxRelativeChange(0), tv_type(tval3c::TVAL3_TV_ANISO) {}
    tval3c::tval3_options to_c() const;
};

template <class Type>
struct tval3_info {
    int total_iters;
    int outer_iters;
    Type rel_chg;
    Type rel_error;
    double secs;
    double outer_secs;
};

template <class Type>
tval3c::tval3_options tval3_options<Type>::to_c() const {
    tval3c::tval3_options o;
    tval3c::tval3_options_default(&o);
    o.mu = mu; o.mu0 = mu0; o.beta = beta; o.beta0 = beta0; o.rate_cnt = rate_cnt; o.tol = tol;
    o.tol_inn = tol_inn; o.maxcnt = maxcnt; o.maxit = maxit; o.c = c; o.gamma = gamma; o.gam = gam;
    o.rate_gam = rate_gam; o.isreal = isreal; o.nonneg = nonneg; o.numInitIterations = numInitIterations;
    o.skipMulRatio = skipMulRatio; o.maxRelativeChange = maxRelativeChange; o.tv_type = tv_type;
    return o;
}

// Host matrix / volume, column-major (y fastest).  Owning or borrowing.
template <class Type>
class mat_host {
   public:
    const int dim_y, dim_x, dim_z, len;
    const T_mat_format format;
    mat_host(int num_elements, bool init = true, bool = false)
        : dim_y(num_elements), dim_x(1), dim_z(1), len(num_elements), format(mat_col_major),
          own_(num_elements > 0 ? num_elements : 0), buf_(own_.data()) {
        if (!init && len) std::memset(buf_, 0, sizeof(Type) * len);
    }
    mat_host(int ny, int nx, T_mat_format storage = mat_col_major, bool = true, bool = false)
        : dim_y(ny), dim_x(nx), dim_z(1), len(ny * nx), format(storage), own_(ny * nx), buf_(own_.data()) {}
    mat_host(int ny, int nx, int nz, bool = true, bool = false)
        : dim_y(ny), dim_x(nx), dim_z(nz), len(ny * nx * nz), format(mat_col_major), own_(ny * nx * nz),
          buf_(own_.data()) {}
    mat_host(int ny, int nx, int nz, Type* buffer)
        : dim_y(ny), dim_x(nx), dim_z(nz), len(ny * nx * nz), format(mat_col_major), buf_(buffer) {}
    mat_host(int num_elements, Type* buffer)
        : dim_y(num_elements), dim_x(1), dim_z(1), len(num_elements), format(mat_col_major), buf_(buffer) {}
    mat_host(const mat_host& m)
        : dim_y(m.dim_y), dim_x(m.dim_x), dim_z(m.dim_z), len(m.len), format(m.format), own_(m.buf_, m.buf_ + m.len),
          buf_(own_.data()) {}
    mat_host& operator=(const mat_host& m) {
        if (m.len != len) throw illegal_mat_gpu_assignment("illegal assignment of mat_host objects");
        std::memcpy(buf_, m.buf_, sizeof(Type) * len);
        return *this;
    }
    Type* data() { return buf_; }
    const Type* data() const { return buf_; }
    Type& operator[](int i) { return buf_[i]; }
    const Type& operator[](int i) const { return buf_[i]; }
    int rows() const { return dim_y; }
    int cols() const { return dim_x * dim_z; }

   private:
    std::vector<Type> own_;
    Type* buf_;
};

// Host sparse matrix A (dim_y = rows = measurements, dim_x = cols = voxels)
// in CSR and/or CSC; the arrays are borrowed.
template <class Type>
class sparse_mat_host {
   public:
    const int dim_y, dim_x, nnz;
    const T_sparse_mat_format format;
    const Type *csr_val, *csc_val;
    const int *csr_ptr, *csr_ind, *csc_ptr, *csc_ind;
    sparse_mat_host(int rows, int cols, int n_nonzero, const Type* csr_v, const int* csr_p, const int* csr_i,
                    const Type* csc_v, const int* csc_p, const int* csc_i)
        : dim_y(rows), dim_x(cols), nnz(n_nonzero),
          format(csr_v && csc_v ? sparse_mat_both : (csr_v ? sparse_mat_csr : sparse_mat_csc)),
          csr_val(csr_v), csc_val(csc_v), csr_ptr(csr_p), csr_ind(csr_i), csc_ptr(csc_p), csc_ind(csc_i) {}
    tval3c::tval3_sparse_host to_c() const {
        using namespace tval3c;
        tval3_sparse_host s;
        s.rows = dim_y; s.cols = dim_x; s.nnz = nnz;
        s.format = (format == sparse_mat_both) ? TVAL3_SPARSE_BOTH
                                               : (format == sparse_mat_csr ? TVAL3_SPARSE_CSR : TVAL3_SPARSE_CSC);
        s.val_type = sizeof(Type) == 8 ? TVAL3_PREC_FP64 : TVAL3_PREC_FP32;
        s.csr_ptr = csr_ptr; s.csr_ind = csr_ind; s.csr_val = csr_val;
        s.csc_ptr = csc_ptr; s.csc_ind = csc_ind; s.csc_val = csc_val;
        return s;
    }
};

// Measurement geometry (fields of geometry_host read by geometry_device,
// 3d/container_device.h:683-750); arrays are borrowed.
struct geometry_host : tval3c::tval3_geometry_host {
    geometry_host() {
        std::memset(static_cast<tval3c::tval3_geometry_host*>(this), 0, sizeof(tval3c::tval3_geometry_host));
        numMPs = 1;
        scale_factor = 1.f;
    }
};

namespace tval3 {
template <class Type>
tval3_info<Type> to_info(const tval3c::tval3_info& i) {
    tval3_info<Type> r;
    r.total_iters = i.total_iters; r.outer_iters = i.outer_iters;
    r.rel_chg = (Type)i.rel_chg; r.rel_error = (Type)i.rel_error;
    r.secs = i.secs; r.outer_secs = i.outer_secs;
    return r;
}
inline const float* ut_ptr(const mat_host<float>* Ut) { return Ut ? Ut->data() : nullptr; }
}  // namespace tval3

// ---------------------------------------------------------------------------
// the reference overloads
// ---------------------------------------------------------------------------
inline const tval3_info<float> tval3_gpu_3d(mat_host<float>& U, const sparse_mat_host<float>& A,
                                            const mat_host<float>& b, const tval3_options<float>& opts,
                                            const mat_host<float>& Ut, bool pagelocked = true, int mainGPU = -1,
                                            int numGPUs = 0, int* gpuArray = nullptr) {
    tval3c::tval3_sparse_host a = A.to_c();
    tval3c::tval3_options o = opts.to_c();
    tval3c::tval3_info i;
    tval3::check(tval3c::tval3_gpu_3d_sparse_f32(U.data(), U.dim_y, U.dim_x, U.dim_z, &a, b.data(), b.len, &o, Ut.data(),
                                         Ut.len, pagelocked, mainGPU, numGPUs, gpuArray, &i));
    return tval3::to_info<float>(i);
}

inline const tval3_info<double> tval3_gpu_3d(mat_host<double>& U, const sparse_mat_host<double>& A,
                                             const mat_host<double>& b, const tval3_options<double>& opts,
                                             const mat_host<double>& Ut, bool pagelocked = true, int mainGPU = -1,
                                             int numGPUs = 0, int* gpuArray = nullptr) {
    tval3c::tval3_sparse_host a = A.to_c();
    tval3c::tval3_options o = opts.to_c();
    tval3c::tval3_info i;
    tval3::check(tval3c::tval3_gpu_3d_sparse_f64(U.data(), U.dim_y, U.dim_x, U.dim_z, &a, b.data(), b.len, &o, Ut.data(),
                                         Ut.len, pagelocked, mainGPU, numGPUs, gpuArray, &i));
    return tval3::to_info<double>(i);
}

inline const tval3_info<float> tval3_gpu_3d(mat_host<float>& U, const mat_host<float>& A, const mat_host<float>& b,
                                            const tval3_options<float>& opts, const mat_host<float>& Ut,
                                            bool pagelocked = true, int mainGPU = -1, int numGPUs = 0,
                                            int* gpuArray = nullptr) {
    if (A.format != mat_col_major) throw tval3_gpu_exception("Argument error: A must be in column major format!");
    tval3c::tval3_dense_host a{A.dim_y, A.dim_x * A.dim_z, 0, tval3c::TVAL3_PREC_FP32, A.data()};
    tval3c::tval3_options o = opts.to_c();
    tval3c::tval3_info i;
    tval3::check(tval3c::tval3_gpu_3d_dense_f32(U.data(), U.dim_y, U.dim_x, U.dim_z, &a, b.data(), b.len, &o, Ut.data(),
                                        Ut.len, pagelocked, mainGPU, numGPUs, gpuArray, &i));
    return tval3::to_info<float>(i);
}

inline const tval3_info<double> tval3_gpu_3d(mat_host<double>& U, const mat_host<double>& A,
                                             const mat_host<double>& b, const tval3_options<double>& opts,
                                             const mat_host<double>& Ut, bool pagelocked = true, int mainGPU = -1,
                                             int numGPUs = 0, int* gpuArray = nullptr) {
    if (A.format != mat_col_major) throw tval3_gpu_exception("Argument error: A must be in column major format!");
    tval3c::tval3_dense_host a{A.dim_y, A.dim_x * A.dim_z, 0, tval3c::TVAL3_PREC_FP64, A.data()};
    tval3c::tval3_options o = opts.to_c();
    tval3c::tval3_info i;
    tval3::check(tval3c::tval3_gpu_3d_dense_f64(U.data(), U.dim_y, U.dim_x, U.dim_z, &a, b.data(), b.len, &o, Ut.data(),
                                        Ut.len, pagelocked, mainGPU, numGPUs, gpuArray, &i));
    return tval3::to_info<double>(i);
}

inline const tval3_info<float> tval3_gpu_3d(mat_host<float>& U, const geometry_host& A, const mat_host<float>& b,
                                            const tval3_options<float>& opts, const mat_host<float>& Ut,
                                            bool pagelocked = true, int mainGPU = -1, int numGPUs = 0,
                                            int* gpuArray = nullptr) {
    tval3c::tval3_options o = opts.to_c();
    tval3c::tval3_info i;
    tval3::check(tval3c::tval3_gpu_3d_geometry_f32(U.data(), U.dim_y, U.dim_x, U.dim_z, &A, b.data(), b.len, &o, Ut.data(),
                                           Ut.len, pagelocked, mainGPU, numGPUs, gpuArray, &i));
    return tval3::to_info<float>(i);
}

inline const tval3_info<float> tval3_gpu_3d(mat_host<float>& U, const geometry_host& A_geo,
                                            sparse_mat_host<float>& A_mat, const mat_host<float>& b,
                                            const tval3_options<float>& opts, const mat_host<float>& Ut,
                                            bool pagelocked = true, int mainGPU = -1, int numGPUs = 0,
                                            int* gpuArray = nullptr) {
    tval3c::tval3_sparse_host a = A_mat.to_c();
    tval3c::tval3_options o = opts.to_c();
    tval3c::tval3_info i;
    tval3::check(tval3c::tval3_gpu_3d_geometry_sparse_f32(U.data(), U.dim_y, U.dim_x, U.dim_z, &A_geo, &a, b.data(), b.len,
                                                  &o, Ut.data(), Ut.len, pagelocked, mainGPU, numGPUs, gpuArray, &i));
    return tval3::to_info<float>(i);
}

inline const tval3_info<double> tval3_gpu_3d(mat_host<double>& U, const geometry_host& A, const mat_host<double>& b,
                                             const tval3_options<double>& opts, const mat_host<double>& Ut,
                                             bool pagelocked = true, int mainGPU = -1, int numGPUs = 0,
                                             int* gpuArray = nullptr) {
    tval3c::tval3_options o = opts.to_c();
    tval3c::tval3_info i;
    tval3::check(tval3c::tval3_gpu_3d_geometry_f64(U.data(), U.dim_y, U.dim_x, U.dim_z, &A, b.data(), b.len, &o,
                                                   Ut.data(), Ut.len, pagelocked, mainGPU, numGPUs, gpuArray, &i));
    return tval3::to_info<double>(i);
}

inline const tval3_info<double> tval3_gpu_3d(mat_host<double>& U, const geometry_host& A_geo,
                                             sparse_mat_host<double>& A_mat, const mat_host<double>& b,
                                             const tval3_options<double>& opts, const mat_host<double>& Ut,
                                             bool pagelocked = true, int mainGPU = -1, int numGPUs = 0,
                                             int* gpuArray = nullptr) {
    tval3c::tval3_sparse_host a = A_mat.to_c();
    tval3c::tval3_options o = opts.to_c();
    tval3c::tval3_info i;
    tval3::check(tval3c::tval3_gpu_3d_geometry_sparse_f64(U.data(), U.dim_y, U.dim_x, U.dim_z, &A_geo, &a, b.data(),
                                                          b.len, &o, Ut.data(), Ut.len, pagelocked, mainGPU, numGPUs,
                                                          gpuArray, &i));
    return tval3::to_info<double>(i);
}

// 2D (2d/tval3_gpu.h:9-19): U is rows x cols.  The 2D reference's untemplated
// containers are in tval3_2d.hpp; these overloads take the 3D templates.
inline const tval3_info<float> tval3_gpu(mat_host<float>& U, const sparse_mat_host<float>& A,
                                         const mat_host<float>& b, const tval3_options<float>& opts,
                                         const mat_host<float>* Ut = nullptr, bool pagelocked = true) {
    tval3c::tval3_sparse_host a = A.to_c();
    tval3c::tval3_options o = opts.to_c();
    tval3c::tval3_info i;
    tval3::check(tval3c::tval3_gpu_sparse(U.data(), U.dim_y, U.dim_x * U.dim_z, &a, b.data(), b.len, &o,
                                  tval3::ut_ptr(Ut), Ut ? Ut->len : 0, pagelocked, &i));
    return tval3::to_info<float>(i);
}

inline const tval3_info<float> tval3_gpu(mat_host<float>& U, const mat_host<float>& A, const mat_host<float>& b,
                                         const tval3_options<float>& opts, const mat_host<float>* Ut = nullptr,
                                         bool pagelocked = true) {
    tval3c::tval3_dense_host a{A.dim_y, A.dim_x * A.dim_z, A.format == mat_row_major ? 1 : 0, tval3c::TVAL3_PREC_FP32,
                               A.data()};
    tval3c::tval3_options o = opts.to_c();
    tval3c::tval3_info i;
    tval3::check(tval3c::tval3_gpu_dense(U.data(), U.dim_y, U.dim_x * U.dim_z, &a, b.data(), b.len, &o, tval3::ut_ptr(Ut),
                                 Ut ? Ut->len : 0, pagelocked, &i));
    return tval3::to_info<float>(i);
}

// ---------------------------------------------------------------------------
// the mat_vec_mul interface on device data
// ---------------------------------------------------------------------------
namespace tval3 {
class op {
   public:
    template <class Type>
    explicit op(const sparse_mat_host<Type>& A, tval3c::tval3_precision p = tval3c::TVAL3_PREC_FP32) {
        tval3c::tval3_sparse_host a = A.to_c();
        check(tval3c::tval3_op_create_sparse(&h_, &a, p));
    }
    explicit op(const geometry_host& G, int mode = 0, tval3c::tval3_precision p = tval3c::TVAL3_PREC_FP32) {
        check(tval3c::tval3_op_create_geometry(&h_, &G, mode, p));
    }
    ~op() {
        if (h_) tval3c::tval3_op_destroy(h_);
    }
    op(const op&) = delete;
    op& operator=(const op&) = delete;
    // y = A x (trans = false) or y = A^T x; device pointers
    void mat_vec_mul(bool trans, const void* x, void* y, void* stream = nullptr) const {
        check(tval3c::tval3_mat_vec_mul(h_, trans ? tval3c::TVAL3_OP_T : tval3c::TVAL3_OP_N, x, y, stream));
    }
    tval3c::tval3_op handle() const { return h_; }

   private:
    tval3c::tval3_op h_ = nullptr;
};
}  // namespace tval3

#endif  // TVAL3_HPP_
