// tval3_2d.hpp -- header-only C++ shim restoring the reference's 2D interface
// (modk/tval3-gpu, directory 2d/) on top of the C ABI in tval3_c.h.
//
//   tval3_gpu(U, A, b, opts, Ut = 0, pagelocked = true)  2d/tval3_gpu.h:9-19
//   mat_host, sparse_mat_host (untemplated, float)        2d/container_host.h:11-127
//   tval3_options, tval3_info, tval3_gpu_exception        2d/tval3_types.h:7-49
//   illegal_mat_gpu_assignment                            2d/container_host.h:18-22
//
// The 2D reference is a project of its own whose containers share their names
// with the 3D class templates of tval3.hpp, so, as there, a translation unit
// includes either this header or tval3.hpp, not both.
//
// Containers hold ordinary host memory: the page-locked flag and the
// allocation flags are accepted and stored for interface compatibility (the
// library copies host arrays itself).  b may hold `layers` columns
// (b.len = A.rows * layers, 2d/tval3.cu:1406-1426); U then holds
// A.cols * layers values, one image per column, solved jointly.
//
// Status codes of the C ABI are rethrown as tval3_gpu_exception (argument and
// shape errors with the library's message, CUDA errors as "Internal error: ...").
#ifndef TVAL3_2D_HPP_
#define TVAL3_2D_HPP_

#include <stddef.h>
#include <stdint.h>

#include <cstdlib>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

namespace tval3c {
#include "tval3_c.h"
}

enum T_alloc { allocated_in_constructor, preallocated_buffer };
enum T_mat_format { mat_col_major, mat_row_major };
enum T_sparse_mat_format { sparse_mat_csc, sparse_mat_csr };

class illegal_mat_gpu_assignment : public std::runtime_error {
   public:
    illegal_mat_gpu_assignment(const std::string& message) : std::runtime_error(message) {}
};

class tval3_gpu_exception : public std::runtime_error {
   public:
    tval3_gpu_exception(const std::string& message) : std::runtime_error(message) {}
};

// Options of the 2D reference: float fields, the reference's defaults.
struct tval3_options {
    float mu, mu0, beta, beta0, rate_cnt, tol, tol_inn;
    int maxcnt, maxit;
    float c, gamma, gam, rate_gam;
    bool isreal, nonneg;
    tval3_options()
        : mu(256.0f), mu0(256.0f), beta(32.0f), beta0(32.0f), rate_cnt(2.0f), tol(1e-6f), tol_inn(1e-3f), maxcnt(10),
          maxit(1025), c(1e-5f), gamma(0.6f), gam(0.9995f), rate_gam(0.9f), isreal(true), nonneg(true) {}
};

struct tval3_info {
    int total_iters;
    int outer_iters;
    float rel_chg;
    float rel_error;
    double secs;
};

// Host matrix, column-major unless constructed with mat_row_major; owning
// (allocated here, zero-filled) or borrowing a caller's buffer.  mat_host(0)
// is the empty matrix the entry points take as "no true image".
class mat_host {
   private:
    std::vector<float> own_;
    float* pbuf;
    T_alloc alloc_info;

   public:
    const int rows;
    const int cols;
    const int len;
    const T_mat_format format;
    const bool pagelocked;
    const unsigned int alloc_flags;

    mat_host(int num_rows, int num_cols, T_mat_format storage = mat_col_major, bool init = true,
             bool mem_pagelocked = false, unsigned int flags = 0u)
        : own_(num_rows > 0 && num_cols > 0 ? (size_t)num_rows * num_cols : 0), pbuf(own_.data()),
          alloc_info(allocated_in_constructor), rows(num_rows), cols(num_cols), len(num_rows * num_cols),
          format(storage), pagelocked(mem_pagelocked), alloc_flags(flags) {
        (void)init;
    }
    mat_host(int num_elements, bool init = true, bool mem_pagelocked = false, unsigned int flags = 0u)
        : own_(num_elements > 0 ? (size_t)num_elements : 0), pbuf(own_.data()), alloc_info(allocated_in_constructor),
          rows(num_elements), cols(1), len(num_elements), format(mat_col_major), pagelocked(mem_pagelocked),
          alloc_flags(flags) {
        (void)init;
    }
    mat_host(int num_rows, int num_cols, float* buffer, T_mat_format storage = mat_col_major,
             bool mem_pagelocked = false, unsigned int flags = 0u)
        : pbuf(buffer), alloc_info(preallocated_buffer), rows(num_rows), cols(num_cols), len(num_rows * num_cols),
          format(storage), pagelocked(mem_pagelocked), alloc_flags(flags) {}
    mat_host(int num_elements, float* buffer, bool mem_pagelocked = false, unsigned int flags = 0u)
        : pbuf(buffer), alloc_info(preallocated_buffer), rows(num_elements), cols(1), len(num_elements),
          format(mat_col_major), pagelocked(mem_pagelocked), alloc_flags(flags) {}
    mat_host(const mat_host& m)
        : own_(m.pbuf, m.pbuf + m.len), pbuf(own_.data()), alloc_info(allocated_in_constructor), rows(m.rows),
          cols(m.cols), len(m.len), format(m.format), pagelocked(m.pagelocked), alloc_flags(m.alloc_flags) {}

    float* data() { return pbuf; }
    const float* data() const { return pbuf; }
    float& operator[](int i) { return pbuf[i]; }
    const float& operator[](int i) const { return pbuf[i]; }

    mat_host& operator=(const mat_host& m) {
        if (m.rows != rows || m.cols != cols || m.format != format)
            throw illegal_mat_gpu_assignment("Illegal assignment: dimension or format mismatch");
        if (len) std::memcpy(pbuf, m.pbuf, sizeof(float) * len);
        return *this;
    }

    // uniform random values in [0, scl) (host rand(), as a test helper)
    void randomFill(float scl) {
        for (int i = 0; i < len; ++i) pbuf[i] = scl * (float)std::rand() / ((float)RAND_MAX + 1.0f);
    }
};

// Host sparse matrix A (rows = measurements, cols = pixels) in ONE format:
// sparse_mat_csr (ptr has rows + 1 entries, ind holds column indices) or
// sparse_mat_csc (ptr has cols + 1 entries, ind holds row indices; the
// reference's default).  Owning or borrowing.
class sparse_mat_host {
   private:
    std::vector<int> own_ptr_, own_ind_;
    std::vector<float> own_val_;
    int* p_ptr;
    int* p_ind;
    float* p_val;
    T_alloc alloc_info;

   public:
    const int rows;
    const int cols;
    const int nnz;
    const T_sparse_mat_format format;
    const bool pagelocked;
    const unsigned int alloc_flags;

    sparse_mat_host(int num_rows, int num_cols, int n_nonzero, T_sparse_mat_format storage_format = sparse_mat_csc,
                    bool init = true, bool mem_pagelocked = false, unsigned int flags = 0u)
        : own_ptr_((storage_format == sparse_mat_csr ? num_rows : num_cols) + 1),
          own_ind_(n_nonzero > 0 ? n_nonzero : 0), own_val_(n_nonzero > 0 ? n_nonzero : 0), p_ptr(own_ptr_.data()),
          p_ind(own_ind_.data()), p_val(own_val_.data()), alloc_info(allocated_in_constructor), rows(num_rows),
          cols(num_cols), nnz(n_nonzero), format(storage_format), pagelocked(mem_pagelocked), alloc_flags(flags) {
        (void)init;
    }
    sparse_mat_host(int num_rows, int num_cols, int n_nonzero, float* buff_val, int* buff_ptr, int* buff_ind,
                    T_sparse_mat_format storage_format = sparse_mat_csc, bool mem_pagelocked = false,
                    unsigned int flags = 0u)
        : p_ptr(buff_ptr), p_ind(buff_ind), p_val(buff_val), alloc_info(preallocated_buffer), rows(num_rows),
          cols(num_cols), nnz(n_nonzero), format(storage_format), pagelocked(mem_pagelocked), alloc_flags(flags) {}
    sparse_mat_host(const sparse_mat_host& m)
        : own_ptr_(m.p_ptr, m.p_ptr + ((m.format == sparse_mat_csr ? m.rows : m.cols) + 1)),
          own_ind_(m.p_ind, m.p_ind + m.nnz), own_val_(m.p_val, m.p_val + m.nnz), p_ptr(own_ptr_.data()),
          p_ind(own_ind_.data()), p_val(own_val_.data()), alloc_info(allocated_in_constructor), rows(m.rows),
          cols(m.cols), nnz(m.nnz), format(m.format), pagelocked(m.pagelocked), alloc_flags(m.alloc_flags) {}

    float* val() { return p_val; }
    const float* val() const { return p_val; }
    int* ptr() { return p_ptr; }
    const int* ptr() const { return p_ptr; }
    int* ind() { return p_ind; }
    const int* ind() const { return p_ind; }

    sparse_mat_host& operator=(const sparse_mat_host& m) {
        if (m.rows != rows || m.cols != cols || m.nnz != nnz || m.format != format)
            throw illegal_mat_gpu_assignment("Illegal assignment: dimension or format mismatch");
        std::memcpy(p_ptr, m.p_ptr, sizeof(int) * ((format == sparse_mat_csr ? rows : cols) + 1));
        if (nnz) {
            std::memcpy(p_ind, m.p_ind, sizeof(int) * nnz);
            std::memcpy(p_val, m.p_val, sizeof(float) * nnz);
        }
        return *this;
    }
};

namespace tval3_2d_detail {
inline void check(tval3c::tval3_status st) {
    if (st == tval3c::TVAL3_OK) return;
    std::string msg = tval3c::tval3_last_error_message();
    if (st == tval3c::TVAL3_ERR_CUDA || st == tval3c::TVAL3_ERR_NOMEM || st == tval3c::TVAL3_ERR_TIMEOUT)
        throw tval3_gpu_exception("Internal error: " + msg);
    throw tval3_gpu_exception(msg);
}
inline tval3c::tval3_options to_c(const tval3_options& opts) {
    tval3c::tval3_options o;
    tval3c::tval3_options_default(&o);
    o.mu = opts.mu; o.mu0 = opts.mu0; o.beta = opts.beta; o.beta0 = opts.beta0; o.rate_cnt = opts.rate_cnt;
    o.tol = opts.tol; o.tol_inn = opts.tol_inn; o.maxcnt = opts.maxcnt; o.maxit = opts.maxit; o.c = opts.c;
    o.gamma = opts.gamma; o.gam = opts.gam; o.rate_gam = opts.rate_gam; o.isreal = opts.isreal;
    o.nonneg = opts.nonneg;
    return o;
}
inline tval3_info from_c(const tval3c::tval3_info& i) {
    tval3_info r;
    r.total_iters = i.total_iters;
    r.outer_iters = i.outer_iters;
    r.rel_chg = (float)i.rel_chg;
    r.rel_error = (float)i.rel_error;
    r.secs = i.secs;
    return r;
}
}  // namespace tval3_2d_detail

// tval3_gpu(U, sparse A, b, opts, Ut, pagelocked), 2d/tval3_gpu.h:9-13.
// U is a rows x cols image (column-major, rows fastest).
inline const tval3_info tval3_gpu(mat_host& U, const sparse_mat_host& A, const mat_host& b,
                                  const tval3_options& opts, const mat_host& Ut = 0, bool pagelocked = true) {
    using namespace tval3c;
    tval3_sparse_host a;
    std::memset(&a, 0, sizeof(a));
    a.rows = A.rows;
    a.cols = A.cols;
    a.nnz = A.nnz;
    a.val_type = TVAL3_PREC_FP32;
    if (A.format == sparse_mat_csr) {
        a.format = TVAL3_SPARSE_CSR;
        a.csr_ptr = A.ptr(); a.csr_ind = A.ind(); a.csr_val = A.val();
    } else {
        a.format = TVAL3_SPARSE_CSC;
        a.csc_ptr = A.ptr(); a.csc_ind = A.ind(); a.csc_val = A.val();
    }
    tval3c::tval3_options o = tval3_2d_detail::to_c(opts);
    tval3c::tval3_info i;
    tval3_2d_detail::check(tval3c::tval3_gpu_sparse(U.data(), U.rows, U.cols, &a, b.data(), b.len, &o,
                                                    Ut.len ? Ut.data() : nullptr, Ut.len, pagelocked, &i));
    return tval3_2d_detail::from_c(i);
}

// tval3_gpu(U, dense A, b, opts, Ut, pagelocked), 2d/tval3_gpu.h:15-19.
inline const tval3_info tval3_gpu(mat_host& U, const mat_host& A, const mat_host& b, const tval3_options& opts,
                                  const mat_host& Ut = 0, bool pagelocked = true) {
    tval3c::tval3_dense_host a;
    a.rows = A.rows;
    a.cols = A.cols;
    a.row_major = A.format == mat_row_major ? 1 : 0;
    a.val_type = tval3c::TVAL3_PREC_FP32;
    a.data = A.data();
    tval3c::tval3_options o = tval3_2d_detail::to_c(opts);
    tval3c::tval3_info i;
    tval3_2d_detail::check(tval3c::tval3_gpu_dense(U.data(), U.rows, U.cols, &a, b.data(), b.len, &o,
                                                   Ut.len ? Ut.data() : nullptr, Ut.len, pagelocked, &i));
    return tval3_2d_detail::from_c(i);
}

#endif  // TVAL3_2D_HPP_
