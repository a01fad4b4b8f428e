// Dense operator (dense_mm, 3d/mat_vec_mul_dense.h:14-73; 2D
// 2d/mat_vec_mul.h:32-104): A is stored row-major (one ray per row) in FP32,
// FP64 or BF16 (with a per-row FP32 scale).  A*x: one warp per row with
// vectorised row loads; A^T*y: column tiles of 256 threads, each block sums a
// slab of rows and the slabs are added by a second pass (deterministic, no
// atomics).  Replaces cublasSgemv.
#include <algorithm>
#include <vector>
#include "dbuf.h"
#include "ops.h"
#include "tval3/tval3_c.h"

namespace tv3 {

template <class T, class V, int EPI>
__global__ void __launch_bounds__(256) k_dense_N(long m, long n, const V* __restrict__ A, const float* __restrict__ rs,
                                                 MatIO<T> io) {
    count_launch(io.ctl);
    const int lane = threadIdx.x & 31;
    const long w = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = ((long)gridDim.x * blockDim.x) >> 5;
    const int sel = io.by_parity ? io.ctl->parity : 0;
    const T* __restrict__ x = io.x[sel];
    T* __restrict__ y = io.y[sel];
    double acc0 = 0.0, acc1 = 0.0;
    for (long r = w; r < m; r += nw) {
        const V* row = A + r * n;
        T s = T(0);
        for (long c = lane; c < n; c += 32) s += (T)Acc<T, V>::load(row + c) * x[c];
        for (int o = 16; o; o >>= 1) s += __shfl_down_sync(FULL, s, o);
        if (lane == 0) {
            if (rs) s *= (T)rs[r];
            if (EPI == SPMV_PLAIN) y[r] = s;
            else if (EPI == SPMV_SUB) y[r] = s - io.sub[r];
            else if (EPI == SPMV_LAM35) {
                y[r] = s;
                double t = (double)s - (double)io.b[r];
                acc0 += t * t;
                acc1 += (double)io.delta[r] * t;
            } else if (EPI == SPMV_NORM2) {
                acc0 += (double)s * s;
            }
        }
    }
    if (EPI == SPMV_LAM35 || EPI == SPMV_NORM2) {
        double v[2] = {acc0, acc1}, tot[2];
        if (grid_reduce<2>(v, io.part, io.ticket, tot) && threadIdx.x == 0) {
            Ctl* c = io.ctl;
            if (EPI == SPMV_LAM35) {
                c->lam3 = tot[0];
                c->lam5 = tot[1];
            } else {
                c->Add = tot[0];
                c->tau = fabs(c->dd / (c->dDd + c->muDbeta * c->Add));
            }
        }
    }
}

// partial column sums over a slab of rows: part[slab][c] = sum_r A[r][c] * s_r y_r
template <class T, class V>
__global__ void __launch_bounds__(256) k_dense_T_part(long m, long n, long rows_per_slab, const V* __restrict__ A,
                                                      const float* __restrict__ rs, MatIO<T> io, T* __restrict__ part) {
    count_launch(io.ctl);
    const int sel = io.by_parity ? io.ctl->parity : 0;
    const T* __restrict__ yv = io.x[sel];
    const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
    const long slab = blockIdx.y;
    const long r0 = slab * rows_per_slab, r1 = min(m, r0 + rows_per_slab);
    if (c >= n) return;
    T s = T(0);
    for (long r = r0; r < r1; ++r) {
        T yr = yv[r];
        if (rs) yr *= (T)rs[r];
        s += (T)Acc<T, V>::load(A + r * n + c) * yr;
    }
    part[slab * n + c] = s;
}

template <class T>
__global__ void k_dense_T_sum(long n, int slabs, const T* __restrict__ part, MatIO<T> io, int sub) {
    count_launch(io.ctl);
    const int sel = io.by_parity ? io.ctl->parity : 0;
    T* __restrict__ out = io.y[sel];
    for (long c = (long)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (long)gridDim.x * blockDim.x) {
        T s = T(0);
        for (int k = 0; k < slabs; ++k) s += part[(long)k * n + c];
        out[c] = sub ? s - io.sub[c] : s;
    }
}

template <class T, class V>
struct DenseOp : LinOp<T> {
    DBuf<V> a;
    DBuf<float> rs;
    mutable DBuf<T> part;
    int slabs = 1;
    long rows_per_slab = 1;

    void apply(int trans, const MatIO<T>& io, int epi, cudaStream_t s) const override {
        const long m = this->m, n = this->n;
        if (!trans) {
            long g = std::min<long>((m * 32 + 255) / 256, (long)num_sms() * 8);
            int grid = (int)std::max<long>(g, 1);
            switch (epi) {
                case SPMV_SUB: k_dense_N<T, V, SPMV_SUB><<<grid, 256, 0, s>>>(m, n, a.p, rs.p, io); break;
                case SPMV_LAM35: k_dense_N<T, V, SPMV_LAM35><<<grid, 256, 0, s>>>(m, n, a.p, rs.p, io); break;
                case SPMV_NORM2: k_dense_N<T, V, SPMV_NORM2><<<grid, 256, 0, s>>>(m, n, a.p, rs.p, io); break;
                default: k_dense_N<T, V, SPMV_PLAIN><<<grid, 256, 0, s>>>(m, n, a.p, rs.p, io); break;
            }
        } else {
            dim3 grid((unsigned)((n + 255) / 256), (unsigned)slabs);
            k_dense_T_part<T, V><<<grid, 256, 0, s>>>(m, n, rows_per_slab, a.p, rs.p, io, part.p);
            long g = std::min<long>((n + 255) / 256, (long)num_sms() * 8);
            k_dense_T_sum<T><<<(int)std::max<long>(g, 1), 256, 0, s>>>(n, slabs, part.p, io, epi == SPMV_SUB);
        }
        TV3_CUDA(cudaGetLastError());
    }
};

template <class T> static __global__ void k_rowmax_dense(long m, long n, const float* A, float* rs) {
    const int lane = threadIdx.x & 31;
    for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < m; r += ((long)gridDim.x * blockDim.x) >> 5) {
        float mx = 0.f;
        for (long c = lane; c < n; c += 32) mx = fmaxf(mx, fabsf(A[r * n + c]));
        for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, o));
        if (lane == 0) rs[r] = mx > 0.f ? mx : 1.f;
    }
}

static __global__ void k_quant_dense(long m, long n, const float* A, const float* rs, __nv_bfloat16* q) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < m * n; i += (long)gridDim.x * blockDim.x)
        q[i] = __float2bfloat16_rn(A[i] / rs[i / n]);
}

template <class T, class V>
static void setup_slabs(DenseOp<T, V>* op) {
    // enough column-tile x slab blocks to cover the SMs several times
    const long tiles = (op->n + 255) / 256;
    long want = std::max<long>(1, (long)num_sms() * 8 / std::max<long>(tiles, 1));
    want = std::min<long>(want, std::max<long>(op->m, 1));
    op->slabs = (int)want;
    op->rows_per_slab = (op->m + want - 1) / want;
    op->part.alloc((size_t)op->slabs * std::max<long>(op->n, 1));
}

// host data (column- or row-major, FP32 or FP64) -> row-major host array of T
template <class T>
static std::vector<T> to_row_major(long m, long n, const void* h, int row_major, int val_type) {
    std::vector<T> out((size_t)m * n);
    for (long r = 0; r < m; ++r)
        for (long c = 0; c < n; ++c) {
            size_t src = row_major ? (size_t)r * n + c : (size_t)c * m + r;
            out[(size_t)r * n + c] = (val_type == TVAL3_PREC_FP64) ? (T)((const double*)h)[src] : (T)((const float*)h)[src];
        }
    return out;
}

template <>
LinOp<float>* make_dense_op<float>(long rows, long cols, const void* h, int row_major, int val_type, int precision,
                                   cudaStream_t s) {
    std::vector<float> rm = to_row_major<float>(rows, cols, h, row_major, val_type);
    if (precision == TVAL3_PREC_BF16) {
        auto* op = new DenseOp<float, __nv_bfloat16>();
        try {
            op->m = rows; op->n = cols; op->nnz = rows * cols; op->kind = 1;
            DBuf<float> tmp(std::max<size_t>(rm.size(), 1));
            TV3_CUDA(cudaMemcpy(tmp.p, rm.data(), rm.size() * sizeof(float), cudaMemcpyHostToDevice));
            op->rs.alloc(std::max<long>(rows, 1));
            op->a.alloc(std::max<size_t>(rm.size(), 1));
            k_rowmax_dense<float><<<std::max<long>(1, std::min<long>((rows * 32 + 255) / 256, 4096)), 256, 0, s>>>(rows, cols, tmp.p, op->rs.p);
            k_quant_dense<<<4096, 256, 0, s>>>(rows, cols, tmp.p, op->rs.p, op->a.p);
            TV3_CUDA(cudaGetLastError());
            TV3_CUDA(cudaStreamSynchronize(s));
            setup_slabs(op);
        } catch (...) {
            delete op;
            throw;
        }
        return op;
    }
    if (precision != TVAL3_PREC_FP32) throw Error{7, "dense FP32-vector operators store FP32 or BF16 values"};
    auto* op = new DenseOp<float, float>();
    try {
        op->m = rows; op->n = cols; op->nnz = rows * cols; op->kind = 1;
        op->a.alloc(std::max<size_t>(rm.size(), 1));
        TV3_CUDA(cudaMemcpy(op->a.p, rm.data(), rm.size() * sizeof(float), cudaMemcpyHostToDevice));
        setup_slabs(op);
    } catch (...) {
        delete op;
        throw;
    }
    return op;
}

template <>
LinOp<double>* make_dense_op<double>(long rows, long cols, const void* h, int row_major, int val_type, int,
                                     cudaStream_t) {
    std::vector<double> rm = to_row_major<double>(rows, cols, h, row_major, val_type);
    auto* op = new DenseOp<double, double>();
    try {
        op->m = rows; op->n = cols; op->nnz = rows * cols; op->kind = 1;
        op->a.alloc(std::max<size_t>(rm.size(), 1));
        TV3_CUDA(cudaMemcpy(op->a.p, rm.data(), rm.size() * sizeof(double), cudaMemcpyHostToDevice));
        setup_slabs(op);
    } catch (...) {
        delete op;
        throw;
    }
    return op;
}

}  // namespace tv3
