// Dense operator (dense_mm, 3d/mat_vec_mul_dense.h:14-73; 2D
// 2d/mat_vec_mul.h:32-104): A is stored row-major (one ray per row) in FP32,
// FP64 or BF16 (with a per-row FP32 scale).  A*x: one warp per row with
// vectorised row loads; A^T*y: column tiles of 256 threads, each block sums a
// slab of rows and the slabs are added by a second pass (deterministic, no
// atomics).  Replaces cublasSgemv.
#include <algorithm>
#include <type_traits>
#include <vector>
#include "dbuf.h"
#include "ops.h"
#include "tval3/tval3_c.h"

namespace tv3 {

// tensor-core multi-RHS products of BF16 operators (dense_tc.cu)
struct UmmaPlan;
bool umma_supported(long m, long n, int L);
UmmaPlan* umma_plan_create(long m, long n, int L, const __nv_bfloat16* Aq);
void umma_plan_destroy(UmmaPlan* p);
void umma_apply(const UmmaPlan* p, int trans, const MatIO<float>& io, int epi, const float* rs, cudaStream_t s);
int umma_take_error(const UmmaPlan* p, cudaStream_t s);

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
                lam35_post(c);
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

// Multi-RHS forms (L > 1, vectors interleaved: element (row, layer) at
// row * L + layer; the reference's cublasSgemm with `layers` columns,
// 2d/mat_vec_mul.h:91-99).  A*X: one warp per row, each lane a strided part
// of the row for up to 32 layers, then a warp reduction per layer.  A^T*Y:
// one warp per (column, layer chunk of 32) over a slab of rows, lanes =
// layers, slab partials added in a fixed order.
template <class T, class V, int EPI>
__global__ void __launch_bounds__(256) k_dense_NL(long m, long n, int L, const V* __restrict__ A,
                                                  const float* __restrict__ rs, MatIO<T> io) {
    count_launch(io.ctl);
    const int lane = threadIdx.x & 31;
    const long w = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5, nw = ((long)gridDim.x * blockDim.x) >> 5;
    const int sel = io.by_parity ? io.ctl->parity : 0;
    const T* __restrict__ x = io.x[sel];
    T* __restrict__ y = io.y[sel];
    double acc0 = 0.0, acc1 = 0.0;
    for (long r = w; r < m; r += nw) {
        const V* row = A + r * n;
        for (int l0 = 0; l0 < L; l0 += 32) {
            const int nl = min(32, L - l0);
            T s[32];
#pragma unroll
            for (int j = 0; j < 32; ++j) s[j] = T(0);
            for (long c = lane; c < n; c += 32) {
                const T a = (T)Acc<T, V>::load(row + c);
                const T* xc = x + c * L + l0;
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (j < nl) s[j] += a * xc[j];
            }
            // lane j ends with the row sum of layer l0 + j
            T mine = T(0);
#pragma unroll
            for (int j = 0; j < 32; ++j) {
                T v = s[j];
                for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
                if (lane == j) mine = v;
            }
            if (lane < nl) {
                if (rs) mine *= (T)rs[r];
                const long o = r * L + l0 + lane;
                if (EPI == SPMV_PLAIN) y[o] = mine;
                else if (EPI == SPMV_SUB) y[o] = mine - io.sub[o];
                else if (EPI == SPMV_LAM35) {
                    y[o] = mine;
                    double t = (double)mine - (double)io.b[o];
                    acc0 += t * t;
                    acc1 += (double)io.delta[o] * t;
                } else if (EPI == SPMV_NORM2) {
                    acc0 += (double)mine * mine;
                }
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
                lam35_post(c);
            } else {
                c->Add = tot[0];
                c->tau = fabs(c->dd / (c->dDd + c->muDbeta * c->Add));
            }
        }
    }
}

// part[slab][c * L + l] = sum over the slab's rows of A[r][c] * s_r * Y[r * L + l]
template <class T, class V>
__global__ void __launch_bounds__(256) k_dense_TL_part(long m, long n, int L, long rows_per_slab,
                                                       const V* __restrict__ A, const float* __restrict__ rs,
                                                       MatIO<T> io, T* __restrict__ part) {
    count_launch(io.ctl);
    const int sel = io.by_parity ? io.ctl->parity : 0;
    const T* __restrict__ yv = io.x[sel];
    const int lane = threadIdx.x & 31;
    const long chunks = (L + 31) / 32;
    const long wi = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;  // (column, chunk)
    if (wi >= n * chunks) return;
    const long c = wi / chunks, l = (wi % chunks) * 32 + lane;
    const long slab = blockIdx.y;
    const long r0 = slab * rows_per_slab, r1 = min(m, r0 + rows_per_slab);
    if (l >= L) return;
    T s = T(0);
    for (long r = r0; r < r1; ++r) {
        T yr = yv[r * L + l];
        if (rs) yr *= (T)rs[r];
        s += (T)Acc<T, V>::load(A + r * n + c) * yr;
    }
    part[slab * n * L + c * L + l] = s;
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
        if (io.L > 1) {
            apply_layers(trans, io, epi, s);
            return;
        }
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

    void apply_layers(int trans, const MatIO<T>& io, int epi, cudaStream_t s) const {
        const long m = this->m, n = this->n;
        const int L = io.L;
        if constexpr (std::is_same<T, float>::value && std::is_same<V, __nv_bfloat16>::value) {
            if (umma && umma_L == L) {
                umma_apply(umma, trans, io, epi, rs.p, s);
                if (!io.ctl) umma_unchecked = true;
                return;
            }
        }
        if (!trans) {
            long g = std::min<long>((m * 32 + 255) / 256, (long)num_sms() * 8);
            int grid = (int)std::max<long>(g, 1);
            switch (epi) {
                case SPMV_SUB: k_dense_NL<T, V, SPMV_SUB><<<grid, 256, 0, s>>>(m, n, L, a.p, rs.p, io); break;
                case SPMV_LAM35: k_dense_NL<T, V, SPMV_LAM35><<<grid, 256, 0, s>>>(m, n, L, a.p, rs.p, io); break;
                case SPMV_NORM2: k_dense_NL<T, V, SPMV_NORM2><<<grid, 256, 0, s>>>(m, n, L, a.p, rs.p, io); break;
                default: k_dense_NL<T, V, SPMV_PLAIN><<<grid, 256, 0, s>>>(m, n, L, a.p, rs.p, io); break;
            }
        } else {
            long tiles, slabs_l, rps;
            layer_slabs(L, tiles, slabs_l, rps);
            if (part_l.n < (size_t)slabs_l * n * L)
                throw Error{1, "dense multi-RHS product used before prepare()"};
            k_dense_TL_part<T, V><<<dim3((unsigned)tiles, (unsigned)slabs_l), 256, 0, s>>>(m, n, L, rps, a.p, rs.p,
                                                                                          io, part_l.p);
            long g = std::min<long>((n * L + 255) / 256, (long)num_sms() * 8);
            k_dense_T_sum<T><<<(int)std::max<long>(g, 1), 256, 0, s>>>(n * L, (int)slabs_l, part_l.p, io,
                                                                       epi == SPMV_SUB);
        }
        TV3_CUDA(cudaGetLastError());
    }
    // column-tile x row-slab split of the multi-RHS A^T*Y
    void layer_slabs(int L, long& tiles, long& slabs_l, long& rps) const {
        const long m = this->m, n = this->n;
        const long chunks = (L + 31) / 32;
        tiles = (n * chunks * 32 + 255) / 256;
        slabs_l = std::max<long>(1, (long)num_sms() * 8 / std::max<long>(tiles, 1));
        slabs_l = std::min<long>(slabs_l, std::max<long>(m, 1));
        rps = std::max<long>(1, (m + slabs_l - 1) / slabs_l);
        slabs_l = std::max<long>(1, (m + rps - 1) / rps);
    }
    void prepare(int L) const override {
        if (L <= 1) return;
        if constexpr (std::is_same<T, float>::value && std::is_same<V, __nv_bfloat16>::value) {
            if (use_umma && umma_supported(this->m, this->n, L)) {
                if (umma && umma_L != L) {
                    umma_plan_destroy(umma);
                    umma = nullptr;
                }
                if (!umma) {
                    umma = umma_plan_create(this->m, this->n, L, a.p);
                    umma_L = L;
                }
                return;
            }
        }
        long tiles, slabs_l, rps;
        layer_slabs(L, tiles, slabs_l, rps);
        const size_t need = (size_t)slabs_l * this->n * L;
        if (part_l.n < need) part_l.alloc(need);
    }
    mutable DBuf<T> part_l;  // slab partials of the multi-RHS A^T*Y
    bool multi_rhs() const override { return true; }
    // standalone tensor-core products record a timed-out wait in the plan's
    // own error word; read (and clear) it once the products have completed
    int take_error(cudaStream_t s) const override {
        if constexpr (std::is_same<T, float>::value && std::is_same<V, __nv_bfloat16>::value) {
            if (umma && umma_unchecked) {
                umma_unchecked = false;
                return umma_take_error(umma, s);
            }
        }
        return 0;
    }
    mutable bool umma_unchecked = false;  // a standalone tensor-core product whose error word is unread
    mutable UmmaPlan* umma = nullptr;  // tensor-core plan of the multi-RHS products (BF16 only)
    mutable int umma_L = 0;
    int use_umma = 1;
    ~DenseOp() override {
        if (umma) umma_plan_destroy(umma);
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
