// CSR operator: device copies of A and of the CSR of A^T, value storage in
// FP32 / FP64 / BF16 / FP16 (16-bit values carry a per-ray FP32 scale), and the
// device-side transpose (replaces cusparseScsr2csc, 2d/mat_vec_mul.h:23-28).
// The single-GPU counterpart in the reference is sparse_mm
// (3d/mat_vec_mul_sparse.h:1599-1781).
#include <cub/cub.cuh>
#include <algorithm>
#include <map>
#include <mutex>
#include <string>
#include <typeinfo>
#include <type_traits>
#include <vector>
#include "dbuf.h"
#include "ops.h"
#include "tiled.h"

namespace tv3 {

void tmp_pool_init() {
    static bool done[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64 || done[dev]) return;
    cudaMemPool_t pool;
    if (cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
        // The threshold counts memory in use too: with live operators holding
        // more than it, every synchronize would return all freed memory to the
        // driver and the next build would map its temporaries again.  Keep up
        // to 1/16 of the device (17.8 GB on a 284 GB part), at least 4 GB.
        size_t free_b = 0, total_b = 0;
        if (cudaMemGetInfo(&free_b, &total_b) != cudaSuccess) total_b = 0;
        unsigned long long keep = std::max<unsigned long long>(4ull << 30, (unsigned long long)total_b / 16);
        cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
    done[dev] = true;
}

void throw_cuda(cudaError_t e, const char* what) {
    int st = (e == cudaErrorMemoryAllocation) ? 4 : 3;
    cudaGetLastError();  // clear a sticky launch error where possible
    throw Error{st, std::string(what) + ": " + cudaGetErrorString(e)};
}

// index / value arrays of a CSR operator: nnz elements plus zeroed slack
// that the four-element loads of the SpMV may touch
template <class X>
static void alloc_padded(DBuf<X>& b, long nnz) {
    b.alloc(nnz + SPMV_PAD);
    TV3_CUDA(cudaMemset(b.p, 0, (nnz + SPMV_PAD) * sizeof(X)));
}

static int pick_lanes(double avg) {
    if (avg > 48) return 32;
    if (avg > 20) return 16;
    if (avg > 8) return 8;
    return 4;
}

static int spmv_grid(long rows, int G) {
    long need = (rows * G + 255) / 256;
    long cap = (long)num_sms() * 8;
    return (int)std::max<long>(1, std::min(need, cap));
}

// ---------------------------------------------------------------------------
// quantisation helpers
// ---------------------------------------------------------------------------
template <class V> __device__ __forceinline__ V to_v(float x);
template <> __device__ __forceinline__ __nv_bfloat16 to_v<__nv_bfloat16>(float x) { return __float2bfloat16_rn(x); }
template <> __device__ __forceinline__ __half to_v<__half>(float x) { return __float2half_rn(x); }
template <class V> __device__ __forceinline__ float from_v(V x);
template <> __device__ __forceinline__ float from_v<__nv_bfloat16>(__nv_bfloat16 x) { return __bfloat162float(x); }
template <> __device__ __forceinline__ float from_v<__half>(__half x) { return __half2float(x); }

// per-row scale = max |a_r| (1 for an empty or all-zero row); one warp per row
__global__ void k_rowmax(long rows, const int* __restrict__ ptr, const float* __restrict__ val, float* __restrict__ s) {
    const int lane = threadIdx.x & 31;
    for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += ((long)gridDim.x * blockDim.x) >> 5) {
        float mx = 0.f;
        for (int k = ptr[r] + lane; k < ptr[r + 1]; k += 32) mx = fmaxf(mx, fabsf(val[k]));
        for (int o = 16; o; o >>= 1) mx = fmaxf(mx, __shfl_xor_sync(FULL, mx, o));
        if (lane == 0) s[r] = (mx > 0.f) ? mx : 1.f;
    }
}

template <class V>
__global__ void k_quant_rows(long rows, const int* __restrict__ ptr, const float* __restrict__ val,
                             const float* __restrict__ s, V* __restrict__ q) {
    const int lane = threadIdx.x & 31;
    for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += ((long)gridDim.x * blockDim.x) >> 5) {
        const float inv = s[r];
        for (int k = ptr[r] + lane; k < ptr[r + 1]; k += 32) q[k] = to_v<V>(val[k] / inv);
    }
}

template <class V>
__global__ void k_quant_entries(long nnz, const int* __restrict__ rowidx, const float* __restrict__ val,
                                const float* __restrict__ s, V* __restrict__ q) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x)
        q[k] = to_v<V>(val[k] / s[rowidx[k]]);
}

template <class V>
__global__ void k_dequant_rows(long rows, const int* __restrict__ ptr, const V* __restrict__ q,
                               const float* __restrict__ s, float* __restrict__ out) {
    const int lane = threadIdx.x & 31;
    for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += ((long)gridDim.x * blockDim.x) >> 5)
        for (int k = ptr[r] + lane; k < ptr[r + 1]; k += 32) out[k] = from_v<V>(q[k]) * s[r];
}

template <class V>
__global__ void k_dequant_entries(long nnz, const int* __restrict__ rowidx, const V* __restrict__ q,
                                  const float* __restrict__ s, float* __restrict__ out) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x)
        out[k] = from_v<V>(q[k]) * s[rowidx[k]];
}

template <class A, class B>
__global__ void k_convert(long n, const A* __restrict__ in, B* __restrict__ out) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        out[k] = (B)in[k];
}

// ---------------------------------------------------------------------------
// device transpose (stable radix sort of the column indices)
// ---------------------------------------------------------------------------
__global__ void k_iota(long n, int* __restrict__ v) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x) v[k] = (int)k;
}

__global__ void k_expand_rows(long rows, const int* __restrict__ ptr, int* __restrict__ rowof) {
    const int lane = threadIdx.x & 31;
    for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += ((long)gridDim.x * blockDim.x) >> 5)
        for (int k = ptr[r] + lane; k < ptr[r + 1]; k += 32) rowof[k] = (int)r;
}

__global__ void k_hist(long nnz, const int* __restrict__ ind, int* __restrict__ cnt) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x)
        atomicAdd(cnt + ind[k], 1);
}

template <class V>
__global__ void k_gather_t(long nnz, const int* __restrict__ perm, const int* __restrict__ rowof,
                           const V* __restrict__ val, int* __restrict__ tind, V* __restrict__ tval) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x) {
        int p = perm[k];
        tind[k] = rowof[p];
        tval[k] = val[p];
    }
}

static int ew(long n) {
    long g = (n + 255) / 256;
    long cap = (long)num_sms() * 32;
    return (int)std::max<long>(1, std::min(g, cap));
}

template <class V>
void csr_transpose_device(long rows, long cols, long nnz, const int* ptr, const int* ind, const V* val, int* tptr,
                          int* tind, V* tval, cudaStream_t s) {
    DBuf<int> cnt(cols + 1);
    TV3_CUDA(cudaMemsetAsync(cnt.p, 0, (cols + 1) * sizeof(int), s));
    if (nnz > 0) {
        DBuf<int> keys_out(nnz), perm_in(nnz), perm_out(nnz), rowof(nnz);
        k_iota<<<ew(nnz), 256, 0, s>>>(nnz, perm_in.p);
        k_expand_rows<<<ew(rows * 32), 256, 0, s>>>(rows, ptr, rowof.p);
        k_hist<<<ew(nnz), 256, 0, s>>>(nnz, ind, cnt.p);
        int end_bit = 1;
        while (end_bit < 31 && (1L << end_bit) < cols) ++end_bit;
        size_t tmp_bytes = 0;
        TV3_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tmp_bytes, ind, keys_out.p, perm_in.p, perm_out.p, (int)nnz,
                                                 0, end_bit, s));
        DBuf<char> tmp(tmp_bytes);
        TV3_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tmp_bytes, ind, keys_out.p, perm_in.p, perm_out.p, (int)nnz,
                                                 0, end_bit, s));
        k_gather_t<V><<<ew(nnz), 256, 0, s>>>(nnz, perm_out.p, rowof.p, val, tind, tval);
        TV3_CUDA(cudaGetLastError());
        size_t scan_bytes = 0;
        TV3_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, scan_bytes, cnt.p, tptr, (int)(cols + 1), s));
        DBuf<char> tmp2(scan_bytes);
        TV3_CUDA(cub::DeviceScan::ExclusiveSum(tmp2.p, scan_bytes, cnt.p, tptr, (int)(cols + 1), s));
        TV3_CUDA(cudaStreamSynchronize(s));  // temporaries are freed on return
    } else {
        TV3_CUDA(cudaMemsetAsync(tptr, 0, (cols + 1) * sizeof(int), s));
        TV3_CUDA(cudaStreamSynchronize(s));
    }
}

template void csr_transpose_device<float>(long, long, long, const int*, const int*, const float*, int*, int*, float*,
                                          cudaStream_t);
template void csr_transpose_device<double>(long, long, long, const int*, const int*, const double*, int*, int*,
                                           double*, cudaStream_t);

// ---------------------------------------------------------------------------
// the operator
// ---------------------------------------------------------------------------
template <class T, class V> struct CsrOp;
template <class T, class V> static void tune_lanes(CsrOp<T, V>* op, int mask);

// Kernel choices of stored operators, per device, value and vector type,
// shape and volume: a later operator of the same key (e.g. the next call of a
// host entry point on the same geometry) takes them without the timing
// contest.  The choice only selects between kernels that compute the same
// products; it fixes their summation order for equal keys within a process.
struct TuneChoice {
    int varN, varT, Gn, Gt, grid_n, grid_t;
    unsigned pend;
};
static std::mutex g_tune_mu;
static std::map<std::string, TuneChoice> g_tune;

static std::string tune_key(const char* types, long m, long n, long nnz, int p, int q, int r) {
    int dev = 0;
    cudaGetDevice(&dev);
    return std::string(types) + "/" + std::to_string(dev) + "/" + std::to_string(m) + "/" + std::to_string(n) + "/" +
           std::to_string(nnz) + "/" + std::to_string(p) + "/" + std::to_string(q) + "/" + std::to_string(r);
}

template <class T, class V>
struct CsrOp : LinOp<T> {
    DBuf<int> ptr, ind, tptr, tind, rowof_t;
    DBuf<V> val, tval;
    DBuf<float> rs;  // per-ray scale (16-bit storage only)
    mutable int Gn = 32, Gt = 8, grid_n = 1, grid_t = 1;
    // products whose CSR lane count is still the untimed default (bit trans):
    // timed on their first CSR use outside stream capture, or never when a
    // tile-staged kernel runs them
    mutable unsigned pend = 0;
    void tune_pending(int trans) const {
        if (!((pend >> trans) & 1u)) return;
        pend &= ~(1u << trans);
        tune_lanes(const_cast<CsrOp*>(this), 1 << trans);
    }
    void ready() const override {
        for (int trans = 0; trans < 2; ++trans)
            if ((trans ? varT : varN) == 0) tune_pending(trans);
    }
    mutable TiledT<T, V> tiled;   // A^T regrouped by voxel tiles (when the volume is known)
    mutable TiledN<T, V> tiledN;  // A cut into per-tile ray segments (when the volume is known)
    // kernel of each product: 0 CSR, 1 tile-staged, 2 (A^T only) tile-staged and pipelined
    mutable int varT = 0, varN = 0;
    mutable int vol[3] = {0, 0, 0};

    void set_volume(int p, int q, int r) const override {
        if (vol[0] == p && vol[1] == q && vol[2] == r) return;
        vol[0] = p; vol[1] = q; vol[2] = r;
        tiled.build(this->n, this->m, p, q, r, tptr.p, tind.p, tval.p, this->nnz, 96 * 1024, 0);
        tiledN.build(this->m, p, q, r, ptr.p, ind.p, val.p, this->nnz, 0);
        varT = tiled.ok ? 1 : 0;
        varN = tiledN.ok ? 1 : 0;
        if (this->nnz < (1L << 22)) return;
        const std::string key = tune_key(typeid(CsrOp).name(), this->m, this->n, this->nnz, p, q, r);
        {
            std::lock_guard<std::mutex> lk(g_tune_mu);
            auto it = g_tune.find(key);
            if (it != g_tune.end()) {
                const TuneChoice& c = it->second;
                varN = (c.varN == 1 && !tiledN.ok) ? 0 : c.varN;
                varT = (c.varT == 1 && !tiled.ok) ? 0 : c.varT;
                Gn = c.Gn; Gt = c.Gt; grid_n = c.grid_n; grid_t = c.grid_t; pend = c.pend;
                return;
            }
        }
        // large operators: the faster kernel of each product, timed here.  The
        // pipelined A^T (variant 2) takes part only when pinned: it lost every
        // measured contest and its tables cost build time.  CSR runs first with
        // its default lanes; its lanes are timed only when it comes within
        // 1.5x of the tile-staged kernel.
        if (this->nnz >= (1L << 22)) {
            for (int trans = 0; trans < 2; ++trans) {
                if (!(trans ? tiled.ok : tiledN.ok)) continue;
                // one round each; two more only when the kernels are within 25 %
                float t1 = time_product(trans, 1, 1);
                const unsigned keep = pend;
                pend &= ~(1u << trans);
                float t0 = time_product(trans, 0, 1);
                pend = keep;
                if (t0 < 1.5f * t1 && ((pend >> trans) & 1u)) {
                    tune_pending(trans);
                    t0 = time_product(trans, 0, 1);
                }
                if (std::max(t0, t1) < 1.25f * std::min(t0, t1)) {
                    t1 = std::min(t1, time_product(trans, 1, 2));
                    t0 = std::min(t0, time_product(trans, 0, 2));
                }
                (trans ? varT : varN) = (t0 < t1) ? 0 : 1;
            }
        }
        std::lock_guard<std::mutex> lk(g_tune_mu);
        g_tune[key] = TuneChoice{varN, varT, Gn, Gt, grid_n, grid_t, pend};
    }

    bool set_variant(int trans, int v) const override {
        if (v < 0 || v > (trans ? 2 : 1)) return false;
        if (v == 1 && !(trans ? tiled.ok : tiledN.ok)) return false;
        if (v == 2 && !tiled.ensure_pipe()) return false;
        (trans ? varT : varN) = v;
        return true;
    }
    int variant(int trans) const override { return trans ? varT : varN; }

    // milliseconds of three products with kernel variant use_variant, best of
    // `rounds` rounds after one warm-up
    float time_product(int trans, int use_variant, int rounds) const {
        int& flag = trans ? varT : varN;
        const int keep = flag;
        flag = use_variant;
        const long lx = trans ? this->m : this->n, ly = trans ? this->n : this->m;
        DBuf<T> x(std::max<long>(lx, 1)), y(std::max<long>(ly, 1));
        TV3_CUDA(cudaMemset(x.p, 0, std::max<long>(lx, 1) * sizeof(T)));
        cudaEvent_t e0, e1;
        TV3_CUDA(cudaEventCreate(&e0));
        TV3_CUDA(cudaEventCreate(&e1));
        MatIO<T> io = plain_io<T>(x.p, y.p);
        apply(trans, io, SPMV_PLAIN, 0);
        float best = 1e30f;
        for (int round = 0; round < rounds; ++round) {
            TV3_CUDA(cudaEventRecord(e0, 0));
            for (int k = 0; k < 3; ++k) apply(trans, io, SPMV_PLAIN, 0);
            TV3_CUDA(cudaEventRecord(e1, 0));
            TV3_CUDA(cudaEventSynchronize(e1));
            float ms = 0.f;
            TV3_CUDA(cudaEventElapsedTime(&ms, e0, e1));
            best = std::min(best, ms);
        }
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        flag = keep;
        return best;
    }

    void apply(int trans, const MatIO<T>& io, int epi, cudaStream_t s) const override {
        if (!trans && io.L <= 1 && varN == 1 && tiledN.ok) {
            TiledNArgs<T, V> t{};
            t.ntiles = tiledN.ntiles;
            t.p = tiledN.p; t.q = tiledN.q; t.r = tiledN.r; t.ty = tiledN.ty; t.tx = tiledN.tx; t.tz = tiledN.tz;
            t.nty = tiledN.nty; t.ntx = tiledN.ntx;
            t.tile_slice = tiledN.tile_slice.p; t.slice_off = tiledN.slice_off.p; t.slot_dest = tiledN.slot_dest.p;
            t.lidx = tiledN.lidx.p; t.val = tiledN.val.p; t.part = tiledN.part.p;
            t.sray = tiledN.sray.p; t.rlen = tiledN.rlen.p;
            t.gbase = tiledN.gbase.p;
            t.m = this->m; t.rscale = rs.p;
            t.x[0] = io.x[0]; t.x[1] = io.x[1]; t.y[0] = io.y[0]; t.y[1] = io.y[1];
            t.by_parity = io.by_parity; t.sub = io.sub; t.b = io.b; t.delta = io.delta; t.ctl = io.ctl;
            t.rpart = io.part; t.ticket = io.ticket;
            tiledN.apply(t, epi, s);
            return;
        }
        if (trans && io.L <= 1 && varT >= 1 && tiled.ok && (epi == SPMV_PLAIN || epi == SPMV_SUB)) {
            TiledArgs<T, V> t{};
            t.ntiles = tiled.ntiles; t.ray_off = tiled.ray_off.p; t.rays = tiled.rays.p;
            t.tile_slice = tiled.tile_slice.p; t.slice_off = tiled.slice_off.p; t.row_voxel = tiled.row_voxel.p;
            t.lidx = tiled.lidx.p; t.val = tiled.val.p;
            t.tile_unit = tiled.tile_unit.p; t.slice_unit = tiled.slice_unit.p; t.unit_slice = tiled.unit_slice.p;
            t.unit_k0 = tiled.unit_k0.p; t.max_rays = tiled.max_rays;
            t.xscale = rs.p;
            t.x[0] = io.x[0]; t.x[1] = io.x[1]; t.y[0] = io.y[0]; t.y[1] = io.y[1];
            t.by_parity = io.by_parity; t.sub = io.sub; t.ctl = io.ctl;
            if (varT == 2) tiled.apply_pipe(t, epi, s);
            else tiled.apply(t, epi, s);
            return;
        }
        SpmvArgs<T, V> a{};
        if (!trans) {
            a.rows = this->m; a.ptr = ptr.p; a.ind = ind.p; a.val = val.p; a.rscale = rs.p; a.xscale = nullptr;
        } else {
            a.rows = this->n; a.ptr = tptr.p; a.ind = tind.p; a.val = tval.p; a.rscale = nullptr; a.xscale = rs.p;
        }
        a.x[0] = io.x[0]; a.x[1] = io.x[1];
        a.y[0] = io.y[0]; a.y[1] = io.y[1];
        a.by_parity = io.by_parity;
        a.sub = io.sub; a.b = io.b; a.delta = io.delta;
        a.ctl = io.ctl; a.part = io.part; a.ticket = io.ticket;
        a.L = io.L;
        if ((pend >> trans) & 1u) {
            cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
            if (cudaStreamIsCapturing(s, &st) == cudaSuccess && st == cudaStreamCaptureStatusNone) tune_pending(trans);
        }
        launch_spmv<T, V>(a, epi, trans ? Gt : Gn, trans ? grid_t : grid_n, s);
        TV3_CUDA(cudaGetLastError());
    }

    void export_csr(int* hptr, int* hind, float* hval, int* htptr, int* htind, float* htval) const override;
    void export_scaled(float* hval, float* hrs, float* htval) const override;
    bool multi_rhs() const override { return true; }
};

template <class T, class V>
static void export_vals(const CsrOp<T, V>& op, float* hval, float* htval);

template <>
void export_vals<float, float>(const CsrOp<float, float>& op, float* hval, float* htval) {
    if (hval) TV3_CUDA(cudaMemcpy(hval, op.val.p, op.nnz * sizeof(float), cudaMemcpyDeviceToHost));
    if (htval) TV3_CUDA(cudaMemcpy(htval, op.tval.p, op.nnz * sizeof(float), cudaMemcpyDeviceToHost));
}
template <>
void export_vals<double, double>(const CsrOp<double, double>& op, float* hval, float* htval) {
    DBuf<float> tmp(std::max<long>(op.nnz, 1));
    if (hval) {
        k_convert<double, float><<<ew(op.nnz), 256>>>(op.nnz, op.val.p, tmp.p);
        TV3_CUDA(cudaMemcpy(hval, tmp.p, op.nnz * sizeof(float), cudaMemcpyDeviceToHost));
    }
    if (htval) {
        k_convert<double, float><<<ew(op.nnz), 256>>>(op.nnz, op.tval.p, tmp.p);
        TV3_CUDA(cudaMemcpy(htval, tmp.p, op.nnz * sizeof(float), cudaMemcpyDeviceToHost));
    }
}
template <class T, class V>
static void export_q(const CsrOp<T, V>& op, float* hval, float* htval) {
    DBuf<float> tmp(std::max<long>(op.nnz, 1));
    if (hval) {
        k_dequant_rows<V><<<ew(op.m * 32), 256>>>(op.m, op.ptr.p, op.val.p, op.rs.p, tmp.p);
        TV3_CUDA(cudaMemcpy(hval, tmp.p, op.nnz * sizeof(float), cudaMemcpyDeviceToHost));
    }
    if (htval) {
        k_dequant_entries<V><<<ew(op.nnz), 256>>>(op.nnz, op.tind.p, op.tval.p, op.rs.p, tmp.p);
        TV3_CUDA(cudaMemcpy(htval, tmp.p, op.nnz * sizeof(float), cudaMemcpyDeviceToHost));
    }
}
template <>
void export_vals<float, __nv_bfloat16>(const CsrOp<float, __nv_bfloat16>& op, float* hval, float* htval) {
    export_q(op, hval, htval);
}
template <>
void export_vals<float, __half>(const CsrOp<float, __half>& op, float* hval, float* htval) {
    export_q(op, hval, htval);
}
template <>
void export_vals<df64, __nv_bfloat16>(const CsrOp<df64, __nv_bfloat16>& op, float* hval, float* htval) {
    export_q(op, hval, htval);
}
template <>
void export_vals<df64, __half>(const CsrOp<df64, __half>& op, float* hval, float* htval) {
    export_q(op, hval, htval);
}

// 16-bit values widened to FP32 (exact), in the layout of the stored arrays
template <class V>
__global__ void k_widen(long n, const V* __restrict__ q, float* __restrict__ out) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < n; k += (long)gridDim.x * blockDim.x)
        out[k] = from_v<V>(q[k]);
}

template <class V>
static constexpr bool is_16bit() {
    return std::is_same<V, __nv_bfloat16>::value || std::is_same<V, __half>::value;
}

template <class T, class V>
void CsrOp<T, V>::export_scaled(float* hval, float* hrs, float* htval) const {
    if constexpr (is_16bit<V>()) {
        DBuf<float> tmp(std::max<long>(this->nnz, 1));
        if (hval && this->nnz) {
            k_widen<V><<<ew(this->nnz), 256>>>(this->nnz, val.p, tmp.p);
            TV3_CUDA(cudaMemcpy(hval, tmp.p, this->nnz * sizeof(float), cudaMemcpyDeviceToHost));
        }
        if (htval && this->nnz) {
            k_widen<V><<<ew(this->nnz), 256>>>(this->nnz, tval.p, tmp.p);
            TV3_CUDA(cudaMemcpy(htval, tmp.p, this->nnz * sizeof(float), cudaMemcpyDeviceToHost));
        }
        if (hrs && this->m) TV3_CUDA(cudaMemcpy(hrs, rs.p, this->m * sizeof(float), cudaMemcpyDeviceToHost));
    } else {
        export_vals<T, V>(*this, hval, htval);
        if (hrs) std::fill(hrs, hrs + this->m, 1.0f);
    }
}

template <class T, class V>
void CsrOp<T, V>::export_csr(int* hptr, int* hind, float* hval, int* htptr, int* htind, float* htval) const {
    if (hptr) TV3_CUDA(cudaMemcpy(hptr, ptr.p, (this->m + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    if (hind) TV3_CUDA(cudaMemcpy(hind, ind.p, this->nnz * sizeof(int), cudaMemcpyDeviceToHost));
    if (htptr) TV3_CUDA(cudaMemcpy(htptr, tptr.p, (this->n + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    if (htind) TV3_CUDA(cudaMemcpy(htind, tind.p, this->nnz * sizeof(int), cudaMemcpyDeviceToHost));
    export_vals<T, V>(*this, hval, htval);
}

// Autotuner: for matrices big enough to matter, time every lanes-per-row
// choice of both products on the operator itself (CUDA events, zero vectors,
// three launches each after one warm-up) and keep the fastest; small matrices
// use the nonzeros-per-row heuristic.
template <class T, class V>
static void tune_lanes(CsrOp<T, V>* op, int mask) {
    const long m = op->m, n = op->n;
    DBuf<T> x(std::max(m, n) + 1), y(std::max(m, n) + 1);
    TV3_CUDA(cudaMemset(x.p, 0, (std::max(m, n) + 1) * sizeof(T)));
    cudaEvent_t e0, e1;
    TV3_CUDA(cudaEventCreate(&e0));
    TV3_CUDA(cudaEventCreate(&e1));
    const int cand[8] = {4, 8, 16, 32, 4 | SPMV_SCALAR, 8 | SPMV_SCALAR, 16 | SPMV_SCALAR, 32 | SPMV_SCALAR};
    for (int trans = 0; trans < 2; ++trans) {
        if (!((mask >> trans) & 1)) continue;
        float best = 1e30f;
        int bestG = trans ? op->Gt : op->Gn;
        for (int G : cand) {
            const int lanes = G & ~SPMV_SCALAR;
            if (trans) { op->Gt = G; op->grid_t = spmv_grid(n, lanes); }
            else { op->Gn = G; op->grid_n = spmv_grid(m, lanes); }
            MatIO<T> io = plain_io<T>(x.p, y.p);
            op->apply(trans, io, SPMV_PLAIN, 0);
            float ms = 1e30f;  // best of two rounds of two launches
            for (int round = 0; round < 2; ++round) {
                TV3_CUDA(cudaEventRecord(e0, 0));
                for (int r = 0; r < 2; ++r) op->apply(trans, io, SPMV_PLAIN, 0);
                TV3_CUDA(cudaEventRecord(e1, 0));
                TV3_CUDA(cudaEventSynchronize(e1));
                float t = 0.f;
                TV3_CUDA(cudaEventElapsedTime(&t, e0, e1));
                ms = std::min(ms, t);
            }
            if (ms < best) { best = ms; bestG = G; }
        }
        if (trans) { op->Gt = bestG; op->grid_t = spmv_grid(n, bestG & ~SPMV_SCALAR); }
        else { op->Gn = bestG; op->grid_n = spmv_grid(m, bestG & ~SPMV_SCALAR); }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

template <class T, class V>
static void finish_layout(CsrOp<T, V>* op, bool tune = true) {
    op->Gn = pick_lanes(op->m ? (double)op->nnz / op->m : 0.0);
    op->Gt = pick_lanes(op->n ? (double)op->nnz / op->n : 0.0);
    op->grid_n = spmv_grid(op->m, op->Gn);
    op->grid_t = spmv_grid(op->n, op->Gt);
    op->pend = (tune && op->nnz >= (1L << 22)) ? 3u : 0u;  // lane timing on first CSR use
}

// Build from device arrays (FP32 values for the FP32/BF16/FP16 precisions,
// FP64 values for FP64).  The transpose is built when d_tptr is null.
template <class T>
LinOp<T>* make_csr_op_device(long rows, long cols, long nnz, const int* d_ptr, const int* d_ind, const T* d_val,
                             const int* d_tptr, const int* d_tind, const T* d_tval, int precision,
                             cudaStream_t s);

template <class T>
static void copy_structure(LinOp<T>* base, DBuf<int>& ptr, DBuf<int>& ind, DBuf<int>& tptr, DBuf<int>& tind,
                           long rows, long cols, long nnz, const int* d_ptr, const int* d_ind) {
    base->m = rows; base->n = cols; base->nnz = nnz; base->kind = 0;
    ptr.alloc(rows + 1);
    alloc_padded(ind, nnz);
    tptr.alloc(cols + 1);
    alloc_padded(tind, nnz);
    TV3_CUDA(cudaMemcpy(ptr.p, d_ptr, (rows + 1) * sizeof(int), cudaMemcpyDeviceToDevice));
    if (nnz) TV3_CUDA(cudaMemcpy(ind.p, d_ind, nnz * sizeof(int), cudaMemcpyDeviceToDevice));
}

template <>
void export_vals<double, float>(const CsrOp<double, float>& op, float* hval, float* htval) {
    if (hval) TV3_CUDA(cudaMemcpy(hval, op.val.p, op.nnz * sizeof(float), cudaMemcpyDeviceToHost));
    if (htval) TV3_CUDA(cudaMemcpy(htval, op.tval.p, op.nnz * sizeof(float), cudaMemcpyDeviceToHost));
}

// FP32 values with FP64 vectors: the matrix stream is that of the FP32
// operator, the products, vectors and reductions are FP64.
LinOp<double>* make_csr_op_f64vec(long rows, long cols, long nnz, const int* d_ptr, const int* d_ind,
                                  const float* d_val, const int* d_tptr, const int* d_tind, const float* d_tval,
                                  cudaStream_t s, bool tune) {
    auto* op = new CsrOp<double, float>();
    try {
        copy_structure<double>(op, op->ptr, op->ind, op->tptr, op->tind, rows, cols, nnz, d_ptr, d_ind);
        alloc_padded(op->val, nnz);
        alloc_padded(op->tval, nnz);
        if (nnz) TV3_CUDA(cudaMemcpy(op->val.p, d_val, nnz * sizeof(float), cudaMemcpyDeviceToDevice));
        if (d_tptr) {
            TV3_CUDA(cudaMemcpy(op->tptr.p, d_tptr, (cols + 1) * sizeof(int), cudaMemcpyDeviceToDevice));
            if (nnz) {
                TV3_CUDA(cudaMemcpy(op->tind.p, d_tind, nnz * sizeof(int), cudaMemcpyDeviceToDevice));
                TV3_CUDA(cudaMemcpy(op->tval.p, d_tval, nnz * sizeof(float), cudaMemcpyDeviceToDevice));
            }
        } else {
            csr_transpose_device<float>(rows, cols, nnz, op->ptr.p, op->ind.p, op->val.p, op->tptr.p, op->tind.p,
                                        op->tval.p, s);
        }
        finish_layout(op, tune);
    } catch (...) {
        delete op;
        throw;
    }
    return op;
}

template <>
void export_vals<df64, float>(const CsrOp<df64, float>& op, float* hval, float* htval) {
    if (hval) TV3_CUDA(cudaMemcpy(hval, op.val.p, op.nnz * sizeof(float), cudaMemcpyDeviceToHost));
    if (htval) TV3_CUDA(cudaMemcpy(htval, op.tval.p, op.nnz * sizeof(float), cudaMemcpyDeviceToHost));
}

__global__ void k_f64_to_df64(long n, const double* __restrict__ in, df64* __restrict__ out) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = df64(in[i]);
}
__global__ void k_df64_to_f64(long n, const df64* __restrict__ in, double* __restrict__ out) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = (double)in[i];
}
void convert_to_df64(const double* in, void* out, long n, cudaStream_t s) {
    if (n > 0) k_f64_to_df64<<<ew(n), 256, 0, s>>>(n, in, static_cast<df64*>(out));
    TV3_CUDA(cudaGetLastError());
}
void convert_from_df64(const void* in, double* out, long n, cudaStream_t s) {
    if (n > 0) k_df64_to_f64<<<ew(n), 256, 0, s>>>(n, static_cast<const df64*>(in), out);
    TV3_CUDA(cudaGetLastError());
}

// Double-float view of an FP32-value / FP64-vector CSR operator: the same
// device arrays (not copied, not freed by the view), products in df64.
LinOp<df64>* make_df64_view(const LinOp<double>* base) {
    auto* b = dynamic_cast<const CsrOp<double, float>*>(base);
    if (!b) throw Error{7, "double-float products need an FP32-value CSR operator"};
    auto* op = new CsrOp<df64, float>();
    op->m = b->m; op->n = b->n; op->nnz = b->nnz; op->kind = b->kind;
    op->ptr.view(b->ptr.p, b->ptr.n);
    op->ind.view(b->ind.p, b->ind.n);
    op->tptr.view(b->tptr.p, b->tptr.n);
    op->tind.view(b->tind.p, b->tind.n);
    op->val.view(b->val.p, b->val.n);
    op->tval.view(b->tval.p, b->tval.n);
    try {
        finish_layout(op);
    } catch (...) {
        delete op;
        throw;
    }
    return op;
}

template <>
LinOp<double>* make_csr_op_device<double>(long rows, long cols, long nnz, const int* d_ptr, const int* d_ind,
                                          const double* d_val, const int* d_tptr, const int* d_tind,
                                          const double* d_tval, int precision, cudaStream_t s) {
    if (precision == 4) {
        DBuf<float> v(std::max<long>(nnz, 1)), tv(std::max<long>(nnz, 1));
        if (nnz) k_convert<double, float><<<ew(nnz), 256, 0, s>>>(nnz, d_val, v.p);
        if (nnz && d_tptr) k_convert<double, float><<<ew(nnz), 256, 0, s>>>(nnz, d_tval, tv.p);
        TV3_CUDA(cudaGetLastError());
        TV3_CUDA(cudaStreamSynchronize(s));
        return make_csr_op_f64vec(rows, cols, nnz, d_ptr, d_ind, v.p, d_tptr, d_tind, d_tptr ? tv.p : nullptr, s, true);
    }
    auto* op = new CsrOp<double, double>();
    try {
        copy_structure<double>(op, op->ptr, op->ind, op->tptr, op->tind, rows, cols, nnz, d_ptr, d_ind);
        alloc_padded(op->val, nnz);
        alloc_padded(op->tval, nnz);
        if (nnz) TV3_CUDA(cudaMemcpy(op->val.p, d_val, nnz * sizeof(double), cudaMemcpyDeviceToDevice));
        if (d_tptr) {
            TV3_CUDA(cudaMemcpy(op->tptr.p, d_tptr, (cols + 1) * sizeof(int), cudaMemcpyDeviceToDevice));
            if (nnz) {
                TV3_CUDA(cudaMemcpy(op->tind.p, d_tind, nnz * sizeof(int), cudaMemcpyDeviceToDevice));
                TV3_CUDA(cudaMemcpy(op->tval.p, d_tval, nnz * sizeof(double), cudaMemcpyDeviceToDevice));
            }
        } else {
            csr_transpose_device<double>(rows, cols, nnz, op->ptr.p, op->ind.p, op->val.p, op->tptr.p, op->tind.p,
                                         op->tval.p, s);
        }
        finish_layout(op);
    } catch (...) {
        delete op;
        throw;
    }
    return op;
}

// 16-bit values with a per-ray FP32 scale (the row's largest magnitude) from
// FP32 device arrays; T is the vector type of the products (float, or df64
// for the mixed-precision modes)
template <class T, class V>
static LinOp<T>* make_q(long rows, long cols, long nnz, const int* d_ptr, const int* d_ind, const float* d_val,
                        const int* d_tptr, const int* d_tind, const float* d_tval, cudaStream_t s) {
    auto* op = new CsrOp<T, V>();
    try {
        copy_structure<T>(op, op->ptr, op->ind, op->tptr, op->tind, rows, cols, nnz, d_ptr, d_ind);
        DBuf<float> tv(std::max<long>(nnz, 1));
        if (d_tptr) {
            TV3_CUDA(cudaMemcpy(op->tptr.p, d_tptr, (cols + 1) * sizeof(int), cudaMemcpyDeviceToDevice));
            if (nnz) {
                TV3_CUDA(cudaMemcpy(op->tind.p, d_tind, nnz * sizeof(int), cudaMemcpyDeviceToDevice));
                TV3_CUDA(cudaMemcpy(tv.p, d_tval, nnz * sizeof(float), cudaMemcpyDeviceToDevice));
            }
        } else {
            csr_transpose_device<float>(rows, cols, nnz, op->ptr.p, op->ind.p, d_val, op->tptr.p, op->tind.p, tv.p, s);
        }
        op->rs.alloc(std::max<long>(rows, 1));
        alloc_padded(op->val, nnz);
        alloc_padded(op->tval, nnz);
        k_rowmax<<<ew(rows * 32), 256, 0, s>>>(rows, op->ptr.p, d_val, op->rs.p);
        k_quant_rows<V><<<ew(rows * 32), 256, 0, s>>>(rows, op->ptr.p, d_val, op->rs.p, op->val.p);
        if (nnz) k_quant_entries<V><<<ew(nnz), 256, 0, s>>>(nnz, op->tind.p, tv.p, op->rs.p, op->tval.p);
        TV3_CUDA(cudaGetLastError());
        TV3_CUDA(cudaStreamSynchronize(s));
        finish_layout(op);
    } catch (...) {
        delete op;
        throw;
    }
    return op;
}

template <>
LinOp<float>* make_csr_op_device<float>(long rows, long cols, long nnz, const int* d_ptr, const int* d_ind,
                                        const float* d_val, const int* d_tptr, const int* d_tind, const float* d_tval,
                                        int precision, cudaStream_t s) {
    if (precision == 2)
        return make_q<float, __nv_bfloat16>(rows, cols, nnz, d_ptr, d_ind, d_val, d_tptr, d_tind, d_tval, s);
    if (precision == 3) return make_q<float, __half>(rows, cols, nnz, d_ptr, d_ind, d_val, d_tptr, d_tind, d_tval, s);
    auto* op = new CsrOp<float, float>();
    try {
        copy_structure<float>(op, op->ptr, op->ind, op->tptr, op->tind, rows, cols, nnz, d_ptr, d_ind);
        alloc_padded(op->val, nnz);
        alloc_padded(op->tval, nnz);
        if (nnz) TV3_CUDA(cudaMemcpy(op->val.p, d_val, nnz * sizeof(float), cudaMemcpyDeviceToDevice));
        if (d_tptr) {
            TV3_CUDA(cudaMemcpy(op->tptr.p, d_tptr, (cols + 1) * sizeof(int), cudaMemcpyDeviceToDevice));
            if (nnz) {
                TV3_CUDA(cudaMemcpy(op->tind.p, d_tind, nnz * sizeof(int), cudaMemcpyDeviceToDevice));
                TV3_CUDA(cudaMemcpy(op->tval.p, d_tval, nnz * sizeof(float), cudaMemcpyDeviceToDevice));
            }
        } else {
            csr_transpose_device<float>(rows, cols, nnz, op->ptr.p, op->ind.p, op->val.p, op->tptr.p, op->tind.p,
                                        op->tval.p, s);
        }
        finish_layout(op);
    } catch (...) {
        delete op;
        throw;
    }
    return op;
}

LinOp<df64>* make_csr_op_df64q(long rows, long cols, long nnz, const int* d_ptr, const int* d_ind,
                               const float* d_val, const int* d_tptr, const int* d_tind, const float* d_tval,
                               int precision, cudaStream_t s) {
    if (precision == 6)
        return make_q<df64, __nv_bfloat16>(rows, cols, nnz, d_ptr, d_ind, d_val, d_tptr, d_tind, d_tval, s);
    if (precision == 7) return make_q<df64, __half>(rows, cols, nnz, d_ptr, d_ind, d_val, d_tptr, d_tind, d_tval, s);
    throw Error{7, "mixed-precision operators store BF16 or FP16 values"};
}

// column-major (rows x k) <-> interleaved (row * k + column)
template <class T>
__global__ void k_interleave(long rows, int k, const T* __restrict__ in, T* __restrict__ out, int inverse) {
    const long tot = rows * k;
    for (long t = (long)blockIdx.x * blockDim.x + threadIdx.x; t < tot; t += (long)gridDim.x * blockDim.x) {
        const long r = t / k, j = t - r * k;  // t = interleaved index
        if (inverse) out[j * rows + r] = in[t];
        else out[t] = in[j * rows + r];
    }
}

template <class T>
void apply_interleaved(const LinOp<T>& op, int trans, int k, const T* X, T* Y, cudaStream_t s) {
    const long lx = trans ? op.m : op.n, ly = trans ? op.n : op.m;
    op.prepare(k);
    DBuf<T> xi(std::max<long>(lx * k, 1)), yi(std::max<long>(ly * k, 1));
    if (lx > 0) k_interleave<T><<<ew(lx * k), 256, 0, s>>>(lx, k, X, xi.p, 0);
    MatIO<T> io = plain_io<T>(xi.p, yi.p);
    io.L = k;
    op.apply(trans, io, SPMV_PLAIN, s);
    if (ly > 0) k_interleave<T><<<ew(ly * k), 256, 0, s>>>(ly, k, yi.p, Y, 1);
    TV3_CUDA(cudaGetLastError());
    TV3_CUDA(cudaStreamSynchronize(s));  // the scratch is freed on return
}
template void apply_interleaved<float>(const LinOp<float>&, int, int, const float*, float*, cudaStream_t);
template void apply_interleaved<double>(const LinOp<double>&, int, int, const double*, double*, cudaStream_t);
template void apply_interleaved<df64>(const LinOp<df64>&, int, int, const df64*, df64*, cudaStream_t);

}  // namespace tv3
