// Dense multi-RHS products on the 5th-generation tensor cores (tcgen05).
//
// The reference multiplies its dense 2D matrix with `layers` right-hand sides
// by cublasSgemm (2d/mat_vec_mul.h:91-99).  Here A is stored in BF16 with a
// per-row FP32 scale (A = diag(rs) * Aq), and both products are GEMMs with
// K-major BF16 operands staged by TMA and FP32 accumulators in tensor memory:
//
//   A*X:    D (m x L)  = Aq (m x n, K = n)   * [Xh + Xl],        y = rs .* D
//   A^T*Y:  D (n x L)  = Aq^T (n x m, K = m) * [(rs.*Y)h + (rs.*Y)l]
//
// The FP32 right-hand side is split into two BF16 parts (hi = bf16(v),
// lo = bf16(v - hi)), so the products carry about 16 mantissa bits of the
// vector and the BF16 rounding of A stays the only quantisation; A^T*Y uses
// the same BF16 values as A*X (a blocked copy of the transpose), so it is the
// exact adjoint of the quantised A.
//
// Kernel structure (one CTA = one 128-row tile of D and one split of K; four
// warps):
//   - thread 0 issues the TMA loads of a STAGES-deep ring (A tile 128 x 64,
//     one contiguous block of the blocked copy of A or A^T; B tiles Npad x 64
//     for hi and lo; 128-byte swizzle) and the
//     tcgen05.mma instructions (M = 128, N = Npad, K = 16 each), then commits
//     each stage's MMAs to the stage's "empty" barrier before refilling it;
//   - warp 0 allocates and frees the TMEM accumulator (Npad columns);
//   - all four warps read the accumulator back (warp w owns TMEM lanes
//     32w..32w+31 = rows of the tile) and write FP32 partial sums per split.
// A second kernel adds the splits in a fixed order and applies the solver
// epilogues (row scale, y - sub, lam3/lam5, ||y||^2) with the deterministic
// grid reduction.
//
// Every mbarrier wait is bounded (about two seconds of SM clock); on a
// timeout the kernel records the error in the control block, waits (bounded)
// for its own outstanding copies and MMAs, frees its TMEM and returns.
#include <cuda.h>
#include <cuda_bf16.h>
#include <algorithm>
#include <mutex>
#include "dbuf.h"
#include "mbar.cuh"
#include "ops.h"
#include "tval3/tval3_c.h"

namespace tv3 {

namespace {

constexpr int UM = 128;          // tile rows (TMEM lanes)
constexpr int UK = 64;           // K per stage: one 128-byte swizzle row of BF16
constexpr int MAX_STAGES = 6;
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* bar) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(map), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// shared-memory matrix descriptor: K-major operand, rows of 128 bytes with the
// 128-byte swizzle, 8-row groups 1024 bytes apart (SBO); LBO unused (1)
__device__ __forceinline__ uint64_t sdesc(const void* p) {
    const uint64_t a = smem_u32(p);
    uint64_t d = (a >> 4) & 0x3FFFull;
    d |= 1ull << 16;
    d |= (uint64_t)(1024 >> 4) << 32;
    d |= 1ull << 46;  // descriptor version of the sm_100 family
    d |= 2ull << 61;  // 128-byte swizzle
    return d;
}

// instruction descriptor of kind::f16: D FP32, A and B BF16, both K-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma(uint32_t tmem_d, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(
            tmem_d),
        "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
        : "memory");
}
__device__ __forceinline__ void umma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }

// 32 consecutive accumulator columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,%"
        "19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}

struct GemmArgs {
    long M;          // rows of D
    long K;          // reduction length
    int L;           // right-hand sides (columns of D written)
    int Npad;        // MMA N (multiple of 16, >= L)
    int tmem_cols;   // power of two >= max(32, Npad)
    int stages;
    int kb_per_split;
    float* part;     // [split][M][L]
    Ctl* ctl;        // launch counter (may be null)
    int* err;        // error word: the solve's Ctl::err, or the plan's own for standalone products
};

__global__ void __launch_bounds__(128, 3) k_umma_gemm(const __grid_constant__ CUtensorMap tmA,
                                                       const __grid_constant__ CUtensorMap tmBh,
                                                       const __grid_constant__ CUtensorMap tmBl, GemmArgs g) {
    count_launch(g.ctl);
    extern __shared__ unsigned char smem_raw[];
    __shared__ uint64_t full[MAX_STAGES], empty[MAX_STAGES], done;
    __shared__ uint32_t tmem_base;
    __shared__ int failed;
    unsigned char* sm = (unsigned char*)(((uintptr_t)smem_raw + 1023) & ~(uintptr_t)1023);
    const int S = g.stages;
    const unsigned a_bytes = UM * 128, b_bytes = (unsigned)g.Npad * 128;
    const unsigned stage_bytes = a_bytes + 2 * b_bytes;
    const int warp = threadIdx.x >> 5;
    // splits of K vary fastest across the grid, so the CTAs resident at one
    // time stream from many different column ranges of A (DRAM pages and
    // channels) rather than from the same offset of every row
    const long ks = blockIdx.x, mt = blockIdx.y;
    const long KB = (g.K + UK - 1) / UK;
    const long kb0 = ks * g.kb_per_split;
    const int nkb = (int)max(0L, min((long)g.kb_per_split, KB - kb0));

    if (threadIdx.x == 0) {
        failed = 0;
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(&done, 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&tmem_base)),
                     "r"(g.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = tmem_base;

    if (threadIdx.x == 0 && nkb > 0) {
        const uint32_t idesc = idesc_bf16(UM, g.Npad);
        // this CTA's k-blocks in a rotated order (start differs per row tile)
        const int rot = (int)((mt * 5) % nkb);
        auto load = [&](int j) {  // the j-th k-block of this split into stage j % S
            const int s = j % S;
            unsigned char* st = sm + (size_t)s * stage_bytes;
            mbar_expect_tx(&full[s], stage_bytes);
            const int jj = (j + rot) % nkb;
            const int kx = (int)((kb0 + jj) * UK);
            tma_load_2d(st, &tmA, 0, (int)((mt * KB + kb0 + jj) * UM), &full[s]);
            tma_load_2d(st + a_bytes, &tmBh, kx, 0, &full[s]);
            tma_load_2d(st + a_bytes + b_bytes, &tmBl, kx, 0, &full[s]);
        };
        int issued = 0, consumed = 0;
        bool ok = true;
        for (; issued < min(S, nkb); ++issued) load(issued);
        for (int i = 0; i < nkb && ok; ++i) {
            const int s = i % S;
            if (!mbar_wait(&full[s], (unsigned)((i / S) & 1))) {
                ok = false;
                break;
            }
            ++consumed;
            tc_fence_after();
            unsigned char* st = sm + (size_t)s * stage_bytes;
            const uint64_t ad = sdesc(st), bh = sdesc(st + a_bytes), bl = sdesc(st + a_bytes + b_bytes);
#pragma unroll
            for (int kk = 0; kk < UK / 16; ++kk) {
                // K = 16 BF16 = 32 bytes further along the swizzled row: +2 in the address field
                umma(tmem, ad + 2 * kk, bh + 2 * kk, idesc, (i > 0 || kk > 0) ? 1u : 0u);
                umma(tmem, ad + 2 * kk, bl + 2 * kk, idesc, 1u);
            }
            umma_commit(&empty[s]);
            // refill the stage the previous iteration used, once its MMAs are done
            if (i > 0 && issued < nkb) {
                const int p = i - 1;
                if (!mbar_wait(&empty[p % S], (unsigned)((p / S) & 1))) {
                    ok = false;
                    break;
                }
                load(issued++);
            }
        }
        umma_commit(&done);
        if (ok) ok = mbar_wait(&done, 0u);
        if (!ok) {
            failed = 1;
            if (g.err) atomicOr(g.err, (int)ERR_UMMA_TIMEOUT);
            // let this CTA's copies and MMAs finish before its shared memory goes away
            for (int j = consumed; j < issued; ++j) mbar_wait(&full[j % S], (unsigned)((j / S) & 1));
            mbar_wait(&done, 0u);
        }
    }
    __syncthreads();
    tc_fence_after();
    if (!failed && nkb > 0) {
        const long row = mt * UM + warp * 32 + (threadIdx.x & 31);
        float* out = g.part + ((size_t)ks * g.M + (size_t)min(row, g.M - 1)) * g.L;
        for (int c0 = 0; c0 < g.Npad; c0 += 32) {
            float v[32];
            tmem_ld32(tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0, v);
            if (row < g.M) {
#pragma unroll
                for (int j = 0; j < 32; ++j)
                    if (c0 + j < g.L) out[c0 + j] = v[j];
            }
        }
    } else if (nkb == 0) {
        const long row = mt * UM + warp * 32 + (threadIdx.x & 31);
        if (row < g.M)
            for (int l = 0; l < g.L; ++l) g.part[((size_t)ks * g.M + row) * g.L + l] = 0.f;
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(g.tmem_cols) : "memory");
    }
}

// B operand of one product: v = x (or rs .* x) as BF16 hi and lo parts, K-major
// rows per right-hand side: B[l * Kp + k].  Rows l >= L stay zero.  A block
// moves QK consecutive k of all L right-hand sides through shared memory, so
// both the interleaved read of x (x[k * L + l]) and the row-wise writes of B
// are coalesced.
constexpr int QK = 32;
__global__ void __launch_bounds__(256) k_umma_quant(long K, int L, long Kp, const float* __restrict__ rs,
                                                    MatIO<float> io, __nv_bfloat16* __restrict__ bh,
                                                    __nv_bfloat16* __restrict__ bl) {
    count_launch(io.ctl);
    __shared__ float t[QK][257];
    const float* __restrict__ x = (io.by_parity && io.ctl->parity) ? io.x[1] : io.x[0];
    for (long k0 = (long)blockIdx.x * QK; k0 < K; k0 += (long)gridDim.x * QK) {
        const int kn = (int)min((long)QK, K - k0);
        __syncthreads();
        for (int idx = threadIdx.x; idx < kn * L; idx += blockDim.x) {
            const int kk = idx / L;
            t[kk][idx - kk * L] = x[k0 * L + idx];
        }
        __syncthreads();
        for (int idx = threadIdx.x; idx < QK * L; idx += blockDim.x) {
            const int l = idx / QK, kk = idx % QK;
            if (kk >= kn) continue;
            float v = t[kk][l];
            if (rs) v *= rs[k0 + kk];
            const __nv_bfloat16 h = __float2bfloat16_rn(v);
            bh[l * Kp + k0 + kk] = h;
            bl[l * Kp + k0 + kk] = __float2bfloat16_rn(v - __bfloat162float(h));
        }
    }
}

// y = (rs .*) sum over splits of the partials, with the solver epilogues
template <int EPI>
__global__ void __launch_bounds__(256) k_umma_reduce(long M, int L, int splits, const float* __restrict__ part,
                                                     const float* __restrict__ rs, MatIO<float> io) {
    count_launch(io.ctl);
    const int sel = io.by_parity ? io.ctl->parity : 0;
    float* __restrict__ y = io.y[sel];
    double acc0 = 0.0, acc1 = 0.0;
    const long tot = M * L;
    for (long o = (long)blockIdx.x * blockDim.x + threadIdx.x; o < tot; o += (long)gridDim.x * blockDim.x) {
        float s = 0.f;
        for (int k = 0; k < splits; ++k) s += part[(size_t)k * tot + o];
        if (rs) s *= rs[o / L];
        if (EPI == SPMV_PLAIN) y[o] = s;
        else if (EPI == SPMV_SUB) y[o] = s - io.sub[o];
        else if (EPI == SPMV_LAM35) {
            y[o] = s;
            double t = (double)s - (double)io.b[o];
            acc0 += t * t;
            acc1 += (double)io.delta[o] * t;
        } else if (EPI == SPMV_NORM2) {
            acc0 += (double)s * s;
        }
    }
    if (EPI == SPMV_LAM35 || EPI == SPMV_NORM2) {
        double v[2] = {acc0, acc1}, tt[2];
        if (grid_reduce<2>(v, io.part, io.ticket, tt) && threadIdx.x == 0) {
            Ctl* c = io.ctl;
            if (EPI == SPMV_LAM35) {
                c->lam3 = tt[0];
                c->lam5 = tt[1];
                lam35_post(c);
            } else {
                c->Add = tt[0];
                c->tau = fabs(c->dd / (c->dDd + c->muDbeta * c->Add));
            }
        }
    }
}

// A (trans = 0) or A^T (trans = 1) of the row-major m x n BF16 array `a` in
// 128 x 64 blocks: block (row tile rt, k-block kb) holds rows rt*128.. and
// columns kb*64.. of the operand, row-major and contiguous (16 KB), blocks in
// (rt, kb) order, zeros outside the matrix.  One TMA box of the GEMM is then a
// single contiguous 16 KB read and one split of K a contiguous run of blocks,
// instead of 128 pieces of 128 bytes one matrix row apart.
__global__ void __launch_bounds__(256) k_bf16_tile(long m, long n, int trans, long KB, long nblocks,
                                                   const __nv_bfloat16* __restrict__ a,
                                                   __nv_bfloat16* __restrict__ dst) {
    __shared__ __nv_bfloat16 t[UK][UM + 2];
    const long R = trans ? n : m, C = trans ? m : n;
    for (long b = blockIdx.x; b < nblocks; b += gridDim.x) {
        const long rt = b / KB, kb = b - rt * KB;
        __nv_bfloat16* __restrict__ o = dst + (size_t)b * (UM * UK);
        if (!trans) {
            for (int idx = threadIdx.x; idx < UM * UK; idx += blockDim.x) {
                const long i = rt * UM + (idx >> 6), k = kb * UK + (idx & 63);
                o[idx] = (i < R && k < C) ? a[i * n + k] : __float2bfloat16_rn(0.f);
            }
        } else {
            __syncthreads();
            for (int idx = threadIdx.x; idx < UM * UK; idx += blockDim.x) {
                const int c = idx >> 7, r = idx & 127;  // operand row rt*128+r = column of a
                const long i = rt * UM + r, k = kb * UK + c;
                t[c][r] = (i < R && k < C) ? a[k * n + i] : __float2bfloat16_rn(0.f);
            }
            __syncthreads();
            for (int idx = threadIdx.x; idx < UM * UK; idx += blockDim.x) o[idx] = t[idx & 63][idx >> 6];
        }
    }
}

using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                 const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                 CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = (EncodeTiled)p;
    });
    if (!fn) throw Error{TVAL3_ERR_CUDA, "cuTensorMapEncodeTiled is not available"};
    return fn;
}

// 2D BF16 tensor map: inner extent `inner` (K), outer extent `outer` rows,
// row pitch `pitch` elements, box 64 x box_rows, 128-byte swizzle, zero fill
CUtensorMap make_map(const void* base, long inner, long outer, long pitch, int box_rows) {
    CUtensorMap m;
    const cuuint64_t dims[2] = {(cuuint64_t)inner, (cuuint64_t)outer};
    const cuuint64_t strides[1] = {(cuuint64_t)pitch * 2};
    const cuuint32_t box[2] = {(cuuint32_t)UK, (cuuint32_t)box_rows};
    const cuuint32_t es[2] = {1, 1};
    CUresult r = encode_fn()(&m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, es,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) throw Error{TVAL3_ERR_CUDA, "cuTensorMapEncodeTiled failed (" + std::to_string((int)r) + ")"};
    return m;
}

}  // namespace

// Everything the two tensor-core products of one (operator, L) need.
struct UmmaPlan {
    long m = 0, n = 0, mp = 0, np = 0;
    int L = 0, Npad = 0, tmem_cols = 0;
    DBuf<__nv_bfloat16> tN, tT;      // Aq and Aq^T in 128 x 64 blocks (k_bf16_tile)
    DBuf<__nv_bfloat16> bN_h, bN_l;  // B of A*X: Npad x np
    DBuf<__nv_bfloat16> bT_h, bT_l;  // B of A^T*Y: Npad x mp
    DBuf<float> part;
    DBuf<int> err;  // error word of products made outside a solve (zero: no error)
    CUtensorMap mapA, mapAt, mapBNh, mapBNl, mapBTh, mapBTl;
    int splitsN = 1, kbN = 1, stagesN = 1, splitsT = 1, kbT = 1, stagesT = 1;
    size_t smemN = 0, smemT = 0;
};

static void plan_split(long M, long K, int& splits, int& kb_per) {
    const long mtiles = (M + UM - 1) / UM, KB = std::max<long>(1, (K + UK - 1) / UK);
    const long target = (long)num_sms() * 6;
    long s = std::max<long>(1, std::min<long>(KB, (target + mtiles - 1) / mtiles));
    kb_per = (int)((KB + s - 1) / s);
    splits = (int)((KB + kb_per - 1) / kb_per);
}

// rows of the blocked copy of an M x K operand (TMA row coordinates are int)
static long blocked_rows(long M, long K) { return (M + UM - 1) / UM * ((K + UK - 1) / UK) * UM; }

bool umma_supported(long m, long n, int L) {
    return L > 1 && L <= 256 && n % 8 == 0 && m > 0 && n > 0 && blocked_rows(m, n) < (1L << 31) &&
           blocked_rows(n, m) < (1L << 31);
}

static void tile_operand(long m, long n, int trans, const __nv_bfloat16* Aq, DBuf<__nv_bfloat16>& dst) {
    const long M = trans ? n : m, K = trans ? m : n;
    const long KB = (K + UK - 1) / UK, nblocks = (M + UM - 1) / UM * KB;
    dst.alloc((size_t)blocked_rows(M, K) * UK);
    const int g = (int)std::min<long>(nblocks, (long)num_sms() * 8);
    k_bf16_tile<<<g, 256>>>(m, n, trans, KB, nblocks, Aq, dst.p);
    TV3_CUDA(cudaGetLastError());
}

UmmaPlan* umma_plan_create(long m, long n, int L, const __nv_bfloat16* Aq) {
    auto* p = new UmmaPlan();
    try {
        p->m = m; p->n = n; p->L = L;
        p->mp = (m + 7) / 8 * 8;
        p->np = n;  // n % 8 == 0
        p->Npad = (L + 15) / 16 * 16;
        int tc = 32;
        while (tc < p->Npad) tc <<= 1;
        p->tmem_cols = tc;
        tile_operand(m, n, 0, Aq, p->tN);
        tile_operand(m, n, 1, Aq, p->tT);
        p->bN_h.alloc((size_t)p->Npad * p->np);
        p->bN_l.alloc((size_t)p->Npad * p->np);
        p->bT_h.alloc((size_t)p->Npad * p->mp);
        p->bT_l.alloc((size_t)p->Npad * p->mp);
        TV3_CUDA(cudaMemset(p->bN_h.p, 0, (size_t)p->Npad * p->np * 2));
        TV3_CUDA(cudaMemset(p->bN_l.p, 0, (size_t)p->Npad * p->np * 2));
        TV3_CUDA(cudaMemset(p->bT_h.p, 0, (size_t)p->Npad * p->mp * 2));
        TV3_CUDA(cudaMemset(p->bT_l.p, 0, (size_t)p->Npad * p->mp * 2));
        plan_split(m, n, p->splitsN, p->kbN);
        plan_split(n, m, p->splitsT, p->kbT);
        p->part.alloc(std::max((size_t)p->splitsN * m * L, (size_t)p->splitsT * n * L));
        p->err.alloc(1);
        TV3_CUDA(cudaMemset(p->err.p, 0, sizeof(int)));
        p->mapA = make_map(p->tN.p, UK, blocked_rows(m, n), UK, UM);
        p->mapAt = make_map(p->tT.p, UK, blocked_rows(n, m), UK, UM);
        p->mapBNh = make_map(p->bN_h.p, n, p->Npad, p->np, p->Npad);
        p->mapBNl = make_map(p->bN_l.p, n, p->Npad, p->np, p->Npad);
        p->mapBTh = make_map(p->bT_h.p, m, p->Npad, p->mp, p->Npad);
        p->mapBTl = make_map(p->bT_l.p, m, p->Npad, p->mp, p->Npad);
        const size_t stage = (size_t)UM * 128 + 2 * (size_t)p->Npad * 128;
        const size_t budget = 72 * 1024;  // three CTAs per SM while a stage is <= 24 KB (Npad <= 32)
        const int st = (int)std::min<size_t>(MAX_STAGES, std::max<size_t>(2, budget / stage));
        p->stagesN = p->stagesT = st;
        p->smemN = p->smemT = st * stage + 1024;
        TV3_CUDA(cudaFuncSetAttribute(k_umma_gemm, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)p->smemN));
        TV3_CUDA(cudaDeviceSynchronize());
    } catch (...) {
        delete p;
        throw;
    }
    return p;
}

void umma_plan_destroy(UmmaPlan* p) { delete p; }

// the error word of the plan's standalone products (after they completed on
// s), cleared for the next product
int umma_take_error(const UmmaPlan* p, cudaStream_t s) {
    int e = 0;
    TV3_CUDA(cudaMemcpyAsync(&e, p->err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    TV3_CUDA(cudaStreamSynchronize(s));
    if (e) TV3_CUDA(cudaMemsetAsync(p->err.p, 0, sizeof(int), s));
    return e;
}

void umma_apply(const UmmaPlan* p, int trans, const MatIO<float>& io, int epi, const float* rs, cudaStream_t s) {
    const long M = trans ? p->n : p->m, K = trans ? p->m : p->n, Kp = trans ? p->mp : p->np;
    __nv_bfloat16* bh = trans ? p->bT_h.p : p->bN_h.p;
    __nv_bfloat16* bl = trans ? p->bT_l.p : p->bN_l.p;
    const int qg = (int)std::max<long>(1, std::min<long>((K + QK - 1) / QK, (long)num_sms() * 8));
    // dependent launches: each kernel waits for its predecessor at entry
    // (count_launch), so its launch overlaps the previous kernel's tail
    launch_k(k_umma_quant, dim3(qg), dim3(256), 0, s, K, p->L, Kp, trans ? rs : nullptr, io, bh, bl);
    GemmArgs g;
    g.M = M; g.K = K; g.L = p->L; g.Npad = p->Npad; g.tmem_cols = p->tmem_cols;
    g.stages = trans ? p->stagesT : p->stagesN;
    g.kb_per_split = trans ? p->kbT : p->kbN;
    g.part = p->part.p;
    g.ctl = io.ctl;
    g.err = io.ctl ? &io.ctl->err : p->err.p;
    const int splits = trans ? p->splitsT : p->splitsN;
    dim3 grid((unsigned)splits, (unsigned)((M + UM - 1) / UM));
    launch_k(k_umma_gemm, grid, dim3(128), trans ? p->smemT : p->smemN, s, trans ? p->mapAt : p->mapA,
             trans ? p->mapBTh : p->mapBNh, trans ? p->mapBTl : p->mapBNl, g);
    const long tot = M * p->L;
    const int rg = (int)std::max<long>(1, std::min<long>((tot + 255) / 256, (long)num_sms() * 4));
    const float* post = trans ? nullptr : rs;
    auto reduce = [&](auto kernel) {
        launch_k(kernel, dim3(rg), dim3(256), 0, s, M, p->L, splits, (const float*)p->part.p, post, io);
    };
    switch (epi) {
        case SPMV_SUB: reduce(k_umma_reduce<SPMV_SUB>); break;
        case SPMV_LAM35: reduce(k_umma_reduce<SPMV_LAM35>); break;
        case SPMV_NORM2: reduce(k_umma_reduce<SPMV_NORM2>); break;
        default: reduce(k_umma_reduce<SPMV_PLAIN>); break;
    }
    TV3_CUDA(cudaGetLastError());
}

}  // namespace tv3
