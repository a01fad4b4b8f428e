// A^T*y with the gathered vector staged in shared memory per voxel tile.
//
// In the CSR of A^T (rows = voxels) every nonzero gathers one y value of a
// ray.  A ray crosses a tile of voxels (16 x 16 x 8 in 3D, 32 x 32 in 2D) in
// a run of about a dozen consecutive voxels, so the ~26,000 nonzeros of a
// tile at 128^3 touch only ~2,000 distinct rays.  The tiled form stores, per
// tile, the ascending list of those rays and, per nonzero, the ray's position
// in that list (16 bits) instead of its index (32 bits).  One CTA per tile
// gathers the tile's y values once into shared memory, then sums its voxel
// rows from shared memory: global gathers drop by an order of magnitude, the
// matrix stream drops from 8 to 6 bytes per FP32 nonzero, and the rows'
// gathers cost shared-memory bandwidth instead of L1/L2 wavefronts.
//
// Inside a tile the voxel rows are sorted by length (longest first) and cut
// into slices of 32 rows stored "sliced ELL" style: entry k of the slice's
// lane l sits at slice_off + 32 k + l, so a warp (one row per lane) reads 32
// entries with one coalesced load of positions and one of values, and the
// slice is padded only to its first (longest) row.  Every row is summed by one
// thread in its original nonzero order (deterministic).
//
// Built once on the device from the CSR of A^T with a radix sort of
// (tile, ray) keys; used for A^T*y when the operator knows the volume's
// dimensions and every tile's ray list fits the shared-memory budget.
//
// Work inside a tile is split into units of at most TILED_UNIT_K steps of
// one slice (32 rows), so the warps of a CTA get near-equal work; each unit
// leaves 32 partial sums in shared memory and every row adds its units'
// partials in order after a barrier (deterministic).
#include <cub/cub.cuh>
#include <algorithm>
#include <type_traits>
#include <vector>
#include "ops.h"
#include "tiled.h"
#include "mbar.cuh"

namespace tv3 {

namespace {

int ewt(long n) {
    long g = (n + 255) / 256;
    long cap = (long)num_sms() * 32;
    return (int)std::max<long>(1, std::min(g, cap));
}

// bits that hold the indices 0 .. count-1 (at least 1)
int index_bits(long count) {
    int b = 1;
    while (b < 62 && (1L << b) < count) ++b;
    return b;
}

template <class V> struct TVT { using type = float; };
template <> struct TVT<double> { using type = double; };

__global__ void k_tile_of_voxel(long n, int p, int q, int ty, int tx, int tz, int nty, int ntx, int* __restrict__ tv,
                                int* __restrict__ iota) {
    for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (long)gridDim.x * blockDim.x) {
        const long y = v % p, x = (v / p) % q, z = v / ((long)p * q);
        tv[v] = (int)((z / tz) * ((long)nty * ntx) + (x / tx) * nty + y / ty);
        iota[v] = (int)v;
    }
}

__global__ void k_rows_of(long rows, const int* __restrict__ ptr, int* __restrict__ rowof) {
    const int lane = threadIdx.x & 31;
    for (long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5; r < rows; r += ((long)gridDim.x * blockDim.x) >> 5)
        for (int k = ptr[r] + lane; k < ptr[r + 1]; k += 32) rowof[k] = (int)r;
}

// (tile, ray) keys: the ray index in the low rb bits, the tile above it, so a
// radix sort needs only the bits the two indices occupy
__global__ void k_keys(long nnz, const int* __restrict__ rowof, const int* __restrict__ tind,
                       const int* __restrict__ tile_of, int rb, unsigned long long* __restrict__ key,
                       int* __restrict__ idx) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x) {
        key[k] = ((unsigned long long)(unsigned)tile_of[rowof[k]] << rb) | (unsigned)tind[k];
        idx[k] = (int)k;
    }
}

// first-of-(tile, ray) flags of the sorted keys, and each tile's first position
__global__ void k_flags(long nnz, const unsigned long long* __restrict__ key, int rb, int* __restrict__ newray,
                        int* __restrict__ tile_first) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x) {
        const unsigned long long c = key[k];
        newray[k] = (k == 0 || key[k - 1] != c) ? 1 : 0;
        if (k == 0 || (key[k - 1] >> rb) != (c >> rb)) tile_first[c >> rb] = (int)k;
    }
}

// uniq[k] = number of distinct (tile, ray) pairs up to and including k
__global__ void k_local(long nnz, const unsigned long long* __restrict__ key, int rb, const int* __restrict__ uniq,
                        const int* __restrict__ idx, const int* __restrict__ tile_first, int* __restrict__ rays,
                        unsigned short* __restrict__ local_of_entry) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x) {
        const unsigned long long c = key[k];
        const int t = (int)(c >> rb);
        const int u = uniq[k] - 1;                 // this (tile, ray) in the concatenated lists
        const int base = uniq[tile_first[t]] - 1;  // the tile's first
        if (k == 0 || key[k - 1] != c) rays[u] = (int)(unsigned)(c & ((1ull << rb) - 1));
        local_of_entry[idx[k]] = (unsigned short)(u - base);
    }
}

__global__ void k_tile_start(int ntiles, const int* __restrict__ tile_first, const int* __restrict__ uniq,
                             int* __restrict__ start) {
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < ntiles; t += gridDim.x * blockDim.x)
        start[t] = tile_first[t] >= 0 ? uniq[tile_first[t]] - 1 : -1;
}

// sorted-row keys: (tile, longest first, voxel order kept by the stable sort)
__global__ void k_row_keys(long n, const int* __restrict__ tile_of, const int* __restrict__ tptr,
                           unsigned long long* __restrict__ key, int* __restrict__ iota, int* __restrict__ too_long) {
    for (long v = (long)blockIdx.x * blockDim.x + threadIdx.x; v < n; v += (long)gridDim.x * blockDim.x) {
        int len = tptr[v + 1] - tptr[v];
        if (len > 0xffff) {
            *too_long = 1;
            len = 0xffff;
        }
        key[v] = ((unsigned long long)(unsigned)tile_of[v] << 16) | (unsigned)(0xffff - len);
        iota[v] = (int)v;
    }
}

template <class V>
__global__ void k_fill_slices(long n, const unsigned long long* __restrict__ key, const int* __restrict__ vox,
                              const int* __restrict__ tile_row, const int* __restrict__ tile_slice,
                              const long long* __restrict__ slice_off, const int* __restrict__ tptr,
                              const unsigned short* __restrict__ local_of, const V* __restrict__ tval,
                              unsigned short* __restrict__ lidx, V* __restrict__ val, int* __restrict__ row_voxel) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) {
        const int t = (int)(key[i] >> 16);
        const int j = (int)(i - tile_row[t]);
        const int sl = tile_slice[t] + j / 32, lane = j % 32;
        const int v = vox[i];
        const int s0 = tptr[v], len = tptr[v + 1] - s0;
        if (len == 0) continue;  // rows without nonzeros sort last and sit in the zero-row list
        row_voxel[(long)sl * 32 + lane] = v;
        const long long o = slice_off[sl] + lane;
        for (int k = 0; k < len; ++k) {
            lidx[o + 32LL * k] = local_of[s0 + k];
            val[o + 32LL * k] = tval[s0 + k];
        }
    }
}

template <class T, class V, int EPI, int U>
__global__ void __launch_bounds__(512) k_spmv_tiled(TiledArgs<T, V> a) {
    count_launch(a.ctl);
    using VV = typename TVT<V>::type;
    extern __shared__ __align__(128) unsigned char sm_raw[];
    T* ysm = reinterpret_cast<T*>(sm_raw);
    T* psm = ysm + a.max_rays;  // partial sums: 32 per work unit
    const int sel = a.by_parity ? a.ctl->parity : 0;
    const T* __restrict__ y = a.x[sel];
    T* __restrict__ out = a.y[sel];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    // one tile per CTA (no tile at all when no row has nonzeros: grid of one
    // CTA that only writes the empty rows)
    const bool has_tile = (int)blockIdx.x < a.nwork;
    const int t = has_tile ? __ldg(a.tile_order + blockIdx.x) : 0;
    const int r0 = __ldg(a.ray_off + t), nr = has_tile ? __ldg(a.ray_off + t + 1) - r0 : 0;
    const int u0 = __ldg(a.tile_unit + t), u1 = has_tile ? __ldg(a.tile_unit + t + 1) : u0;
    const int s0 = __ldg(a.tile_slice + t), s1 = has_tile ? __ldg(a.tile_slice + t + 1) : s0;
    // this thread's row of the final sums (a tile has at most 512 rows): its
    // voxel, unit range and subtrahend, loaded now so their latency hides
    // behind the staging and the products
    int rv = -1, re0 = 0, re1 = 0;
    T rsub = T(0);
    if ((int)threadIdx.x < (s1 - s0) * 32) {
        const int sl = s0 + warp;
        rv = __ldg(a.row_voxel + (long)sl * 32 + lane);
        re0 = __ldg(a.slice_unit + sl) - u0;
        re1 = __ldg(a.slice_unit + sl + 1) - u0;
        if (EPI == SPMV_SUB && rv >= 0) rsub = a.sub[rv];
    }
    // stage the tile's y values: 8 independent index loads, then 8 gathers
    for (int j0 = threadIdx.x; j0 < nr; j0 += 8 * blockDim.x) {
        int ray[8];
        T v[8];
#pragma unroll
        for (int u = 0; u < 8; ++u) {
            const int j = j0 + u * blockDim.x;
            ray[u] = (j < nr) ? __ldg(a.rays + r0 + j) : -1;
        }
#pragma unroll
        for (int u = 0; u < 8; ++u) v[u] = (ray[u] >= 0) ? y[ray[u]] : T(0);
        if (a.xscale) {
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (ray[u] >= 0) v[u] *= (T)__ldg(a.xscale + ray[u]);
        }
#pragma unroll
        for (int u = 0; u < 8; ++u)
            if (ray[u] >= 0) ysm[j0 + u * blockDim.x] = v[u];
    }
    __syncthreads();
    // work units: at most UNIT_K steps of one slice, so warps get equal work.
    // A unit is one 16-byte descriptor (its first entry and its steps); the
    // warp's next descriptor is loaded while it sums the current unit.
    longlong2 dnext = make_longlong2(0, 0);
    if (u0 + warp < u1) dnext = __ldg(a.unit_desc + u0 + warp);
    for (int w = u0 + warp; w < u1; w += nwarps) {
        const longlong2 dc = dnext;
        if (w + nwarps < u1) dnext = __ldg(a.unit_desc + w + nwarps);
        const unsigned short* __restrict__ li = a.lidx + dc.x + lane;
        const V* __restrict__ va = a.val + dc.x + lane;
        const int k1 = (int)dc.y;
        RowAcc<T> acc;
        int k = 0;
        for (; k + U <= k1; k += U) {
            unsigned short ii[U];
            VV vv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                ii[u] = __ldcs(li + 32 * (k + u));
                vv[u] = (VV)Acc<VV, V>::load(va + 32 * (k + u));
            }
#pragma unroll
            for (int u = 0; u < U; ++u) madd(acc, vv[u], ysm[ii[u]]);
        }
        for (; k < k1; ++k) madd(acc, (VV)Acc<VV, V>::load(va + 32 * k), ysm[__ldcs(li + 32 * k)]);
        psm[(w - u0) * 32 + lane] = acc.value();
    }
    __syncthreads();
    // every row: its units' partials in order
    if (rv >= 0) {
        T sum = T(0);
        for (int e = re0; e < re1; ++e) sum += psm[e * 32 + lane];
        out[rv] = (EPI == SPMV_SUB) ? sum - rsub : sum;
    }
    // rows without nonzeros, (A^T y)_v = 0, shared out over the tile CTAs (a
    // CTA of their own would hold a tile's shared memory for a few stores)
    for (long z = (long)blockIdx.x * blockDim.x + threadIdx.x; z < a.nzero; z += (long)gridDim.x * blockDim.x) {
        const int v = __ldg(a.zrows + z);
        out[v] = (EPI == SPMV_SUB) ? T(0) - a.sub[v] : T(0);
    }
}

// ---------------------------------------------------------------------------
// Pipelined A^T*y.  One persistent CTA per SM takes the tiles with work in
// largest-first order, snaking over the CTAs (tile k*G + b for even k,
// k*G + G-1-b for odd k).  Warp PIPE_CONSUMERS is a producer: per tile it
// bulk-copies the tile's ray list into shared memory and gathers the tile's y
// values with 4/8-byte asynchronous copies into one of two y buffers, so the
// gather of the next tile runs while the PIPE_CONSUMERS consumer warps sum
// the current one (the staging phase of k_spmv_tiled, which no streaming
// overlaps inside its CTA).  The consumers stream the units from global
// memory exactly as k_spmv_tiled does (unit j of a tile to warp j mod 31; the
// sums and the row sums in unit order are the same, bit for bit).
//
// Every mbarrier wait is bounded.  On a timeout the warp records
// ERR_TILED_TIMEOUT, stops computing, keeps taking part in the consumers'
// named barriers so no warp is left waiting, releases a y buffer only after a
// second bounded wait for its gathers, and the producer waits (bounded) for
// its own copies in flight before it returns.
// ---------------------------------------------------------------------------
template <class T, class V, int EPI, int U>
__global__ void __launch_bounds__(32 * (PIPE_CONSUMERS + 1), 1) k_spmv_tiled_pipe(TiledArgs<T, V> a, PipeArgs pa) {
    count_launch(a.ctl);
    using VV = typename TVT<V>::type;
    extern __shared__ __align__(128) unsigned char sm_raw[];
    uint64_t* yfull = reinterpret_cast<uint64_t*>(sm_raw);  // 2
    uint64_t* yempty = yfull + 2;                             // 2
    uint64_t* rbar = yempty + 2;                              // 1
    T* ybuf = reinterpret_cast<T*>(sm_raw + 64);
    int* ridx = reinterpret_cast<int*>(ybuf + 2 * (size_t)pa.ybuf_elems);
    T* psm = reinterpret_cast<T*>(ridx + pa.ybuf_elems);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) {
        for (int i = 0; i < 2; ++i) {
            mbar_init(&yfull[i], 32);
            mbar_init(&yempty[i], PIPE_CONSUMERS);
        }
        mbar_init(rbar, 1);
        mbar_fence_init();
    }
    __syncthreads();
    const int sel = a.by_parity ? a.ctl->parity : 0;
    const T* __restrict__ y = a.x[sel];
    T* __restrict__ out = a.y[sel];
    const int G = gridDim.x, b = blockIdx.x;
    auto tile_at = [&](int i) {  // this CTA's i-th tile (position in the largest-first order)
        return i * G + ((i & 1) ? G - 1 - b : b);
    };
    auto sched_of = [&](int i, int4& s0, int4& s1) {  // this CTA's i-th tile record (or none)
        const int k = tile_at(i);
        if (k < a.nwork) {
            s0 = __ldg(pa.sched + 2 * k);
            s1 = __ldg(pa.sched + 2 * k + 1);
        } else {
            s0 = make_int4(-1, 0, 0, 0);
            s1 = make_int4(0, 0, 0, 0);
        }
    };
    bool ok = true;
    if (warp == PIPE_CONSUMERS) {
        // ------------------------------------------------------- producer: per
        // tile, the ray list by one bulk copy, then the tile's y values by
        // 4/8-byte asynchronous copies into the free y buffer (a tile ahead)
        int rpend = -1;  // parity of a ray-list copy not yet seen complete
        int4 ta, tb, na, nb4;
        sched_of(0, ta, tb);
        for (int i = 0; ok && ta.x >= 0; ++i, ta = na, tb = nb4) {
            sched_of(i + 1, na, nb4);  // the next record loads while this tile is served
            const int yb = i & 1, nr = tb.z;
            if (i >= 2) ok = __all_sync(FULL, mbar_wait(&yempty[yb], (unsigned)(((i - 2) >> 1) & 1)));
            if (!ok) break;
            const unsigned nbytes = (unsigned)((nr + 3) & ~3) * 4u;
            if (lane == 0) {
                mbar_expect_tx(rbar, nbytes);
                bulk_g2s(ridx, pa.rays_pad + tb.w, nbytes, rbar);
            }
            rpend = i & 1;
            ok = __all_sync(FULL, mbar_wait(rbar, (unsigned)rpend));
            if (!ok) break;
            rpend = -1;
            T* ys = ybuf + (size_t)yb * pa.ybuf_elems;
            for (int j = lane; j < nr; j += 32) cp_async<(int)sizeof(T)>(ys + j, y + ridx[j]);
            cp_async_arrive(&yfull[yb]);
            __syncwarp();  // every lane has read ridx before the next list overwrites it
        }
        if (!ok && lane == 0 && a.ctl) atomicOr(&a.ctl->err, (int)ERR_TILED_TIMEOUT);
        cp_async_wait_all();  // the gathers land before the CTA may exit
        if (lane == 0 && rpend >= 0) mbar_wait(rbar, (unsigned)rpend);
        return;
    }
    // ---------------------------------------------------------------- consumers
    int4 ta, tb, na, nb4;
    sched_of(0, ta, tb);
    for (int i = 0; ta.x >= 0; ++i, ta = na, tb = nb4) {
        sched_of(i + 1, na, nb4);
        const int yb = i & 1;
        const int u0 = ta.y, s0 = ta.z, s1 = ta.w, u1 = tb.x;
        // this thread's row of the final sums, loaded before the wait
        int rv = -1, re0 = 0, re1 = 0;
        T rsub = T(0);
        if ((int)threadIdx.x < (s1 - s0) * 32) {
            const int sl = s0 + warp;
            rv = __ldg(a.row_voxel + (long)sl * 32 + lane);
            re0 = __ldg(a.slice_unit + sl) - u0;
            re1 = __ldg(a.slice_unit + sl + 1) - u0;
            if (EPI == SPMV_SUB && rv >= 0) rsub = a.sub[rv];
        }
        // the y buffer is released only after its gathers have landed: a wait
        // that ran out (or a warp already failed) waits once more for them
        if (!(ok && __all_sync(FULL, mbar_wait(&yfull[yb], (unsigned)((i >> 1) & 1))))) {
            ok = false;
            mbar_wait(&yfull[yb], (unsigned)((i >> 1) & 1));
        }
        const T* ysm = ybuf + (size_t)yb * pa.ybuf_elems;
        if (ok) {
            for (int w = u0 + warp; w < u1; w += PIPE_CONSUMERS) {
                const int sl = __ldg(a.unit_slice + w);
                const long long off = a.slice_off[sl];
                const int len = (int)((a.slice_off[sl + 1] - off) >> 5);
                const int k0 = __ldg(a.unit_k0 + w), k1 = min(len, k0 + TILED_UNIT_K);
                const unsigned short* __restrict__ li = a.lidx + off + lane;
                const V* __restrict__ va = a.val + off + lane;
                RowAcc<T> acc;
                int k = k0;
                for (; k + U <= k1; k += U) {
                    unsigned short ii[U];
                    VV vv[U];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        ii[u] = __ldcs(li + 32 * (k + u));
                        vv[u] = (VV)Acc<VV, V>::load(va + 32 * (k + u));
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) madd(acc, vv[u], ysm[ii[u]]);
                }
                for (; k < k1; ++k) madd(acc, (VV)Acc<VV, V>::load(va + 32 * k), ysm[__ldcs(li + 32 * k)]);
                psm[(w - u0) * 32 + lane] = acc.value();
            }
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&yempty[yb]);
        named_sync(1, 32 * PIPE_CONSUMERS);  // every unit's partials are in psm
        if (ok && rv >= 0) {
            T sum = T(0);
            for (int e = re0; e < re1; ++e) sum += psm[e * 32 + lane];
            out[rv] = (EPI == SPMV_SUB) ? sum - rsub : sum;
        }
        named_sync(1, 32 * PIPE_CONSUMERS);  // psm is free for the next tile
    }
    if (!ok && lane == 0 && a.ctl) atomicOr(&a.ctl->err, (int)ERR_TILED_TIMEOUT);
    // rows without nonzeros, spread over the CTAs
    for (long z = (long)b * (32 * PIPE_CONSUMERS) + threadIdx.x; z < a.nzero; z += (long)G * (32 * PIPE_CONSUMERS)) {
        const int v = __ldg(a.zrows + z);
        out[v] = (EPI == SPMV_SUB) ? T(0) - a.sub[v] : T(0);
    }
}

// ---- slicing tables from rows sorted by key (tile << 16) | (0xffff - length):
// tiles in order, longest rows first, rows without entries last
__global__ void k_fill_value(long n, int v, int* __restrict__ a) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) a[i] = v;
}

// first[t]: the tile's first row; nzend[t]: its first row without entries
__global__ void k_tile_bounds(long N, const unsigned long long* __restrict__ key, int* __restrict__ first,
                              int* __restrict__ nzend) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
        const unsigned long long k = key[i];
        const int t = (int)(k >> 16);
        const bool head = (i == 0) || (int)(key[i - 1] >> 16) != t;
        if (head) first[t] = (int)i;
        if ((k & 0xffff) == 0xffff && (head || (key[i - 1] & 0xffff) != 0xffff)) nzend[t] = (int)i;
    }
}

// every 32nd row of a tile's rows with entries opens a slice as long as that row
__global__ void k_slice_len(long N, const unsigned long long* __restrict__ key, const int* __restrict__ first,
                            const int* __restrict__ nzend, const int* __restrict__ tsl, int* __restrict__ slen) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x) {
        const unsigned long long k = key[i];
        const int t = (int)(k >> 16);
        const long j = i - first[t];
        if ((j & 31) == 0 && i < nzend[t]) slen[tsl[t] + j / 32] = 0xffff - (int)(k & 0xffff);
    }
}

__global__ void k_empty_flags(long N, const unsigned long long* __restrict__ key, char* __restrict__ f) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < N; i += (long)gridDim.x * blockDim.x)
        f[i] = (key[i] & 0xffff) == 0xffff;
}

// Host copies of the slicing tables, computed by two passes on the device:
// first[t] (first[ntiles] = N) and nzend[t] bound tile t's rows and its rows
// with entries; tile t owns slices tsl[t] .. tsl[t+1]-1; slen[sl] is the
// length of slice sl.  first_d receives first[] for the fill kernels.
struct SliceTables {
    std::vector<int> first, nzend, tsl, slen;
};

void slice_tables(long N, int ntiles, const unsigned long long* key_s, TmpBuf<int>& first_d, cudaStream_t s,
                  SliceTables& o) {
    TmpBuf<int> nz_d(ntiles), tsl_d(ntiles + 1);
    k_fill_value<<<ewt(ntiles + 1), 256, 0, s>>>(ntiles + 1, (int)N, first_d.p);
    TV3_CUDA(cudaMemsetAsync(nz_d.p, 0xff, ntiles * sizeof(int), s));
    k_tile_bounds<<<ewt(N), 256, 0, s>>>(N, key_s, first_d.p, nz_d.p);
    TV3_CUDA(cudaGetLastError());
    o.first.assign(ntiles + 1, 0);
    o.nzend.assign(ntiles, 0);
    TV3_CUDA(cudaMemcpyAsync(o.first.data(), first_d.p, ntiles * sizeof(int), cudaMemcpyDeviceToHost, s));
    TV3_CUDA(cudaMemcpyAsync(o.nzend.data(), nz_d.p, ntiles * sizeof(int), cudaMemcpyDeviceToHost, s));
    TV3_CUDA(cudaStreamSynchronize(s));
    o.first[ntiles] = (int)N;
    // a tile without rows starts where the next one does
    for (int t = ntiles - 1; t >= 0; --t) o.first[t] = std::min(o.first[t], o.first[t + 1]);
    o.tsl.assign(ntiles + 1, 0);
    for (int t = 0; t < ntiles; ++t) {
        if (o.nzend[t] < 0) o.nzend[t] = o.first[t + 1];
        o.tsl[t + 1] = o.tsl[t] + (o.nzend[t] - o.first[t] + 31) / 32;
    }
    const int ns = o.tsl[ntiles];
    o.slen.assign(std::max(ns, 1), 0);
    TV3_CUDA(cudaMemcpyAsync(first_d.p, o.first.data(), (ntiles + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
    TV3_CUDA(cudaMemcpyAsync(nz_d.p, o.nzend.data(), ntiles * sizeof(int), cudaMemcpyHostToDevice, s));
    TV3_CUDA(cudaMemcpyAsync(tsl_d.p, o.tsl.data(), (ntiles + 1) * sizeof(int), cudaMemcpyHostToDevice, s));
    if (ns > 0) {
        TmpBuf<int> slen_d(ns);
        k_slice_len<<<ewt(N), 256, 0, s>>>(N, key_s, first_d.p, nz_d.p, tsl_d.p, slen_d.p);
        TV3_CUDA(cudaGetLastError());
        TV3_CUDA(cudaMemcpyAsync(o.slen.data(), slen_d.p, ns * sizeof(int), cudaMemcpyDeviceToHost, s));
        TV3_CUDA(cudaStreamSynchronize(s));
    }
    TV3_CUDA(cudaStreamSynchronize(s));
}

template <class T, class V>
void set_smem_attr(size_t smem) {
    const int b = (int)smem;
    TV3_CUDA(cudaFuncSetAttribute(k_spmv_tiled<T, V, SPMV_PLAIN, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
    TV3_CUDA(cudaFuncSetAttribute(k_spmv_tiled<T, V, SPMV_SUB, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, b));
}

}  // namespace

template <class T, class V>
void TiledT<T, V>::build(long n_, long m, int p, int q, int r, const int* tptr, const int* tind, const V* tval,
                         long nnz, size_t max_smem, cudaStream_t s) {
    // tile shapes, largest first: 8 x 8 x 8 voxels in 3D (16 x 16 in 2D); a
    // volume crossed by so many rays that a tile's ray list overflows shared
    // memory takes smaller tiles (fewer rays cross each)
    static const int shapes3[][3] = {{8, 8, 8}, {8, 8, 4}, {4, 4, 4}, {4, 4, 2}};
    static const int shapes2[][3] = {{16, 16, 1}, {8, 8, 1}, {4, 4, 1}};
    const bool flat = r <= 1;
    const int ns = flat ? 3 : 4;
    for (int i = 0; i < ns && !ok; ++i) {
        const int* sh = flat ? shapes2[i] : shapes3[i];
        build_shape(n_, m, p, q, r, tptr, tind, tval, nnz, max_smem, s, sh[0], sh[1], sh[2]);
    }
}

template <class T, class V>
void TiledT<T, V>::build_shape(long n_, long m, int p, int q, int r, const int* tptr, const int* tind, const V* tval,
                               long nnz, size_t max_smem, cudaStream_t s, int ty0, int tx0, int tz0) {
    ok = false;
    n = n_;
    if (nnz <= 0 || n <= 0 || m <= 0 || (long)p * q * r != n || nnz >= (1L << 31)) return;
    const int ty = std::min(p, ty0), tx = std::min(q, tx0), tz = std::min(r, tz0);
    const int nty = (p + ty - 1) / ty, ntx = (q + tx - 1) / tx, ntz = (r + tz - 1) / tz;
    const long nt = (long)nty * ntx * ntz;
    if (nt >= (1L << 24) || (long)ty * tx * tz > 512) return;  // the kernel gives each row of a tile one thread
    ntiles = (int)nt;

    // ---- (tile, ray) keys of every nonzero, sorted: the tiles' ray lists
    TmpBuf<int> tile_of(n), iota(n), tile_first(ntiles);
    TmpBuf<unsigned short> local_of(nnz);
    int nuniq = 0;
    {
        TmpBuf<int> rowof(nnz), idx(nnz), idx_s(nnz), newray(nnz), uniq(nnz);
        TmpBuf<unsigned long long> key(nnz), key_s(nnz);
        k_tile_of_voxel<<<ewt(n), 256, 0, s>>>(n, p, q, ty, tx, tz, nty, ntx, tile_of.p, iota.p);
        k_rows_of<<<ewt(n * 32), 256, 0, s>>>(n, tptr, rowof.p);
        const int ray_bits = index_bits(m), end_bit = ray_bits + index_bits(ntiles);
        k_keys<<<ewt(nnz), 256, 0, s>>>(nnz, rowof.p, tind, tile_of.p, ray_bits, key.p, idx.p);
        TV3_CUDA(cudaGetLastError());
        size_t tb = 0;
        TV3_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, key.p, key_s.p, idx.p, idx_s.p, (int)nnz, 0, end_bit, s));
        {
            TmpBuf<char> tmp(std::max<size_t>(tb, 1));
            TV3_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, key.p, key_s.p, idx.p, idx_s.p, (int)nnz, 0, end_bit,
                                                     s));
            TV3_CUDA(cudaStreamSynchronize(s));
        }
        TV3_CUDA(cudaMemsetAsync(tile_first.p, 0xff, ntiles * sizeof(int), s));
        k_flags<<<ewt(nnz), 256, 0, s>>>(nnz, key_s.p, ray_bits, newray.p, tile_first.p);
        size_t sb = 0;
        TV3_CUDA(cub::DeviceScan::InclusiveSum(nullptr, sb, newray.p, uniq.p, (int)nnz, s));
        {
            TmpBuf<char> tmp(std::max<size_t>(sb, 1));
            TV3_CUDA(cub::DeviceScan::InclusiveSum(tmp.p, sb, newray.p, uniq.p, (int)nnz, s));
            TV3_CUDA(cudaStreamSynchronize(s));
        }
        TV3_CUDA(cudaMemcpy(&nuniq, uniq.p + nnz - 1, sizeof(int), cudaMemcpyDeviceToHost));
        rays.alloc(std::max(nuniq, 1));
        k_local<<<ewt(nnz), 256, 0, s>>>(nnz, key_s.p, ray_bits, uniq.p, idx_s.p, tile_first.p, rays.p, local_of.p);
        TV3_CUDA(cudaGetLastError());
        // per-tile ray offsets: start of tile t's list = uniq[tile_first[t]] - 1;
        // a tile without nonzeros takes the next tile's start
        std::vector<int> roff(ntiles + 1, 0);
        TmpBuf<int> st(ntiles);
        k_tile_start<<<ewt(ntiles), 256, 0, s>>>(ntiles, tile_first.p, uniq.p, st.p);
        std::vector<int> start(ntiles);
        TV3_CUDA(cudaMemcpyAsync(start.data(), st.p, ntiles * sizeof(int), cudaMemcpyDeviceToHost, s));
        TV3_CUDA(cudaStreamSynchronize(s));
        roff[ntiles] = nuniq;
        for (int t = ntiles - 1; t >= 0; --t) roff[t] = (start[t] >= 0) ? start[t] : roff[t + 1];
        max_rays = 0;
        for (int t = 0; t < ntiles; ++t) max_rays = std::max(max_rays, roff[t + 1] - roff[t]);
        if (max_rays > 65535 || (size_t)max_rays * sizeof(T) > max_smem) {
            rays.release();
            return;
        }
        ray_off.alloc(ntiles + 1);
        TV3_CUDA(cudaMemcpy(ray_off.p, roff.data(), (ntiles + 1) * sizeof(int), cudaMemcpyHostToDevice));
    }

    // ---- rows sorted by (tile, length descending), cut into slices of 32
    TmpBuf<unsigned long long> rkey(n), rkey_s(n);
    TmpBuf<int> vox(n), too_long(1);
    TV3_CUDA(cudaMemsetAsync(too_long.p, 0, sizeof(int), s));
    k_row_keys<<<ewt(n), 256, 0, s>>>(n, tile_of.p, tptr, rkey.p, iota.p, too_long.p);
    int rbits = 17;
    while (rbits < 64 && (1LL << (rbits - 16)) < ntiles) ++rbits;
    size_t rb = 0;
    TV3_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, rb, rkey.p, rkey_s.p, iota.p, vox.p, (int)n, 0, rbits, s));
    {
        TmpBuf<char> tmp(std::max<size_t>(rb, 1));
        TV3_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, rb, rkey.p, rkey_s.p, iota.p, vox.p, (int)n, 0, rbits, s));
        TV3_CUDA(cudaStreamSynchronize(s));
    }
    int tl = 0;
    TV3_CUDA(cudaMemcpy(&tl, too_long.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (tl) {
        rays.release();
        ray_off.release();
        return;
    }
    // slices: each tile's rows with entries in runs of 32; the rows without
    // entries (sorted last in their tile) go to one list of voxels whose
    // result is 0 (or -sub), in row order
    TmpBuf<int> trow_d(ntiles + 1);
    SliceTables st;
    slice_tables(n, ntiles, rkey_s.p, trow_d, s, st);
    std::vector<int>& tsl = st.tsl;
    nslices = tsl[ntiles];
    std::vector<long long> soff(nslices + 1, 0);
    for (int sl = 0; sl < nslices; ++sl) soff[sl + 1] = soff[sl] + 32LL * st.slen[sl];
    long nz = 0;
    for (int t = 0; t < ntiles; ++t) nz += st.first[t + 1] - st.nzend[t];
    nzero = nz;
    zrows.alloc(std::max<long>(nzero, 1));
    if (nzero) {
        TmpBuf<char> flags(n);
        TmpBuf<int> nsel(1);
        k_empty_flags<<<ewt(n), 256, 0, s>>>(n, rkey_s.p, flags.p);
        size_t fb = 0;
        TV3_CUDA(cub::DeviceSelect::Flagged(nullptr, fb, vox.p, flags.p, zrows.p, nsel.p, (int)n, s));
        TmpBuf<char> tmp(std::max<size_t>(fb, 1));
        TV3_CUDA(cub::DeviceSelect::Flagged(tmp.p, fb, vox.p, flags.p, zrows.p, nsel.p, (int)n, s));
        TV3_CUDA(cudaStreamSynchronize(s));
    }
    // tiles with work, largest first: the longest tiles start in the first
    // wave and the last wave is made of the smallest ones
    {
        std::vector<std::pair<long long, int>> w;
        for (int t = 0; t < ntiles; ++t)
            if (tsl[t + 1] > tsl[t]) w.push_back({-(soff[tsl[t + 1]] - soff[tsl[t]]), t});
        std::sort(w.begin(), w.end());
        std::vector<int> o(w.size());
        for (size_t i = 0; i < w.size(); ++i) o[i] = w[i].second;
        nwork = (int)o.size();
        tile_order.alloc(std::max(nwork, 1));
        if (nwork) TV3_CUDA(cudaMemcpy(tile_order.p, o.data(), nwork * sizeof(int), cudaMemcpyHostToDevice));
    }
    // work units of at most TILED_UNIT_K steps per slice (a slice of length 0 still gets one)
    std::vector<int> uslice, tunit(ntiles + 1, 0), sunit(nslices + 1, 0);
    std::vector<unsigned short> uk0;
    max_units = 0;
    for (int t = 0; t < ntiles; ++t) {
        tunit[t] = (int)uslice.size();
        for (int sl = tsl[t]; sl < tsl[t + 1]; ++sl) {
            sunit[sl] = (int)uslice.size();
            const long len = (soff[sl + 1] - soff[sl]) / 32;
            for (long k0 = 0; k0 < std::max(len, 1L); k0 += TILED_UNIT_K) {
                uslice.push_back(sl);
                uk0.push_back((unsigned short)k0);
            }
        }
        max_units = std::max(max_units, (int)uslice.size() - tunit[t]);
    }
    tunit[ntiles] = (int)uslice.size();
    sunit[nslices] = (int)uslice.size();
    if ((size_t)max_rays * sizeof(T) + (size_t)max_units * 32 * sizeof(T) > max_smem) {
        rays.release();
        ray_off.release();
        return;
    }
    nunits = (int)uslice.size();
    {
        std::vector<longlong2> desc(std::max(nunits, 1), make_longlong2(0, 0));
        for (int u = 0; u < nunits; ++u) {
            const int sl = uslice[u];
            const long long len = (soff[sl + 1] - soff[sl]) / 32;
            const long long k0 = uk0[u], k1 = std::min(len, k0 + (long long)TILED_UNIT_K);
            desc[u] = make_longlong2(soff[sl] + 32LL * k0, std::max(k1 - k0, 0LL));
        }
        unit_desc.alloc(desc.size());
        TV3_CUDA(cudaMemcpy(unit_desc.p, desc.data(), desc.size() * sizeof(longlong2), cudaMemcpyHostToDevice));
    }
    tile_unit.alloc(ntiles + 1);
    slice_unit.alloc(nslices + 1);
    unit_slice.alloc(std::max(nunits, 1));
    unit_k0.alloc(std::max(nunits, 1));
    TV3_CUDA(cudaMemcpy(tile_unit.p, tunit.data(), (ntiles + 1) * sizeof(int), cudaMemcpyHostToDevice));
    TV3_CUDA(cudaMemcpy(slice_unit.p, sunit.data(), (nslices + 1) * sizeof(int), cudaMemcpyHostToDevice));
    if (nunits) {
        TV3_CUDA(cudaMemcpy(unit_slice.p, uslice.data(), nunits * sizeof(int), cudaMemcpyHostToDevice));
        TV3_CUDA(cudaMemcpy(unit_k0.p, uk0.data(), nunits * sizeof(unsigned short), cudaMemcpyHostToDevice));
    }
    const long long padded = soff.back();
    tile_slice.alloc(ntiles + 1);
    slice_off.alloc(nslices + 1);
    TV3_CUDA(cudaMemcpy(tile_slice.p, tsl.data(), (ntiles + 1) * sizeof(int), cudaMemcpyHostToDevice));
    TV3_CUDA(cudaMemcpy(slice_off.p, soff.data(), (nslices + 1) * sizeof(long long), cudaMemcpyHostToDevice));
    lidx.alloc(std::max<long long>(padded, 1));
    val.alloc(std::max<long long>(padded, 1));
    row_voxel.alloc((size_t)std::max(nslices, 1) * 32);
    TV3_CUDA(cudaMemsetAsync(lidx.p, 0, std::max<long long>(padded, 1) * sizeof(unsigned short), s));
    TV3_CUDA(cudaMemsetAsync(val.p, 0, std::max<long long>(padded, 1) * sizeof(V), s));
    TV3_CUDA(cudaMemsetAsync(row_voxel.p, 0xff, (size_t)std::max(nslices, 1) * 32 * sizeof(int), s));
    k_fill_slices<V><<<ewt(n), 256, 0, s>>>(n, rkey_s.p, vox.p, trow_d.p, tile_slice.p, slice_off.p, tptr, local_of.p,
                                            tval, lidx.p, val.p, row_voxel.p);
    TV3_CUDA(cudaGetLastError());
    padded_entries = padded;
    // the attribute is per kernel, shared by every operator: always the full budget
    set_smem_attr<T, V>(max_smem);
    // kept for the pipelined form, built on first use
    h_tsl = std::move(tsl);
    h_tunit = std::move(tunit);
    pipe_tried = false;
    pipe_ok = false;
    TV3_CUDA(cudaStreamSynchronize(s));
    ok = true;
}

// Tile records and padded ray lists of the pipelined form, when its shared
// memory (two y buffers, the ray list and the unit partials) fits one CTA.
template <class T, class V>
bool TiledT<T, V>::ensure_pipe() const {
    if (!pipe_tried) {
        pipe_tried = true;
        if (ok) const_cast<TiledT*>(this)->build_pipe();
    }
    return pipe_ok;
}

template <class T, class V>
void TiledT<T, V>::build_pipe() {
    const std::vector<int>& tsl = h_tsl;
    const std::vector<int>& tunit = h_tunit;
    pipe_ok = false;
    if (!(std::is_same<V, float>::value || std::is_same<V, double>::value) || ntiles <= 0) return;
    int dev = 0, optin = 0;
    TV3_CUDA(cudaGetDevice(&dev));
    TV3_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
    const int ybe = (max_rays + 3) & ~3;
    const size_t smem = 64 + 2 * (size_t)ybe * sizeof(T) + (size_t)ybe * 4 + (size_t)max_units * 32 * sizeof(T);
    if (smem > (size_t)optin) return;
    // ray lists starting at multiples of four entries (16-byte bulk copies)
    std::vector<int> roff(ntiles + 1);
    TV3_CUDA(cudaMemcpy(roff.data(), ray_off.p, (ntiles + 1) * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<int> hr(std::max(roff[ntiles], 1));
    if (roff[ntiles] > 0)
        TV3_CUDA(cudaMemcpy(hr.data(), rays.p, roff[ntiles] * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<int> rpo(ntiles), rp;
    for (int t = 0; t < ntiles; ++t) {
        rpo[t] = (int)rp.size();
        for (int j = roff[t]; j < roff[t + 1]; ++j) rp.push_back(hr[j]);
        while (rp.size() % 4) rp.push_back(0);
    }
    if (rp.empty()) rp.assign(4, 0);
    // per position of the largest-first order: the tile's two records
    std::vector<int> ord(std::max(nwork, 1));
    if (nwork) TV3_CUDA(cudaMemcpy(ord.data(), tile_order.p, nwork * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<int4> sc(2 * (size_t)std::max(nwork, 1), make_int4(0, 0, 0, 0));
    for (int k = 0; k < nwork; ++k) {
        const int t = ord[k];
        sc[2 * k] = make_int4(t, tunit[t], tsl[t], tsl[t + 1]);
        sc[2 * k + 1] = make_int4(tunit[t + 1], 0, roff[t + 1] - roff[t], rpo[t]);
    }
    sched.alloc(sc.size());
    TV3_CUDA(cudaMemcpy(sched.p, sc.data(), sc.size() * sizeof(int4), cudaMemcpyHostToDevice));
    rays_pad.alloc(rp.size());
    TV3_CUDA(cudaMemcpy(rays_pad.p, rp.data(), rp.size() * sizeof(int), cudaMemcpyHostToDevice));
    TV3_CUDA(cudaFuncSetAttribute(k_spmv_tiled_pipe<T, V, SPMV_PLAIN, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  optin));
    TV3_CUDA(cudaFuncSetAttribute(k_spmv_tiled_pipe<T, V, SPMV_SUB, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  optin));
    pipe_ybe = ybe;
    pipe_smem = smem;
    pipe_ok = true;
}

template <class T, class V>
void TiledT<T, V>::apply_pipe(const TiledArgs<T, V>& a, int epi, cudaStream_t s) const {
    if (!pipe_ok || a.xscale) {
        apply(a, epi, s);
        return;
    }
    TiledArgs<T, V> b = a;
    b.tile_order = tile_order.p;
    b.nwork = nwork;
    b.zrows = zrows.p;
    b.nzero = nzero;
    PipeArgs pa{sched.p, rays_pad.p, pipe_ybe};
    const int grid = std::max(1, num_sms());
    const int threads = 32 * (PIPE_CONSUMERS + 1);
    if (epi == SPMV_SUB) launch_k(k_spmv_tiled_pipe<T, V, SPMV_SUB, 8>, dim3(grid), dim3(threads), pipe_smem, s, b, pa);
    else launch_k(k_spmv_tiled_pipe<T, V, SPMV_PLAIN, 8>, dim3(grid), dim3(threads), pipe_smem, s, b, pa);
    TV3_CUDA(cudaGetLastError());
}

template <class T, class V>
void TiledT<T, V>::apply(const TiledArgs<T, V>& a, int epi, cudaStream_t s) const {
    const size_t smem = std::max<size_t>(((size_t)max_rays + (size_t)max_units * 32) * sizeof(T), 16);
    TiledArgs<T, V> b = a;
    b.tile_order = tile_order.p;
    b.nwork = nwork;
    b.zrows = zrows.p;
    b.nzero = nzero;
    b.unit_desc = unit_desc.p;
    const long grid = std::max<long>((long)nwork, 1);
    if (epi == SPMV_SUB) launch_k(k_spmv_tiled<T, V, SPMV_SUB, 8>, dim3((unsigned)grid), dim3(512), smem, s, b);
    else launch_k(k_spmv_tiled<T, V, SPMV_PLAIN, 8>, dim3((unsigned)grid), dim3(512), smem, s, b);
    TV3_CUDA(cudaGetLastError());
}

// ---------------------------------------------------------------------------
// tile-staged A*x
// ---------------------------------------------------------------------------
namespace {

// (tile, ray) keys, the ray in the low rb bits
__global__ void k_n_keys(long nnz, const int* __restrict__ rowof, const int* __restrict__ ind,
                         const int* __restrict__ tile_of, int rb, unsigned long long* __restrict__ key,
                         int* __restrict__ idx) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x) {
        key[k] = ((unsigned long long)(unsigned)tile_of[ind[k]] << rb) | (unsigned)rowof[k];
        idx[k] = (int)k;
    }
}

__global__ void k_n_newseg(long nnz, const unsigned long long* __restrict__ key, int* __restrict__ f) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x)
        f[k] = (k == 0 || key[k - 1] != key[k]) ? 1 : 0;
}

// per segment: its (tile, ray) key and first position in the sorted entries
__global__ void k_n_segs(long nnz, const unsigned long long* __restrict__ key, const int* __restrict__ segid,
                         unsigned long long* __restrict__ seg_key, int* __restrict__ seg_start) {
    for (long k = (long)blockIdx.x * blockDim.x + threadIdx.x; k < nnz; k += (long)gridDim.x * blockDim.x)
        if (k == 0 || key[k - 1] != key[k]) {
            seg_key[segid[k] - 1] = key[k];
            seg_start[segid[k] - 1] = (int)k;
        }
}

// segment keys for the slicing sort (tile, longest first) and the ray-major sort (ray, tile)
__global__ void k_n_segkeys(long nseg, const unsigned long long* __restrict__ seg_key, const int* __restrict__ seg_start,
                            long nnz, int rb, int tb, unsigned long long* __restrict__ k_slice,
                            unsigned long long* __restrict__ k_ray, int* __restrict__ iota, int* __restrict__ too_long) {
    for (long s = (long)blockIdx.x * blockDim.x + threadIdx.x; s < nseg; s += (long)gridDim.x * blockDim.x) {
        const unsigned long long c = seg_key[s];
        const long end = (s + 1 < nseg) ? seg_start[s + 1] : nnz;
        long len = end - seg_start[s];
        if (len > 0xffff) {
            *too_long = 1;
            len = 0xffff;
        }
        const unsigned tile = (unsigned)(c >> rb), ray = (unsigned)(c & ((1ull << rb) - 1));
        k_slice[s] = ((unsigned long long)tile << 16) | (unsigned)(0xffff - len);
        k_ray[s] = ((unsigned long long)ray << tb) | tile;
        iota[s] = (int)s;
    }
}

// partials per lane that the per-ray reduction stages in shared memory
constexpr int RED_K0 = 16;

__global__ void k_n_count(long nseg, const unsigned long long* __restrict__ k_ray_s, int tb, int* __restrict__ rcount) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nseg; i += (long)gridDim.x * blockDim.x)
        atomicAdd(rcount + (k_ray_s[i] >> tb), 1);
}

// Layout of the partials.  The rays of each window of 256 consecutive rays are
// ranked by their number of partials (longest first, ties by ray), and the
// rank gives each ray a slot: slot 256 w + rank.  Slots 32G .. 32G+31 form
// group G, whose partials are interleaved: partial k of the ray in slot s at
// gbase[G] + 32 k + s % 32, the group padded to its longest ray (rays of
// similar length share a group, so the padding is small).
__global__ void __launch_bounds__(256) k_n_slots(long m, const int* __restrict__ rcount, int* __restrict__ rslot,
                                                 int* __restrict__ sray, int* __restrict__ slen) {
    __shared__ int wl[256];
    const long r = (long)blockIdx.x * 256 + threadIdx.x;
    const int len = (r < m) ? rcount[r] : -1;
    wl[threadIdx.x] = len;
    __syncthreads();
    if (r >= m) return;
    int rank = 0;
    for (int j = 0; j < 256; ++j) {
        const int lj = wl[j];
        rank += (lj > len) || (lj == len && j < (int)threadIdx.x);
    }
    const long sl = (long)blockIdx.x * 256 + rank;
    rslot[r] = (int)sl;
    sray[sl] = (int)r;
    slen[sl] = len;
}

__global__ void k_n_group_len(long m, const int* __restrict__ slen, long long* __restrict__ glen) {
    const long ng = (m + 31) / 32;
    for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < ng; g += (long)gridDim.x * blockDim.x) {
        int mx = 0;
        for (long sl = 32 * g; sl < min(m, 32 * g + 32); ++sl) mx = max(mx, slen[sl]);
        glen[g] = 32LL * mx;
    }
}

// destination of each segment's partial; the ray-major order i (ray, then
// tile) gives the segment's place k = i - rseg[ray] among its ray's partials
__global__ void k_n_dest(long nseg, const int* __restrict__ by_ray, const unsigned long long* __restrict__ k_ray_s,
                         int tb, const int* __restrict__ rseg, const int* __restrict__ rslot,
                         const long long* __restrict__ gbase, int* __restrict__ dest) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nseg; i += (long)gridDim.x * blockDim.x) {
        const long ray = (long)(k_ray_s[i] >> tb);
        const long sl = rslot[ray];
        dest[by_ray[i]] = (int)(gbase[sl >> 5] + 32LL * (i - rseg[ray]) + (sl & 31));
    }
}

template <class V>
__global__ void k_n_fill(long nseg, const int* __restrict__ order, const unsigned long long* __restrict__ k_slice_s,
                         const int* __restrict__ tile_seg0, const int* __restrict__ tile_slice,
                         const long long* __restrict__ slice_off, const int* __restrict__ seg_start, long nnz,
                         const int* __restrict__ idx_s, const int* __restrict__ ind, const V* __restrict__ valin,
                         const int* __restrict__ dest, int p, int q, int ty, int tx, int tz,
                         unsigned short* __restrict__ lidx, V* __restrict__ val, int* __restrict__ slot_dest) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < nseg; i += (long)gridDim.x * blockDim.x) {
        const int sid = order[i];
        const int t = (int)(k_slice_s[i] >> 16);
        const int j = (int)(i - tile_seg0[t]);
        const int sl = tile_slice[t] + j / 32, lane = j % 32;
        slot_dest[(long)sl * 32 + lane] = dest[sid];
        const long long o = slice_off[sl] + lane;
        const long b0 = seg_start[sid], b1 = (sid + 1 < nseg) ? seg_start[sid + 1] : nnz;
        for (long k = b0; k < b1; ++k) {
            const int e = idx_s[k];
            const long v = ind[e];
            const long y = v % p, x = (v / p) % q, z = v / ((long)p * q);
            lidx[o + 32LL * (k - b0)] = (unsigned short)((y % ty) + ty * ((x % tx) + tx * (z % tz)));
            val[o + 32LL * (k - b0)] = valin[e];
        }
    }
}

// a matrix value read from shared memory, in the accumulation type
__device__ __forceinline__ float smem_val(float v) { return v; }
__device__ __forceinline__ double smem_val(double v) { return v; }
__device__ __forceinline__ float smem_val(__nv_bfloat16 v) { return __bfloat162float(v); }
__device__ __forceinline__ float smem_val(__half v) { return __half2float(v); }

constexpr size_t align128(size_t b) { return (b + 127) & ~(size_t)127; }
// one stage: positions, values, the slices' destinations (32 each), places
constexpr size_t BULK_LB = align128((size_t)BULK_CHUNK * 2);
template <class V> constexpr size_t bulk_val_bytes() { return align128((size_t)BULK_CHUNK * sizeof(V)); }
constexpr size_t BULK_DB = (size_t)BULK_MAXS * 32 * 4;
template <class V> constexpr size_t bulk_stage_bytes() {
    return BULK_LB + bulk_val_bytes<V>() + BULK_DB + (size_t)BULK_MAXS * 16;
}

// x values of tile t into xs (shared memory) by asynchronous copies; voxels
// outside the volume (boundary tiles) are zero
template <class T, class V>
__device__ __forceinline__ void stage_x_async(const TiledNArgs<T, V>& a, const T* __restrict__ x, int t, T* xs) {
    const int tvox = a.ty * a.tx * a.tz;
    const int tzi = t / (a.nty * a.ntx), rem = t - tzi * a.nty * a.ntx, txi = rem / a.nty, tyi = rem - txi * a.nty;
    const long y0 = (long)tyi * a.ty, x0 = (long)txi * a.tx, z0 = (long)tzi * a.tz;
    for (int j = threadIdx.x; j < tvox; j += 32 * BULK_NC) {
        const int ly = j % a.ty, lx = (j / a.ty) % a.tx, lz = j / (a.ty * a.tx);
        const long yy = y0 + ly, xx = x0 + lx, zz = z0 + lz;
        if (yy < a.p && xx < a.q && zz < a.r) cp_async<(int)sizeof(T)>(xs + j, x + yy + (long)a.p * (xx + (long)a.q * zz));
        else xs[j] = T(0);
    }
    cp_async_commit();
}

// Tile-staged A*x.  A persistent CTA of BULK_NC consumer warps and one
// producer warp takes the tiles with segments in largest-first order,
// snaking over the CTAs (position k*G + b for even k, k*G + G-1-b for odd
// k).  The tiles' slices are consecutive in memory; the producer (one lane)
// bulk-copies them chunk by chunk, across tile boundaries, into a ring of
// BULK_STAGES shared-memory stages (positions, values, and the chunk's
// per-slice destinations and places; mbarrier full[s] counts the bytes), so
// the matrix stream stays in flight without registers or per-warp load
// chains and without draining between tiles.  The consumers keep two x
// buffers: while they sum tile k, the x values of tile k+1 arrive by
// asynchronous copies.  A chunk's slice j goes to warp j mod BULK_NC (one
// segment per lane, steps in order); the warp releases the stage (mbarrier
// empty[s], one arrival per consumer warp).  Every wait is bounded: on a
// timeout a warp records ERR_TILED_TIMEOUT and stops computing but keeps
// releasing stages, each only after a second bounded wait for its copy, and
// the producer waits (bounded) for its last copies before it returns, so no
// copy lands in a released stage or after the CTA exits.
template <class T, class V>
__global__ void __launch_bounds__(32 * (BULK_NC + 1)) k_spmv_tiledN(TiledNArgs<T, V> a, BulkArgs bk) {
    count_launch(a.ctl);
    using VV = typename TVT<V>::type;
    constexpr int S = BULK_STAGES, NC = BULK_NC;
    constexpr size_t VB = bulk_val_bytes<V>(), SB = bulk_stage_bytes<V>();
    extern __shared__ __align__(128) unsigned char sm_raw[];
    uint64_t* full = reinterpret_cast<uint64_t*>(sm_raw);
    uint64_t* empty = full + S;
    unsigned char* stages = sm_raw + 128;
    T* xbuf = reinterpret_cast<T*>(stages + S * SB);
    const int xstride = (a.ty * a.tx * a.tz + 1) & ~1;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int G = gridDim.x, b = blockIdx.x;
    auto tile_pos = [&](int k) { return k * G + ((k & 1) ? G - 1 - b : b); };  // this CTA's k-th tile position
    int ntl = 0;  // tiles of this CTA
    while (tile_pos(ntl) < bk.nwork) ++ntl;
    if (threadIdx.x == 0) {
        for (int i = 0; i < S; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], NC);
        }
        mbar_fence_init();
    }
    __syncthreads();
    if (warp == NC) {
        // ---- producer: one lane issues the bulk copies of every chunk of every tile
        if (lane == 0) {
            bool ok = true;
            int i = 0;  // chunks issued
            for (int k = 0; k < ntl && ok; ++k) {
                const int t = __ldg(a.tile_order + tile_pos(k));
                const int c0 = __ldg(bk.tile_chunk + t), c1 = __ldg(bk.tile_chunk + t + 1);
                for (int c = c0; c < c1; ++c, ++i) {
                    const int st = i % S;
                    if (i >= S && !mbar_wait(&empty[st], (unsigned)(((i / S) - 1) & 1))) {
                        ok = false;
                        break;
                    }
                    const long long e0 = __ldg(bk.chunk_e0 + c), ne = __ldg(bk.chunk_e0 + c + 1) - e0;
                    const int cs0 = __ldg(bk.chunk_slice + c), ns = __ldg(bk.chunk_slice + c + 1) - cs0;
                    const unsigned bl = (unsigned)(ne * 2), bv = (unsigned)(ne * sizeof(V));
                    const unsigned bd = (unsigned)ns * 128u, bi = (unsigned)ns * 16u;
                    unsigned char* dst = stages + st * SB;
                    mbar_expect_tx(&full[st], bl + bv + bd + bi);
                    bulk_g2s(dst, a.lidx + e0, bl, &full[st]);
                    bulk_g2s(dst + BULK_LB, a.val + e0, bv, &full[st]);
                    bulk_g2s(dst + BULK_LB + VB, a.slot_dest + (long)cs0 * 32, bd, &full[st]);
                    bulk_g2s(dst + BULK_LB + VB + BULK_DB, bk.slice_info + cs0, bi, &full[st]);
                }
            }
            // the last copies of each stage land before this thread (and so the CTA) exits
            for (int j = max(0, i - S); j < i; ++j)
                if (!mbar_wait(&full[j % S], (unsigned)((j / S) & 1))) ok = false;
            if (!ok && a.ctl) atomicOr(&a.ctl->err, (int)ERR_TILED_TIMEOUT);
        }
        return;
    }
    // ---- consumers
    const T* __restrict__ x = a.x[a.by_parity ? a.ctl->parity : 0];
    bool ok = true;
    int i = 0;  // chunks consumed
    if (ntl > 0) stage_x_async(a, x, __ldg(a.tile_order + tile_pos(0)), xbuf);
    for (int k = 0; k < ntl; ++k) {
        const int t = __ldg(a.tile_order + tile_pos(k));
        const int c0 = __ldg(bk.tile_chunk + t), nch = __ldg(bk.tile_chunk + t + 1) - c0;
        const int cfirst = (lane <= nch) ? __ldg(bk.chunk_slice + c0 + lane) : 0;  // lane j: chunk j's first slice
        named_sync(1, 32 * NC);  // every consumer is done with tile k-1: its x buffer is free
        if (k + 1 < ntl) {
            stage_x_async(a, x, __ldg(a.tile_order + tile_pos(k + 1)), xbuf + ((k + 1) & 1) * xstride);
            cp_async_wait_group<1>();  // this thread's copies of tile k have landed
        } else {
            cp_async_wait_group<0>();
        }
        named_sync(1, 32 * NC);  // ... and every thread's
        const T* xsm = xbuf + (k & 1) * xstride;
        for (int j = 0; j < nch; ++j, ++i) {
            const int st = i % S;
            int cs0, cs1;
            if (j < 31) {
                cs0 = __shfl_sync(FULL, cfirst, j);
                cs1 = __shfl_sync(FULL, cfirst, j + 1);
            } else {  // a tile of more than 31 chunks: read the bounds directly
                cs0 = __ldg(bk.chunk_slice + c0 + j);
                cs1 = __ldg(bk.chunk_slice + c0 + j + 1);
            }
            // a stage is released only after its copy has landed: a wait that
            // ran out (or a warp already failed) waits once more for the copy,
            // so the producer never re-arms a barrier whose phase is pending
            if (!(ok && mbar_wait(&full[st], (unsigned)((i / S) & 1)))) {
                ok = false;
                mbar_wait(&full[st], (unsigned)((i / S) & 1));
            }
            if (ok) {
                const unsigned char* base = stages + st * SB;
                const unsigned short* L = reinterpret_cast<const unsigned short*>(base);
                const V* W = reinterpret_cast<const V*>(base + BULK_LB);
                const int* D = reinterpret_cast<const int*>(base + BULK_LB + VB);
                const int4* I = reinterpret_cast<const int4*>(base + BULK_LB + VB + BULK_DB);
                for (int js = warp; js < cs1 - cs0; js += NC) {
                    const int4 info = I[js];
                    const int off = info.x, len = info.y;
                    const unsigned short* li = L + off + lane;
                    const V* wv = W + off + lane;
                    // two independent accumulations (even and odd steps), so
                    // that the dependent chain of one step is half as long
                    RowAcc<T> acc0, acc1;
                    int kk = 0;
                    for (; kk + 4 <= len; kk += 4) {
                        unsigned short ii[4];
                        VV vv[4];
#pragma unroll
                        for (int u = 0; u < 4; ++u) {
                            ii[u] = li[32 * (kk + u)];
                            vv[u] = (VV)smem_val(wv[32 * (kk + u)]);
                        }
                        madd(acc0, vv[0], xsm[ii[0]]);
                        madd(acc1, vv[1], xsm[ii[1]]);
                        madd(acc0, vv[2], xsm[ii[2]]);
                        madd(acc1, vv[3], xsm[ii[3]]);
                    }
                    for (; kk < len; ++kk) {
                        if (kk & 1) madd(acc1, (VV)smem_val(wv[32 * kk]), xsm[li[32 * kk]]);
                        else madd(acc0, (VV)smem_val(wv[32 * kk]), xsm[li[32 * kk]]);
                    }
                    combine(acc0, acc1);
                    const int d = D[js * 32 + lane];
                    if (d >= 0) a.part[d] = acc0.value();
                }
            }
            __syncwarp();
            if (lane == 0) mbar_arrive(&empty[st]);
        }
    }
    cp_async_wait_group<0>();
    if (!ok && lane == 0 && a.ctl) atomicOr(&a.ctl->err, (int)ERR_TILED_TIMEOUT);
}

// Blocks per SM of the per-ray reduction: six for float and double-float
// partials (at most 40 registers), which its shared-memory stage allows; the
// lam3/lam5 form otherwise takes 56 registers and runs four.  FP64 partials
// would spill at 40.
template <class T>
constexpr int red_min_blocks() { return std::is_same<T, double>::value ? 1 : 6; }

// Each ray's partials in tile order, one warp per group of 32 ray slots and
// one lane per slot (rays of similar length, from one window of 256 rays).
// The group's partials are interleaved (partial k of the ray in lane l's slot
// at gbase + 32 k + l), so the k-th copies of the 32 lanes are one coalesced
// row.  Each lane copies its first K0 partials into its own column of shared
// memory with asynchronous copies (all in flight at once, no registers held),
// waits for its own copies and adds them in order (for double-float partials
// a compensated sum: high parts by TwoSum, low parts and errors in one FP32
// term); longer rays load the rest directly.  Then the solver epilogues.
template <class T, class V, int EPI>
__global__ void __launch_bounds__(256, red_min_blocks<T>()) k_tiledN_reduce(TiledNArgs<T, V> a) {
    count_launch(a.ctl);
    constexpr int K0 = RED_K0;
    __shared__ T stage[8][K0][32];
    const int sel = a.by_parity ? a.ctl->parity : 0;
    T* __restrict__ y = a.y[sel];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    double acc0 = 0.0, acc1 = 0.0;
    const long nwarps = (long)gridDim.x * 8;
    for (long g = (long)blockIdx.x * 8 + warp; 32 * g < a.m; g += nwarps) {
        const long sl = 32 * g + lane;
        const long r = (sl < a.m) ? __ldg(a.sray + sl) : a.m;  // the slot's ray
        const int len = (sl < a.m) ? __ldg(a.rlen + sl) : 0;
        const T* __restrict__ pp = a.part + __ldg(a.gbase + g) + lane;
#pragma unroll
        for (int u = 0; u < K0; ++u)
            if (u < len) cp_async<(int)sizeof(T)>(&stage[warp][u][lane], pp + 32 * u);
        cp_async_commit();
        // the epilogue's inputs, loaded before the sums so their latency overlaps them
        T eb = T(0), ed = T(0);
        float esc = 1.f;
        if (r < a.m) {
            if (EPI == SPMV_LAM35) {
                eb = a.b[r];
                ed = a.delta[r];
            } else if (EPI == SPMV_SUB) {
                eb = a.sub[r];
            }
            if (a.rscale) esc = __ldg(a.rscale + r);
        }
        RowAcc<T> acc;
        cp_async_wait_group<0>();  // this lane's copies have landed
        const int l0 = min(len, K0);
        for (int u = 0; u < l0; ++u) add(acc, stage[warp][u][lane]);
        for (int k = K0; k < len; k += 8) {
            T v[8];
#pragma unroll
            for (int u = 0; u < 8; ++u) v[u] = (k + u < len) ? pp[32 * (k + u)] : T(0);
#pragma unroll
            for (int u = 0; u < 8; ++u)
                if (k + u < len) add(acc, v[u]);
        }
        T s = acc.value();
        if (r < a.m) {
            if (a.rscale) s *= (T)esc;
            if (EPI == SPMV_PLAIN) {
                y[r] = s;
            } else if (EPI == SPMV_SUB) {
                y[r] = s - eb;
            } else if (EPI == SPMV_LAM35) {
                y[r] = s;
                double t = acc_d(to_acc(s) - to_acc(eb));
                acc0 += t * t;
                acc1 += acc_d(to_acc(ed)) * t;
            } else if (EPI == SPMV_NORM2) {
                const double sd = acc_d(to_acc(s));
                acc0 += sd * sd;
            }
        }
    }
    if (EPI == SPMV_LAM35 || EPI == SPMV_NORM2) {
        double v[2] = {acc0, acc1}, tot[2];
        if (grid_reduce<2>(v, a.rpart, a.ticket, tot) && threadIdx.x == 0) {
            Ctl* c = a.ctl;
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

}  // namespace

template <class T, class V>
void TiledN<T, V>::build(long m_, int p_, int q_, int r_, const int* ptr, const int* ind, const V* valin, long nnz,
                         cudaStream_t s) {
    ok = false;
    m = m_; p = p_; q = q_; r = r_;
    const long n = (long)p * q * r;
    if (nnz <= 0 || n <= 0 || m <= 0 || nnz >= (1L << 31) || m >= (1L << 31)) return;
    // tile shape: 8 x 8 x 8 voxels in 3D (16 x 16 in 2D); a volume with many
    // more tiles than the SMs can use takes 16 x 8 x 8 tiles, which halve the
    // (ray, tile) segments and so the partials written and re-read, while
    // still leaving dozens of tiles per SM for the load balance
    ty = std::min(p, r > 1 ? 8 : 16); tx = std::min(q, r > 1 ? 8 : 16); tz = std::min(r, 8);
    if (r > 1) {
        const long n8 = (long)((p + 7) / 8) * ((q + 7) / 8) * ((r + 7) / 8);
        if (n8 >= 48L * num_sms()) ty = std::min(p, 16);
    }
    nty = (p + ty - 1) / ty; ntx = (q + tx - 1) / tx;
    const int ntz = (r + tz - 1) / tz;
    const long nt = (long)nty * ntx * ntz;
    if (nt >= (1L << 24) || (long)ty * tx * tz > 65535) return;
    ntiles = (int)nt;

    // entries sorted by (tile, ray), ray order kept inside each segment
    TmpBuf<int> tile_of(n), iota_v(n), rowof(nnz), idx(nnz), idx_s(nnz), flag(nnz), segid(nnz);
    TmpBuf<unsigned long long> key(nnz), key_s(nnz);
    k_tile_of_voxel<<<ewt(n), 256, 0, s>>>(n, p, q, ty, tx, tz, nty, ntx, tile_of.p, iota_v.p);
    k_rows_of<<<ewt(m * 32), 256, 0, s>>>(m, ptr, rowof.p);
    const int ray_bits = index_bits(m), tile_bits = index_bits(ntiles), end_bit = ray_bits + tile_bits;
    k_n_keys<<<ewt(nnz), 256, 0, s>>>(nnz, rowof.p, ind, tile_of.p, ray_bits, key.p, idx.p);
    TV3_CUDA(cudaGetLastError());
    {
        size_t tb = 0;
        TV3_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, key.p, key_s.p, idx.p, idx_s.p, (int)nnz, 0, end_bit, s));
        TmpBuf<char> tmp(std::max<size_t>(tb, 1));
        TV3_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, key.p, key_s.p, idx.p, idx_s.p, (int)nnz, 0, end_bit, s));
        TV3_CUDA(cudaStreamSynchronize(s));
    }
    key.release();
    idx.release();
    k_n_newseg<<<ewt(nnz), 256, 0, s>>>(nnz, key_s.p, flag.p);
    {
        size_t sb = 0;
        TV3_CUDA(cub::DeviceScan::InclusiveSum(nullptr, sb, flag.p, segid.p, (int)nnz, s));
        TmpBuf<char> tmp(std::max<size_t>(sb, 1));
        TV3_CUDA(cub::DeviceScan::InclusiveSum(tmp.p, sb, flag.p, segid.p, (int)nnz, s));
        TV3_CUDA(cudaStreamSynchronize(s));
    }
    int ns = 0;
    TV3_CUDA(cudaMemcpy(&ns, segid.p + nnz - 1, sizeof(int), cudaMemcpyDeviceToHost));
    nseg = ns;
    TmpBuf<unsigned long long> seg_key(nseg), k_slice(nseg), k_slice_s(nseg), k_ray(nseg), k_ray_s(nseg);
    TmpBuf<int> seg_start(nseg), iota_s(nseg), order(nseg), by_ray(nseg), dest(nseg), too_long(1);
    k_n_segs<<<ewt(nnz), 256, 0, s>>>(nnz, key_s.p, segid.p, seg_key.p, seg_start.p);
    TV3_CUDA(cudaMemsetAsync(too_long.p, 0, sizeof(int), s));
    k_n_segkeys<<<ewt(nseg), 256, 0, s>>>(nseg, seg_key.p, seg_start.p, nnz, ray_bits, tile_bits, k_slice.p, k_ray.p,
                                          iota_s.p, too_long.p);
    // slicing order: (tile, longest first), stable
    int sbits = 17;
    while (sbits < 64 && (1LL << (sbits - 16)) < ntiles) ++sbits;
    {
        size_t tb = 0;
        TV3_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, k_slice.p, k_slice_s.p, iota_s.p, order.p, (int)nseg, 0,
                                                 sbits, s));
        TmpBuf<char> tmp(std::max<size_t>(tb, 1));
        TV3_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, k_slice.p, k_slice_s.p, iota_s.p, order.p, (int)nseg, 0,
                                                 sbits, s));
        TV3_CUDA(cudaStreamSynchronize(s));
    }
    // segments in (ray, tile) order: each ray's partials are numbered in tile order
    const int rbits = ray_bits + tile_bits;
    {
        size_t tb = 0;
        TV3_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, tb, k_ray.p, k_ray_s.p, iota_s.p, by_ray.p, (int)nseg, 0,
                                                 rbits, s));
        TmpBuf<char> tmp(std::max<size_t>(tb, 1));
        TV3_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, tb, k_ray.p, k_ray_s.p, iota_s.p, by_ray.p, (int)nseg, 0,
                                                 rbits, s));
        TV3_CUDA(cudaStreamSynchronize(s));
    }
    int tl = 0;
    TV3_CUDA(cudaMemcpy(&tl, too_long.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (tl) return;
    TmpBuf<int> rcnt(m + 1), rseg(m + 1), rslot(std::max<long>(m, 1));
    TV3_CUDA(cudaMemsetAsync(rcnt.p, 0, (m + 1) * sizeof(int), s));
    k_n_count<<<ewt(nseg), 256, 0, s>>>(nseg, k_ray_s.p, tile_bits, rcnt.p);
    const long ngroups = (m + 31) / 32;
    sray.alloc(std::max<long>(m, 1));
    rlen.alloc(std::max<long>(m, 1));
    if (m > 0) k_n_slots<<<(int)((m + 255) / 256), 256, 0, s>>>(m, rcnt.p, rslot.p, sray.p, rlen.p);
    TmpBuf<long long> glen(ngroups + 1);
    gbase.alloc(ngroups + 1);
    TV3_CUDA(cudaMemsetAsync(glen.p + ngroups, 0, sizeof(long long), s));
    k_n_group_len<<<ewt(ngroups), 256, 0, s>>>(m, rlen.p, glen.p);
    {
        size_t sb = 0, sg = 0;
        TV3_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, sb, rcnt.p, rseg.p, (int)(m + 1), s));
        TV3_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, sg, glen.p, gbase.p, (int)(ngroups + 1), s));
        TmpBuf<char> tmp(std::max<size_t>(std::max(sb, sg), 1));
        TV3_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, sb, rcnt.p, rseg.p, (int)(m + 1), s));
        TV3_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, sg, glen.p, gbase.p, (int)(ngroups + 1), s));
        TV3_CUDA(cudaStreamSynchronize(s));
    }
    long long npart = 0;
    TV3_CUDA(cudaMemcpy(&npart, gbase.p + ngroups, sizeof(long long), cudaMemcpyDeviceToHost));
    if (npart >= (1LL << 31)) return;  // destinations are int
    k_n_dest<<<ewt(nseg), 256, 0, s>>>(nseg, by_ray.p, k_ray_s.p, tile_bits, rseg.p, rslot.p, gbase.p, dest.p);
    // slices: each tile's segments in runs of 32 (every segment has entries)
    TmpBuf<int> tseg_d(ntiles + 1);
    SliceTables st;
    slice_tables(nseg, ntiles, k_slice_s.p, tseg_d, s, st);
    std::vector<int>& tsl = st.tsl;
    nslices = tsl[ntiles];
    std::vector<long long> soff(nslices + 1, 0);
    for (int sl = 0; sl < nslices; ++sl) soff[sl + 1] = soff[sl] + 32LL * st.slen[sl];
    {
        std::vector<std::pair<long long, int>> w;
        for (int t = 0; t < ntiles; ++t)
            if (tsl[t + 1] > tsl[t]) w.push_back({-(soff[tsl[t + 1]] - soff[tsl[t]]), t});
        std::sort(w.begin(), w.end());
        std::vector<int> o(w.size());
        for (size_t i = 0; i < w.size(); ++i) o[i] = w[i].second;
        nwork = (int)o.size();
        tile_order.alloc(std::max(nwork, 1));
        if (nwork) TV3_CUDA(cudaMemcpy(tile_order.p, o.data(), nwork * sizeof(int), cudaMemcpyHostToDevice));
    }
    const long long padded = soff.back();
    tile_slice.alloc(ntiles + 1);
    slice_off.alloc(nslices + 1);
    TV3_CUDA(cudaMemcpy(tile_slice.p, tsl.data(), (ntiles + 1) * sizeof(int), cudaMemcpyHostToDevice));
    TV3_CUDA(cudaMemcpy(slice_off.p, soff.data(), (nslices + 1) * sizeof(long long), cudaMemcpyHostToDevice));
    lidx.alloc(std::max<long long>(padded, 1));
    val.alloc(std::max<long long>(padded, 1));
    slot_dest.alloc((size_t)std::max(nslices, 1) * 32);
    part.alloc(std::max<long long>(npart, 1));
    TV3_CUDA(cudaMemsetAsync(lidx.p, 0, std::max<long long>(padded, 1) * sizeof(unsigned short), s));
    TV3_CUDA(cudaMemsetAsync(val.p, 0, std::max<long long>(padded, 1) * sizeof(V), s));
    TV3_CUDA(cudaMemsetAsync(slot_dest.p, 0xff, (size_t)std::max(nslices, 1) * 32 * sizeof(int), s));
    k_n_fill<V><<<ewt(nseg), 256, 0, s>>>(nseg, order.p, k_slice_s.p, tseg_d.p, tile_slice.p, slice_off.p,
                                          seg_start.p, nnz, idx_s.p, ind, valin, dest.p, p, q, ty, tx, tz, lidx.p,
                                          val.p, slot_dest.p);
    TV3_CUDA(cudaGetLastError());
    // chunks of the streamed form: per tile, runs of consecutive slices with
    // at most BULK_CHUNK entries and 32 slices per consumer warp
    {
        std::vector<int> tch(ntiles + 1, 0), csl;
        std::vector<long long> ce0;
        std::vector<int4> sinfo(std::max(nslices, 1), make_int4(0, 0, 0, 0));
        for (int t = 0; t < ntiles; ++t) {
            tch[t] = (int)csl.size();
            int sl = tsl[t];
            while (sl < tsl[t + 1]) {
                csl.push_back(sl);
                ce0.push_back(soff[sl]);
                long long ent = 0;
                int cnt = 0;
                while (sl < tsl[t + 1] && cnt < BULK_MAXS && ent + (soff[sl + 1] - soff[sl]) <= BULK_CHUNK) {
                    sinfo[sl] = make_int4((int)(soff[sl] - ce0.back()), (int)((soff[sl + 1] - soff[sl]) / 32), 0, 0);
                    ent += soff[sl + 1] - soff[sl];
                    ++cnt;
                    ++sl;
                }
                if (cnt == 0) return;  // a slice longer than a chunk (not met by ray segments of a tile)
            }
        }
        tch[ntiles] = (int)csl.size();
        csl.push_back(nslices);
        ce0.push_back(soff[nslices]);
        tile_chunk.alloc(ntiles + 1);
        chunk_slice.alloc(csl.size());
        chunk_e0.alloc(ce0.size());
        slice_info.alloc(sinfo.size());
        TV3_CUDA(cudaMemcpy(tile_chunk.p, tch.data(), tch.size() * sizeof(int), cudaMemcpyHostToDevice));
        TV3_CUDA(cudaMemcpy(chunk_slice.p, csl.data(), csl.size() * sizeof(int), cudaMemcpyHostToDevice));
        TV3_CUDA(cudaMemcpy(chunk_e0.p, ce0.data(), ce0.size() * sizeof(long long), cudaMemcpyHostToDevice));
        TV3_CUDA(cudaMemcpy(slice_info.p, sinfo.data(), sinfo.size() * sizeof(int4), cudaMemcpyHostToDevice));
    }
    TV3_CUDA(cudaFuncSetAttribute(k_spmv_tiledN<T, V>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem_bytes()));
    // persistent CTAs: as many as fit on the GPU at once (at most one per tile)
    int per = 0;
    TV3_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_spmv_tiledN<T, V>, 32 * (BULK_NC + 1),
                                                           smem_bytes()));
    grid_n = std::max(1, std::min(std::max(nwork, 1), std::max(per, 1) * num_sms()));
    TV3_CUDA(cudaStreamSynchronize(s));
    ok = true;
}

template <class T, class V>
size_t TiledN<T, V>::smem_bytes() const {
    const size_t xs = ((size_t)ty * tx * tz + 1) & ~(size_t)1;
    return 128 + BULK_STAGES * bulk_stage_bytes<V>() + 2 * xs * sizeof(T);
}

template <class T, class V>
void TiledN<T, V>::apply(const TiledNArgs<T, V>& a, int epi, cudaStream_t s) const {
    TiledNArgs<T, V> b = a;
    b.tile_order = tile_order.p;
    const BulkArgs bk{tile_chunk.p, chunk_slice.p, chunk_e0.p, slice_info.p, nwork};
    if (nwork > 0) launch_k(k_spmv_tiledN<T, V>, dim3(grid_n), dim3(32 * (BULK_NC + 1)), smem_bytes(), s, b, bk);
    const int g = (int)std::max<long>(1, std::min<long>((a.m + 255) / 256, (long)num_sms() * 8));
    switch (epi) {
        case SPMV_SUB: launch_k(k_tiledN_reduce<T, V, SPMV_SUB>, dim3(g), dim3(256), 0, s, b); break;
        case SPMV_LAM35: launch_k(k_tiledN_reduce<T, V, SPMV_LAM35>, dim3(g), dim3(256), 0, s, b); break;
        case SPMV_NORM2: launch_k(k_tiledN_reduce<T, V, SPMV_NORM2>, dim3(g), dim3(256), 0, s, b); break;
        default: launch_k(k_tiledN_reduce<T, V, SPMV_PLAIN>, dim3(g), dim3(256), 0, s, b); break;
    }
    TV3_CUDA(cudaGetLastError());
}

template struct TiledN<float, float>;
template struct TiledN<double, double>;
template struct TiledN<double, float>;
template struct TiledN<df64, float>;
template struct TiledN<float, __nv_bfloat16>;
template struct TiledN<float, __half>;
template struct TiledN<df64, __nv_bfloat16>;
template struct TiledN<df64, __half>;

template struct TiledT<float, float>;
template struct TiledT<double, double>;
template struct TiledT<double, float>;
template struct TiledT<df64, float>;
template struct TiledT<float, __nv_bfloat16>;
template struct TiledT<float, __half>;
template struct TiledT<df64, __nv_bfloat16>;
template struct TiledT<df64, __half>;

}  // namespace tv3
