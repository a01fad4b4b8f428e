// Tile-staged A^T*y (tiled.cu): the CSR of A^T regrouped by voxel tiles, with
// per-tile ray lists so that a CTA can stage the tile's y values in shared
// memory.
#pragma once

#include <cuda_runtime.h>
#include <vector>
#include "dbuf.h"
#include "launch.h"
#include "tval3_internal.cuh"

namespace tv3 {

constexpr int TILED_UNIT_K = 16;  // steps of one slice per work unit

template <class T, class V>
struct TiledArgs {
    int ntiles;
    const int* ray_off;          // ntiles + 1: the tile's rays are rays[ray_off[t] .. ray_off[t+1])
    const int* rays;             // ray indices, ascending inside each tile
    const int* tile_slice;       // ntiles + 1: the tile's slices of 32 rows
    const long long* slice_off;  // nslices + 1: entry k of lane l of slice s at slice_off[s] + 32 k + l
    const int* row_voxel;        // 32 per slice: the voxel of each lane's row (-1: padding)
    const unsigned short* lidx;  // position of the nonzero's ray in its tile's list (0 in padding)
    const V* val;                // value (0 in padding)
    const int* tile_unit;        // ntiles + 1: the tile's work units
    const int* slice_unit;       // nslices + 1: the slice's work units
    const int* unit_slice;       // slice of each unit
    const unsigned short* unit_k0;  // first step of each unit
    const longlong2* unit_desc;     // per unit: {its first entry (lane 0), its steps}
    int max_rays;                // shared memory: max_rays values of y, then 32 partials per unit
    const float* xscale;       // per-ray scale of the gathered y (16-bit storage), or null
    const T* x[2];             // y (the input of A^T), ping-pong by parity
    T* y[2];                   // the output volume
    int by_parity;
    const T* sub;              // SPMV_SUB: out = A^T y - sub
    Ctl* ctl;
    const int* tile_order;     // tiles with nonzeros, largest first (one per CTA)
    int nwork;
    const int* zrows;          // voxels whose row of A^T is empty (result 0 or -sub)
    long nzero;
};

// Pipelined A^T*y (k_spmv_tiled_pipe): one persistent CTA per SM of
// PIPE_CONSUMERS consumer warps and one producer warp that stages the next
// tile's y values while the consumers sum the current tile.
constexpr int PIPE_CONSUMERS = 31;

struct PipeArgs {
    // per position k of the largest-first order, two 16-byte records:
    // {tile, first unit, first slice, end slice}, {end unit, 0, rays, start of
    // the ray list in rays_pad}
    const int4* sched;
    const int* rays_pad;         // ray lists, each starting at a multiple of 4 entries
    int ybuf_elems;              // y elements per buffer (max rays rounded up to 4)
};

template <class T, class V>
struct TiledT {
    bool ok = false;
    long n = 0;
    int ntiles = 0, nslices = 0, nunits = 0, max_rays = 0, max_units = 0, nwork = 0;
    long nzero = 0;
    DBuf<int> tile_order, zrows;
    long long padded_entries = 0;
    DBuf<int> ray_off, rays, tile_slice, row_voxel, tile_unit, slice_unit, unit_slice;
    DBuf<unsigned short> unit_k0;
    DBuf<longlong2> unit_desc;
    DBuf<long long> slice_off;
    DBuf<unsigned short> lidx;
    DBuf<V> val;
    // build from the CSR of A^T (n voxel rows, ray indices < m) of a p x q x r
    // volume; leaves ok = false when, with the smallest tiles, some tile's ray
    // list exceeds max_smem bytes of T or 65,535 entries
    void build(long n, long m, int p, int q, int r, const int* tptr, const int* tind, const V* tval, long nnz,
               size_t max_smem, cudaStream_t s);
    // one attempt with tiles of ty x tx x tz voxels (clipped to the volume)
    void build_shape(long n, long m, int p, int q, int r, const int* tptr, const int* tind, const V* tval, long nnz,
                     size_t max_smem, cudaStream_t s, int ty, int tx, int tz);
    void apply(const TiledArgs<T, V>& a, int epi, cudaStream_t s) const;
    // pipelined form: one CTA per SM; a producer warp gathers the next tile's
    // y values (bulk copy of the ray list, then asynchronous copies) while 31
    // consumer warps sum the current tile; FP32/FP64 values only
    mutable bool pipe_ok = false;
    mutable int pipe_ybe = 0;
    mutable size_t pipe_smem = 0;
    mutable DBuf<int4> sched;
    mutable DBuf<int> rays_pad;
    void apply_pipe(const TiledArgs<T, V>& a, int epi, cudaStream_t s) const;
    // the pipelined form's tables are built on first use (a caller pinning
    // variant 2); the slice and unit layout they need is kept from build()
    bool ensure_pipe() const;
    mutable bool pipe_tried = false;
    std::vector<int> h_tsl, h_tunit;
    void build_pipe();
};

// Tile-staged A*x: the rays' nonzeros cut into segments (the part of a ray
// inside one voxel tile).  A CTA stages its tile's x values in shared memory
// and sums every segment (sliced ELL, one lane per segment); the partial sums
// land ray by ray in `part`, and a second kernel adds each ray's partials in
// tile order and applies the epilogues.
// Streaming of a tile's slices through shared memory (tile-staged A*x): a
// producer warp bulk-copies chunks of consecutive slices (at most
// BULK_CHUNK entries and BULK_MAXS slices, two per consumer warp, with the
// slices' destinations and places) into a ring of BULK_STAGES stages while
// BULK_NC consumer warps sum the slices of the chunks already landed.
constexpr int BULK_NC = 8;
constexpr int BULK_STAGES = 2;
constexpr int BULK_CHUNK = 4096;
constexpr int BULK_MAXS = 2 * BULK_NC;

struct BulkArgs {
    const int* tile_chunk;        // ntiles + 1: the tile's chunks
    const int* chunk_slice;       // nchunks + 1: the chunk's first slice (the next chunk's first ends it)
    const long long* chunk_e0;    // nchunks + 1: the chunk's first entry
    const int4* slice_info;       // per slice: {first entry - its chunk's first entry, steps, 0, 0}
    int nwork;                    // tiles with segments (positions of tile_order)
};

template <class T, class V>
struct TiledNArgs {
    int ntiles;
    int p, q, r, ty, tx, tz, nty, ntx;  // volume and tile shape (for staging x)
    const int* tile_slice;       // ntiles + 1
    const long long* slice_off;  // nslices + 1
    const int* slot_dest;        // 32 per slice: index of the segment's partial in `part` (-1: padding)
    const unsigned short* lidx;  // local voxel of each nonzero in its tile (0 in padding)
    const V* val;                // value (0 in padding)
    T* part;                     // one partial per segment, in groups of 32 ray slots (gbase)
    const int* sray;             // m: the ray of each slot (slots: rays ranked by length in windows of 256)
    const int* rlen;             // m: partials (segments) of the ray in each slot
    const long long* gbase;      // per 32 slots: partial k of the ray in slot s is part[gbase[s/32] + 32 k + s%32]
    long m;
    const float* rscale;         // per-ray scale of the row sum (16-bit storage), or null
    const T* x[2];
    T* y[2];
    int by_parity;
    const T* sub;
    const T* b;
    const T* delta;
    Ctl* ctl;
    double* rpart;               // grid-reduction scratch of the epilogues
    unsigned* ticket;
    const int* tile_order;       // tiles with segments, largest first (one per CTA)
};

template <class T, class V>
struct TiledN {
    bool ok = false;
    int ntiles = 0, nslices = 0, nwork = 0;
    DBuf<int> tile_order;
    int p = 0, q = 0, r = 0, ty = 0, tx = 0, tz = 0, nty = 0, ntx = 0;
    long m = 0, nseg = 0;
    DBuf<int> tile_slice, slot_dest, sray, rlen;
    DBuf<long long> gbase;
    DBuf<long long> slice_off;
    DBuf<unsigned short> lidx;
    DBuf<V> val;
    mutable DBuf<T> part;
    DBuf<int> tile_chunk, chunk_slice;
    DBuf<long long> chunk_e0;
    DBuf<int4> slice_info;
    mutable int grid_n = 0;  // persistent CTAs of the streamed A*x
    size_t smem_bytes() const;
    // build from the CSR of A (m ray rows over the p x q x r volume)
    void build(long m, int p, int q, int r, const int* ptr, const int* ind, const V* val, long nnz, cudaStream_t s);
    void apply(const TiledNArgs<T, V>& a, int epi, cudaStream_t s) const;
};

}  // namespace tv3
