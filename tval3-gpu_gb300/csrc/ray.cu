// Ray-geometry operators: the measurement matrix of straight rays between
// emitters and receivers, either built on the device as CSR (then used by the
// CSR products of ops.cu) or traversed on the fly in every product.
//
// Ray list: 3d/mat_vec_mul_dynamic.h:477-556 compacts the use_path flags of
// numMPs x E x R signals into (emitter, receiver) pairs; signal i gives
// emitter i / R and receiver (i / (E*R)) * R + i % R.
//
// Bresenham: the integer 3D walk of dyn_calc_kernel
// (3d/tval3_gpu_3d_kernels.cu:1612-1764).  The walk of m1 = max|d| steps is
// restated in closed form: after step j the dominant coordinate has moved j
// voxels and a secondary coordinate with extent m has moved
// s(j) = (2*m*j + m1 - 1) / (2*m1) voxels (integer division), which equals the
// error-term recursion of the reference step for step, so every voxel of a ray
// can be computed independently (lane-parallel traversal).  Every voxel gets
// the weight scale_factor (mult_elementN/T, :1461-1507).
//
// Siddon: exact intersection lengths of the segment with the voxel grid,
// evaluated in FP64 with explicitly rounded operations (no contraction), so
// the voxel sequence and the FP32 lengths equal a CPU evaluation of the same
// formulas bit for bit.  Not present in the reference.
#include <cub/cub.cuh>
#include <algorithm>
#include <cmath>
#include <memory>
#include <vector>
#include "dbuf.h"
#include "ops.h"
#include "tval3/tval3_c.h"

namespace tv3 {

struct RayGeom {
    long nrays = 0;
    int nx = 0, ny = 0, nz = 0;  // rv_x, rv_y (fastest), rv_z
    int traversal = 0;
    double scale = 1.0;
    DBuf<unsigned> pairs;        // 2 per ray
    DBuf<int> ie;                // integer coordinates: xe ye ze (E) then xr yr zr (R)
    DBuf<double> pe;             // continuous coordinates, same layout
    long ne = 0, nr = 0;         // emitter / receiver counts (all MPs)
};

// ---------------------------------------------------------------------------
// device walkers
// ---------------------------------------------------------------------------
struct BresRay {
    int s1, s2, s3, inc1, inc2, inc3, m1, m2, m3;
    int a1, a2, a3;  // which of x, y, z is the dominant / 2nd / 3rd axis (0 x, 1 y, 2 z)
};

__device__ __forceinline__ BresRay bres_setup(int xs, int ys, int zs, int xe, int ye, int ze) {
    int d1 = xe - xs, d2 = ye - ys, d3 = ze - zs;
    int m1 = abs(d1), m2 = abs(d2), m3 = abs(d3);
    BresRay b;
    int st[3] = {xs, ys, zs};
    if (m1 >= m2 && m1 >= m3) {
        b.a1 = 0; b.a2 = 1; b.a3 = 2;
    } else if (m2 >= m1 && m2 >= m3) {
        int t = d1; d1 = d2; d2 = t;
        b.a1 = 1; b.a2 = 0; b.a3 = 2;
    } else {
        int t = d1; d1 = d3; d3 = d2; d2 = t;
        b.a1 = 2; b.a2 = 0; b.a3 = 1;
    }
    b.inc1 = d1 < 0 ? -1 : 1;
    b.inc2 = d2 < 0 ? -1 : 1;
    b.inc3 = d3 < 0 ? -1 : 1;
    b.m1 = abs(d1); b.m2 = abs(d2); b.m3 = abs(d3);
    b.s1 = (b.a1 == 0) ? st[0] : (b.a1 == 1) ? st[1] : st[2];
    b.s2 = (b.a2 == 0) ? st[0] : (b.a2 == 1) ? st[1] : st[2];
    b.s3 = (b.a3 == 0) ? st[0] : (b.a3 == 1) ? st[1] : st[2];
    return b;
}

// voxel j (0 = emitter voxel) of a Bresenham ray: coordinates (x, y, z) and
// linear index
__device__ __forceinline__ void bres_coords(const BresRay& b, int j, int c[3]) {
    long twom1 = 2L * b.m1;
    int k2 = b.m1 ? (int)((2L * b.m2 * j + b.m1 - 1) / twom1) : 0;
    int k3 = b.m1 ? (int)((2L * b.m3 * j + b.m1 - 1) / twom1) : 0;
    const int v1 = b.s1 + b.inc1 * j, v2 = b.s2 + b.inc2 * k2, v3 = b.s3 + b.inc3 * k3;
    // selects instead of c[b.a1] = ... keep c in registers
#pragma unroll
    for (int a = 0; a < 3; ++a) c[a] = (b.a1 == a) ? v1 : (b.a2 == a) ? v2 : v3;
}

__device__ __forceinline__ long bres_voxel(const BresRay& b, int j, int nx, int ny) {
    int c[3];
    bres_coords(b, j, c);
    return (long)c[2] * nx * ny + (long)c[0] * ny + c[1];
}

__device__ __forceinline__ double dmin_(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double dmax_(double a, double b) { return (a < b) ? b : a; }

// Siddon walk, split into the ray's constants (sid_setup), the walk state
// (t, the next plane k[a] of each axis and its crossing parameter tn[a]) and
// one iteration of the walk loop (sid_event), so that the CSR builder, the
// on-the-fly A*x and the tile-resumed A^T*y run the same operations.  Every
// floating-point operation is an explicitly rounded intrinsic so that it
// matches the host evaluation (compiled without contraction) bit for bit.
struct SidRay {
    double P0[3], dv[3];
    double L, tmin, tmax;
    int k0[3];  // the first plane of each axis (the walk state at tmin)
    int pad;
};

struct SidState {
    double t, tn[3];
    int k[3];
};

// false when the segment misses the volume (or has no length)
__device__ __forceinline__ bool sid_setup(const double P0[3], const double P1[3], const int N[3], SidRay& R) {
    for (int a = 0; a < 3; ++a) {
        R.P0[a] = P0[a];
        R.dv[a] = __dsub_rn(P1[a], P0[a]);
        R.k0[a] = 0;
    }
    R.pad = 0;
    R.tmin = 0.0;
    R.tmax = 0.0;
    R.L = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(R.dv[0], R.dv[0]), __dmul_rn(R.dv[1], R.dv[1])),
                               __dmul_rn(R.dv[2], R.dv[2])));
    if (!(R.L > 0.0)) return false;
    double tmin = 0.0, tmax = 1.0;
    for (int a = 0; a < 3; ++a) {
        if (R.dv[a] == 0.0) {
            if (!(P0[a] >= 0.0 && P0[a] < (double)N[a])) return false;
        } else {
            double t0 = __ddiv_rn(__dsub_rn(0.0, P0[a]), R.dv[a]);
            double t1 = __ddiv_rn(__dsub_rn((double)N[a], P0[a]), R.dv[a]);
            double lo = dmin_(t0, t1), hi = dmax_(t0, t1);
            tmin = dmax_(tmin, lo);
            tmax = dmin_(tmax, hi);
        }
    }
    if (!(tmin < tmax)) return false;
    R.tmin = tmin;
    R.tmax = tmax;
    for (int a = 0; a < 3; ++a) {
        if (R.dv[a] == 0.0) continue;
        const int st = R.dv[a] > 0 ? 1 : -1;
        double pos = __dadd_rn(P0[a], __dmul_rn(tmin, R.dv[a]));
        // (round-down / round-up conversions: floor and ceil in one instruction)
        long k = (st > 0) ? (long)__double2ll_rd(pos) + 1 : (long)__double2ll_ru(pos) - 1;
        double tn = __ddiv_rn(__dsub_rn((double)k, P0[a]), R.dv[a]);
        for (int guard = 0; tn <= tmin && guard < 4; ++guard) {
            k += st;
            tn = __ddiv_rn(__dsub_rn((double)k, P0[a]), R.dv[a]);
        }
        R.k0[a] = (int)k;
    }
    return true;
}

// the walk state at parameter t with next planes k (tn follows from k)
__device__ __forceinline__ void sid_start(const SidRay& R, double t, const int k[3], SidState& s) {
    s.t = t;
    for (int a = 0; a < 3; ++a) {
        s.k[a] = k[a];
        s.tn[a] = (R.dv[a] == 0.0) ? INFINITY : __ddiv_rn(__dsub_rn((double)k[a], R.P0[a]), R.dv[a]);
    }
}

// one iteration of the walk loop: the segment [t, te] to the nearest crossing
// (returned with its clamped voxel c and FP32 length v when te > t), then the
// advance of every axis whose plane lies at te
__device__ __forceinline__ bool sid_event(const SidRay& R, const int N[3], double scale, SidState& s, int c[3],
                                          float& v) {
    const double te = dmin_(dmin_(s.tn[0], s.tn[1]), dmin_(s.tn[2], R.tmax));
    bool out = false;
    if (te > s.t) {
        const double mid = __dmul_rn(0.5, __dadd_rn(s.t, te));
        for (int a = 0; a < 3; ++a) {
            const double cc = __dadd_rn(R.P0[a], __dmul_rn(mid, R.dv[a]));
            long q = (long)__double2ll_rd(cc);
            if (q < 0) q = 0;
            if (q > N[a] - 1) q = N[a] - 1;
            c[a] = (int)q;
        }
        const double len = __dmul_rn(__dsub_rn(te, s.t), R.L);
        v = __double2float_rn(__dmul_rn(len, scale));
        out = true;
    }
    for (int a = 0; a < 3; ++a)
        if (s.tn[a] == te) {
            s.k[a] += R.dv[a] > 0 ? 1 : -1;
            s.tn[a] = __ddiv_rn(__dsub_rn((double)s.k[a], R.P0[a]), R.dv[a]);
        }
    s.t = te;
    return out;
}

// iterations of the walk loop: at most one segment per crossed plane (the
// bound only matters for degenerate input)
__device__ __forceinline__ int sid_guard(const int N[3]) { return N[0] + N[1] + N[2] + 8; }

__device__ __forceinline__ long vox_index(const int c[3], const int N[3]) {
    return (long)c[2] * N[0] * N[1] + (long)c[0] * N[1] + c[1];
}

// Siddon walk; emit(index, float length) for each segment of positive length
template <class F>
__device__ void siddon_walk_dev(const double P0[3], const double P1[3], const int N[3], double scale, F emit) {
    SidRay R;
    if (!sid_setup(P0, P1, N, R)) return;
    SidState s;
    sid_start(R, R.tmin, R.k0, s);
    for (int guard = sid_guard(N); s.t < R.tmax && guard > 0; --guard) {
        int c[3];
        float v;
        if (sid_event(R, N, scale, s, c, v)) emit(vox_index(c, N), v);
    }
}

struct GeomView {
    long nrays;
    int nx, ny, nz;
    long ne, nr;
    const unsigned* pairs;
    const int* ie;
    const double* pe;
    double scale;
};

__device__ __forceinline__ void ray_ends_int(const GeomView& g, long r, int& xs, int& ys, int& zs, int& xe, int& ye,
                                             int& ze) {
    unsigned e = g.pairs[2 * r], q = g.pairs[2 * r + 1];
    xs = g.ie[e]; ys = g.ie[g.ne + e]; zs = g.ie[2 * g.ne + e];
    const int* R = g.ie + 3 * g.ne;
    xe = R[q]; ye = R[g.nr + q]; ze = R[2 * g.nr + q];
}

__device__ __forceinline__ void ray_ends_pos(const GeomView& g, long r, double P0[3], double P1[3]) {
    unsigned e = g.pairs[2 * r], q = g.pairs[2 * r + 1];
    P0[0] = g.pe[e]; P0[1] = g.pe[g.ne + e]; P0[2] = g.pe[2 * g.ne + e];
    const double* R = g.pe + 3 * g.ne;
    P1[0] = R[q]; P1[1] = R[g.nr + q]; P1[2] = R[2 * g.nr + q];
}

// ---------------------------------------------------------------------------
// CSR build: count, scan, fill
// ---------------------------------------------------------------------------
__global__ void k_ray_count(GeomView g, int traversal, int* __restrict__ len) {
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < g.nrays; r += (long)gridDim.x * blockDim.x) {
        int c = 0;
        if (traversal == TVAL3_TRAVERSAL_BRESENHAM) {
            int xs, ys, zs, xe, ye, ze;
            ray_ends_int(g, r, xs, ys, zs, xe, ye, ze);
            c = max(abs(xe - xs), max(abs(ye - ys), abs(ze - zs))) + 1;
        } else {
            double P0[3], P1[3];
            ray_ends_pos(g, r, P0, P1);
            const int N[3] = {g.nx, g.ny, g.nz};
            siddon_walk_dev(P0, P1, N, g.scale, [&](long, float) { ++c; });
        }
        len[r] = c;
    }
}

__global__ void k_ray_fill(GeomView g, int traversal, const int* __restrict__ ptr, int* __restrict__ ind,
                           float* __restrict__ val) {
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < g.nrays; r += (long)gridDim.x * blockDim.x) {
        long k = ptr[r];
        if (traversal == TVAL3_TRAVERSAL_BRESENHAM) {
            int xs, ys, zs, xe, ye, ze;
            ray_ends_int(g, r, xs, ys, zs, xe, ye, ze);
            BresRay b = bres_setup(xs, ys, zs, xe, ye, ze);
            const float w = (float)g.scale;
            for (int j = 0; j <= b.m1; ++j) {
                ind[k] = (int)bres_voxel(b, j, g.nx, g.ny);
                val[k] = w;
                ++k;
            }
        } else {
            double P0[3], P1[3];
            ray_ends_pos(g, r, P0, P1);
            const int N[3] = {g.nx, g.ny, g.nz};
            siddon_walk_dev(P0, P1, N, g.scale, [&](long idx, float v) {
                ind[k] = (int)idx;
                val[k] = v;
                ++k;
            });
        }
    }
}

// ---------------------------------------------------------------------------
// on-the-fly A*x
// ---------------------------------------------------------------------------
// row epilogues of A*x: store the row (PLAIN, LAM35) and add the row's terms
// of lam3 = ||Ax - b||^2 and lam5 = <delta, Ax - b> (LAM35) or of ||Ax||^2
// (NORM2)
template <int EPI>
__device__ __forceinline__ void ray_row_epi(const MatIO<float>& io, float* y, long r, float s, double& acc0,
                                            double& acc1) {
    if (EPI == SPMV_PLAIN) y[r] = s;
    else if (EPI == SPMV_LAM35) {
        y[r] = s;
        double t = (double)s - (double)io.b[r];
        acc0 += t * t;
        acc1 += (double)io.delta[r] * t;
    } else if (EPI == SPMV_NORM2) {
        acc0 += (double)s * s;
    }
}

// grid reduction of the epilogue sums into the solver's scalars
template <int EPI>
__device__ __forceinline__ void ray_epi_finish(const MatIO<float>& io, double acc0, double acc1) {
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

// Bresenham: G lanes per ray, each lane a stride of the ray's voxels (the
// closed-form walk makes every voxel independent)
template <int G, int EPI>
__global__ void __launch_bounds__(256) k_bres_N(GeomView g, MatIO<float> io) {
    count_launch(io.ctl);
    const int lane = threadIdx.x % G;
    const long grp = ((long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const long ngrp = ((long)gridDim.x * blockDim.x) / G;
    const int sel = io.by_parity ? io.ctl->parity : 0;
    const float* __restrict__ x = io.x[sel];
    float* __restrict__ y = io.y[sel];
    const unsigned gmask = (G == 32) ? FULL : (((1u << G) - 1u) << ((threadIdx.x & 31) / G * G));
    const float w = (float)g.scale;
    double acc0 = 0.0, acc1 = 0.0;
    for (long r = grp; r < g.nrays; r += ngrp) {
        int xs, ys, zs, xe, ye, ze;
        ray_ends_int(g, r, xs, ys, zs, xe, ye, ze);
        BresRay b = bres_setup(xs, ys, zs, xe, ye, ze);
        float s = 0.f;
        for (int j = lane; j <= b.m1; j += G) s += x[bres_voxel(b, j, g.nx, g.ny)];
#pragma unroll
        for (int o = G / 2; o; o >>= 1) s += __shfl_down_sync(gmask, s, o, G);
        if (lane == 0) ray_row_epi<EPI>(io, y, r, s * w, acc0, acc1);
    }
    ray_epi_finish<EPI>(io, acc0, acc1);
}

// Siddon: one thread per ray walks the segments from the ray's stored
// constants (the builder's exact FP64 arithmetic, so the implied matrix is
// the stored CSR's bit for bit) and gathers x
template <int EPI>
__global__ void __launch_bounds__(256) k_sid_N(GeomView g, const SidRay* __restrict__ rec, MatIO<float> io) {
    count_launch(io.ctl);
    const int sel = io.by_parity ? io.ctl->parity : 0;
    const float* __restrict__ x = io.x[sel];
    float* __restrict__ y = io.y[sel];
    const int N[3] = {g.nx, g.ny, g.nz};
    double acc0 = 0.0, acc1 = 0.0;
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < g.nrays; r += (long)gridDim.x * blockDim.x) {
        const SidRay R = rec[r];
        float s = 0.f;
        if (R.tmin < R.tmax) {
            SidState st;
            sid_start(R, R.tmin, R.k0, st);
            for (int guard = sid_guard(N); st.t < R.tmax && guard > 0; --guard) {
                int c[3];
                float v;
                if (sid_event(R, N, g.scale, st, c, v)) s = fmaf(v, x[vox_index(c, N)], s);
            }
        }
        ray_row_epi<EPI>(io, y, r, s, acc0, acc1);
    }
    ray_epi_finish<EPI>(io, acc0, acc1);
}

// ---------------------------------------------------------------------------
// on-the-fly A^T*y over tile runs
// ---------------------------------------------------------------------------
// A ray's segments are cut into runs: consecutive segments whose voxels lie
// in one voxel tile.  A run is stored as the walk state before its first
// segment and its segment count, and the runs are grouped by tile.  One CTA
// per tile resumes every run through its tile and sums A^T y for the tile's
// voxels in shared memory: each warp owns a private row of accumulators, a
// warp step combines the lanes that hit one voxel in lane order, and the rows
// are added in warp order, so the result is the same on every run (no global
// atomics).
struct RunEntry {
    double t;     // Siddon: the walk parameter before the run's first segment
    int ray;
    unsigned pk;  // bits 0-7: segments of the run.  Siddon: bits 8-31 the next
                  // planes of x, y, z (8 bits each, relative to the tile's first
                  // voxel, plus 128).  Bresenham: bits 8-31 the step of the
                  // run's first voxel
};

constexpr int RUN_WARPS = 8;
constexpr int RUN_TV = 512;  // voxels of a tile at most (8 x 8 x 8, or 16 x 16 x 1)
constexpr unsigned RUN_ERR_COUNT = 1u, RUN_ERR_PLANE = 2u, RUN_ERR_STEP = 4u;

struct RunView {
    int T[3];               // tile extent along x, y, z in voxels
    int nt[3];              // tiles along x, y, z
    int ntiles;
    const long long* tile_off;  // ntiles + 1: the tile's runs
    const int* tile_order;      // every tile, most runs first
    const RunEntry* ent;
    const SidRay* rec;          // Siddon: the rays' constants
};

__device__ __forceinline__ int tile_of(const RunView& v, const int c[3]) {
    return (c[2] / v.T[2]) * v.nt[0] * v.nt[1] + (c[0] / v.T[0]) * v.nt[1] + c[1] / v.T[1];
}

__device__ __forceinline__ void tile_base(const RunView& v, int tile, int b[3]) {
    const int per = v.nt[0] * v.nt[1];
    b[2] = (tile / per) * v.T[2];
    b[0] = ((tile % per) / v.nt[1]) * v.T[0];
    b[1] = (tile % v.nt[1]) * v.T[1];
}

__device__ __forceinline__ unsigned run_pack_sid(const RunView& v, int tile, const SidRay& R, const int k[3], int cnt,
                                                 unsigned& err) {
    int b[3];
    tile_base(v, tile, b);
    if (cnt > 255) err |= RUN_ERR_COUNT;
    unsigned pk = (unsigned)min(cnt, 255);
    for (int a = 0; a < 3; ++a) {
        int rel = (R.dv[a] == 0.0) ? 0 : k[a] - b[a];
        if (rel < -128 || rel > 127) {
            err |= RUN_ERR_PLANE;
            rel = 0;
        }
        pk |= (unsigned)(rel + 128) << (8 + 8 * a);
    }
    return pk;
}

__device__ __forceinline__ unsigned run_pack_bres(int j0, int cnt, unsigned& err) {
    if (cnt > 255) err |= RUN_ERR_COUNT;
    if (j0 >= (1 << 24)) err |= RUN_ERR_STEP;
    return (unsigned)min(cnt, 255) | ((unsigned)(j0 & 0xffffff) << 8);
}

// the runs of ray r in walk order: flush(tile, entry) per run; Siddon rays
// also store their constants in rec_out
template <int TRAV, class F>
__device__ void ray_runs(const GeomView& g, const RunView& v, long r, SidRay* rec_out, unsigned& err, F flush) {
    const int N[3] = {g.nx, g.ny, g.nz};
    if (TRAV == TVAL3_TRAVERSAL_SIDDON) {
        double P0[3], P1[3];
        ray_ends_pos(g, r, P0, P1);
        SidRay R;
        const bool hit = sid_setup(P0, P1, N, R);
        rec_out[r] = R;
        if (!hit) return;
        SidState s, s0;
        sid_start(R, R.tmin, R.k0, s);
        s0 = s;
        int cur = -1, cnt = 0;
        for (int guard = sid_guard(N); s.t < R.tmax && guard > 0; --guard) {
            const SidState before = s;
            int c[3];
            float val;
            if (sid_event(R, N, g.scale, s, c, val)) {
                const int tl = tile_of(v, c);
                if (tl != cur) {
                    if (cur >= 0) flush(cur, RunEntry{s0.t, (int)r, run_pack_sid(v, cur, R, s0.k, cnt, err)});
                    cur = tl;
                    s0 = before;
                    cnt = 0;
                }
                ++cnt;
            }
        }
        if (cur >= 0) flush(cur, RunEntry{s0.t, (int)r, run_pack_sid(v, cur, R, s0.k, cnt, err)});
    } else {
        int xs, ys, zs, xe, ye, ze;
        ray_ends_int(g, r, xs, ys, zs, xe, ye, ze);
        const BresRay b = bres_setup(xs, ys, zs, xe, ye, ze);
        int cur = -1, cnt = 0, j0 = 0;
        for (int j = 0; j <= b.m1; ++j) {
            int c[3];
            bres_coords(b, j, c);
            const int tl = tile_of(v, c);
            if (tl != cur) {
                if (cur >= 0) flush(cur, RunEntry{0.0, (int)r, run_pack_bres(j0, cnt, err)});
                cur = tl;
                j0 = j;
                cnt = 0;
            }
            ++cnt;
        }
        if (cur >= 0) flush(cur, RunEntry{0.0, (int)r, run_pack_bres(j0, cnt, err)});
    }
}

// per ray: runs and segments (and the Siddon constants)
template <int TRAV>
__global__ void k_runs_count(GeomView g, RunView v, SidRay* rec, long long* runs, long long* segs, unsigned* err) {
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < g.nrays; r += (long)gridDim.x * blockDim.x) {
        unsigned e = 0;
        long long nr = 0, ns = 0;
        ray_runs<TRAV>(g, v, r, rec, e, [&](int, const RunEntry& en) {
            ++nr;
            ns += en.pk & 255u;
        });
        runs[r] = nr;
        segs[r] = ns;
        if (e) atomicOr(err, e);
    }
}

// per ray: its runs at run_off[r] .. (tile keys beside them) and the tiles' run counts
template <int TRAV>
__global__ void k_runs_fill(GeomView g, RunView v, SidRay* rec, const long long* __restrict__ run_off,
                            RunEntry* __restrict__ ent, int* __restrict__ key, int* __restrict__ tile_cnt) {
    for (long r = (long)blockIdx.x * blockDim.x + threadIdx.x; r < g.nrays; r += (long)gridDim.x * blockDim.x) {
        unsigned e = 0;
        long long k = run_off[r];
        ray_runs<TRAV>(g, v, r, rec, e, [&](int tile, const RunEntry& en) {
            ent[k] = en;
            key[k] = tile;
            atomicAdd(tile_cnt + tile, 1);
            ++k;
        });
    }
}

__global__ void k_iota(int* a, long n) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) a[i] = (int)i;
}

__global__ void k_gather_runs(const RunEntry* __restrict__ in, const int* __restrict__ idx, RunEntry* __restrict__ out,
                              long n) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x)
        out[i] = in[idx[i]];
}

__global__ void k_widen_count(const int* __restrict__ in, long long* __restrict__ out, long n) {
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) out[i] = in[i];
}

template <int TRAV, int EPI>
__global__ void __launch_bounds__(256) k_run_T(GeomView g, RunView v, MatIO<float> io) {
    __shared__ float acc[RUN_WARPS * RUN_TV];
    count_launch(io.ctl);
    const int sel = io.by_parity ? io.ctl->parity : 0;
    const float* __restrict__ yv = io.x[sel];
    float* __restrict__ out = io.y[sel];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int N[3] = {g.nx, g.ny, g.nz};
    const int TV = v.T[0] * v.T[1] * v.T[2];
    const float w = (float)g.scale;
    float* my = acc + warp * RUN_TV;
    for (int pos = blockIdx.x; pos < v.ntiles; pos += gridDim.x) {
        const int tile = v.tile_order[pos];
        for (int i = threadIdx.x; i < RUN_WARPS * RUN_TV; i += blockDim.x) acc[i] = 0.f;
        __syncthreads();
        int b[3];
        tile_base(v, tile, b);
        const long long e0 = v.tile_off[tile];
        const int cnt = (int)(v.tile_off[tile + 1] - e0);
        for (int base = warp * 32; base < cnt; base += RUN_WARPS * 32) {
            const int e = base + lane;
            int rem = 0;
            float yr = 0.f;
            SidRay R;
            SidState st;
            BresRay br;
            int j = 0;
            int guard = sid_guard(N);
            if (e < cnt) {
                const RunEntry en = v.ent[e0 + e];
                rem = (int)(en.pk & 255u);
                yr = yv[en.ray];
                if (TRAV == TVAL3_TRAVERSAL_SIDDON) {
                    R = v.rec[en.ray];
                    int k[3];
                    for (int a = 0; a < 3; ++a) k[a] = b[a] + (int)((en.pk >> (8 + 8 * a)) & 255u) - 128;
                    sid_start(R, en.t, k, st);
                } else {
                    int xs, ys, zs, xe, ye, ze;
                    ray_ends_int(g, en.ray, xs, ys, zs, xe, ye, ze);
                    br = bres_setup(xs, ys, zs, xe, ye, ze);
                    j = (int)(en.pk >> 8);
                    yr *= w;
                }
            }
            while (__any_sync(FULL, rem > 0)) {
                bool emit = false;
                int vloc = 0;
                float contrib = 0.f;
                if (rem > 0) {
                    int c[3];
                    if (TRAV == TVAL3_TRAVERSAL_SIDDON) {
                        float val;
                        if (!(st.t < R.tmax) || guard-- <= 0) rem = 0;
                        else if (sid_event(R, N, g.scale, st, c, val)) {
                            emit = true;
                            contrib = val * yr;
                        }
                    } else {
                        bres_coords(br, j, c);
                        ++j;
                        emit = true;
                        contrib = yr;
                    }
                    if (emit) {
                        --rem;
                        int l[3];
                        for (int a = 0; a < 3; ++a) l[a] = min(max(c[a] - b[a], 0), v.T[a] - 1);
                        vloc = (l[2] * v.T[0] + l[0]) * v.T[1] + l[1];
                    }
                }
                // lanes on one voxel: the lowest lane adds the group's values in lane order
                const unsigned grp = __match_any_sync(FULL, emit ? (unsigned)vloc : (0x80000000u | (unsigned)lane));
                const int gsz = __reduce_max_sync(FULL, emit ? (unsigned)__popc(grp) : 0u);
                float s = contrib;
                if (gsz > 1) {
                    unsigned rest = grp & (grp - 1u);
                    for (int i = 1; i < gsz; ++i) {
                        const int src = rest ? __ffs(rest) - 1 : lane;
                        const float o = __shfl_sync(FULL, contrib, src);
                        if (rest) {
                            s += o;
                            rest &= rest - 1u;
                        }
                    }
                }
                if (emit && lane == __ffs(grp) - 1) my[vloc] += s;
            }
        }
        __syncthreads();
        for (int i = threadIdx.x; i < TV; i += blockDim.x) {
            const int lz = i / (v.T[0] * v.T[1]), rxy = i % (v.T[0] * v.T[1]);
            const int c[3] = {b[0] + rxy / v.T[1], b[1] + rxy % v.T[1], b[2] + lz};
            if (c[0] < N[0] && c[1] < N[1] && c[2] < N[2]) {
                float s = acc[i];
#pragma unroll
                for (int k = 1; k < RUN_WARPS; ++k) s += acc[k * RUN_TV + i];
                const long idx = vox_index(c, N);
                out[idx] = (EPI == SPMV_SUB) ? s - io.sub[idx] : s;
            }
        }
        __syncthreads();
    }
}

static int grid_for(long items, int per_block) {
    long g = (items + per_block - 1) / per_block;
    long cap = (long)num_sms() * 8;
    return (int)std::max<long>(1, std::min(g, cap));
}

// ---------------------------------------------------------------------------
// construction from a host geometry
// ---------------------------------------------------------------------------
static void upload_geometry(const tval3_geometry_host* G, RayGeom& g) {
    if (!G) throw Error{1, "Argument error: geometry is NULL!"};
    if (G->numMPs < 0 || G->num_emitters < 0 || G->num_receivers < 0 || G->rv_x <= 0 || G->rv_y <= 0 || G->rv_z <= 0)
        throw Error{2, "Argument error: bad geometry dimensions!"};
    if (G->traversal != TVAL3_TRAVERSAL_BRESENHAM && G->traversal != TVAL3_TRAVERSAL_SIDDON)
        throw Error{1, "Argument error: unknown traversal!"};
    const long E = G->num_emitters, R = G->num_receivers, M = G->numMPs;
    g.nx = G->rv_x; g.ny = G->rv_y; g.nz = G->rv_z;
    g.traversal = G->traversal;
    g.scale = G->scale_factor;
    g.ne = M * E; g.nr = M * R;
    // ray list (3d/mat_vec_mul_dynamic.h:477-556)
    std::vector<unsigned> pairs;
    const long per = E * R;
    for (long i = 0; i < per * M; ++i) {
        if (G->use_path && G->use_path[i % per] == 0) continue;
        pairs.push_back((unsigned)(i / R));
        pairs.push_back((unsigned)((i / per) * R + (i % R)));
    }
    g.nrays = (long)pairs.size() / 2;
    const bool have_int = G->x_emitters && G->y_emitters && G->z_emitters && G->x_receivers && G->y_receivers &&
                          G->z_receivers;
    const bool have_pos = G->xe_pos && G->ye_pos && G->ze_pos && G->xr_pos && G->yr_pos && G->zr_pos;
    if (G->traversal == TVAL3_TRAVERSAL_BRESENHAM && !have_int)
        throw Error{1, "Argument error: Bresenham traversal needs integer coordinates!"};
    if (G->traversal == TVAL3_TRAVERSAL_SIDDON && !have_int && !have_pos)
        throw Error{1, "Argument error: Siddon traversal needs coordinates!"};
    std::vector<int> ie;
    if (have_int) {
        ie.resize(3 * (g.ne + g.nr));
        const int* src[6] = {G->x_emitters, G->y_emitters, G->z_emitters, G->x_receivers, G->y_receivers, G->z_receivers};
        const int lim[3] = {g.nx, g.ny, g.nz};
        for (int a = 0; a < 3; ++a) {
            for (long e = 0; e < g.ne; ++e) {
                int v = src[a][e];
                if (G->traversal == TVAL3_TRAVERSAL_BRESENHAM && (v < 0 || v >= lim[a]))
                    throw Error{2, "Argument error: emitter coordinate outside the volume!"};
                ie[a * g.ne + e] = v;
            }
            for (long q = 0; q < g.nr; ++q) {
                int v = src[3 + a][q];
                if (G->traversal == TVAL3_TRAVERSAL_BRESENHAM && (v < 0 || v >= lim[a]))
                    throw Error{2, "Argument error: receiver coordinate outside the volume!"};
                ie[3 * g.ne + a * g.nr + q] = v;
            }
        }
        g.ie.alloc(ie.size());
        TV3_CUDA(cudaMemcpy(g.ie.p, ie.data(), ie.size() * sizeof(int), cudaMemcpyHostToDevice));
    }
    if (G->traversal == TVAL3_TRAVERSAL_SIDDON) {
        std::vector<double> pe(3 * (g.ne + g.nr));
        const double* src[6] = {G->xe_pos, G->ye_pos, G->ze_pos, G->xr_pos, G->yr_pos, G->zr_pos};
        for (int a = 0; a < 3; ++a) {
            for (long e = 0; e < g.ne; ++e) {
                double v = have_pos ? src[a][e] : ie[a * g.ne + e] + 0.5;
                if (!std::isfinite(v)) throw Error{6, "Argument error: non-finite coordinate!"};
                if (std::fabs(v) > 1e6) throw Error{1, "Argument error: coordinate beyond 1e6 voxels!"};
                pe[a * g.ne + e] = v;
            }
            for (long q = 0; q < g.nr; ++q) {
                double v = have_pos ? src[3 + a][q] : ie[3 * g.ne + a * g.nr + q] + 0.5;
                if (!std::isfinite(v)) throw Error{6, "Argument error: non-finite coordinate!"};
                if (std::fabs(v) > 1e6) throw Error{1, "Argument error: coordinate beyond 1e6 voxels!"};
                pe[3 * g.ne + a * g.nr + q] = v;
            }
        }
        g.pe.alloc(pe.size());
        TV3_CUDA(cudaMemcpy(g.pe.p, pe.data(), pe.size() * sizeof(double), cudaMemcpyHostToDevice));
    }
    g.pairs.alloc(std::max<size_t>(pairs.size(), 2));
    if (!pairs.empty())
        TV3_CUDA(cudaMemcpy(g.pairs.p, pairs.data(), pairs.size() * sizeof(unsigned), cudaMemcpyHostToDevice));
}

static GeomView view_of(const RayGeom& geo) {
    GeomView v;
    v.nrays = geo.nrays; v.nx = geo.nx; v.ny = geo.ny; v.nz = geo.nz; v.ne = geo.ne; v.nr = geo.nr;
    v.pairs = geo.pairs.p; v.ie = geo.ie.p; v.pe = geo.pe.p; v.scale = geo.scale;
    return v;
}

// the device CSR of a geometry: count pass, exclusive scan, fill pass
struct RayCsr {
    long m = 0, n = 0;
    int nnz = 0;
    DBuf<int> ptr, ind;
    DBuf<float> val;
};

static RayCsr build_ray_csr(const tval3_geometry_host* G, cudaStream_t s) {
    RayGeom geo;
    upload_geometry(G, geo);
    RayCsr c;
    c.m = geo.nrays;
    c.n = (long)geo.nx * geo.ny * geo.nz;
    const long m = c.m;
    GeomView v = view_of(geo);
    DBuf<int> len(std::max<long>(m, 1) + 1);
    c.ptr.alloc(m + 1);
    TV3_CUDA(cudaMemsetAsync(len.p, 0, (m + 1) * sizeof(int), s));
    const int grid = grid_for(m, 128);
    if (m) k_ray_count<<<grid, 128, 0, s>>>(v, geo.traversal, len.p);
    TV3_CUDA(cudaGetLastError());
    size_t tmp_bytes = 0;
    TV3_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tmp_bytes, len.p, c.ptr.p, (int)(m + 1), s));
    DBuf<char> tmp(tmp_bytes);
    TV3_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tmp_bytes, len.p, c.ptr.p, (int)(m + 1), s));
    TV3_CUDA(cudaMemcpyAsync(&c.nnz, c.ptr.p + m, sizeof(int), cudaMemcpyDeviceToHost, s));
    TV3_CUDA(cudaStreamSynchronize(s));
    if (c.nnz < 0) throw Error{2, "ray matrix exceeds 2^31 nonzeros"};
    c.ind.alloc(std::max(c.nnz, 1));
    c.val.alloc(std::max(c.nnz, 1));
    if (m) k_ray_fill<<<grid, 128, 0, s>>>(v, geo.traversal, c.ptr.p, c.ind.p, c.val.p);
    TV3_CUDA(cudaGetLastError());
    TV3_CUDA(cudaStreamSynchronize(s));
    return c;
}

// On-the-fly operator of a geometry: A*x walks the rays (k_bres_N, k_sid_N),
// A^T*y resumes the stored tile runs (k_run_T).  Held on the device: the
// geometry, the Siddon rays' constants (88 bytes a ray) and the runs (16
// bytes a run), no matrix values or voxel indices.
struct RayFlyOp : LinOp<float> {
    RayGeom geo;
    DBuf<SidRay> rec;
    DBuf<RunEntry> ent;
    DBuf<long long> tile_off;
    DBuf<int> tile_order;
    RunView rv{};
    long long nruns = 0;

    template <int TRAV>
    void build_runs(cudaStream_t s) {
        GeomView g = view_of(geo);
        const int N[3] = {geo.nx, geo.ny, geo.nz};
        const int T3[3] = {8, 8, 8}, T2[3] = {16, 16, 1};
        const int* T = (geo.nz == 1) ? T2 : T3;
        long long ntl = 1;
        for (int a = 0; a < 3; ++a) {
            rv.T[a] = T[a];
            rv.nt[a] = (N[a] + T[a] - 1) / T[a];
            ntl *= rv.nt[a];
        }
        if (ntl > (1LL << 30)) throw Error{2, "volume has too many voxel tiles"};
        rv.ntiles = (int)ntl;
        const long m = geo.nrays;
        if (TRAV == TVAL3_TRAVERSAL_SIDDON) rec.alloc(std::max<long>(m, 1));
        // runs and segments per ray, then their totals and the runs' offsets
        DBuf<long long> runs(m + 1), segs(m + 1), run_off(m + 1), seg_total(1);
        DBuf<unsigned> err(1);
        TV3_CUDA(cudaMemsetAsync(runs.p, 0, (m + 1) * sizeof(long long), s));
        TV3_CUDA(cudaMemsetAsync(segs.p, 0, (m + 1) * sizeof(long long), s));
        TV3_CUDA(cudaMemsetAsync(err.p, 0, sizeof(unsigned), s));
        const int grid = grid_for(m, 128);
        if (m) k_runs_count<TRAV><<<grid, 128, 0, s>>>(g, rv, rec.p, runs.p, segs.p, err.p);
        TV3_CUDA(cudaGetLastError());
        {
            size_t tb = 0, tb2 = 0;
            TV3_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, tb, runs.p, run_off.p, (int)(m + 1), s));
            TV3_CUDA(cub::DeviceReduce::Sum(nullptr, tb2, segs.p, seg_total.p, (int)(m + 1), s));
            DBuf<char> tmp(std::max(tb, tb2));
            TV3_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, tb, runs.p, run_off.p, (int)(m + 1), s));
            TV3_CUDA(cub::DeviceReduce::Sum(tmp.p, tb2, segs.p, seg_total.p, (int)(m + 1), s));
            long long h[2] = {0, 0};
            unsigned herr = 0;
            TV3_CUDA(cudaMemcpyAsync(&h[0], run_off.p + m, sizeof(long long), cudaMemcpyDeviceToHost, s));
            TV3_CUDA(cudaMemcpyAsync(&h[1], seg_total.p, sizeof(long long), cudaMemcpyDeviceToHost, s));
            TV3_CUDA(cudaMemcpyAsync(&herr, err.p, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
            TV3_CUDA(cudaStreamSynchronize(s));
            if (herr) throw Error{2, "a ray's tile run exceeds the packed run format"};
            nruns = h[0];
            nnz = (long)h[1];
        }
        if (nruns >= (long long)INT32_MAX) throw Error{2, "ray walk has more than 2^31 tile runs"};
        const long E = (long)nruns, E1 = std::max<long>(E, 1);
        const int nt = rv.ntiles;
        // the runs in ray order with their tiles, and the tiles' run counts
        DBuf<RunEntry> raw(E1);
        DBuf<int> key(E1), key_s(E1), idx(E1), idx_s(E1), tcnt(nt), tcnt_s(nt), tids(nt);
        TV3_CUDA(cudaMemsetAsync(tcnt.p, 0, nt * sizeof(int), s));
        if (m) k_runs_fill<TRAV><<<grid, 128, 0, s>>>(g, rv, rec.p, run_off.p, raw.p, key.p, tcnt.p);
        k_iota<<<grid_for(E1, 256), 256, 0, s>>>(idx.p, E);
        k_iota<<<grid_for(nt, 256), 256, 0, s>>>(tids.p, nt);
        DBuf<long long> c64(nt + 1);
        TV3_CUDA(cudaMemsetAsync(c64.p, 0, (nt + 1) * sizeof(long long), s));
        k_widen_count<<<grid_for(nt, 256), 256, 0, s>>>(tcnt.p, c64.p, nt);
        TV3_CUDA(cudaGetLastError());
        int bits = 1;
        while ((1LL << bits) < nt) ++bits;
        ent.alloc(E1);
        tile_off.alloc(nt + 1);
        tile_order.alloc(nt);
        size_t sb = 0, sb2 = 0, sb3 = 0;
        TV3_CUDA(cub::DeviceRadixSort::SortPairs(nullptr, sb, key.p, key_s.p, idx.p, idx_s.p, (int)E1, 0, bits, s));
        TV3_CUDA(cub::DeviceRadixSort::SortPairsDescending(nullptr, sb2, tcnt.p, tcnt_s.p, tids.p, tile_order.p, nt,
                                                           0, 32, s));
        TV3_CUDA(cub::DeviceScan::ExclusiveSum(nullptr, sb3, c64.p, tile_off.p, nt + 1, s));
        DBuf<char> tmp(std::max(sb, std::max(sb2, sb3)));
        // stable sort by tile: inside a tile the runs stay in ray order
        if (E) {
            TV3_CUDA(cub::DeviceRadixSort::SortPairs(tmp.p, sb, key.p, key_s.p, idx.p, idx_s.p, (int)E, 0, bits, s));
            k_gather_runs<<<grid_for(E, 256), 256, 0, s>>>(raw.p, idx_s.p, ent.p, E);
            TV3_CUDA(cudaGetLastError());
        }
        TV3_CUDA(cub::DeviceScan::ExclusiveSum(tmp.p, sb3, c64.p, tile_off.p, nt + 1, s));
        // every tile, most runs first (equal counts in tile order: the sort is stable)
        TV3_CUDA(cub::DeviceRadixSort::SortPairsDescending(tmp.p, sb2, tcnt.p, tcnt_s.p, tids.p, tile_order.p, nt, 0,
                                                           32, s));
        TV3_CUDA(cudaStreamSynchronize(s));
        rv.tile_off = tile_off.p;
        rv.tile_order = tile_order.p;
        rv.ent = ent.p;
        rv.rec = rec.p;
    }

    void apply(int trans, const MatIO<float>& io, int epi, cudaStream_t s) const override {
        if (io.L > 1) throw Error{7, "on-the-fly ray operators take one right-hand side"};
        const GeomView g = view_of(geo);
        const bool sid = geo.traversal == TVAL3_TRAVERSAL_SIDDON;
        if (!trans) {
            if (sid) {
                const int grid = grid_for(g.nrays, 256);
                switch (epi) {
                    case SPMV_LAM35: k_sid_N<SPMV_LAM35><<<grid, 256, 0, s>>>(g, rec.p, io); break;
                    case SPMV_NORM2: k_sid_N<SPMV_NORM2><<<grid, 256, 0, s>>>(g, rec.p, io); break;
                    default: k_sid_N<SPMV_PLAIN><<<grid, 256, 0, s>>>(g, rec.p, io); break;
                }
            } else {
                const int G = 32;
                const int grid = grid_for(g.nrays * G, 256);
                switch (epi) {
                    case SPMV_LAM35: k_bres_N<G, SPMV_LAM35><<<grid, 256, 0, s>>>(g, io); break;
                    case SPMV_NORM2: k_bres_N<G, SPMV_NORM2><<<grid, 256, 0, s>>>(g, io); break;
                    default: k_bres_N<G, SPMV_PLAIN><<<grid, 256, 0, s>>>(g, io); break;
                }
            }
        } else {
            const int grid = rv.ntiles;
            const bool sub = epi == SPMV_SUB;
            if (sid) {
                if (sub) k_run_T<TVAL3_TRAVERSAL_SIDDON, SPMV_SUB><<<grid, 256, 0, s>>>(g, rv, io);
                else k_run_T<TVAL3_TRAVERSAL_SIDDON, SPMV_PLAIN><<<grid, 256, 0, s>>>(g, rv, io);
            } else {
                if (sub) k_run_T<TVAL3_TRAVERSAL_BRESENHAM, SPMV_SUB><<<grid, 256, 0, s>>>(g, rv, io);
                else k_run_T<TVAL3_TRAVERSAL_BRESENHAM, SPMV_PLAIN><<<grid, 256, 0, s>>>(g, rv, io);
            }
        }
        TV3_CUDA(cudaGetLastError());
    }
};

template <>
LinOp<float>* make_geometry_op<float>(const void* gh, int mode, int precision, cudaStream_t s) {
    const tval3_geometry_host* G = static_cast<const tval3_geometry_host*>(gh);
    if (mode == 1) {
        std::unique_ptr<RayFlyOp> op(new RayFlyOp());
        upload_geometry(G, op->geo);
        op->m = op->geo.nrays;
        op->n = (long)op->geo.nx * op->geo.ny * op->geo.nz;
        op->kind = 2;
        if (op->geo.traversal == TVAL3_TRAVERSAL_SIDDON) op->build_runs<TVAL3_TRAVERSAL_SIDDON>(s);
        else op->build_runs<TVAL3_TRAVERSAL_BRESENHAM>(s);
        return op.release();
    }
    RayCsr c = build_ray_csr(G, s);
    return make_csr_op_device<float>(c.m, c.n, c.nnz, c.ptr.p, c.ind.p, c.val.p, nullptr, nullptr, nullptr, precision,
                                     s);
}

template <>
LinOp<double>* make_geometry_op<double>(const void* gh, int mode, int precision, cudaStream_t s) {
    // precision 4: FP64-vector products; 5: the storage behind a double-float
    // view, which runs no products of its own (so no lane timing)
    if (mode != 0 || (precision != 4 && precision != 5))
        throw Error{7, "FP64-vector geometry operators are stored (mode 0) with FP32 values"};
    RayCsr c = build_ray_csr(static_cast<const tval3_geometry_host*>(gh), s);
    return make_csr_op_f64vec(c.m, c.n, c.nnz, c.ptr.p, c.ind.p, c.val.p, nullptr, nullptr, nullptr, s,
                              precision == 4);
}

template <>
LinOp<df64>* make_geometry_op<df64>(const void* gh, int mode, int precision, cudaStream_t s) {
    // precision 6 / 7: the ray matrix in BF16 / FP16 with per-ray FP32 scales,
    // double-float products
    if (mode != 0 || (precision != 6 && precision != 7))
        throw Error{7, "mixed-precision geometry operators are stored (mode 0) with BF16 or FP16 values"};
    RayCsr c = build_ray_csr(static_cast<const tval3_geometry_host*>(gh), s);
    return make_csr_op_df64q(c.m, c.n, c.nnz, c.ptr.p, c.ind.p, c.val.p, nullptr, nullptr, nullptr, precision, s);
}

}  // namespace tv3
