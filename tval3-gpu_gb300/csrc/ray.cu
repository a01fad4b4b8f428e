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
    b.s1 = st[b.a1]; b.s2 = st[b.a2]; b.s3 = st[b.a3];
    return b;
}

// linear index of voxel j (0 = emitter voxel) of a Bresenham ray
__device__ __forceinline__ long bres_voxel(const BresRay& b, int j, int nx, int ny) {
    long twom1 = 2L * b.m1;
    int k2 = b.m1 ? (int)((2L * b.m2 * j + b.m1 - 1) / twom1) : 0;
    int k3 = b.m1 ? (int)((2L * b.m3 * j + b.m1 - 1) / twom1) : 0;
    int c[3];
    c[b.a1] = b.s1 + b.inc1 * j;
    c[b.a2] = b.s2 + b.inc2 * k2;
    c[b.a3] = b.s3 + b.inc3 * k3;
    return (long)c[2] * nx * ny + (long)c[0] * ny + c[1];
}

__device__ __forceinline__ double dmin_(double a, double b) { return (b < a) ? b : a; }
__device__ __forceinline__ double dmax_(double a, double b) { return (a < b) ? b : a; }

// Siddon walk; emit(index, float length) for each segment of positive length.
// Every floating-point operation is an explicitly rounded intrinsic so that it
// matches the host evaluation (compiled without contraction) bit for bit.
template <class F>
__device__ void siddon_walk_dev(const double P0[3], const double P1[3], const int N[3], double scale, F emit) {
    double dv[3];
    for (int a = 0; a < 3; ++a) dv[a] = __dsub_rn(P1[a], P0[a]);
    double L = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dv[0], dv[0]), __dmul_rn(dv[1], dv[1])), __dmul_rn(dv[2], dv[2])));
    if (!(L > 0.0)) return;
    double tmin = 0.0, tmax = 1.0;
    for (int a = 0; a < 3; ++a) {
        if (dv[a] == 0.0) {
            if (!(P0[a] >= 0.0 && P0[a] < (double)N[a])) return;
        } else {
            double t0 = __ddiv_rn(__dsub_rn(0.0, P0[a]), dv[a]);
            double t1 = __ddiv_rn(__dsub_rn((double)N[a], P0[a]), dv[a]);
            double lo = dmin_(t0, t1), hi = dmax_(t0, t1);
            tmin = dmax_(tmin, lo);
            tmax = dmin_(tmax, hi);
        }
    }
    if (!(tmin < tmax)) return;
    double tn[3];
    long k[3];
    int st[3];
    for (int a = 0; a < 3; ++a) {
        if (dv[a] == 0.0) {
            tn[a] = INFINITY; k[a] = 0; st[a] = 0;
            continue;
        }
        st[a] = dv[a] > 0 ? 1 : -1;
        double pos = __dadd_rn(P0[a], __dmul_rn(tmin, dv[a]));
        k[a] = (st[a] > 0) ? (long)floor(pos) + 1 : (long)ceil(pos) - 1;
        tn[a] = __ddiv_rn(__dsub_rn((double)k[a], P0[a]), dv[a]);
        for (int guard = 0; tn[a] <= tmin && guard < 4; ++guard) {
            k[a] += st[a];
            tn[a] = __ddiv_rn(__dsub_rn((double)k[a], P0[a]), dv[a]);
        }
    }
    double t = tmin;
    // at most one segment per crossed plane (the guard only bounds degenerate input)
    for (int guard = N[0] + N[1] + N[2] + 8; t < tmax && guard > 0; --guard) {
        double te = dmin_(dmin_(tn[0], tn[1]), dmin_(tn[2], tmax));
        if (te > t) {
            double mid = __dmul_rn(0.5, __dadd_rn(t, te));
            int idx[3];
            for (int a = 0; a < 3; ++a) {
                double c = __dadd_rn(P0[a], __dmul_rn(mid, dv[a]));
                long v = (long)floor(c);
                if (v < 0) v = 0;
                if (v > N[a] - 1) v = N[a] - 1;
                idx[a] = (int)v;
            }
            double len = __dmul_rn(__dsub_rn(te, t), L);
            emit((long)idx[2] * N[0] * N[1] + (long)idx[0] * N[1] + idx[1], __double2float_rn(__dmul_rn(len, scale)));
        }
        for (int a = 0; a < 3; ++a)
            if (tn[a] == te) {
                k[a] += st[a];
                tn[a] = __ddiv_rn(__dsub_rn((double)k[a], P0[a]), dv[a]);
            }
        t = te;
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
// on-the-fly Bresenham operator: G lanes per ray, each lane a stride of voxels
// ---------------------------------------------------------------------------
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
        if (lane == 0) {
            s *= w;
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

// A^T y by scattering: out must be zero on entry
template <int G>
__global__ void __launch_bounds__(256) k_bres_T(GeomView g, MatIO<float> io) {
    count_launch(io.ctl);
    const int lane = threadIdx.x % G;
    const long grp = ((long)blockIdx.x * blockDim.x + threadIdx.x) / G;
    const long ngrp = ((long)gridDim.x * blockDim.x) / G;
    const int sel = io.by_parity ? io.ctl->parity : 0;
    const float* __restrict__ yv = io.x[sel];
    float* __restrict__ out = io.y[sel];
    const float w = (float)g.scale;
    for (long r = grp; r < g.nrays; r += ngrp) {
        int xs, ys, zs, xe, ye, ze;
        ray_ends_int(g, r, xs, ys, zs, xe, ye, ze);
        BresRay b = bres_setup(xs, ys, zs, xe, ye, ze);
        const float v = yv[r] * w;
        if (v != 0.f)
            for (int j = lane; j <= b.m1; j += G) atomicAdd(out + bres_voxel(b, j, g.nx, g.ny), v);
    }
}

__global__ void k_zero_sel(MatIO<float> io, long n) {
    count_launch(io.ctl);
    const int sel = io.by_parity ? io.ctl->parity : 0;
    float* y = io.y[sel];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) y[i] = 0.f;
}

__global__ void k_sub_sel(MatIO<float> io, long n) {
    count_launch(io.ctl);
    const int sel = io.by_parity ? io.ctl->parity : 0;
    float* y = io.y[sel];
    for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (long)gridDim.x * blockDim.x) y[i] -= io.sub[i];
}

static int grid_for(long items, int per_block) {
    long g = (items + per_block - 1) / per_block;
    long cap = (long)num_sms() * 8;
    return (int)std::max<long>(1, std::min(g, cap));
}

struct BresOp : LinOp<float> {
    RayGeom geo;
    GeomView view() const {
        GeomView v;
        v.nrays = geo.nrays; v.nx = geo.nx; v.ny = geo.ny; v.nz = geo.nz; v.ne = geo.ne; v.nr = geo.nr;
        v.pairs = geo.pairs.p; v.ie = geo.ie.p; v.pe = geo.pe.p; v.scale = geo.scale;
        return v;
    }
    void apply(int trans, const MatIO<float>& io, int epi, cudaStream_t s) const override {
        if (io.L > 1) throw Error{7, "on-the-fly ray operators take one right-hand side"};
        const GeomView g = view();
        const int G = 32;
        const int grid = grid_for(g.nrays * G, 256);
        if (!trans) {
            switch (epi) {
                case SPMV_LAM35: k_bres_N<G, SPMV_LAM35><<<grid, 256, 0, s>>>(g, io); break;
                case SPMV_NORM2: k_bres_N<G, SPMV_NORM2><<<grid, 256, 0, s>>>(g, io); break;
                default: k_bres_N<G, SPMV_PLAIN><<<grid, 256, 0, s>>>(g, io); break;
            }
        } else {
            const long nv = (long)geo.nx * geo.ny * geo.nz;
            k_zero_sel<<<grid_for(nv, 256), 256, 0, s>>>(io, nv);
            k_bres_T<G><<<grid, 256, 0, s>>>(g, io);
            if (epi == SPMV_SUB) k_sub_sel<<<grid_for(nv, 256), 256, 0, s>>>(io, nv);
        }
        TV3_CUDA(cudaGetLastError());
    }
};

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

template <>
LinOp<float>* make_geometry_op<float>(const void* gh, int mode, int precision, cudaStream_t s) {
    const tval3_geometry_host* G = static_cast<const tval3_geometry_host*>(gh);
    if (mode == 1) {
        if (G && G->traversal != TVAL3_TRAVERSAL_BRESENHAM)
            throw Error{7, "on-the-fly traversal is provided for the Bresenham rays of the reference"};
        auto* op = new BresOp();
        try {
            upload_geometry(G, op->geo);
            op->m = op->geo.nrays;
            op->n = (long)op->geo.nx * op->geo.ny * op->geo.nz;
            op->kind = 2;
            // nnz of the implied matrix: sum of m1 + 1 (host arithmetic from the coordinates)
            op->nnz = 0;
        } catch (...) {
            delete op;
            throw;
        }
        return op;
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
