/*
 * tval3_c.h -- C ABI of the GB300 (sm_103a) TVAL3 reconstructor.
 *
 * Drop-in boundary for the reference's tval3_gpu_3d / tval3_gpu entry points
 * and its mat_vec_mul operator interface (modk/tval3-gpu).  Plain C types and
 * pointers only; every function returns a tval3_status and, on failure, sets
 * a thread-local message readable with tval3_last_error_message().  The C++
 * header tval3.hpp restores the reference's overloads, container classes and
 * exception types on top of these functions.
 *
 * Data layout: volumes are column-major with y fastest (the reference's
 * mat_host with dim_y, dim_x, dim_z; 3d/tval3_gpu_3d_kernels.cu:1501):
 * voxel (y, x, z) is element y + dim_y*(x + dim_x*z).  Sparse matrices are
 * A (rays x voxels) in CSR, plus optionally the CSR of A^T (the reference's
 * CSC arrays, 3d/tval3_gpu_3d.cpp:1463).
 */
#ifndef TVAL3_C_H_
#define TVAL3_C_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#if defined(_WIN32)
#define TVAL3_API
#else
#define TVAL3_API __attribute__((visibility("default")))
#endif

/* Status codes.  Replace the reference's exceptions (tval3_gpu_exception,
 * cuda_exception, illegal_mat_gpu_assignment; 2d/tval3_types.h:45-49,
 * 2d/handle_error.h:14-41). */
typedef enum tval3_status {
    TVAL3_OK = 0,
    TVAL3_ERR_ARG = 1,        /* argument error (reference: "Argument error: ...") */
    TVAL3_ERR_SHAPE = 2,      /* inconsistent dimensions */
    TVAL3_ERR_CUDA = 3,       /* CUDA runtime error */
    TVAL3_ERR_NOMEM = 4,      /* device or host allocation failed */
    TVAL3_ERR_TIMEOUT = 5,    /* a bounded device wait expired */
    TVAL3_ERR_NONFINITE = 6,  /* NaN/Inf in an input */
    TVAL3_ERR_UNSUPPORTED = 7 /* combination not provided by this build */
} tval3_status;

typedef enum tval3_tv { TVAL3_TV_ANISO = 0, TVAL3_TV_ISO = 1 } tval3_tv;

/* Storage precision of operator values. */
typedef enum tval3_precision {
    TVAL3_PREC_FP32 = 0,
    TVAL3_PREC_FP64 = 1,
    TVAL3_PREC_BF16 = 2, /* BF16 values with per-row FP32 scale, FP32 accumulation */
    TVAL3_PREC_FP16 = 3, /* FP16 values with per-row FP32 scale, FP32 accumulation */
    TVAL3_PREC_FP32_F64VEC = 4, /* FP32 values, FP64 vectors, products and reductions */
    TVAL3_PREC_FP32_DF64 = 5,   /* FP32 values; vectors, products and reductions in double-float
                                   (pairs of FP32, ~48 bits) on the FP32 pipes; FP64 at the interface */
    TVAL3_PREC_BF16_DF64 = 6,   /* mixed: BF16 values with a per-row FP32 scale (the matrix stream
                                   shrinks to 2 bytes per value); vectors, products, the step size,
                                   line-search inner products and stopping norms in double-float;
                                   FP64 at the interface */
    TVAL3_PREC_FP16_DF64 = 7    /* mixed: as TVAL3_PREC_BF16_DF64 with FP16 values */
} tval3_precision;

typedef enum tval3_trans { TVAL3_OP_N = 0, TVAL3_OP_T = 1 } tval3_trans;

/* Options: the fields of tval3_options (2d/tval3_types.h:7-35) and the 3D
 * skip-multiplication fields (3d/tval3_gpu_3d.cpp:194-197), plus tv_type.
 * tval3_options_default() sets the reference defaults (2d/tval3_types.h:29-33). */
typedef struct tval3_options {
    double mu;        /* maximum mu */
    double mu0;       /* initial mu */
    double beta;      /* maximum beta */
    double beta0;     /* initial beta */
    double rate_cnt;  /* continuation rate of mu and beta */
    double tol;       /* outer tolerance */
    double tol_inn;   /* inner tolerance */
    int maxcnt;       /* maximum outer iterations */
    int maxit;        /* maximum total iterations */
    double c;         /* Armijo parameter */
    double gamma;     /* backtracking factor */
    double gam;       /* nonmonotone weight */
    double rate_gam;  /* shrink rate of gam after a failed backtracking */
    int isreal;       /* kept for interface compatibility (unused, as in the reference) */
    int nonneg;       /* project onto U >= 0 */
    unsigned numInitIterations; /* skip-A^T heuristic (3d/tval3_gpu_3d.cpp:398-468): A^T Au is always */
    double skipMulRatio;        /* formed during the first numInitIterations get_g calls, then skipped */
    double maxRelativeChange;   /* by this ratio unless ||Au - last_Au|| / ||Au|| > maxRelativeChange;
                                   skipMulRatio = 0 (the default) forms it every time */
    int tv_type;      /* tval3_tv; the reference is anisotropic */
    int precision;    /* internal arithmetic of the host entry points: -1 = the entry point's
                         type; TVAL3_PREC_FP32_DF64 with an _f64 entry and FP32 matrix values
                         runs the solve in double-float; TVAL3_PREC_BF16_DF64 / FP16_DF64
                         with an _f64 sparse or geometry entry store the matrix in 16 bits
                         (per-row FP32 scale) and run the solve in double-float */
} tval3_options;

/* Result summary (tval3_info, 2d/tval3_types.h:37-43; outer_secs
 * 3d/tval3_gpu_3d.cpp:1507) plus line-search counters. */
typedef struct tval3_info {
    int total_iters;
    int outer_iters;
    double rel_chg;
    double rel_error;
    double secs;
    double outer_secs;
    int backtracks;
    int restarts;
    double final_f;
    int launches;     /* kernels the solve ran on the device */
    int products_T;   /* A^T products formed by get_g under the skip heuristic (-1: heuristic off) */
} tval3_info;

/* Sparse matrix in host memory (sparse_mat_host, 2d/container_host.h:78-127).
 * rows = m (measurements, reference A.dim_y), cols = n (voxels, A.dim_x).
 * format: 1 = CSR only, 2 = CSC only, 3 = both (the 3D reference requires 3,
 * 3d/tval3_gpu_3d.cpp:1463; this library builds whichever part is missing).
 * val_type: TVAL3_PREC_FP32 or TVAL3_PREC_FP64 (type of csr_val / csc_val). */
typedef struct tval3_sparse_host {
    int rows, cols, nnz;
    int format;
    int val_type;
    const int* csr_ptr;
    const int* csr_ind;
    const void* csr_val;
    const int* csc_ptr;
    const int* csc_ind;
    const void* csc_val;
} tval3_sparse_host;

#define TVAL3_SPARSE_CSR 1
#define TVAL3_SPARSE_CSC 2
#define TVAL3_SPARSE_BOTH 3

/* Dense matrix in host memory (mat_host, column-major by default;
 * 3d/tval3_gpu_3d.cpp:1404 requires column-major). row_major = 1 accepts a
 * row-major array too.  rows = m, cols = n. */
typedef struct tval3_dense_host {
    int rows, cols;
    int row_major;
    int val_type;
    const void* data;
} tval3_dense_host;

/* Measurement geometry (geometry_host; fields read by geometry_device,
 * 3d/container_device.h:683-750).  Coordinates are voxel indices per
 * measurement position: x_emitters[numMPs*num_emitters] etc.  use_path
 * (num_emitters*num_receivers flags, may be NULL = all) selects the rays; the
 * ray list is compacted as in 3d/mat_vec_mul_dynamic.h:477-556.
 * traversal 0 = integer Bresenham (dyn_calc_kernel, weight scale_factor);
 * traversal 1 = Siddon exact path lengths from the continuous coordinates
 * *_pos (voxel units, NULL = voxel centres of the integer coordinates),
 * multiplied by scale_factor. */
typedef struct tval3_geometry_host {
    int numMPs;
    int num_emitters, num_receivers;
    const int *x_emitters, *y_emitters, *z_emitters;
    const int *x_receivers, *y_receivers, *z_receivers;
    const unsigned* use_path;
    int rv_x, rv_y, rv_z;
    float scale_factor;
    int traversal;
    const double *xe_pos, *ye_pos, *ze_pos;
    const double *xr_pos, *yr_pos, *zr_pos;
} tval3_geometry_host;

#define TVAL3_TRAVERSAL_BRESENHAM 0
#define TVAL3_TRAVERSAL_SIDDON 1

/* ---------------------------------------------------------------------- */
TVAL3_API void tval3_options_default(tval3_options* opts);
TVAL3_API const char* tval3_last_error_message(void);
/* Seconds spent in the phases of the calling thread's last call of a
 * reference entry point (tval3_gpu_3d_* / tval3_gpu_*): [0] operator (input
 * checks, upload, transpose or quantisation, ray-matrix build), [1] set-up
 * (b upload, solver workspace, tile-staged layouts and kernel choice), [2]
 * solve (graph capture and instantiation on first use, then the solve), [3]
 * download of U; then parts of those: [4] matrix upload, [5] input
 * validation, [6] operator layout (device copies, transpose, quantisation,
 * ray-matrix build), [7] tile-staged layouts and kernel choice, [8] graph
 * capture and instantiation, [9] the host-to-device copies alone (inside
 * [4], which also holds the device allocations).  n entries are written (at
 * most 10).  No counterpart in the reference. */
TVAL3_API tval3_status tval3_last_call_phases(double* secs, int n);
TVAL3_API const char* tval3_version(void);
/* Self-test of the bounded device waits: one warp waits `cycles` of SM clock
 * (at most 4e9, about two seconds) on an mbarrier phase that nothing
 * completes.  *timed_out = 1 when the wait gave up, as it must;
 * *waited_cycles = the cycles it waited.  The pipelined kernels use the same
 * wait with a limit of 4e9 cycles.  No counterpart in the reference. */
TVAL3_API tval3_status tval3_selftest_bounded_wait(int64_t cycles, int* timed_out, int64_t* waited_cycles);

/* ---------------------------------------------------------------------- *
 * Reference entry points.  U (dim_y x dim_x x dim_z, column-major) is output
 * only; A and b are read; Ut (length n or NULL) enables info->rel_error.
 * pagelocked / mainGPU / numGPUs / gpuArray are accepted for compatibility;
 * this library runs on the current device only (one GPU).
 * ---------------------------------------------------------------------- */

/* tval3_gpu_3d(U, sparse_mat_host<float> A, b, opts, Ut, ...),
 * 3d/tval3_gpu_3d.cpp:23-27 and :1454-1530 */
TVAL3_API tval3_status tval3_gpu_3d_sparse_f32(float* U, int dim_y, int dim_x, int dim_z,
                                               const tval3_sparse_host* A, const float* b, int b_len,
                                               const tval3_options* opts, const float* Ut, int Ut_len,
                                               int pagelocked, int mainGPU, int numGPUs, const int* gpuArray,
                                               tval3_info* info);
/* double instantiation, 3d/tval3_gpu_3d.cpp:46-50 */
TVAL3_API tval3_status tval3_gpu_3d_sparse_f64(double* U, int dim_y, int dim_x, int dim_z,
                                               const tval3_sparse_host* A, const double* b, int b_len,
                                               const tval3_options* opts, const double* Ut, int Ut_len,
                                               int pagelocked, int mainGPU, int numGPUs, const int* gpuArray,
                                               tval3_info* info);
/* tval3_gpu_3d(U, mat_host<float> A, ...), 3d/tval3_gpu_3d.cpp:29-33, :1395-1448 */
TVAL3_API tval3_status tval3_gpu_3d_dense_f32(float* U, int dim_y, int dim_x, int dim_z,
                                              const tval3_dense_host* A, const float* b, int b_len,
                                              const tval3_options* opts, const float* Ut, int Ut_len,
                                              int pagelocked, int mainGPU, int numGPUs, const int* gpuArray,
                                              tval3_info* info);
TVAL3_API tval3_status tval3_gpu_3d_dense_f64(double* U, int dim_y, int dim_x, int dim_z,
                                              const tval3_dense_host* A, const double* b, int b_len,
                                              const tval3_options* opts, const double* Ut, int Ut_len,
                                              int pagelocked, int mainGPU, int numGPUs, const int* gpuArray,
                                              tval3_info* info);
/* tval3_gpu_3d(U, geometry_host A, ...), 3d/tval3_gpu_3d.cpp:35-39, :1533-1600:
 * evaluated on the fly as in the reference (no matrix stored), for Bresenham
 * and Siddon rays; A^T*y is deterministic (tile runs summed in a fixed order). */
TVAL3_API tval3_status tval3_gpu_3d_geometry_f32(float* U, int dim_y, int dim_x, int dim_z,
                                                 const tval3_geometry_host* A, const float* b, int b_len,
                                                 const tval3_options* opts, const float* Ut, int Ut_len,
                                                 int pagelocked, int mainGPU, int numGPUs, const int* gpuArray,
                                                 tval3_info* info);
/* tval3_gpu_3d(U, geometry_host, sparse_mat_host, ...) (on-the-fly A*x,
 * sparse A^T*y; sparse_geom_mm), 3d/tval3_gpu_3d.cpp:41-44, :1606-1667 */
TVAL3_API tval3_status tval3_gpu_3d_geometry_sparse_f32(float* U, int dim_y, int dim_x, int dim_z,
                                                        const tval3_geometry_host* A_geo,
                                                        const tval3_sparse_host* A_mat, const float* b,
                                                        int b_len, const tval3_options* opts, const float* Ut,
                                                        int Ut_len, int pagelocked, int mainGPU, int numGPUs,
                                                        const int* gpuArray, tval3_info* info);
/* double instantiations of the geometry overloads, 3d/tval3_gpu_3d.cpp:58-69:
 * the ray matrix is built on the device and stored with FP32 values (the
 * reference evaluates it on the fly); the solve runs with FP64 vectors, or in
 * double-float (opts->precision = TVAL3_PREC_FP32_DF64), or in double-float
 * over a BF16/FP16 copy of the matrix (TVAL3_PREC_BF16_DF64 / FP16_DF64). */
TVAL3_API tval3_status tval3_gpu_3d_geometry_f64(double* U, int dim_y, int dim_x, int dim_z,
                                                 const tval3_geometry_host* A, const double* b, int b_len,
                                                 const tval3_options* opts, const double* Ut, int Ut_len,
                                                 int pagelocked, int mainGPU, int numGPUs, const int* gpuArray,
                                                 tval3_info* info);
/* (U, geometry_host, sparse_mat_host<double>, ...): A*x from the geometry's
 * ray matrix, A^T*y from A_mat, FP64 vectors. */
TVAL3_API tval3_status tval3_gpu_3d_geometry_sparse_f64(double* U, int dim_y, int dim_x, int dim_z,
                                                        const tval3_geometry_host* A_geo,
                                                        const tval3_sparse_host* A_mat, const double* b,
                                                        int b_len, const tval3_options* opts, const double* Ut,
                                                        int Ut_len, int pagelocked, int mainGPU, int numGPUs,
                                                        const int* gpuArray, tval3_info* info);
/* 2D: tval3_gpu(U, sparse_mat_host A, b, opts, Ut, pagelocked), 2d/tval3_gpu.h:9-13;
 * U is rows x cols (dim_y x dim_x), periodic D in 2D (2d/tval3.cu:202-331).
 * layers = b_len / A.rows columns of b share A (2d/tval3.cu:1406-1426): U
 * (and Ut) then hold rows*cols*layers values, one image per column, solved
 * jointly (shared step sizes and penalties, D inside each image). */
TVAL3_API tval3_status tval3_gpu_sparse(float* U, int rows, int cols, const tval3_sparse_host* A, const float* b,
                                        int b_len, const tval3_options* opts, const float* Ut, int Ut_len,
                                        int pagelocked, tval3_info* info);
/* 2D dense: tval3_gpu(U, mat_host A, ...), 2d/tval3_gpu.h:15-19; layers as
 * above.  opts->precision = TVAL3_PREC_BF16 stores A in BF16 with a per-row
 * FP32 scale. */
TVAL3_API tval3_status tval3_gpu_dense(float* U, int rows, int cols, const tval3_dense_host* A, const float* b,
                                       int b_len, const tval3_options* opts, const float* Ut, int Ut_len,
                                       int pagelocked, tval3_info* info);

/* ---------------------------------------------------------------------- *
 * Operator handles: the mat_vec_mul interface (3d/mat_vec_mul_sparse.h:1703,
 * 3d/mat_vec_mul_dense.h:37, 3d/mat_vec_mul_dynamic.h:683,
 * 3d/mat_vec_mul.h:733).  A handle owns device copies of the operator; the
 * products take DEVICE pointers and a stream.
 * ---------------------------------------------------------------------- */
typedef struct tval3_op_s* tval3_op;

/* From host CSR (+ optional CSR of A^T).  precision selects the stored value
 * type: FP32, BF16 or FP16 (the vector type of products is FP32), or FP64
 * (vector type FP64), FP32_F64VEC (FP32 values, vector type FP64), or
 * FP32_DF64 / BF16_DF64 / FP16_DF64 (FP32, BF16 or FP16 values, vector type
 * double-float).  16-bit values carry a per-row FP32 scale (the row's largest
 * magnitude), quantised from FP32 values.  The transpose is built on the
 * device when absent. */
TVAL3_API tval3_status tval3_op_create_sparse(tval3_op* op, const tval3_sparse_host* A, int precision);
/* From device CSR arrays (copied; the caller keeps ownership).  val is FP32. */
TVAL3_API tval3_status tval3_op_create_sparse_device(tval3_op* op, int rows, int cols, int nnz, const int* d_ptr,
                                                     const int* d_ind, const float* d_val, int precision,
                                                     void* stream);
/* From a geometry: the ray matrix (Bresenham or Siddon) is built on the
 * device.  mode 0: stored as CSR; mode 1 (FP32 only): on-the-fly traversal,
 * no matrix stored: A*x walks every ray and gathers x; A^T*y resumes each
 * ray's runs through a voxel tile (16 bytes a run, plus 88 bytes a Siddon
 * ray) and sums the tile's voxels in shared memory in a fixed order, so it is
 * deterministic.  The implied matrix equals the mode-0 CSR bit for bit. */
TVAL3_API tval3_status tval3_op_create_geometry(tval3_op* op, const tval3_geometry_host* G, int mode, int precision);
TVAL3_API tval3_status tval3_op_create_dense(tval3_op* op, const tval3_dense_host* A, int precision);
TVAL3_API tval3_status tval3_op_destroy(tval3_op op);
TVAL3_API tval3_status tval3_op_shape(tval3_op op, int* rows, int* cols, int64_t* nnz);
/* Device memory the operator kept from its creation (matrix storage, the
 * transposed copy, tile layouts, geometry tables); layouts that a solver
 * builds later on first use are not included. */
TVAL3_API tval3_status tval3_op_device_bytes(tval3_op op, int64_t* bytes);
/* Copy the device CSR (A and A^T) of a stored operator to host arrays
 * (ptr: rows+1 / cols+1 ints, ind: nnz ints, val: nnz floats); any pointer may
 * be NULL to skip that array.  Values are FP32 (dequantised for the 16-bit
 * storages: the FP32 rounding of value x row scale). */
TVAL3_API tval3_status tval3_op_export_csr(tval3_op op, int* ptr, int* ind, float* val, int* tptr, int* tind,
                                           float* tval);
/* The stored matrix as the products see it: values val/tval (FP32) and a
 * per-row scale row_scale (rows floats), so that entry (r, c) is exactly
 * val * row_scale[r] (and tval * row_scale[r] in the CSR of A^T) when
 * evaluated in FP64.  For 16-bit storage val holds the 16-bit values widened
 * to FP32 (exact) and row_scale the per-ray scales; for other storage
 * row_scale is all ones and val is what tval3_op_export_csr returns.  Lets a
 * checker rebuild the quantised matrix without the rounding of an FP32
 * product.  Any pointer may be NULL.  No counterpart in the reference. */
TVAL3_API tval3_status tval3_op_export_csr_scaled(tval3_op op, int* ptr, int* ind, float* val, float* row_scale,
                                                  int* tptr, int* tind, float* tval);
/* mat_vec_mul(trans, A, x, y, stream): y = A x (trans = 0) or y = A^T x.
 * x, y are device pointers of the operator's vector type: float (FP32, BF16,
 * FP16 operators), double (FP64, FP32_F64VEC), or double-float pairs
 * {float hi, lo} (FP32_DF64, BF16_DF64, FP16_DF64; see tval3_df64_from_f64).
 * Batched multi-RHS
 * form: nrhs columns, leading dimension = vector length (the reference's
 * `layers`, 2d/mat_vec_mul.h:65-71, :96-99).  Products on the tensor cores
 * (BF16 dense operators with several right-hand sides) have bounded device
 * waits: these calls then wait for the stream and return TVAL3_ERR_TIMEOUT
 * if a wait ran out (the output is incomplete); all other products return
 * without waiting. */
TVAL3_API tval3_status tval3_mat_vec_mul(tval3_op op, int trans, const void* x, void* y, void* stream);
TVAL3_API tval3_status tval3_mat_mat_mul(tval3_op op, int trans, int nrhs, const void* X, void* Y, void* stream);
/* Kernel of the single-vector products of a stored operator whose volume is
 * known (geometry operators, or any operator once a solver has been created
 * on it): variant 0 = CSR kernels, 1 = tile-staged (the vector staged per
 * voxel tile in shared memory), 2 (A^T only, FP32/FP64 matrix values) =
 * tile-staged and pipelined (one CTA per SM; a producer warp stages the next
 * tile's y with bulk and asynchronous copies while the other warps sum the
 * current tile; same sums as variant 1, bit for bit; built on first use and
 * never chosen by the timing).  The library picks between CSR and
 * tile-staged by timing when it builds the tiled form; pinning a variant
 * makes a program's results independent of that timing.
 * TVAL3_ERR_UNSUPPORTED if the variant is not available. */
TVAL3_API tval3_status tval3_op_set_variant(tval3_op op, int trans, int variant);
TVAL3_API tval3_status tval3_op_get_variant(tval3_op op, int trans, int* variant);
/* The same product on interleaved data: element (row, column j) at
 * row * nrhs + j, the layout the multi-layer solver keeps.  One SpMM (CSR),
 * tensor-core GEMM (BF16 dense) or SIMT GEMM (FP32/FP64 dense) launch
 * sequence; the first call for a given nrhs sets up the operator's scratch
 * (make it before any stream capture), later calls allocate nothing.  On the
 * tensor-core path the call waits for the stream and reports a timed-out
 * device wait as TVAL3_ERR_TIMEOUT (see tval3_mat_vec_mul). */
TVAL3_API tval3_status tval3_mat_mat_mul_interleaved(tval3_op op, int trans, int nrhs, const void* X, void* Y,
                                                     void* stream);
/* Device conversions between double and the double-float pairs used by
 * FP32_DF64 operators (hi = round(x), lo = round(x - hi)). */
TVAL3_API tval3_status tval3_df64_from_f64(const double* d_in, void* d_pairs, int64_t n, void* stream);
TVAL3_API tval3_status tval3_df64_to_f64(const void* d_pairs, double* d_out, int64_t n, void* stream);

/* ---------------------------------------------------------------------- *
 * Device-resident solver: a workspace bound to an operator and a volume;
 * solve() takes DEVICE b and writes DEVICE U.  Repeated solves reuse the
 * workspace (no allocation per call).
 * ---------------------------------------------------------------------- */
typedef struct tval3_solver_s* tval3_solver;
TVAL3_API tval3_status tval3_solver_create(tval3_solver* s, tval3_op A, int dim_y, int dim_x, int dim_z,
                                           const tval3_options* opts);
/* The same with `layers` right-hand sides sharing A (the 2D entries' layers):
 * d_b is rows(A) x layers and d_U cols(A) x layers, column-major. */
TVAL3_API tval3_status tval3_solver_create_layers(tval3_solver* s, tval3_op A, int dim_y, int dim_x, int dim_z,
                                                  int layers, const tval3_options* opts);
/* mode 0: host-driven loop with device-resident scalars; mode 1: the whole
 * solve as one CUDA graph with conditional nodes (no host round trips). */
TVAL3_API tval3_status tval3_solver_set_mode(tval3_solver s, int mode);
TVAL3_API tval3_status tval3_solver_solve(tval3_solver s, const void* d_b, void* d_U, const void* d_Ut,
                                          tval3_info* info, void* stream);
/* Solver state (no counterpart in the reference; checkpoint/resume): the
 * control block and every workspace vector of a finished solve, in a host
 * buffer of tval3_solver_state_size bytes.  tval3_solver_resume loads such a
 * state into a solver of the same operator shape, volume, layers and vector
 * type and continues the loop from it under this solver's maxit/maxcnt and
 * pause, writing U like tval3_solver_solve.  A state saved at a pause
 * continues exactly as if the solve had not stopped; a state saved after a
 * stop by maxit continues after that outer step (which the stop completed). */
/* Pause: solves and resumes of this solver stop once the total iteration
 * count reaches `iterations` (0 = never) without ending the outer iteration
 * in progress, so that save_state + resume continue exactly as an
 * uninterrupted solve would (U is written at the pause). */
TVAL3_API tval3_status tval3_solver_set_pause(tval3_solver s, int iterations);
TVAL3_API tval3_status tval3_solver_state_size(tval3_solver s, size_t* bytes);
TVAL3_API tval3_status tval3_solver_save_state(tval3_solver s, void* host_state, void* stream);
TVAL3_API tval3_status tval3_solver_resume(tval3_solver s, const void* host_state, void* d_U, const void* d_Ut,
                                           tval3_info* info, void* stream);
/* Record ||U_k/scl - xstar|| after every iteration k (xstar on device, length
 * n; NULL disables).  Read with tval3_solver_trace (host array of maxit). */
TVAL3_API tval3_status tval3_solver_set_trace(tval3_solver s, const void* d_xstar);
TVAL3_API tval3_status tval3_solver_trace(tval3_solver s, double* host_err, int len);
TVAL3_API tval3_status tval3_solver_destroy(tval3_solver s);

/* ---------------------------------------------------------------------- *
 * Batched solves: many independent problems (the slices of a 2D stack, each
 * with its own size and geometry) solved by ONE CUDA graph launch in which
 * every problem is a parallel branch with its own loops.  The reference
 * solves one image per tval3_gpu call (2d/tval3_gpu.h:9-19, 2d/tval3.cu:
 * 1435-1513); these replace a host loop over that call.
 * ---------------------------------------------------------------------- */
typedef struct tval3_batch_s* tval3_batch;
/* One solver per problem i over ops[i] (borrowed: keep the operators alive
 * until the batch is destroyed) with volume dims[3i .. 3i+2] = (dim_y, dim_x,
 * dim_z).  All operators must have the same vector type. */
TVAL3_API tval3_status tval3_batch_create(tval3_batch* batch, const tval3_op* ops, const int* dims, int count,
                                          const tval3_options* opts);
/* d_b[i], d_U[i] and d_Ut[i] (d_Ut may be NULL, or hold NULL entries) are
 * device vectors of the operators' vector type; infos (count entries, may be
 * NULL) get each problem's counters, and secs = the time of the whole batch. */
TVAL3_API tval3_status tval3_batch_solve(tval3_batch batch, const void* const* d_b, void* const* d_U,
                                         const void* const* d_Ut, tval3_info* infos, void* stream);
/* Elements per block of the vector kernels that the batch's first solve
 * chose by timing short solves of the whole batch (512 ... 4,096; 1,024
 * unless another was at least 3 % faster).  Solvers created later in the
 * process for the same vector type and problem shape take the same grid, so
 * their results equal the batch's bit for bit. */
TVAL3_API tval3_status tval3_batch_tuned_grid(tval3_batch batch, int64_t* elems_per_block);
TVAL3_API tval3_status tval3_batch_destroy(tval3_batch batch);

/* Host form: tval3_gpu(U, sparse A, b, opts, Ut) of every slice (FP32,
 * U rows x cols), all slices in one launch. */
typedef struct {
    float* U;
    int rows, cols;
    const tval3_sparse_host* A;
    const float* b;
    int b_len;
    const float* Ut;
    int Ut_len;
} tval3_slice_host;
TVAL3_API tval3_status tval3_gpu_batched(const tval3_slice_host* slices, int count, const tval3_options* opts,
                                         tval3_info* infos);

/* ---------------------------------------------------------------------- *
 * Stencil operators on device arrays (D_gpu / Dt_gpu, 3d/tval3_gpu_3d.cpp:
 * 271-361).  DU holds 3 consecutive n-vectors (along y, x, z).
 * ---------------------------------------------------------------------- */
TVAL3_API tval3_status tval3_D_f32(int dim_y, int dim_x, int dim_z, const float* d_U, float* d_DU, void* stream);
TVAL3_API tval3_status tval3_Dt_f32(int dim_y, int dim_x, int dim_z, const float* d_V, float* d_out, void* stream);
TVAL3_API tval3_status tval3_D_f64(int dim_y, int dim_x, int dim_z, const double* d_U, double* d_DU, void* stream);
TVAL3_API tval3_status tval3_Dt_f64(int dim_y, int dim_x, int dim_z, const double* d_V, double* d_out,
                                    void* stream);

/* ---------------------------------------------------------------------- *
 * Shrinkage as a differentiable operator (no reference counterpart as an
 * entry point; the forward map is shrinkage_kernel,
 * 3d/tval3_gpu_3d_kernels.cu:1249-1300, plus isotropic TV).  v, W, gW, gv
 * hold 3 n-vectors; W = shrink(v, t) with threshold t (= 1/beta).  The
 * adjoint writes gv = J^T gW and, when gt is not NULL, the n per-voxel terms
 * of dL/dt (sum them for the scalar).  iso: tval3_tv.
 * ---------------------------------------------------------------------- */
TVAL3_API tval3_status tval3_shrink_f32(int64_t n, const float* d_v, double t, int iso, float* d_W, void* stream);
TVAL3_API tval3_status tval3_shrink_f64(int64_t n, const double* d_v, double t, int iso, double* d_W, void* stream);
TVAL3_API tval3_status tval3_shrink_adjoint_f32(int64_t n, const float* d_v, double t, int iso, const float* d_gW,
                                                float* d_gv, float* d_gt, void* stream);
TVAL3_API tval3_status tval3_shrink_adjoint_f64(int64_t n, const double* d_v, double t, int iso, const double* d_gW,
                                                double* d_gv, double* d_gt, void* stream);

/* ---------------------------------------------------------------------- *
 * One differentiable inner step of the TVAL3 u-subproblem and its adjoint
 * (the autograd path; the reference's inner iteration,
 * 3d/tval3_gpu_3d.cpp:823-1029, without the discrete Armijo decision):
 *   DU = D U, W = shrink(DU - sigma/beta, 1/beta),
 *   g2 = D^T (DU - W - sigma/beta), g = A^T (A U - b - delta/mu),
 *   d = g2 + (mu/beta) g, tau = |<s,s>/<s,y>| with s = U - Up,
 *   y = g2 - g2p + (mu/beta)(g - gp)   (first = 1: tau = |<d,d> /
 *   (||D d||^2 + (mu/beta)||A d||^2)|, and Up, gp, g2p are not read),
 *   Un = max(U - tau d, 0) (nonneg) or U - tau d.
 * Device vectors: U, Up, gp, g2p, Un, g, g2 (dim_y*dim_x*dim_z), b, delta
 * (op rows), sigma (3 volumes); sigma and delta may be NULL (zero).  mub is
 * a device array {mu, beta}.  op's products must take the entry point's
 * vector type (an FP32 operator for _f32, FP64 vectors for _f64).
 * The adjoint takes the adjoints gUn, gg, gg2 of the outputs (any NULL =
 * zero), recomputes the step's intermediates from the same inputs, and
 * writes the adjoints of U, Up, gp, g2p (NULL to skip; not written for the
 * first step), b (NULL to skip) and {mu, beta} (device array of 2, NULL to
 * skip).  All work is queued on `stream`; scratch comes from the
 * stream-ordered pool.
 * ---------------------------------------------------------------------- */
TVAL3_API tval3_status tval3_unroll_step_f32(tval3_op op, int dim_y, int dim_x, int dim_z, int first, int iso,
                                             int nonneg, const double* d_mub, const float* d_U, const float* d_Up,
                                             const float* d_gp, const float* d_g2p, const float* d_b,
                                             const float* d_sigma, const float* d_delta, float* d_Un, float* d_g,
                                             float* d_g2, void* stream);
TVAL3_API tval3_status tval3_unroll_step_f64(tval3_op op, int dim_y, int dim_x, int dim_z, int first, int iso,
                                             int nonneg, const double* d_mub, const double* d_U, const double* d_Up,
                                             const double* d_gp, const double* d_g2p, const double* d_b,
                                             const double* d_sigma, const double* d_delta, double* d_Un,
                                             double* d_g, double* d_g2, void* stream);
TVAL3_API tval3_status tval3_unroll_step_adjoint_f32(tval3_op op, int dim_y, int dim_x, int dim_z, int first,
                                                     int iso, int nonneg, const double* d_mub, const float* d_U,
                                                     const float* d_Up, const float* d_gp, const float* d_g2p,
                                                     const float* d_b, const float* d_sigma, const float* d_delta,
                                                     const float* d_gUn, const float* d_gg, const float* d_gg2,
                                                     float* d_gU, float* d_gUp, float* d_ggp, float* d_gg2p,
                                                     float* d_gb, double* d_gmub, void* stream);
TVAL3_API tval3_status tval3_unroll_step_adjoint_f64(tval3_op op, int dim_y, int dim_x, int dim_z, int first,
                                                     int iso, int nonneg, const double* d_mub, const double* d_U,
                                                     const double* d_Up, const double* d_gp, const double* d_g2p,
                                                     const double* d_b, const double* d_sigma,
                                                     const double* d_delta, const double* d_gUn,
                                                     const double* d_gg, const double* d_gg2, double* d_gU,
                                                     double* d_gUp, double* d_ggp, double* d_gg2p, double* d_gb,
                                                     double* d_gmub, void* stream);

/* ---------------------------------------------------------------------- *
 * Dense A^T*y without any device allocation (no counterpart in the
 * reference; same result as tval3_mat_vec_mul(trans = 1) on a dense FP32
 * operator up to summation order).  For callers that must not allocate
 * device memory while running (fixed memory budgets, their own pool
 * allocator, no cudaMalloc inside a stream capture): A (rows x cols,
 * row-major, one ray per row), y (rows) and x (cols) are the caller's device
 * arrays; the slab partial sums live in one static device array of
 * 1,048,576 floats, so cols must not exceed that (TVAL3_ERR_SHAPE
 * otherwise).  A call on a stream that is not capturing looks up that
 * array's address on the current device; calls under capture use the
 * address remembered from an earlier call, so make the first call on a
 * device before any stream capture.  Calls that overlap in time on one
 * device share the array and race; order them.  rows = 0 writes x = 0.
 * ---------------------------------------------------------------------- */
#define TVAL3_NOALLOC_SCRATCH_FLOATS 1048576
TVAL3_API tval3_status tval3_dense_rmatvec_f32_noalloc(int rows, int cols, const float* d_A, const float* d_y,
                                                       float* d_x, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TVAL3_C_H_ */
