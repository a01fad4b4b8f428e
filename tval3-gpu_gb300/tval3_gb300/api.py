"""Python mirror of the reference's TVAL3 interface over the C ABI.

Names follow modk/tval3-gpu: ``tval3_gpu_3d`` (3d/tval3_gpu_3d.cpp:23-69) and
``tval3_gpu`` (2d/tval3_gpu.h:9-19) take U's shape, the matrix A (sparse,
dense or geometry), b, the options and an optional true image Ut, and return
the reconstruction with a ``tval3_info``; errors raise ``Tval3Error`` (the
reference raises tval3_gpu_exception).  ``Operator.mat_vec_mul`` is the
reference's ``mat_vec_mul(trans, A, x, y, stream)``.

Volumes are numpy arrays indexed [z, x, y] (C order), which is the
reference's column-major layout with y fastest.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import capi
from .capi import (PREC_BF16, PREC_FP16, PREC_FP32, PREC_FP64, SPARSE_BOTH, SPARSE_CSC, SPARSE_CSR,
                   TRAV_BRESENHAM, TRAV_SIDDON, Info, Options, check, default_options, load)

__all__ = ["SparseMatrix", "DenseMatrix", "Geometry", "tval3_gpu_3d", "tval3_gpu", "Operator", "Solver",
           "last_call_phases",
           "D", "Dt", "default_options", "Options", "Info"]


def _ptr(a) -> int | None:
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        return a.ctypes.data
    if hasattr(a, "data_ptr"):
        return a.data_ptr()
    return int(a)


def _stream(stream) -> int | None:
    if stream is None:
        try:
            import torch
            if torch.cuda.is_available():
                return torch.cuda.current_stream().cuda_stream
        except ImportError:
            pass
        return None
    if hasattr(stream, "cuda_stream"):
        return stream.cuda_stream
    return int(stream)


@dataclass
class SparseMatrix:
    """sparse_mat_host: A (rows = rays, cols = voxels) as CSR and/or the CSC arrays."""
    rows: int
    cols: int
    csr_ptr: np.ndarray | None = None
    csr_ind: np.ndarray | None = None
    csr_val: np.ndarray | None = None
    csc_ptr: np.ndarray | None = None
    csc_ind: np.ndarray | None = None
    csc_val: np.ndarray | None = None

    def __post_init__(self):
        def c(a, dt):
            return None if a is None else np.ascontiguousarray(a, dtype=dt)
        vt = np.float64 if (self.csr_val is not None and np.asarray(self.csr_val).dtype == np.float64) or \
            (self.csr_val is None and self.csc_val is not None and np.asarray(self.csc_val).dtype == np.float64) \
            else np.float32
        self.csr_ptr, self.csr_ind, self.csr_val = c(self.csr_ptr, np.int32), c(self.csr_ind, np.int32), c(self.csr_val, vt)
        self.csc_ptr, self.csc_ind, self.csc_val = c(self.csc_ptr, np.int32), c(self.csc_ind, np.int32), c(self.csc_val, vt)

    @property
    def nnz(self) -> int:
        return int(self.csr_ind.size if self.csr_ind is not None else self.csc_ind.size)

    @property
    def format(self) -> int:
        return (SPARSE_CSR if self.csr_ptr is not None else 0) | (SPARSE_CSC if self.csc_ptr is not None else 0)

    def struct(self) -> capi.SparseHost:
        s = capi.SparseHost()
        s.rows, s.cols, s.nnz, s.format = self.rows, self.cols, self.nnz, self.format
        v = self.csr_val if self.csr_val is not None else self.csc_val
        s.val_type = PREC_FP64 if v.dtype == np.float64 else PREC_FP32
        s.csr_ptr, s.csr_ind, s.csr_val = _ptr(self.csr_ptr), _ptr(self.csr_ind), _ptr(self.csr_val)
        s.csc_ptr, s.csc_ind, s.csc_val = _ptr(self.csc_ptr), _ptr(self.csc_ind), _ptr(self.csc_val)
        return s


@dataclass
class DenseMatrix:
    """mat_host A (rows x cols).  ``data`` is row-major unless row_major=False."""
    data: np.ndarray
    row_major: bool = True

    def __post_init__(self):
        dt = np.float64 if self.data.dtype == np.float64 else np.float32
        self.data = np.ascontiguousarray(self.data, dtype=dt)

    @property
    def rows(self):
        return self.data.shape[0] if self.row_major else self.data.shape[1]

    @property
    def cols(self):
        return self.data.shape[1] if self.row_major else self.data.shape[0]

    def struct(self) -> capi.DenseHost:
        s = capi.DenseHost()
        s.rows, s.cols, s.row_major = self.rows, self.cols, 1 if self.row_major else 0
        s.val_type = PREC_FP64 if self.data.dtype == np.float64 else PREC_FP32
        s.data = _ptr(self.data)
        return s


@dataclass
class Geometry:
    """geometry_host: transducer voxel coordinates per measurement position,
    use_path flags (E*R) and the volume size; optional continuous positions for
    Siddon traversal (voxel units)."""
    rv_x: int
    rv_y: int
    rv_z: int
    x_emitters: np.ndarray
    y_emitters: np.ndarray
    z_emitters: np.ndarray
    x_receivers: np.ndarray
    y_receivers: np.ndarray
    z_receivers: np.ndarray
    num_emitters: int = 0
    num_receivers: int = 0
    numMPs: int = 1
    use_path: np.ndarray | None = None
    scale_factor: float = 1.0
    traversal: int = TRAV_BRESENHAM
    pos: tuple | None = None  # (xe, ye, ze, xr, yr, zr) float64 arrays
    _keep: list = field(default_factory=list, repr=False)

    def __post_init__(self):
        for k in ("x_emitters", "y_emitters", "z_emitters", "x_receivers", "y_receivers", "z_receivers"):
            setattr(self, k, np.ascontiguousarray(getattr(self, k), dtype=np.int32))
        if not self.num_emitters:
            self.num_emitters = self.x_emitters.size // self.numMPs
        if not self.num_receivers:
            self.num_receivers = self.x_receivers.size // self.numMPs
        if self.use_path is not None:
            self.use_path = np.ascontiguousarray(self.use_path, dtype=np.uint32)
        if self.pos is not None:
            self.pos = tuple(np.ascontiguousarray(p, dtype=np.float64) for p in self.pos)

    def with_traversal(self, traversal: int) -> "Geometry":
        return Geometry(self.rv_x, self.rv_y, self.rv_z, self.x_emitters, self.y_emitters, self.z_emitters,
                        self.x_receivers, self.y_receivers, self.z_receivers, self.num_emitters,
                        self.num_receivers, self.numMPs, self.use_path, self.scale_factor, traversal, self.pos)

    def ray_pairs(self) -> np.ndarray:
        """(emitter, receiver) of every ray in the reference's compaction order."""
        E, R, M = self.num_emitters, self.num_receivers, self.numMPs
        i = np.arange(M * E * R, dtype=np.int64)
        if self.use_path is not None:
            i = i[self.use_path[i % (E * R)] != 0]
        return np.stack([i // R, (i // (E * R)) * R + i % R], axis=1).astype(np.uint32)

    @property
    def nrays(self) -> int:
        if self.use_path is None:
            return self.numMPs * self.num_emitters * self.num_receivers
        return int(self.numMPs * np.count_nonzero(self.use_path))

    def struct(self) -> capi.GeometryHost:
        s = capi.GeometryHost()
        s.numMPs, s.num_emitters, s.num_receivers = self.numMPs, self.num_emitters, self.num_receivers
        s.x_emitters, s.y_emitters, s.z_emitters = _ptr(self.x_emitters), _ptr(self.y_emitters), _ptr(self.z_emitters)
        s.x_receivers, s.y_receivers, s.z_receivers = (_ptr(self.x_receivers), _ptr(self.y_receivers),
                                                       _ptr(self.z_receivers))
        s.use_path = _ptr(self.use_path)
        s.rv_x, s.rv_y, s.rv_z = self.rv_x, self.rv_y, self.rv_z
        s.scale_factor = self.scale_factor
        s.traversal = self.traversal
        if self.pos is not None:
            s.xe_pos, s.ye_pos, s.ze_pos, s.xr_pos, s.yr_pos, s.zr_pos = (_ptr(p) for p in self.pos)
        return s


def _opts(opts) -> Options:
    if opts is None:
        return default_options()
    if isinstance(opts, Options):
        return opts
    return default_options(**opts)


def tval3_gpu_3d(shape, A, b, opts=None, Ut=None, *, dtype=np.float32, pagelocked=True, mainGPU=-1,
                 numGPUs=0, gpuArray=None):
    """Reconstruct U (shape (dim_y, dim_x, dim_z)) from b = A U.  Returns
    (U as a [z, x, y] array, info dict).  A: SparseMatrix, DenseMatrix or
    Geometry, or (Geometry, SparseMatrix) for the combined operator."""
    lib = load()
    dim_y, dim_x, dim_z = shape
    n = dim_y * dim_x * dim_z
    dt = np.float64 if dtype == np.float64 else np.float32
    b = np.ascontiguousarray(b, dtype=dt)
    U = np.zeros((dim_z, dim_x, dim_y), dtype=dt)
    Ut_a = None if Ut is None else np.ascontiguousarray(Ut, dtype=dt).reshape(-1)
    o = _opts(opts)
    info = Info()
    common = (_ptr(b), b.size, C.byref(o), _ptr(Ut_a), 0 if Ut_a is None else Ut_a.size, int(pagelocked),
              mainGPU, numGPUs, None, C.byref(info))
    if isinstance(A, tuple):
        geo, mat = A
        gs, ms = geo.struct(), mat.struct()
        fn = lib.tval3_gpu_3d_geometry_sparse_f64 if dt == np.float64 else lib.tval3_gpu_3d_geometry_sparse_f32
        st = fn(_ptr(U), dim_y, dim_x, dim_z, C.byref(gs), C.byref(ms), *common)
    elif isinstance(A, SparseMatrix):
        s = A.struct()
        fn = lib.tval3_gpu_3d_sparse_f64 if dt == np.float64 else lib.tval3_gpu_3d_sparse_f32
        st = fn(_ptr(U), dim_y, dim_x, dim_z, C.byref(s), *common)
    elif isinstance(A, DenseMatrix):
        s = A.struct()
        fn = lib.tval3_gpu_3d_dense_f64 if dt == np.float64 else lib.tval3_gpu_3d_dense_f32
        st = fn(_ptr(U), dim_y, dim_x, dim_z, C.byref(s), *common)
    elif isinstance(A, Geometry):
        s = A.struct()
        fn = lib.tval3_gpu_3d_geometry_f64 if dt == np.float64 else lib.tval3_gpu_3d_geometry_f32
        st = fn(_ptr(U), dim_y, dim_x, dim_z, C.byref(s), *common)
    else:
        raise TypeError(f"unsupported matrix type {type(A).__name__}")
    check(st)
    assert U.size == n
    return U, info.as_dict()


def last_call_phases() -> dict:
    """Seconds of the phases of this thread's last reference entry-point
    call: operator, setup, solve, download, and inside them the matrix
    upload, validation, operator layout, tile layouts + kernel choice and
    graph build (tval3_last_call_phases)."""
    names = ("operator_s", "setup_s", "solve_s", "download_s", "upload_s", "validate_s", "layout_s", "tiles_s",
             "graph_s", "copy_s")
    out = (C.c_double * len(names))()
    check(load().tval3_last_call_phases(out, len(names)))
    return dict(zip(names, list(out)))


def tval3_gpu(shape, A, b, opts=None, Ut=None, pagelocked=True):
    """2D entry (2d/tval3_gpu.h:9-19): shape = (rows, cols); returns U [cols, rows].
    b may hold `layers` columns (b.size = A.rows * layers, column-major), which
    share A and are solved jointly; U is then [layers, cols, rows]."""
    lib = load()
    rows, cols = shape
    b = np.ascontiguousarray(b, dtype=np.float32)
    nrows = A.rows
    layers = b.size // nrows if nrows and b.size % nrows == 0 else 1
    U = np.zeros((cols, rows) if layers == 1 else (layers, cols, rows), dtype=np.float32)
    Ut_a = None if Ut is None else np.ascontiguousarray(Ut, dtype=np.float32).reshape(-1)
    o = _opts(opts)
    info = Info()
    s = A.struct()
    fn = lib.tval3_gpu_sparse if isinstance(A, SparseMatrix) else lib.tval3_gpu_dense
    check(fn(_ptr(U), rows, cols, C.byref(s), _ptr(b), b.size, C.byref(o), _ptr(Ut_a),
             0 if Ut_a is None else Ut_a.size, int(pagelocked), C.byref(info)))
    return U, info.as_dict()


class Operator:
    """A device operator (tval3_op): the reference's mat_vec_mul interface."""

    def __init__(self, handle: C.c_void_p, keep=None):
        self._h = handle
        self._keep = keep
        r, c, z = C.c_int(), C.c_int(), C.c_int64()
        check(load().tval3_op_shape(self._h, C.byref(r), C.byref(c), C.byref(z)))
        self.rows, self.cols, self.nnz = r.value, c.value, z.value

    @classmethod
    def from_sparse(cls, A: SparseMatrix, precision: int = PREC_FP32) -> "Operator":
        h = C.c_void_p()
        s = A.struct()
        check(load().tval3_op_create_sparse(C.byref(h), C.byref(s), precision))
        return cls(h)

    @classmethod
    def from_device_csr(cls, rows, cols, ptr, ind, val, precision=PREC_FP32, stream=None) -> "Operator":
        h = C.c_void_p()
        check(load().tval3_op_create_sparse_device(C.byref(h), rows, cols, int(ind.numel()), _ptr(ptr), _ptr(ind),
                                                   _ptr(val), precision, _stream(stream)))
        return cls(h)

    @classmethod
    def from_geometry(cls, G: Geometry, mode: int = 0, precision: int = PREC_FP32) -> "Operator":
        h = C.c_void_p()
        s = G.struct()
        check(load().tval3_op_create_geometry(C.byref(h), C.byref(s), mode, precision))
        return cls(h)

    @classmethod
    def from_dense(cls, A: DenseMatrix, precision: int = PREC_FP32) -> "Operator":
        h = C.c_void_p()
        s = A.struct()
        check(load().tval3_op_create_dense(C.byref(h), C.byref(s), precision))
        return cls(h)

    @property
    def handle(self):
        return self._h

    @property
    def device_bytes(self) -> int:
        """Device memory the operator kept from its creation."""
        z = C.c_int64()
        check(load().tval3_op_device_bytes(self._h, C.byref(z)))
        return z.value

    def mat_vec_mul(self, trans: int, x, y, stream=None) -> None:
        check(load().tval3_mat_vec_mul(self._h, int(trans), _ptr(x), _ptr(y), _stream(stream)))

    def mat_mat_mul(self, trans: int, nrhs: int, X, Y, stream=None) -> None:
        check(load().tval3_mat_mat_mul(self._h, int(trans), nrhs, _ptr(X), _ptr(Y), _stream(stream)))

    def set_variant(self, trans: int, variant: int) -> None:
        """Pin the kernel of A*x (trans 0) or A^T*y (trans 1): 0 CSR, 1 tile-staged."""
        check(load().tval3_op_set_variant(self._h, int(trans), int(variant)))

    def variant(self, trans: int) -> int:
        v = C.c_int()
        check(load().tval3_op_get_variant(self._h, int(trans), C.byref(v)))
        return v.value

    def mat_mat_mul_interleaved(self, trans: int, nrhs: int, X, Y, stream=None) -> None:
        """Y = A X (or A^T X) for nrhs right-hand sides stored interleaved
        (element (row, j) at row * nrhs + j)."""
        check(load().tval3_mat_mat_mul_interleaved(self._h, trans, nrhs, _ptr(X), _ptr(Y), _stream(stream)))

    def export_csr(self):
        m, n, z = self.rows, self.cols, self.nnz
        ptr, tptr = np.empty(m + 1, np.int32), np.empty(n + 1, np.int32)
        ind, tind = np.empty(z, np.int32), np.empty(z, np.int32)
        val, tval = np.empty(z, np.float32), np.empty(z, np.float32)
        check(load().tval3_op_export_csr(self._h, _ptr(ptr), _ptr(ind), _ptr(val), _ptr(tptr), _ptr(tind),
                                         _ptr(tval)))
        return ptr, ind, val, tptr, tind, tval

    def export_csr_scaled(self):
        """(ptr, ind, val, row_scale, tptr, tind, tval): entry (r, c) is exactly
        val * row_scale[r] in FP64 (16-bit storage: val holds the 16-bit values,
        row_scale the per-ray scales; otherwise row_scale is all ones)."""
        m, n, z = self.rows, self.cols, self.nnz
        ptr, tptr = np.empty(m + 1, np.int32), np.empty(n + 1, np.int32)
        ind, tind = np.empty(z, np.int32), np.empty(z, np.int32)
        val, tval, rs = np.empty(z, np.float32), np.empty(z, np.float32), np.empty(m, np.float32)
        check(load().tval3_op_export_csr_scaled(self._h, _ptr(ptr), _ptr(ind), _ptr(val), _ptr(rs), _ptr(tptr),
                                                _ptr(tind), _ptr(tval)))
        return ptr, ind, val, rs, tptr, tind, tval

    def close(self):
        if self._h:
            load().tval3_op_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Solver:
    """Device-resident workspace (tval3_solver) for repeated solves."""

    def __init__(self, op: Operator, shape, opts=None, mode: int = 0, layers: int = 1):
        self.op = op
        self.shape = shape
        self.layers = layers
        self._h = C.c_void_p()
        o = _opts(opts)
        self.maxit = o.maxit
        if layers == 1:
            check(load().tval3_solver_create(C.byref(self._h), op.handle, *shape, C.byref(o)))
        else:
            check(load().tval3_solver_create_layers(C.byref(self._h), op.handle, *shape, layers, C.byref(o)))
        self.set_mode(mode)

    def set_mode(self, mode: int):
        check(load().tval3_solver_set_mode(self._h, mode))

    def set_trace(self, xstar_dev):
        check(load().tval3_solver_set_trace(self._h, _ptr(xstar_dev)))

    def trace(self) -> np.ndarray:
        out = np.zeros(max(self.maxit, 1), dtype=np.float64)
        check(load().tval3_solver_trace(self._h, _ptr(out), out.size))
        return out

    def solve(self, b_dev, U_dev, Ut_dev=None, stream=None) -> dict:
        info = Info()
        check(load().tval3_solver_solve(self._h, _ptr(b_dev), _ptr(U_dev), _ptr(Ut_dev), C.byref(info),
                                        _stream(stream)))
        return info.as_dict()

    def set_pause(self, iterations: int):
        """Stop solves (resumably) after this many total iterations; 0 = never."""
        check(load().tval3_solver_set_pause(self._h, int(iterations)))

    def save_state(self, stream=None) -> bytes:
        """The solver's state after a solve (checkpoint), as bytes."""
        size = C.c_size_t()
        check(load().tval3_solver_state_size(self._h, C.byref(size)))
        buf = C.create_string_buffer(size.value)
        check(load().tval3_solver_save_state(self._h, buf, _stream(stream)))
        return buf.raw

    def resume(self, state: bytes, U_dev, Ut_dev=None, stream=None) -> dict:
        """Continue a saved state under this solver's iteration limits."""
        info = Info()
        buf = C.create_string_buffer(bytes(state), len(state))
        check(load().tval3_solver_resume(self._h, buf, _ptr(U_dev), _ptr(Ut_dev), C.byref(info), _stream(stream)))
        return info.as_dict()

    def close(self):
        if self._h:
            load().tval3_solver_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Batch:
    """Independent problems solved by one CUDA graph launch (tval3_batch_*):
    ops[i] with volume shapes[i] = (dim_y, dim_x, dim_z).  The operators are
    borrowed and kept alive by this object."""

    def __init__(self, ops, shapes, opts=None):
        self.ops = list(ops)
        self.count = len(self.ops)
        dims = (C.c_int * (3 * self.count))(*[int(v) for sh in shapes for v in sh])
        handles = (C.c_void_p * self.count)(*[op.handle.value for op in self.ops])
        self._h = C.c_void_p()
        o = _opts(opts)
        check(load().tval3_batch_create(C.byref(self._h), handles, dims, self.count, C.byref(o)))

    def solve(self, b_devs, U_devs, Ut_devs=None, stream=None) -> list[dict]:
        k = self.count
        pb = (C.c_void_p * k)(*[_ptr(x) for x in b_devs])
        pU = (C.c_void_p * k)(*[_ptr(x) for x in U_devs])
        pUt = None if Ut_devs is None else (C.c_void_p * k)(*[_ptr(x) for x in Ut_devs])
        infos = (Info * k)()
        check(load().tval3_batch_solve(self._h, pb, pU, pUt, infos, _stream(stream)))
        return [i.as_dict() for i in infos]

    @property
    def tuned_grid(self) -> int:
        """Elements per block of the vector kernels chosen by the first solve."""
        v = C.c_int64()
        check(load().tval3_batch_tuned_grid(self._h, C.byref(v)))
        return v.value

    def close(self):
        if self._h:
            load().tval3_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def tval3_gpu_batched(slices, opts=None):
    """tval3_gpu for every slice in one launch.  slices: list of (shape
    (rows, cols), SparseMatrix A, b[, Ut]).  Returns ([U [cols, rows]], [info])."""
    lib = load()
    k = len(slices)
    arr = (capi.SliceHost * k)()
    keep = []
    outs = []
    for i, sl in enumerate(slices):
        (rows, cols), A, b = sl[0], sl[1], sl[2]
        Ut = sl[3] if len(sl) > 3 else None
        b = np.ascontiguousarray(b, dtype=np.float32)
        U = np.zeros((cols, rows), dtype=np.float32)
        Ut_a = None if Ut is None else np.ascontiguousarray(Ut, dtype=np.float32).reshape(-1)
        st = A.struct()
        keep += [b, Ut_a, st]
        outs.append(U)
        arr[i] = capi.SliceHost(_ptr(U), rows, cols, C.cast(C.pointer(st), C.c_void_p), _ptr(b), b.size,
                                _ptr(Ut_a), 0 if Ut_a is None else Ut_a.size)
    o = _opts(opts)
    infos = (Info * k)()
    check(lib.tval3_gpu_batched(arr, k, C.byref(o), infos))
    return outs, [i.as_dict() for i in infos]


def D(U_dev, shape, DU_dev, stream=None):
    """DU (3 n-vectors along y, x, z) = D U on device arrays (float32 or float64)."""
    f = load().tval3_D_f64 if _is_f64(U_dev) else load().tval3_D_f32
    check(f(*shape, _ptr(U_dev), _ptr(DU_dev), _stream(stream)))


def Dt(V_dev, shape, out_dev, stream=None):
    f = load().tval3_Dt_f64 if _is_f64(V_dev) else load().tval3_Dt_f32
    check(f(*shape, _ptr(V_dev), _ptr(out_dev), _stream(stream)))


def _is_f64(t) -> bool:
    return str(getattr(t, "dtype", "")) in ("torch.float64", "float64")
