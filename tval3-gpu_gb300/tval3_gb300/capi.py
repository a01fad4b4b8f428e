"""ctypes binding of the C ABI (include/tval3/tval3_c.h).

Loads the in-tree libtval3_gb300.so.  There is no fallback: if the library is
missing or fails to load, every entry point raises, so no computation ever
silently runs anywhere but in the CUDA library.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libtval3_gb300.so"

TVAL3_OK = 0
STATUS = {0: "OK", 1: "ERR_ARG", 2: "ERR_SHAPE", 3: "ERR_CUDA", 4: "ERR_NOMEM", 5: "ERR_TIMEOUT",
          6: "ERR_NONFINITE", 7: "ERR_UNSUPPORTED"}
PREC_FP32, PREC_FP64, PREC_BF16, PREC_FP16, PREC_FP32_F64VEC, PREC_FP32_DF64 = 0, 1, 2, 3, 4, 5
PREC_BF16_DF64, PREC_FP16_DF64 = 6, 7
TV_ANISO, TV_ISO = 0, 1
SPARSE_CSR, SPARSE_CSC, SPARSE_BOTH = 1, 2, 3
TRAV_BRESENHAM, TRAV_SIDDON = 0, 1


class Tval3Error(RuntimeError):
    """A non-OK status of the C ABI (the reference raises tval3_gpu_exception)."""

    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status
        self.message = message


class Options(C.Structure):
    """tval3_options; defaults from tval3_options_default (2d/tval3_types.h:29-33)."""
    _fields_ = [("mu", C.c_double), ("mu0", C.c_double), ("beta", C.c_double), ("beta0", C.c_double),
                ("rate_cnt", C.c_double), ("tol", C.c_double), ("tol_inn", C.c_double),
                ("maxcnt", C.c_int), ("maxit", C.c_int), ("c", C.c_double), ("gamma", C.c_double),
                ("gam", C.c_double), ("rate_gam", C.c_double), ("isreal", C.c_int), ("nonneg", C.c_int),
                ("numInitIterations", C.c_uint), ("skipMulRatio", C.c_double), ("maxRelativeChange", C.c_double),
                ("tv_type", C.c_int), ("precision", C.c_int)]


class Info(C.Structure):
    _fields_ = [("total_iters", C.c_int), ("outer_iters", C.c_int), ("rel_chg", C.c_double),
                ("rel_error", C.c_double), ("secs", C.c_double), ("outer_secs", C.c_double),
                ("backtracks", C.c_int), ("restarts", C.c_int), ("final_f", C.c_double), ("launches", C.c_int),
                ("products_T", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class SparseHost(C.Structure):
    _fields_ = [("rows", C.c_int), ("cols", C.c_int), ("nnz", C.c_int), ("format", C.c_int), ("val_type", C.c_int),
                ("csr_ptr", C.c_void_p), ("csr_ind", C.c_void_p), ("csr_val", C.c_void_p),
                ("csc_ptr", C.c_void_p), ("csc_ind", C.c_void_p), ("csc_val", C.c_void_p)]


class DenseHost(C.Structure):
    _fields_ = [("rows", C.c_int), ("cols", C.c_int), ("row_major", C.c_int), ("val_type", C.c_int),
                ("data", C.c_void_p)]


class GeometryHost(C.Structure):
    _fields_ = [("numMPs", C.c_int), ("num_emitters", C.c_int), ("num_receivers", C.c_int),
                ("x_emitters", C.c_void_p), ("y_emitters", C.c_void_p), ("z_emitters", C.c_void_p),
                ("x_receivers", C.c_void_p), ("y_receivers", C.c_void_p), ("z_receivers", C.c_void_p),
                ("use_path", C.c_void_p), ("rv_x", C.c_int), ("rv_y", C.c_int), ("rv_z", C.c_int),
                ("scale_factor", C.c_float), ("traversal", C.c_int),
                ("xe_pos", C.c_void_p), ("ye_pos", C.c_void_p), ("ze_pos", C.c_void_p),
                ("xr_pos", C.c_void_p), ("yr_pos", C.c_void_p), ("zr_pos", C.c_void_p)]


class SliceHost(C.Structure):
    _fields_ = [("U", C.c_void_p), ("rows", C.c_int), ("cols", C.c_int), ("A", C.c_void_p), ("b", C.c_void_p),
                ("b_len", C.c_int), ("Ut", C.c_void_p), ("Ut_len", C.c_int)]


_P = C.c_void_p
_I = C.c_int
_SIG = {
    "tval3_options_default": (None, [C.POINTER(Options)]),
    "tval3_last_error_message": (C.c_char_p, []),
    "tval3_version": (C.c_char_p, []),
    "tval3_selftest_bounded_wait": (_I, [C.c_int64, _P, _P]),
    "tval3_last_call_phases": (_I, [_P, _I]),
    "tval3_gpu_3d_sparse_f32": (_I, [_P, _I, _I, _I, _P, _P, _I, _P, _P, _I, _I, _I, _I, _P, _P]),
    "tval3_gpu_3d_sparse_f64": (_I, [_P, _I, _I, _I, _P, _P, _I, _P, _P, _I, _I, _I, _I, _P, _P]),
    "tval3_gpu_3d_dense_f32": (_I, [_P, _I, _I, _I, _P, _P, _I, _P, _P, _I, _I, _I, _I, _P, _P]),
    "tval3_gpu_3d_dense_f64": (_I, [_P, _I, _I, _I, _P, _P, _I, _P, _P, _I, _I, _I, _I, _P, _P]),
    "tval3_gpu_3d_geometry_f32": (_I, [_P, _I, _I, _I, _P, _P, _I, _P, _P, _I, _I, _I, _I, _P, _P]),
    "tval3_gpu_3d_geometry_sparse_f32": (_I, [_P, _I, _I, _I, _P, _P, _P, _I, _P, _P, _I, _I, _I, _I, _P, _P]),
    "tval3_gpu_3d_geometry_f64": (_I, [_P, _I, _I, _I, _P, _P, _I, _P, _P, _I, _I, _I, _I, _P, _P]),
    "tval3_gpu_3d_geometry_sparse_f64": (_I, [_P, _I, _I, _I, _P, _P, _P, _I, _P, _P, _I, _I, _I, _I, _P, _P]),
    "tval3_gpu_sparse": (_I, [_P, _I, _I, _P, _P, _I, _P, _P, _I, _I, _P]),
    "tval3_gpu_dense": (_I, [_P, _I, _I, _P, _P, _I, _P, _P, _I, _I, _P]),
    "tval3_op_create_sparse": (_I, [_P, _P, _I]),
    "tval3_op_create_sparse_device": (_I, [_P, _I, _I, _I, _P, _P, _P, _I, _P]),
    "tval3_op_create_geometry": (_I, [_P, _P, _I, _I]),
    "tval3_op_create_dense": (_I, [_P, _P, _I]),
    "tval3_op_destroy": (_I, [_P]),
    "tval3_op_shape": (_I, [_P, _P, _P, _P]),
    "tval3_op_device_bytes": (_I, [_P, _P]),
    "tval3_op_export_csr": (_I, [_P, _P, _P, _P, _P, _P, _P]),
    "tval3_op_export_csr_scaled": (_I, [_P, _P, _P, _P, _P, _P, _P, _P]),
    "tval3_mat_vec_mul": (_I, [_P, _I, _P, _P, _P]),
    "tval3_mat_mat_mul": (_I, [_P, _I, _I, _P, _P, _P]),
    "tval3_mat_mat_mul_interleaved": (_I, [_P, _I, _I, _P, _P, _P]),
    "tval3_op_set_variant": (_I, [_P, _I, _I]),
    "tval3_op_get_variant": (_I, [_P, _I, _P]),
    "tval3_unroll_step_f32": (_I, [_P, _I, _I, _I, _I, _I, _I] + [_P] * 12),
    "tval3_unroll_step_f64": (_I, [_P, _I, _I, _I, _I, _I, _I] + [_P] * 12),
    "tval3_unroll_step_adjoint_f32": (_I, [_P, _I, _I, _I, _I, _I, _I] + [_P] * 18),
    "tval3_unroll_step_adjoint_f64": (_I, [_P, _I, _I, _I, _I, _I, _I] + [_P] * 18),
    "tval3_shrink_f32": (_I, [C.c_int64, _P, C.c_double, _I, _P, _P]),
    "tval3_shrink_f64": (_I, [C.c_int64, _P, C.c_double, _I, _P, _P]),
    "tval3_shrink_adjoint_f32": (_I, [C.c_int64, _P, C.c_double, _I, _P, _P, _P, _P]),
    "tval3_shrink_adjoint_f64": (_I, [C.c_int64, _P, C.c_double, _I, _P, _P, _P, _P]),
    "tval3_df64_from_f64": (_I, [_P, _P, C.c_int64, _P]),
    "tval3_df64_to_f64": (_I, [_P, _P, C.c_int64, _P]),
    "tval3_solver_create": (_I, [_P, _P, _I, _I, _I, _P]),
    "tval3_solver_create_layers": (_I, [_P, _P, _I, _I, _I, _I, _P]),
    "tval3_solver_set_mode": (_I, [_P, _I]),
    "tval3_solver_solve": (_I, [_P, _P, _P, _P, _P, _P]),
    "tval3_solver_set_pause": (_I, [_P, _I]),
    "tval3_solver_state_size": (_I, [_P, _P]),
    "tval3_solver_save_state": (_I, [_P, _P, _P]),
    "tval3_solver_resume": (_I, [_P, _P, _P, _P, _P, _P]),
    "tval3_solver_set_trace": (_I, [_P, _P]),
    "tval3_solver_trace": (_I, [_P, _P, _I]),
    "tval3_solver_destroy": (_I, [_P]),
    "tval3_D_f32": (_I, [_I, _I, _I, _P, _P, _P]),
    "tval3_Dt_f32": (_I, [_I, _I, _I, _P, _P, _P]),
    "tval3_D_f64": (_I, [_I, _I, _I, _P, _P, _P]),
    "tval3_Dt_f64": (_I, [_I, _I, _I, _P, _P, _P]),
    "tval3_batch_create": (_I, [_P, _P, _P, _I, _P]),
    "tval3_batch_solve": (_I, [_P, _P, _P, _P, _P, _P]),
    "tval3_batch_destroy": (_I, [_P]),
    "tval3_batch_tuned_grid": (_I, [_P, _P]),
    "tval3_gpu_batched": (_I, [_P, _I, _P, _P]),
    "tval3_dense_rmatvec_f32_noalloc": (_I, [_I, _I, _P, _P, _P, _P]),
}

_lib = None


def load(path: Path | str | None = None) -> C.CDLL:
    """Load libtval3_gb300.so (raises if it is absent; no fallback)."""
    global _lib
    if _lib is not None and path is None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise OSError(f"{p} is missing: build it with tval3_gb300.build.build_library()")
    lib = C.CDLL(str(p))
    for name, (res, args) in _SIG.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if path is None:
        _lib = lib
    return lib


def check(status: int) -> None:
    if status != TVAL3_OK:
        msg = load().tval3_last_error_message()
        raise Tval3Error(status, msg.decode() if msg else "")


def default_options(**kw) -> Options:
    o = Options()
    load().tval3_options_default(C.byref(o))
    for k, v in kw.items():
        if not hasattr(o, k):
            raise AttributeError(f"tval3_options has no field {k!r}")
        setattr(o, k, v)
    return o


def exported_symbols() -> list[str]:
    return sorted(_SIG)
