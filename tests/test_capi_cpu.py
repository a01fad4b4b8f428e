"""The C-ABI library loads and exports every function that
include/tval3/tval3_c.h declares; argument validation (which runs before any
device call) behaves like the reference's check_params.  No GPU needed."""
import ctypes as C
import re
from pathlib import Path

import numpy as np
import pytest

HEADER = Path(__file__).resolve().parents[1] / "include" / "tval3" / "tval3_c.h"


def declared_functions():
    text = HEADER.read_text()
    return sorted(set(re.findall(r"TVAL3_API\s+[\w\s\*]+?\b(tval3_\w+)\s*\(", text)))


def test_every_declared_symbol_exported(lib):
    names = declared_functions()
    assert len(names) >= 30
    for name in names:
        assert hasattr(lib, name), name
    from tval3_gb300 import capi
    assert set(capi.exported_symbols()) == set(names)


def test_options_defaults_are_the_references(lib):
    from tval3_gb300 import default_options
    o = default_options()
    assert (o.mu, o.mu0, o.beta, o.beta0, o.rate_cnt) == (256.0, 256.0, 32.0, 32.0, 2.0)
    assert (o.tol, o.tol_inn, o.maxcnt, o.maxit, o.c) == (1e-6, 1e-3, 10, 1025, 1e-5)
    assert (o.gamma, o.gam, o.rate_gam, o.isreal, o.nonneg) == (0.6, 0.9995, 0.9, 1, 1)


def _tiny():
    from tval3_gb300 import SparseMatrix
    ptr = np.array([0, 1, 2], np.int32)
    ind = np.array([0, 1], np.int32)
    return SparseMatrix(2, 2, ptr, ind, np.array([1.0, 1.0], np.float32))


@pytest.mark.parametrize("case,status,text", [
    ("u_len", 2, "the length of U must be equal to A.dim_x"),
    ("b_len", 2, "b.len must be equal to A.dim_y"),
    ("ut_len", 2, "U and Ut must have the same size"),
    ("nan_b", 6, "non-finite"),
    ("skip", 1, "skipMulRatio"),
    ("bad_ptr", 2, "pointer"),
    ("bad_ind", 2, "index out of range"),
])
def test_argument_errors(lib, case, status, text):
    from tval3_gb300 import SparseMatrix, Tval3Error, tval3_gpu_3d
    A = _tiny()
    shape, b, Ut, opts = (2, 1, 1), np.array([1.0, 2.0]), None, None
    if case == "u_len":
        shape = (3, 1, 1)
    elif case == "b_len":
        b = np.array([1.0, 2.0, 3.0])
    elif case == "ut_len":
        Ut = np.ones(5)
    elif case == "nan_b":
        b = np.array([1.0, np.nan])
    elif case == "skip":
        opts = dict(skipMulRatio=-0.5)
    elif case == "bad_ptr":
        A = SparseMatrix(2, 2, np.array([0, 2, 1], np.int32), np.array([0, 1], np.int32), np.ones(2, np.float32))
    elif case == "bad_ind":
        A = SparseMatrix(2, 2, np.array([0, 1, 2], np.int32), np.array([0, 5], np.int32), np.ones(2, np.float32))
    with pytest.raises(Tval3Error) as e:
        tval3_gpu_3d(shape, A, b, opts, Ut=Ut)
    assert e.value.status == status
    assert text in e.value.message


def test_null_arguments(lib):
    from tval3_gb300.capi import Info
    info = Info()
    st = lib.tval3_gpu_3d_sparse_f32(None, 1, 1, 1, None, None, 0, None, None, 0, 1, -1, 0, None, C.byref(info))
    assert st != 0
    assert lib.tval3_last_error_message()
    assert lib.tval3_mat_vec_mul(None, 0, None, None, None) == 1
    assert lib.tval3_solver_solve(None, None, None, None, None, None) == 1
    assert lib.tval3_batch_create(None, None, None, 0, None) == 1
    assert lib.tval3_batch_solve(None, None, None, None, None, None) == 1
    assert lib.tval3_gpu_batched(None, 0, None, None) == 1
    t, w = C.c_int(-1), C.c_int64(0)
    assert lib.tval3_selftest_bounded_wait(1000, None, None) == 1
    assert lib.tval3_selftest_bounded_wait(-1, C.byref(t), C.byref(w)) == 1  # limit out of range
    assert lib.tval3_selftest_bounded_wait(5_000_000_000, C.byref(t), C.byref(w)) == 1


def test_batched_slice_errors(lib):
    """tval3_gpu_batched validates every slice (like tval3_gpu) before any
    device work: a slice whose b does not match its matrix is rejected."""
    import ctypes as C
    from tval3_gb300 import capi, default_options
    A = _tiny()
    st_A = A.struct()
    U = np.zeros(2, np.float32)
    b = np.ones(3, np.float32)
    arr = (capi.SliceHost * 1)()
    arr[0] = capi.SliceHost(U.ctypes.data, 2, 1, C.cast(C.pointer(st_A), C.c_void_p), b.ctypes.data, 3, None, 0)
    o = default_options()
    assert lib.tval3_gpu_batched(arr, 1, C.byref(o), None) == 2
    assert b"b.len must be equal" in lib.tval3_last_error_message()


def test_python_mirror_names():
    import tval3_gb300 as T
    for name in ("tval3_gpu_3d", "tval3_gpu", "Operator", "Solver", "SparseMatrix", "DenseMatrix", "Geometry"):
        assert hasattr(T, name)
    assert hasattr(T.Operator, "mat_vec_mul")
