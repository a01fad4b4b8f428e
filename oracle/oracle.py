"""TEST INFRASTRUCTURE ONLY: ctypes view of the CPU oracle (tval3_oracle.cpp).

Only tests/, __graft_entry__.smoke() and the cpu_baseline / reference legs of
bench.py use this module, always as the checker or as the timed CPU baseline,
never inside the library.  See tval3_oracle.cpp for what it restates and for
its parity status ("parity unpinned" against the reference's own outputs).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
LIB = HERE / "liboracle.so"
SRC = HERE / "tval3_oracle.cpp"


def build(force: bool = False) -> Path:
    if force or not LIB.exists() or LIB.stat().st_mtime < SRC.stat().st_mtime:
        subprocess.run(["make", "-s", "-C", str(HERE)], check=True)
    return LIB


class OracleOpts(C.Structure):
    _fields_ = [("mu", C.c_double), ("mu0", C.c_double), ("beta", C.c_double), ("beta0", C.c_double),
                ("rate_cnt", C.c_double), ("tol", C.c_double), ("tol_inn", C.c_double), ("maxcnt", C.c_int),
                ("maxit", C.c_int), ("c", C.c_double), ("gamma", C.c_double), ("gam", C.c_double),
                ("rate_gam", C.c_double), ("nonneg", C.c_int), ("tv_iso", C.c_int),
                ("num_init_iterations", C.c_uint), ("skip_mul_ratio", C.c_double),
                ("max_relative_change", C.c_double)]


class OracleInfo(C.Structure):
    _fields_ = [("total_iters", C.c_int), ("outer_iters", C.c_int), ("rel_chg", C.c_double),
                ("rel_error", C.c_double), ("backtracks", C.c_int), ("restarts", C.c_int),
                ("final_f", C.c_double), ("scl", C.c_double), ("products_T", C.c_int)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        L.oracle_ray_list.restype = C.c_long
        L.oracle_ray_list.argtypes = [C.c_int, C.c_int, C.c_int, P, P]
        L.oracle_bresenham_csr.restype = C.c_long
        L.oracle_bresenham_csr.argtypes = [C.c_long, P, P, P, P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_float,
                                           P, P, P]
        L.oracle_siddon_csr.restype = C.c_long
        L.oracle_siddon_csr.argtypes = [C.c_long, P, P, P, P, P, P, P, C.c_int, C.c_int, C.c_int, C.c_double,
                                        P, P, P]
        L.oracle_csr_transpose.restype = None
        L.oracle_csr_transpose.argtypes = [C.c_long, C.c_long, P, P, P, P, P, P]
        L.oracle_spmv_f64.restype = None
        L.oracle_spmv_f64.argtypes = [C.c_long, P, P, P, P, P]
        L.oracle_D_f64.restype = None
        L.oracle_D_f64.argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, P]
        L.oracle_Dt_f64.restype = None
        L.oracle_Dt_f64.argtypes = [C.c_int, C.c_int, C.c_int, P, P, P, P]
        L.oracle_shrink_f64.restype = C.c_double
        L.oracle_shrink_f64.argtypes = [C.c_long, P, P, P, P, P, P, C.c_double, C.c_int, P, P, P]
        L.oracle_tval3_csr.restype = C.c_int
        L.oracle_tval3_csr.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_long, P, P, P, P, P, P, P,
                                       C.POINTER(OracleOpts), P, P, C.POINTER(OracleInfo), P, P, P]
        L.oracle_tval3_csr_scaled.restype = C.c_int
        L.oracle_tval3_csr_scaled.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_long, P, P, P, P, P, P, P, P,
                                              C.POINTER(OracleOpts), P, P, C.POINTER(OracleInfo), P, P, P]
        L.oracle_spmv_scaled_f64.restype = None
        L.oracle_spmv_scaled_f64.argtypes = [C.c_long, P, P, P, P, P, P]
        L.oracle_tval3_dense.restype = C.c_int
        L.oracle_tval3_dense.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_long, P, P,
                                         C.POINTER(OracleOpts), P, P, C.POINTER(OracleInfo), P]
        L.oracle_tval3_csr_layers.restype = C.c_int
        L.oracle_tval3_csr_layers.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_long, P, P, P, P, P,
                                              P, P, C.POINTER(OracleOpts), P, P, C.POINTER(OracleInfo)]
        L.oracle_tval3_dense_layers.restype = C.c_int
        L.oracle_tval3_dense_layers.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_long, P, P,
                                                C.POINTER(OracleOpts), P, P, C.POINTER(OracleInfo)]
        L.oracle_num_threads.restype = C.c_int
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data


def ray_list(numMPs, E, R, use_path=None) -> np.ndarray:
    up = None if use_path is None else np.ascontiguousarray(use_path, np.uint32)
    cnt = lib().oracle_ray_list(numMPs, E, R, _p(up), None)
    out = np.empty((cnt, 2), np.uint32)
    lib().oracle_ray_list(numMPs, E, R, _p(up), _p(out))
    return out


def bresenham_csr(geo):
    """CSR (ptr, ind, val) of the reference's Bresenham ray matrix."""
    pairs = ray_list(geo.numMPs, geo.num_emitters, geo.num_receivers, geo.use_path)
    m = pairs.shape[0]
    arrs = [np.ascontiguousarray(a, np.int32) for a in (geo.x_emitters, geo.y_emitters, geo.z_emitters,
                                                        geo.x_receivers, geo.y_receivers, geo.z_receivers)]
    ptr = np.zeros(m + 1, np.int32)
    args = [m, _p(pairs)] + [_p(a) for a in arrs] + [geo.rv_x, geo.rv_y, geo.rv_z, geo.scale_factor, _p(ptr)]
    nnz = lib().oracle_bresenham_csr(*args, None, None)
    if nnz < 0:
        raise ValueError("endpoint outside the volume")
    ind = np.empty(nnz, np.int32)
    val = np.empty(nnz, np.float32)
    lib().oracle_bresenham_csr(*args, _p(ind), _p(val))
    return ptr, ind, val


def siddon_csr(geo):
    pairs = ray_list(geo.numMPs, geo.num_emitters, geo.num_receivers, geo.use_path)
    m = pairs.shape[0]
    if geo.pos is not None:
        pos = [np.ascontiguousarray(p, np.float64) for p in geo.pos]
    else:
        pos = [np.asarray(a, np.float64) + 0.5 for a in (geo.x_emitters, geo.y_emitters, geo.z_emitters,
                                                           geo.x_receivers, geo.y_receivers, geo.z_receivers)]
    ptr = np.zeros(m + 1, np.int32)
    args = [m, _p(pairs)] + [_p(a) for a in pos] + [geo.rv_x, geo.rv_y, geo.rv_z, float(geo.scale_factor), _p(ptr)]
    nnz = lib().oracle_siddon_csr(*args, None, None)
    ind = np.empty(nnz, np.int32)
    val = np.empty(nnz, np.float32)
    lib().oracle_siddon_csr(*args, _p(ind), _p(val))
    return ptr, ind, val


def transpose(m, n, ptr, ind, val):
    tptr = np.empty(n + 1, np.int32)
    tind = np.empty(ind.size, np.int32)
    tval = np.empty(ind.size, np.float32)
    lib().oracle_csr_transpose(m, n, _p(ptr), _p(ind), _p(val), _p(tptr), _p(tind), _p(tval))
    return tptr, tind, tval


def spmv(ptr, ind, val, x, rscale=None):
    """y = A x in FP64; rscale: optional per-row scale (entry = val * rscale[row])."""
    x = np.ascontiguousarray(x, np.float64).reshape(-1)
    y = np.empty(ptr.size - 1, np.float64)
    if rscale is None:
        lib().oracle_spmv_f64(ptr.size - 1, _p(ptr), _p(ind), _p(val), _p(x), _p(y))
    else:
        rs = np.ascontiguousarray(rscale, np.float32)
        lib().oracle_spmv_scaled_f64(ptr.size - 1, _p(ptr), _p(ind), _p(val), _p(rs), _p(x), _p(y))
    return y


def D(U, dims):
    p, q, r = dims
    U = np.ascontiguousarray(U, np.float64).reshape(-1)
    out = np.empty((3, U.size), np.float64)
    lib().oracle_D_f64(p, q, r, _p(U), _p(out[0]), _p(out[1]), _p(out[2]))
    return out


def Dt(V, dims):
    p, q, r = dims
    V = np.ascontiguousarray(V, np.float64).reshape(3, -1)
    out = np.empty(V.shape[1], np.float64)
    lib().oracle_Dt_f64(p, q, r, _p(V[0]), _p(V[1]), _p(V[2]), _p(out))
    return out


def shrink(DU, sig, beta, iso):
    DU = np.ascontiguousarray(DU, np.float64).reshape(3, -1)
    sig = np.ascontiguousarray(sig, np.float64).reshape(3, -1)
    W = np.empty_like(DU)
    lam1 = lib().oracle_shrink_f64(DU.shape[1], _p(DU[0]), _p(DU[1]), _p(DU[2]), _p(sig[0]), _p(sig[1]),
                                   _p(sig[2]), beta, int(iso), _p(W[0]), _p(W[1]), _p(W[2]))
    return W, lam1


def make_opts(**kw) -> OracleOpts:
    o = OracleOpts(mu=256.0, mu0=256.0, beta=32.0, beta0=32.0, rate_cnt=2.0, tol=1e-6, tol_inn=1e-3, maxcnt=10,
                   maxit=1025, c=1e-5, gamma=0.6, gam=0.9995, rate_gam=0.9, nonneg=1, tv_iso=0)
    for k, v in kw.items():
        k = {"tv_type": "tv_iso", "numInitIterations": "num_init_iterations", "skipMulRatio": "skip_mul_ratio",
             "maxRelativeChange": "max_relative_change"}.get(k, k)
        if k in ("isreal", "precision"):
            continue
        setattr(o, k, v)
    return o


def tval3_csr(dims, ptr, ind, val, b, opts=None, prec=0, Ut=None, tptr=None, tind=None, tval=None, trace=False,
              xstar=None, rscale=None):
    """Solve with the oracle.  prec 0: FP64 vectors, 1: FP32 vectors.
    rscale: optional per-row scale of A (entry (r, c) = val * rscale[r]; the
    library's 16-bit storage as tval3_op_export_csr_scaled returns it), with
    tval then holding the unscaled values of the transpose.
    Returns (U as [z, x, y] array, info dict[, per-iteration f][, per-iteration
    relative error vs xstar])."""
    p, q, r = dims
    n = p * q * r
    m = ptr.size - 1
    if tptr is None:
        tptr, tind, tval = transpose(m, n, ptr, ind, val)
    dt = np.float64 if prec == 0 else np.float32
    b = np.ascontiguousarray(b, dt).reshape(-1)
    U = np.zeros(n, dt)
    Ut_a = None if Ut is None else np.ascontiguousarray(Ut, dt).reshape(-1)
    o = opts if isinstance(opts, OracleOpts) else make_opts(**(opts or {}))
    info = OracleInfo()
    tr = np.zeros(max(o.maxit, 1), np.float64) if trace else None
    xs = None if xstar is None else np.ascontiguousarray(xstar, np.float64).reshape(-1)
    te = None if xs is None else np.full(max(o.maxit, 1), np.nan)
    if rscale is None:
        lib().oracle_tval3_csr(prec, p, q, r, m, _p(ptr), _p(ind), _p(val), _p(tptr), _p(tind), _p(tval), _p(b),
                               C.byref(o), _p(U), _p(Ut_a), C.byref(info), _p(tr), _p(xs), _p(te))
    else:
        rs = np.ascontiguousarray(rscale, np.float32)
        lib().oracle_tval3_csr_scaled(prec, p, q, r, m, _p(ptr), _p(ind), _p(val), _p(rs), _p(tptr), _p(tind),
                                      _p(tval), _p(b), C.byref(o), _p(U), _p(Ut_a), C.byref(info), _p(tr), _p(xs),
                                      _p(te))
    out = (U.reshape(r, q, p), info.as_dict())
    if trace:
        out = out + (tr,)
    if xs is not None:
        out = out + (te,)
    return out


def tval3_dense(dims, A, b, opts=None, prec=0, Ut=None):
    p, q, r = dims
    n = p * q * r
    A = np.ascontiguousarray(A, np.float32)
    dt = np.float64 if prec == 0 else np.float32
    b = np.ascontiguousarray(b, dt).reshape(-1)
    U = np.zeros(n, dt)
    Ut_a = None if Ut is None else np.ascontiguousarray(Ut, dt).reshape(-1)
    o = opts if isinstance(opts, OracleOpts) else make_opts(**(opts or {}))
    info = OracleInfo()
    lib().oracle_tval3_dense(prec, p, q, r, A.shape[0], _p(A), _p(b), C.byref(o), _p(U), _p(Ut_a), C.byref(info),
                             None)
    return U.reshape(r, q, p), info.as_dict()


def tval3_layers(dims, L, A, b, opts=None, prec=0, Ut=None):
    """Joint solve of L layers sharing one matrix (the reference 2D entry with
    b.len = A.rows * layers).  A: (ptr, ind, val) CSR or a dense row-major
    array; b: m x L column-major (layer slowest).  Returns (U [L, z, x, y],
    info)."""
    p, q, r = dims
    n = p * q * r
    dt = np.float64 if prec == 0 else np.float32
    b = np.ascontiguousarray(b, dt).reshape(-1)
    U = np.zeros(n * L, dt)
    Ut_a = None if Ut is None else np.ascontiguousarray(Ut, dt).reshape(-1)
    o = opts if isinstance(opts, OracleOpts) else make_opts(**(opts or {}))
    info = OracleInfo()
    if isinstance(A, tuple):
        ptr, ind, val = A
        m = ptr.size - 1
        tptr, tind, tval = transpose(m, n, ptr, ind, val)
        lib().oracle_tval3_csr_layers(prec, p, q, r, L, m, _p(ptr), _p(ind), _p(val), _p(tptr), _p(tind), _p(tval),
                                      _p(b), C.byref(o), _p(U), _p(Ut_a), C.byref(info))
    else:
        A = np.ascontiguousarray(A, np.float32)
        lib().oracle_tval3_dense_layers(prec, p, q, r, L, A.shape[0], _p(A), _p(b), C.byref(o), _p(U), _p(Ut_a),
                                        C.byref(info))
    return U.reshape(L, r, q, p), info.as_dict()


def num_threads() -> int:
    return lib().oracle_num_threads()


if __name__ == "__main__":
    print(build(force=True), os.cpu_count())
