"""GPU parity of the mixed-precision modes (BF16 / FP16 matrix values with a
per-ray FP32 scale, double-float vectors, FP64 scalars) and of the double
geometry entry points, against the CPU oracle.

The oracle runs on the SAME quantised matrix the device stores: the device
exports its 16-bit values widened to FP32 (exact) and its per-ray scales, and
the oracle applies entry (r, c) = value * scale[r] in FP64.  Against that
matrix the double-float solve must follow the FP64 oracle as the FP32_DF64
mode does over the FP32 matrix: identical control flow over the short 2D
horizon (1e-6), and the 1e-3 bound over a full 32^3 hemisphere solve.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MIXED = [6, 7]  # TVAL3_PREC_BF16_DF64, TVAL3_PREC_FP16_DF64


def _pairs(torch, lib, capi, v, cuda):
    out = torch.empty(2 * v.numel(), dtype=torch.float32, device=cuda)
    capi.check(lib.tval3_df64_from_f64(v.to(cuda).data_ptr(), out.data_ptr(), v.numel(), None))
    return out


def _unpairs(torch, lib, capi, p, k, cuda):
    out = torch.empty(k, dtype=torch.float64, device=cuda)
    capi.check(lib.tval3_df64_to_f64(p.data_ptr(), out.data_ptr(), k, None))
    return out


@pytest.mark.parametrize("prec", MIXED)
def test_mixed_products_match_oracle(cuda, oracle, prec):
    """A x and A^T y of the mixed operators against the oracle's FP64 products
    of the exported quantised matrix (1e-12 relative: double-float
    accumulation), the same 16-bit values and scales as the FP32-vector
    BF16/FP16 operator, and the adjoint identity <Ax, y> = <x, A^T y>."""
    import torch
    from tval3_gb300 import Operator, capi
    from tval3_gb300 import workloads as W
    cfg, geo, x0 = W.config_3d(24, 20, 20, seed=0)
    op = Operator.from_geometry(geo, mode=0, precision=prec)
    ptr, ind, val, rs, tptr, tind, tval = op.export_csr_scaled()
    # the storage equals the FP32-vector 16-bit operator's (same quantisation)
    q = Operator.from_geometry(geo, mode=0, precision=prec - 4)
    qptr, qind, qval, qrs, qtptr, qtind, qtval = q.export_csr_scaled()
    assert np.array_equal(ind, qind) and np.array_equal(val, qval) and np.array_equal(rs, qrs)
    assert np.array_equal(tval, qtval)
    # the widened values are 16-bit numbers and the rows are scaled by their maximum
    assert np.all(np.abs(val) <= 1.0) and np.all(rs > 0)
    rptr, rind, rval = oracle.siddon_csr(geo)
    assert np.array_equal(ptr, rptr) and np.array_equal(ind, rind)
    rel = np.abs(val.astype(np.float64) * rs[np.repeat(np.arange(ptr.size - 1), np.diff(ptr))] - rval)
    half_ulp = 2.0 ** -8 if prec == 6 else 2.0 ** -11
    assert np.all(rel <= half_ulp * np.abs(rval) * 1.001 + 2.0 ** -24 * 2.0)
    m, n = op.rows, op.cols
    lib = capi.load()
    g = torch.Generator(device="cpu").manual_seed(3)
    x = torch.randn(n, generator=g, dtype=torch.float64)
    y = torch.randn(m, generator=g, dtype=torch.float64)
    Axp = torch.empty(2 * m, dtype=torch.float32, device=cuda)
    Atyp = torch.empty(2 * n, dtype=torch.float32, device=cuda)
    op.mat_vec_mul(0, _pairs(torch, lib, capi, x, cuda), Axp)
    op.mat_vec_mul(1, _pairs(torch, lib, capi, y, cuda), Atyp)
    torch.cuda.synchronize()
    Ax = _unpairs(torch, lib, capi, Axp, m, cuda).cpu().numpy()
    Aty = _unpairs(torch, lib, capi, Atyp, n, cuda).cpu().numpy()
    ref_Ax = oracle.spmv(ptr, ind, val, x.numpy(), rscale=rs)
    # A^T y with the row scales applied to the gathered y
    ref_Aty = oracle.spmv(tptr, tind, tval, (y.numpy() * rs.astype(np.float64)))
    assert np.linalg.norm(Ax - ref_Ax) <= 1e-12 * np.linalg.norm(ref_Ax)
    assert np.linalg.norm(Aty - ref_Aty) <= 1e-12 * np.linalg.norm(ref_Aty)
    lhs, rhs = float(np.dot(Ax, y.numpy())), float(np.dot(x.numpy(), Aty))
    assert abs(lhs - rhs) <= 1e-12 * max(abs(lhs), 1.0)
    # both product kernels (CSR and tile-staged) give the same products
    for trans in (0, 1):
        for v in (0, 1):
            op.set_variant(trans, v)
            out = torch.empty(2 * (n if trans else m), dtype=torch.float32, device=cuda)
            op.mat_vec_mul(trans, _pairs(torch, lib, capi, y if trans else x, cuda), out)
            torch.cuda.synchronize()
            got = _unpairs(torch, lib, capi, out, n if trans else m, cuda).cpu().numpy()
            ref = ref_Aty if trans else ref_Ax
            assert np.linalg.norm(got - ref) <= 1e-12 * np.linalg.norm(ref)


def _ring(oracle, n=64, nt=128, seed=0):
    from tval3_gb300 import workloads as W
    geo = W.ring_geometry(n, nt)
    x = W.ellipse_phantom(n, 3, seed=seed, axes=(2.0, 0.4 * n))
    ptr, ind, val = oracle.siddon_csr(geo)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), 0.01, seed)
    return geo, x, ptr, ind, val, b


OPTS = dict(mu=256., mu0=256., beta=32., beta0=32., rate_cnt=2., tol=1e-4, tol_inn=1e-3, maxcnt=10, maxit=60,
            c=1e-5, gamma=0.6, gam=0.9995, rate_gam=0.9, nonneg=1)


@pytest.mark.parametrize("prec", MIXED)
@pytest.mark.parametrize("iso", [0, 1])
def test_mixed_short_horizon_2d(cuda, oracle, prec, iso):
    """The 64^2 ring problem, 60 iterations: the mixed solve follows the FP64
    oracle run on the same quantised matrix (identical control flow, 1e-6),
    through the device solver (host-driven and graph modes) and through the
    reference-facing FP64 entry point."""
    import torch
    from tval3_gb300 import Operator, Solver, SparseMatrix, tval3_gpu_3d
    geo, x, ptr0, ind0, val0, b = _ring(oracle)
    A = SparseMatrix(ptr0.size - 1, x.size, ptr0, ind0, val0)
    op = Operator.from_sparse(A, precision=prec)
    ptr, ind, val, rs, tptr, tind, tval = op.export_csr_scaled()
    o = dict(OPTS, tv_type=iso)
    Uo, io = oracle.tval3_csr((64, 64, 1), ptr, ind, val, b.astype(np.float64), o, prec=0, rscale=rs,
                              tptr=tptr, tind=tind, tval=tval)
    key = ("total_iters", "outer_iters", "backtracks", "restarts")
    for mode in (0, 1):
        s = Solver(op, (64, 64, 1), o, mode=mode)
        U = torch.empty(x.size, dtype=torch.float64, device=cuda)
        ig = s.solve(torch.tensor(b, dtype=torch.float64, device=cuda), U)
        torch.cuda.synchronize()
        assert tuple(ig[k] for k in key) == tuple(io[k] for k in key)
        assert np.linalg.norm(U.cpu().numpy() - Uo.reshape(-1)) <= 1e-6 * np.linalg.norm(Uo)
        s.close()
    Uh, ih = tval3_gpu_3d((64, 64, 1), A, b.astype(np.float64), dict(o, precision=prec), dtype=np.float64)
    assert tuple(ih[k] for k in key) == tuple(io[k] for k in key)
    assert np.linalg.norm(Uh - Uo) <= 1e-6 * np.linalg.norm(Uo)


@pytest.mark.parametrize("prec", MIXED)
def test_mixed_full_solve_3d(cuda, oracle, prec):
    """A full solve of the small hemisphere problem (the 128^3 workload's
    geometry and options at 32^3, 48 x 48 rays) in the mixed mode ends inside
    the 1e-3 bound of the FP64 oracle on the same quantised matrix, with the
    same iteration counts, through the FP64 geometry entry point."""
    from tval3_gb300 import Operator, tval3_gpu_3d
    from tval3_gb300 import workloads as W
    cfg, geo, x = W.config_3d(32, 48, 48, seed=1)
    rptr, rind, rval = oracle.siddon_csr(geo)
    b = W.add_noise(oracle.spmv(rptr, rind, rval, x), cfg.noise, cfg.seed).astype(np.float64)
    op = Operator.from_geometry(geo, mode=0, precision=prec)
    ptr, ind, val, rs, tptr, tind, tval = op.export_csr_scaled()
    Uo, io = oracle.tval3_csr(cfg.dims, ptr, ind, val, b, cfg.opts, prec=0, rscale=rs, tptr=tptr, tind=tind,
                              tval=tval)
    Ug, ig = tval3_gpu_3d(cfg.dims, geo, b, dict(cfg.opts, precision=prec), dtype=np.float64)
    assert (ig["total_iters"], ig["outer_iters"]) == (io["total_iters"], io["outer_iters"])
    assert np.linalg.norm(Ug - Uo) <= 1e-3 * np.linalg.norm(Uo)


@pytest.mark.parametrize("precision", [-1, 5])
def test_geometry_f64_entry(cuda, oracle, precision):
    """tval3_gpu_3d(U, geometry_host, ...) in double (3d/tval3_gpu_3d.cpp:58-63):
    FP64 vectors (precision -1) follow the FP64 oracle on the Siddon matrix with
    identical control flow and 1e-7; double-float (precision 5) within 1e-6
    over the 60-iteration horizon."""
    from tval3_gb300 import tval3_gpu_3d
    geo, x, ptr, ind, val, b = _ring(oracle)
    o = dict(OPTS, tv_type=1)
    Uo, io = oracle.tval3_csr((64, 64, 1), ptr, ind, val, b.astype(np.float64), o, prec=0, Ut=x)
    Ug, ig = tval3_gpu_3d((64, 64, 1), geo, b.astype(np.float64), dict(o, precision=precision), Ut=x,
                          dtype=np.float64)
    key = ("total_iters", "outer_iters", "backtracks", "restarts")
    assert tuple(ig[k] for k in key) == tuple(io[k] for k in key)
    tol = 1e-7 if precision == -1 else 1e-6
    assert np.linalg.norm(Ug - Uo) <= tol * np.linalg.norm(Uo)
    assert abs(ig["rel_error"] - io["rel_error"]) <= 10 * tol


def test_geometry_sparse_f64_entry(cuda, oracle):
    """tval3_gpu_3d(U, geometry_host, sparse_mat_host<double>, ...)
    (3d/tval3_gpu_3d.cpp:64-69): A x from the geometry, A^T y from the given
    matrix (here FP64 values), FP64 vectors; identical control flow and 1e-7
    against the FP64 oracle."""
    from tval3_gb300 import SparseMatrix, tval3_gpu_3d
    geo, x, ptr, ind, val, b = _ring(oracle)
    o = dict(OPTS, tv_type=0)
    Uo, io = oracle.tval3_csr((64, 64, 1), ptr, ind, val, b.astype(np.float64), o, prec=0)
    A = SparseMatrix(ptr.size - 1, x.size, ptr, ind, val.astype(np.float64))
    Ug, ig = tval3_gpu_3d((64, 64, 1), (geo, A), b.astype(np.float64), o, dtype=np.float64)
    key = ("total_iters", "outer_iters", "backtracks", "restarts")
    assert tuple(ig[k] for k in key) == tuple(io[k] for k in key)
    assert np.linalg.norm(Ug - Uo) <= 1e-7 * np.linalg.norm(Uo)
