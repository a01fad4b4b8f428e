"""GPU parity of the whole TVAL3 solve against the CPU oracle.

The loop's Barzilai-Borwein steps make trajectories sensitive to rounding:
two FP64 implementations that sum in different orders agree to ~1e-9 after
25 iterations on the 16^2 problem, while FP32 and FP64 runs of the same
algorithm separate by ~2e-5 after 5 iterations and ~1e-2 after 20 on the 64^2
ring problem (measured with the oracle).  So the tests check
  - FP64 GPU vs FP64 oracle over full solves: identical control flow
    (iterations, outer iterations, backtracks, restarts) and a tight result;
  - FP32 GPU vs FP32 oracle within 1e-4 relative L2 over the short horizon
    where FP32 rounding has not yet been amplified;
  - host-driven and CUDA-graph solves bit-identical.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problem(oracle, n=16, nt=24, seed=2):
    from tval3_gb300 import workloads as W
    geo = W.ring_geometry(n, nt)
    x = W.ellipse_phantom(n, 3, seed=seed, axes=(2.0, 0.4 * n))
    ptr, ind, val = oracle.siddon_csr(geo)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), 0.01, seed)
    return geo, x, ptr, ind, val, b


OPTS = dict(mu=256., mu0=64., beta=32., beta0=8., rate_cnt=2., tol=1e-4, tol_inn=1e-3, maxcnt=10, maxit=300,
            c=1e-5, gamma=0.6, gam=0.9995, rate_gam=0.9, nonneg=1)


@pytest.mark.parametrize("iso", [0, 1])
def test_fp64_solve_matches_oracle(cuda, oracle, iso):
    from tval3_gb300 import SparseMatrix, tval3_gpu_3d
    geo, x, ptr, ind, val, b = _problem(oracle)
    o = dict(OPTS, tv_type=iso, maxit=60)
    Uo, io = oracle.tval3_csr((16, 16, 1), ptr, ind, val, b.astype(np.float64), o, prec=0, Ut=x)
    A = SparseMatrix(ptr.size - 1, x.size, ptr, ind, val.astype(np.float64))
    Ug, ig = tval3_gpu_3d((16, 16, 1), A, b.astype(np.float64), o, Ut=x, dtype=np.float64)
    assert (ig["total_iters"], ig["outer_iters"], ig["backtracks"], ig["restarts"]) == \
        (io["total_iters"], io["outer_iters"], io["backtracks"], io["restarts"])
    assert np.linalg.norm(Ug - Uo) <= 1e-7 * np.linalg.norm(Uo)
    assert abs(ig["rel_error"] - io["rel_error"]) <= 1e-7


@pytest.mark.parametrize("iso", [0, 1])
def test_double_float_short_horizon_2d(cuda, oracle, iso):
    """Double-float vectors (FP32 pairs, ~48 bits) over the FP32 matrix track
    the FP64 oracle closely while the loop's amplification of rounding is
    still small: identical control flow and 1e-6 after 60 iterations of the
    64^2 ring problem (over its full 300-iteration horizon this problem
    amplifies FP64 rounding alone to ~3e-5, so no 48-bit arithmetic can stay
    within 1e-3 of it; see the 3D test below for a full horizon)."""
    import torch
    from tval3_gb300 import PREC_FP32_DF64, Operator, Solver, SparseMatrix, tval3_gpu_3d
    geo, x, ptr, ind, val, b = _problem(oracle, 64, 128, seed=0)
    o = dict(OPTS, tv_type=iso, mu0=256., beta0=32., maxit=60)
    Uo, io = oracle.tval3_csr((64, 64, 1), ptr, ind, val, b.astype(np.float64), o, prec=0, Ut=x)
    op = Operator.from_sparse(SparseMatrix(ptr.size - 1, x.size, ptr, ind, val), precision=PREC_FP32_DF64)
    for mode in (0, 1):
        s = Solver(op, (64, 64, 1), o, mode=mode)
        U = torch.empty(x.size, dtype=torch.float64, device=cuda)
        ig = s.solve(torch.tensor(b, dtype=torch.float64, device=cuda), U)
        torch.cuda.synchronize()
        assert (ig["total_iters"], ig["outer_iters"], ig["backtracks"], ig["restarts"]) == \
            (io["total_iters"], io["outer_iters"], io["backtracks"], io["restarts"])
        assert np.linalg.norm(U.cpu().numpy() - Uo.reshape(-1)) <= 1e-6 * np.linalg.norm(Uo)
        s.close()
    # the reference-facing FP64 entry point with FP32 values, run in double-float
    Uh, ih = tval3_gpu_3d((64, 64, 1), SparseMatrix(ptr.size - 1, x.size, ptr, ind, val), b.astype(np.float64),
                          dict(o, precision=PREC_FP32_DF64), dtype=np.float64)
    assert ih["total_iters"] == io["total_iters"]
    assert np.linalg.norm(Uh - Uo) <= 1e-6 * np.linalg.norm(Uo)


def test_double_float_full_solve_3d(cuda, oracle):
    """A full solve of a small hemisphere problem (the 128^3 workload's
    geometry and options at 32^3, 48 x 48 rays) in double-float ends inside
    the 1e-3 bound of the FP64 oracle with the same control flow."""
    import torch
    from tval3_gb300 import PREC_FP32_DF64, Operator, Solver
    from tval3_gb300 import workloads as W
    cfg, geo, x = W.config_3d(32, 48, 48, seed=1)
    ptr, ind, val = oracle.siddon_csr(geo)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), cfg.noise, cfg.seed).astype(np.float64)
    Uo, io = oracle.tval3_csr(cfg.dims, ptr, ind, val, b, cfg.opts, prec=0)
    op = Operator.from_geometry(geo, mode=0, precision=PREC_FP32_DF64)
    s = Solver(op, cfg.dims, cfg.opts, mode=1)
    U = torch.empty(x.size, dtype=torch.float64, device=cuda)
    ig = s.solve(torch.tensor(b, device=cuda), U)
    torch.cuda.synchronize()
    assert (ig["total_iters"], ig["outer_iters"]) == (io["total_iters"], io["outer_iters"])
    assert np.linalg.norm(U.cpu().numpy() - Uo.reshape(-1)) <= 1e-3 * np.linalg.norm(Uo)


@pytest.mark.parametrize("iso", [0, 1])
def test_fp32_solve_matches_oracle_short_horizon(cuda, oracle, iso):
    from tval3_gb300 import SparseMatrix, tval3_gpu_3d
    geo, x, ptr, ind, val, b = _problem(oracle, 64, 128, seed=0)
    o = dict(OPTS, tv_type=iso, maxit=5, mu0=256., beta0=32.)
    Uo, io = oracle.tval3_csr((64, 64, 1), ptr, ind, val, b, o, prec=1)
    Ug, ig = tval3_gpu_3d((64, 64, 1), SparseMatrix(ptr.size - 1, x.size, ptr, ind, val), b, o)
    assert ig["total_iters"] == io["total_iters"] == 5
    assert np.linalg.norm(Ug.astype(np.float64) - Uo) <= 1e-4 * np.linalg.norm(Uo)


def test_fp32_full_solve_objective_close(cuda, oracle):
    """Over a full 300-iteration solve the FP32 path ends within the spread
    that FP32 rounding alone produces in the oracle."""
    from tval3_gb300 import SparseMatrix, tval3_gpu_3d
    geo, x, ptr, ind, val, b = _problem(oracle, 64, 128, seed=0)
    o = dict(OPTS, mu0=256., beta0=32.)
    Uo64, io64 = oracle.tval3_csr((64, 64, 1), ptr, ind, val, b, o, prec=0, Ut=x)
    Ug, ig = tval3_gpu_3d((64, 64, 1), SparseMatrix(ptr.size - 1, x.size, ptr, ind, val), b, o, Ut=x)
    assert ig["total_iters"] > 50
    assert abs(ig["rel_error"] - io64["rel_error"]) < 0.05
    assert np.linalg.norm(Ug - Uo64) <= 0.2 * np.linalg.norm(Uo64)


@pytest.mark.parametrize("f64", [False, True])
def test_graph_mode_bit_identical(cuda, oracle, f64):
    import torch
    from tval3_gb300 import Operator, Solver, SparseMatrix
    geo, x, ptr, ind, val, b = _problem(oracle, 32, 48, seed=1)
    dt = torch.float64 if f64 else torch.float32
    A = SparseMatrix(ptr.size - 1, x.size, ptr, ind, val.astype(np.float64) if f64 else val)
    op = Operator.from_sparse(A, precision=1 if f64 else 0)
    bd = torch.tensor(b, dtype=dt, device=cuda)
    outs = []
    for mode in (0, 1, 1):
        s = Solver(op, (32, 32, 1), dict(OPTS, maxit=120), mode=mode)
        U = torch.empty(x.size, dtype=dt, device=cuda)
        info = s.solve(bd, U)
        torch.cuda.synchronize()
        outs.append((U.cpu().numpy(), info))
        s.close()
    for U, info in outs[1:]:
        assert np.array_equal(U, outs[0][0])
        for k in ("total_iters", "outer_iters", "backtracks", "restarts"):
            assert info[k] == outs[0][1][k]


def test_repeated_solves_reuse_workspace(cuda, oracle):
    import torch
    from tval3_gb300 import Operator, Solver, SparseMatrix
    geo, x, ptr, ind, val, b = _problem(oracle, 32, 48, seed=1)
    op = Operator.from_sparse(SparseMatrix(ptr.size - 1, x.size, ptr, ind, val))
    s = Solver(op, (32, 32, 1), dict(OPTS, maxit=80), mode=1)
    bd = torch.tensor(b, device=cuda)
    U1 = torch.empty(x.size, device=cuda)
    U2 = torch.empty(x.size, device=cuda)
    s.solve(bd, U1)
    s.solve(bd, U2)
    torch.cuda.synchronize()
    assert torch.equal(U1, U2)


def test_geometry_entry_points(cuda, oracle):
    """tval3_gpu_3d with a geometry (on-the-fly Bresenham) and with
    (geometry, sparse) give the result of the CSR path within FP32 noise over
    a short horizon."""
    from tval3_gb300 import SparseMatrix, tval3_gpu_3d
    from tval3_gb300 import workloads as W
    geo = W.ring_geometry(32, 48).with_traversal(0)
    x = W.ellipse_phantom(32, 3, seed=4, axes=(3.0, 10.0))
    ptr, ind, val = oracle.bresenham_csr(geo)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), 0.01, 4)
    o = dict(OPTS, maxit=4)
    Uc, ic = tval3_gpu_3d((32, 32, 1), SparseMatrix(ptr.size - 1, x.size, ptr, ind, val), b, o)
    Ug, ig = tval3_gpu_3d((32, 32, 1), geo, b, o)
    tptr, tind, tval = oracle.transpose(ptr.size - 1, x.size, ptr, ind, val)
    Us, is_ = tval3_gpu_3d((32, 32, 1), (geo, SparseMatrix(ptr.size - 1, x.size, ptr, ind, val, tptr, tind, tval)), b, o)
    for U in (Ug, Us):
        assert np.linalg.norm(U - Uc) <= 1e-4 * np.linalg.norm(Uc)


@pytest.mark.parametrize("iso", [0, 1])
def test_geometry_siddon_on_the_fly_solve(cuda, oracle, iso):
    """tval3_gpu_3d(U, geometry_host, ...) with Siddon rays runs on the fly
    (no stored matrix: per-ray FP64 walks for A x, tile runs summed in a fixed
    order for A^T y) on the 32^3 hemisphere problem.  Over the short horizon
    it follows the FP32 oracle on the Siddon CSR within 1e-4, as the stored
    CSR solve does; over a full solve it ends where the FP64 oracle ends
    within the spread FP32 rounding produces, and two on-the-fly solves are
    bit-identical (deterministic A^T y)."""
    from tval3_gb300 import SparseMatrix, tval3_gpu_3d
    from tval3_gb300 import workloads as W
    cfg, geo, x = W.config_3d(32, 48, 48, seed=1)
    ptr, ind, val = oracle.siddon_csr(geo)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), cfg.noise, cfg.seed).astype(np.float32)
    A = SparseMatrix(ptr.size - 1, x.size, ptr, ind, val)
    o = dict(cfg.opts, tv_type=iso, maxit=5)
    Uo, io = oracle.tval3_csr(cfg.dims, ptr, ind, val, b, o, prec=1)
    Ug, ig = tval3_gpu_3d(cfg.dims, geo, b, o)
    Uc, ic = tval3_gpu_3d(cfg.dims, A, b, o)
    assert ig["total_iters"] == ic["total_iters"] == io["total_iters"] == 5
    assert np.linalg.norm(Ug.astype(np.float64) - Uo) <= 1e-4 * np.linalg.norm(Uo)
    assert np.linalg.norm(Uc.astype(np.float64) - Uo) <= 1e-4 * np.linalg.norm(Uo)
    of = dict(cfg.opts, tv_type=iso)
    Uo64, io64 = oracle.tval3_csr(cfg.dims, ptr, ind, val, b.astype(np.float64), of, prec=0, Ut=x)
    U1, i1 = tval3_gpu_3d(cfg.dims, geo, b, of, Ut=x)
    U2, i2 = tval3_gpu_3d(cfg.dims, geo, b, of, Ut=x)
    assert np.array_equal(U1, U2) and i1["total_iters"] == i2["total_iters"]
    assert abs(i1["rel_error"] - io64["rel_error"]) < 0.05
    assert np.linalg.norm(U1 - Uo64) <= 0.2 * np.linalg.norm(Uo64)


def test_entry_phases_reported(cuda, oracle):
    """tval3_last_call_phases after a host entry call: ten non-negative
    figures; the upload, validation and layout parts fit inside the operator
    phase, the tile and graph parts inside set-up plus solve, and the four
    main phases inside the call's wall time."""
    import time
    from tval3_gb300 import SparseMatrix, tval3_gpu_3d
    from tval3_gb300.api import last_call_phases
    geo, x, ptr, ind, val, b = _problem(oracle, 64, 128, seed=0)
    A = SparseMatrix(ptr.size - 1, x.size, ptr, ind, val)
    t0 = time.perf_counter()
    tval3_gpu_3d((64, 64, 1), A, b, dict(OPTS, maxit=20))
    wall = time.perf_counter() - t0
    ph = last_call_phases()
    assert len(ph) == 10 and all(v >= 0.0 for v in ph.values())
    assert ph["copy_s"] <= ph["upload_s"] + ph["setup_s"] + 1e-6
    main = ph["operator_s"] + ph["setup_s"] + ph["solve_s"] + ph["download_s"]
    assert 0.0 < main <= wall
    assert ph["upload_s"] + ph["validate_s"] + ph["layout_s"] <= ph["operator_s"] + 1e-6
    assert ph["tiles_s"] + ph["graph_s"] <= ph["setup_s"] + ph["solve_s"] + 1e-6


def test_uploads_from_unaligned_host_arrays(cuda, oracle):
    """Host arrays that start 4 bytes past a 16-byte boundary (numpy views)
    upload like aligned ones: the host entry's result is bit-identical."""
    from tval3_gb300 import SparseMatrix, tval3_gpu_3d
    geo, x, ptr, ind, val, b = _problem(oracle, 32, 48, seed=3)

    def shifted(a):
        buf = np.zeros(a.size + 4, dtype=a.dtype)
        out = buf[1:1 + a.size]
        out[:] = a
        return out

    o = dict(OPTS, maxit=30)
    U1, i1 = tval3_gpu_3d((32, 32, 1), SparseMatrix(ptr.size - 1, x.size, ptr, ind, val), b, o)
    sp, si, sv, sb = shifted(ptr), shifted(ind), shifted(val), shifted(np.asarray(b, dtype=np.float32))
    assert sp.ctypes.data % 16 != 0 and si.ctypes.data % 16 != 0
    U2, i2 = tval3_gpu_3d((32, 32, 1), SparseMatrix(ptr.size - 1, x.size, sp, si, sv), sb, o)
    assert np.array_equal(U1, U2) and i1["total_iters"] == i2["total_iters"]


def test_dense_entry_points(cuda, oracle):
    from tval3_gb300 import DenseMatrix, tval3_gpu
    geo, x, ptr, ind, val, b = _problem(oracle)
    A = np.zeros((ptr.size - 1, x.size), np.float32)
    for r in range(ptr.size - 1):
        A[r, ind[ptr[r]:ptr[r + 1]]] += val[ptr[r]:ptr[r + 1]]
    o = dict(OPTS, maxit=6)
    Ud, idn = tval3_gpu((16, 16), DenseMatrix(A), b, o)
    Uo, io = oracle.tval3_dense((16, 16, 1), A, b.astype(np.float64), o, prec=0)
    assert idn["total_iters"] == io["total_iters"]
    assert np.linalg.norm(Ud - Uo) <= 1e-3 * np.linalg.norm(Uo)


@pytest.mark.parametrize("max_rel", [1e-3, 0.0])
def test_skip_heuristic_matches_oracle(cuda, oracle, max_rel):
    """The skip-A^T heuristic (skipMulRatio, numInitIterations,
    maxRelativeChange; 3d/tval3_gpu_3d.cpp:398-468) decided on the device:
    FP64 solves take the oracle's decisions (same number of A^T products,
    iterations, backtracks) and land within 1e-7; host-driven and graph forms
    agree bit for bit."""
    import torch
    from tval3_gb300 import PREC_FP64, Operator, Solver, SparseMatrix
    geo, x, ptr, ind, val, b = _problem(oracle)
    o = dict(OPTS, tv_type=0, maxit=80, skipMulRatio=0.5, numInitIterations=4, maxRelativeChange=max_rel)
    Uo, io = oracle.tval3_csr((16, 16, 1), ptr, ind, val, b.astype(np.float64), o, prec=0)
    op = Operator.from_sparse(SparseMatrix(ptr.size - 1, x.size, ptr, ind, val.astype(np.float64)),
                              precision=PREC_FP64)
    outs = []
    for mode in (0, 1):
        s = Solver(op, (16, 16, 1), o, mode=mode)
        U = torch.empty(x.size, dtype=torch.float64, device=cuda)
        ig = s.solve(torch.tensor(b, dtype=torch.float64, device=cuda), U)
        assert (ig["total_iters"], ig["backtracks"], ig["restarts"], ig["products_T"]) == \
            (io["total_iters"], io["backtracks"], io["restarts"], io["products_T"])
        assert np.linalg.norm(U.cpu().numpy() - Uo.reshape(-1)) <= 1e-7 * np.linalg.norm(Uo)
        outs.append(U.cpu().numpy())
        s.close()
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("dims", [(15, 14, 1), (9, 7, 5), (16, 12, 6), (70, 9, 3), (2, 3, 4), (130, 17, 2)])
def test_fp64_odd_and_even_volumes(cuda, oracle, dims):
    """The pass-per-vector kernels take two voxels per 16-byte access when the
    fastest dimension (stencils) or the volume (plain streams) is even, one
    voxel otherwise; FP64 solves of odd and even volumes keep the oracle's
    control flow and result (p = 2: a single voxel pair along y, its own
    periodic neighbour)."""
    from tval3_gb300 import SparseMatrix, tval3_gpu_3d
    from tval3_gb300 import workloads as W
    p, q, r = dims
    rng = np.random.default_rng(p * 100 + q * 10 + r)
    n = p * q * r
    m = 3 * n // 2
    rows = []
    for _ in range(m):
        k = rng.integers(3, 9)
        rows.append(np.sort(rng.choice(n, size=k, replace=False)))
    ptr = np.zeros(m + 1, np.int32)
    ptr[1:] = np.cumsum([len(x) for x in rows])
    ind = np.concatenate(rows).astype(np.int32)
    val = rng.uniform(0.2, 1.0, ind.size).astype(np.float32)
    x = rng.uniform(0.0, 1.0, n)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), 0.01, 3).astype(np.float64)
    o = dict(OPTS, tv_type=1, maxit=40)
    Uo, io = oracle.tval3_csr(dims, ptr, ind, val, b, o)
    Ug, ig = tval3_gpu_3d(dims, SparseMatrix(m, n, ptr, ind, val.astype(np.float64)), b, o, dtype=np.float64)
    assert (ig["total_iters"], ig["outer_iters"], ig["backtracks"], ig["restarts"]) == \
        (io["total_iters"], io["outer_iters"], io["backtracks"], io["restarts"])
    assert np.linalg.norm(Ug.reshape(-1) - Uo.reshape(-1)) <= 1e-7 * np.linalg.norm(Uo)

