"""Layers: `layers` columns of b sharing one matrix, solved jointly (the
reference 2D entry with b.len = A.rows * layers, 2d/tval3.cu:1406-1426).
The GPU keeps the layers interleaved (element (voxel, layer) at
voxel * L + layer) and multiplies all of them in one sparse (SpMM) or dense
multi-RHS product; the oracle stores them one after the other.

  - FP64 CSR and FP64 dense solves through the device solver match the FP64
    oracle's joint solve with identical control flow and 1e-7 relative L2;
  - the FP32 2D host entry with layers matches the oracle over a short
    horizon (1e-4), and a single-layer call is unchanged by the layers code.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OPTS = dict(mu=256., mu0=64., beta=32., beta0=8., rate_cnt=2., tol=1e-4, tol_inn=1e-3, maxcnt=10, maxit=60,
            c=1e-5, gamma=0.6, gam=0.9995, rate_gam=0.9, nonneg=1, tv_type=0)


def _problem(oracle, n=20, nt=28, L=3):
    from tval3_gb300 import workloads as W
    geo = W.ring_geometry(n, nt)
    xs = [W.ellipse_phantom(n, 3, seed=10 + l, axes=(2.0, 0.4 * n)) for l in range(L)]
    ptr, ind, val = oracle.siddon_csr(geo)
    b = np.concatenate([W.add_noise(oracle.spmv(ptr, ind, val, x), 0.01, 20 + l) for l, x in enumerate(xs)])
    return ptr, ind, val, np.stack(xs), b


@pytest.mark.parametrize("L", [3, 40])
def test_layers_csr_fp64_matches_oracle(cuda, oracle, L):
    import torch
    from tval3_gb300 import PREC_FP64, Operator, Solver, SparseMatrix
    n = 16 if L > 8 else 20
    ptr, ind, val, xs, b = _problem(oracle, n, 24, L)
    Uo, io = oracle.tval3_layers((n, n, 1), L, (ptr, ind, val), b, OPTS, Ut=xs)
    op = Operator.from_sparse(SparseMatrix(ptr.size - 1, n * n, ptr, ind, val.astype(np.float64)),
                              precision=PREC_FP64)
    for mode in (0, 1):
        s = Solver(op, (n, n, 1), OPTS, mode=mode, layers=L)
        U = torch.empty(n * n * L, dtype=torch.float64, device=cuda)
        ig = s.solve(torch.tensor(b, dtype=torch.float64, device=cuda), U,
                     torch.tensor(xs.reshape(-1), dtype=torch.float64, device=cuda))
        assert (ig["total_iters"], ig["outer_iters"], ig["backtracks"], ig["restarts"]) == \
            (io["total_iters"], io["outer_iters"], io["backtracks"], io["restarts"])
        assert np.linalg.norm(U.cpu().numpy() - Uo.reshape(-1)) <= 1e-7 * np.linalg.norm(Uo)
        assert abs(ig["rel_error"] - io["rel_error"]) <= 1e-7
        s.close()


def test_layers_dense_fp64_matches_oracle(cuda, oracle):
    import torch
    from tval3_gb300 import PREC_FP64, DenseMatrix, Operator, Solver
    n, L = 12, 4
    ptr, ind, val, xs, b = _problem(oracle, n, 20, L)
    m = ptr.size - 1
    A = np.zeros((m, n * n), np.float32)
    for r in range(m):
        A[r, ind[ptr[r]:ptr[r + 1]]] = val[ptr[r]:ptr[r + 1]]
    Uo, io = oracle.tval3_layers((n, n, 1), L, A, b, OPTS)
    op = Operator.from_dense(DenseMatrix(A.astype(np.float64)), precision=PREC_FP64)
    s = Solver(op, (n, n, 1), OPTS, mode=1, layers=L)
    U = torch.empty(n * n * L, dtype=torch.float64, device=cuda)
    ig = s.solve(torch.tensor(b, dtype=torch.float64, device=cuda), U)
    assert (ig["total_iters"], ig["outer_iters"], ig["backtracks"]) == \
        (io["total_iters"], io["outer_iters"], io["backtracks"])
    assert np.linalg.norm(U.cpu().numpy() - Uo.reshape(-1)) <= 1e-7 * np.linalg.norm(Uo)


def test_layers_host_entry_fp32(cuda, oracle):
    from tval3_gb300 import SparseMatrix, tval3_gpu
    n, L = 20, 3
    ptr, ind, val, xs, b = _problem(oracle, n, 28, L)
    o = dict(OPTS, maxit=5)
    Uo, io = oracle.tval3_layers((n, n, 1), L, (ptr, ind, val), b, o, prec=1)
    A = SparseMatrix(ptr.size - 1, n * n, ptr, ind, val)
    Ug, ig = tval3_gpu((n, n), A, b, o, Ut=xs)
    assert Ug.shape == (L, n, n)
    assert ig["total_iters"] == io["total_iters"]
    assert np.linalg.norm(Ug.reshape(-1) - Uo.reshape(-1)) <= 1e-4 * np.linalg.norm(Uo)
    # one layer through the same entry: the single-image path
    U1, i1 = tval3_gpu((n, n), A, b[: ptr.size - 1], o)
    U1o, io1 = oracle.tval3_csr((n, n, 1), ptr, ind, val, b[: ptr.size - 1].astype(np.float32), o, prec=1)
    assert U1.shape == (n, n)
    assert np.linalg.norm(U1.reshape(-1) - U1o.reshape(-1)) <= 1e-4 * np.linalg.norm(U1o)
