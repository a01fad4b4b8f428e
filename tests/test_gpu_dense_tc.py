"""Multi-RHS products: tval3_mat_mat_mul (column-major, k columns) runs one
interleaved product — SpMM for CSR operators, the tensor-core (tcgen05) BF16
GEMM for BF16 dense operators, a SIMT kernel for FP32/FP64 dense ones — and
must match the per-column products (tval3_mat_vec_mul).

The tensor-core GEMM multiplies the BF16 matrix by the vector split into two
BF16 parts (hi + lo), accumulating in FP32; against the exact product of the
same quantised matrix with the FP32 vector its error is bounded by
2^-16 * sum|q||x| (the dropped tail of the split) plus FP32 accumulation;
the test allows 4e-5 * sum|a||x| per output.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _quantised(A):
    """Row scale and BF16 values as the library stores them (rs = max |row|)."""
    import torch
    rs = np.abs(A).max(axis=1).astype(np.float32)
    rs[rs == 0] = 1.0
    q = torch.from_numpy((A / rs[:, None]).astype(np.float32)).to(torch.bfloat16).float().numpy()
    return rs, q


@pytest.mark.parametrize("m,n,k", [(1000, 512, 32), (333, 200, 5), (4096, 1024, 48), (300, 128, 2)])
@pytest.mark.parametrize("trans", [0, 1])
def test_tensor_core_bf16_products(cuda, m, n, k, trans):
    import torch
    from tval3_gb300 import PREC_BF16, DenseMatrix, Operator
    rng = np.random.default_rng(m + n + k)
    A = rng.standard_normal((m, n)).astype(np.float32)
    op = Operator.from_dense(DenseMatrix(A), precision=PREC_BF16)
    rs, q = _quantised(A)
    Aq = (q.astype(np.float64) * rs[:, None].astype(np.float64))
    lx, ly = (m, n) if trans else (n, m)
    X = rng.standard_normal((k, lx)).astype(np.float32)  # k columns of length lx
    Xd = torch.from_numpy(X).to(cuda).contiguous()
    Yd = torch.full((k, ly), float("nan"), dtype=torch.float32, device=cuda)
    op.mat_mat_mul(trans, k, Xd, Yd)
    torch.cuda.synchronize()
    Y = Yd.cpu().numpy()
    M = Aq.T if trans else Aq
    ref = (M @ X.astype(np.float64).T).T
    bound = 4e-5 * (np.abs(M) @ np.abs(X.astype(np.float64)).T).T + 1e-30
    assert np.all(np.abs(Y - ref) <= bound), float(np.max(np.abs(Y - ref) / bound))
    # the same operator, one column at a time (the single-vector kernels)
    y0 = torch.empty(ly, dtype=torch.float32, device=cuda)
    op.mat_vec_mul(trans, Xd[0], y0)
    torch.cuda.synchronize()
    assert np.all(np.abs(y0.cpu().numpy() - ref[0]) <= bound[0])


@pytest.mark.parametrize("kind", ["csr32", "csr64", "dense32", "dense64"])
def test_mat_mat_mul_matches_columns(cuda, oracle, kind):
    import torch
    from tval3_gb300 import PREC_FP32, PREC_FP64, DenseMatrix, Operator, SparseMatrix
    from tval3_gb300 import workloads as W
    geo = W.ring_geometry(24, 40)
    ptr, ind, val = oracle.siddon_csr(geo)
    m, n = ptr.size - 1, 24 * 24
    f64 = kind.endswith("64")
    dt = torch.float64 if f64 else torch.float32
    if kind.startswith("csr"):
        op = Operator.from_sparse(SparseMatrix(m, n, ptr, ind, val.astype(np.float64) if f64 else val),
                                  precision=PREC_FP64 if f64 else PREC_FP32)
    else:
        A = np.zeros((m, n), np.float32)
        for r in range(m):
            A[r, ind[ptr[r]:ptr[r + 1]]] = val[ptr[r]:ptr[r + 1]]
        op = Operator.from_dense(DenseMatrix(A.astype(np.float64) if f64 else A),
                                 precision=PREC_FP64 if f64 else PREC_FP32)
    k = 7
    g = torch.Generator().manual_seed(3)
    for trans in (0, 1):
        lx, ly = (m, n) if trans else (n, m)
        X = torch.randn(k, lx, dtype=dt, generator=g).to(cuda)
        Y = torch.empty(k, ly, dtype=dt, device=cuda)
        op.mat_mat_mul(trans, k, X, Y)
        for j in range(k):
            y = torch.empty(ly, dtype=dt, device=cuda)
            op.mat_vec_mul(trans, X[j].contiguous(), y)
            tol = 1e-12 if f64 else 1e-5
            assert torch.allclose(Y[j], y, rtol=tol, atol=tol * float(y.abs().max()))


def test_dense_bf16_layers_solve(cuda, oracle):
    """2D dense solve with 32 right-hand sides (noise realisations) on the
    BF16 operator (tensor-core products) against the FP64 oracle run on the
    same quantised matrix, over 8 iterations."""
    from tval3_gb300 import PREC_BF16, DenseMatrix, tval3_gpu
    from tval3_gb300 import workloads as W
    n, nt, L = 24, 36, 32
    geo = W.ring_geometry(n, nt)
    ptr, ind, val = oracle.siddon_csr(geo)
    m = ptr.size - 1
    A = np.zeros((m, n * n), np.float32)
    for r in range(m):
        A[r, ind[ptr[r]:ptr[r + 1]]] = val[ptr[r]:ptr[r + 1]]
    x = W.ellipse_phantom(n, 3, seed=4, axes=(2.0, 0.4 * n))
    Ax = A.astype(np.float64) @ x.reshape(-1)
    b = np.concatenate([W.add_noise(Ax, 0.01, 100 + l) for l in range(L)]).astype(np.float32)
    rs, q = _quantised(A)
    Aq = (q * rs[:, None]).astype(np.float32)
    o = dict(mu=256., mu0=64., beta=32., beta0=8., tol=1e-4, maxit=8, tv_type=0)
    Uo, io = oracle.tval3_layers((n, n, 1), L, Aq, b.astype(np.float64), o)
    Ug, ig = tval3_gpu((n, n), DenseMatrix(A), b, dict(o, precision=PREC_BF16))
    assert Ug.shape == (L, n, n)
    assert ig["total_iters"] == io["total_iters"]
    assert np.linalg.norm(Ug.reshape(-1) - Uo.reshape(-1)) <= 1e-3 * np.linalg.norm(Uo)


@pytest.mark.parametrize("prec", ["bf16", "csr32"])
def test_interleaved_product_matches_column_major(cuda, oracle, prec):
    import torch
    from tval3_gb300 import PREC_BF16, PREC_FP32, DenseMatrix, Operator, SparseMatrix
    from tval3_gb300 import workloads as W
    geo = W.ring_geometry(32, 48)
    ptr, ind, val = oracle.siddon_csr(geo)
    m, n = ptr.size - 1, 32 * 32
    if prec == "bf16":
        A = np.zeros((m, n), np.float32)
        for r in range(m):
            A[r, ind[ptr[r]:ptr[r + 1]]] = val[ptr[r]:ptr[r + 1]]
        op = Operator.from_dense(DenseMatrix(A), precision=PREC_BF16)
    else:
        op = Operator.from_sparse(SparseMatrix(m, n, ptr, ind, val), precision=PREC_FP32)
    k = 32
    g = torch.Generator().manual_seed(9)
    for trans in (0, 1):
        lx, ly = (m, n) if trans else (n, m)
        Xc = torch.randn(k, lx, generator=g).to(cuda)
        Yc = torch.empty(k, ly, device=cuda)
        op.mat_mat_mul(trans, k, Xc, Yc)
        Xi = Xc.t().contiguous()
        Yi = torch.empty(ly, k, device=cuda)
        for _ in range(2):  # second call: the plan set up by the first is reused
            op.mat_mat_mul_interleaved(trans, k, Xi, Yi)
            torch.cuda.synchronize()
            assert torch.equal(Yi.t(), Yc)
