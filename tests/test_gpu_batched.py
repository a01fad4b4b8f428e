"""Batched solves (tval3_batch_* and tval3_gpu_batched): independent slices
of different sizes and geometries in one CUDA graph launch.

  - FP64: every slice of the batch matches its own FP64 oracle solve with
    identical control flow (iterations, outer iterations, backtracks,
    restarts) and 1e-7 relative L2, as a single FP64 solve does;
  - FP32: the batched host entry point gives bit-identical results and
    counters to solving each slice alone through tval3_gpu (the same kernels
    in the same order, only run side by side);
  - a repeated batch solve reuses its graph and gives the same result;
  - the first batch solve tunes the vector kernels' grid on short solves of
    the whole batch, and solvers created later for the same shapes take the
    same grid (so the single solves above equal the batched ones).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SLICES = [(20, 24), (28, 40), (36, 32), (24, 48), (32, 36), (16, 30)]  # (side, N_t)
OPTS = dict(mu=256., mu0=64., beta=32., beta0=8., rate_cnt=2., tol=1e-4, tol_inn=1e-3, maxcnt=10, maxit=80,
            c=1e-5, gamma=0.6, gam=0.9995, rate_gam=0.9, nonneg=1, tv_type=0)


def _slices(oracle):
    from tval3_gb300 import workloads as W
    out = []
    for k, (n, nt) in enumerate(SLICES):
        geo = W.ring_geometry(n, nt)
        x = W.ellipse_phantom(n, 3, seed=k, axes=(2.0, 0.4 * n))
        ptr, ind, val = oracle.siddon_csr(geo)
        b = W.add_noise(oracle.spmv(ptr, ind, val, x), 0.01, k)
        out.append((n, x, ptr, ind, val, b))
    return out


def test_batch_fp64_matches_oracle_per_slice(cuda, oracle):
    import torch
    from tval3_gb300 import PREC_FP64, Batch, Operator, SparseMatrix
    sl = _slices(oracle)
    ops = [Operator.from_sparse(SparseMatrix(p.size - 1, x.size, p, i, v.astype(np.float64)), precision=PREC_FP64)
           for (n, x, p, i, v, b) in sl]
    bt = Batch(ops, [(n, n, 1) for (n, *_) in sl], OPTS)
    bs = [torch.tensor(b, dtype=torch.float64, device=cuda) for (*_, b) in sl]
    Us = [torch.empty(x.size, dtype=torch.float64, device=cuda) for (n, x, *_) in sl]
    Uts = [torch.tensor(x.reshape(-1), dtype=torch.float64, device=cuda) for (n, x, *_) in sl]
    infos = bt.solve(bs, Us, Uts)
    # the first solve tuned the vector kernels' grid (one of the candidates)
    assert bt.tuned_grid in (512, 1024, 2048, 4096)
    for (n, x, p, i, v, b), U, ig in zip(sl, Us, infos):
        Uo, io = oracle.tval3_csr((n, n, 1), p, i, v, b.astype(np.float64), OPTS, prec=0, Ut=x)
        assert (ig["total_iters"], ig["outer_iters"], ig["backtracks"], ig["restarts"]) == \
            (io["total_iters"], io["outer_iters"], io["backtracks"], io["restarts"])
        assert np.linalg.norm(U.cpu().numpy() - Uo.reshape(-1)) <= 1e-7 * np.linalg.norm(Uo)
        assert abs(ig["rel_error"] - io["rel_error"]) <= 1e-7
    # the same batch again (graph reused): identical
    first = [U.clone() for U in Us]
    infos2 = bt.solve(bs, Us, Uts)
    assert all(torch.equal(a, b) for a, b in zip(first, Us))
    assert [i["total_iters"] for i in infos2] == [i["total_iters"] for i in infos]
    bt.close()


def test_batched_host_entry_equals_single_solves(cuda, oracle):
    from tval3_gb300 import SparseMatrix, tval3_gpu, tval3_gpu_batched
    sl = _slices(oracle)
    mats = [SparseMatrix(p.size - 1, x.size, p, i, v) for (n, x, p, i, v, b) in sl]
    outs, infos = tval3_gpu_batched([((n, n), A, b, x) for (n, x, p, i, v, b), A in zip(sl, mats)], OPTS)
    key = ("total_iters", "outer_iters", "backtracks", "restarts")
    for (n, x, p, i, v, b), A, Ub, ib in zip(sl, mats, outs, infos):
        Us, is_ = tval3_gpu((n, n), A, b, OPTS, Ut=x)
        assert [ib[k] for k in key] == [is_[k] for k in key]
        assert np.array_equal(Ub, Us)
        assert ib["rel_error"] == is_["rel_error"]
