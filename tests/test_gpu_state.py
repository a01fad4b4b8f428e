"""Checkpoint/resume of the solver state (tval3_solver_set_pause /
save_state / resume): a solve paused after K iterations, saved, and resumed
in a fresh solver gives bit for bit the result and counters of one
uninterrupted solve, in both the graph and the host-driven forms; a state of
another shape is rejected."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(oracle):
    from tval3_gb300 import PREC_FP64, Operator, SparseMatrix
    from tval3_gb300 import workloads as W
    cfg, geo, x = W.config_3d(20, 24, 24, seed=4)
    ptr, ind, val = oracle.siddon_csr(geo)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), cfg.noise, 4).astype(np.float64)
    op = Operator.from_sparse(SparseMatrix(ptr.size - 1, x.size, ptr, ind, val.astype(np.float64)),
                              precision=PREC_FP64)
    return cfg, op, b, x.size


@pytest.mark.parametrize("mode", [1, 0])
def test_resume_equals_uninterrupted_solve(cuda, oracle, mode):
    import torch
    from tval3_gb300 import Solver
    cfg, op, b, n = _setup(oracle)
    bd = torch.tensor(b, device=cuda)
    full = dict(cfg.opts, maxit=60)
    s_full = Solver(op, cfg.dims, full, mode=mode)
    U_full = torch.empty(n, dtype=torch.float64, device=cuda)
    i_full = s_full.solve(bd, U_full)
    s1 = Solver(op, cfg.dims, full, mode=mode)
    s1.set_pause(25)
    U1 = torch.empty(n, dtype=torch.float64, device=cuda)
    i1 = s1.solve(bd, U1)
    assert i1["total_iters"] == 25 < i_full["total_iters"]
    state = s1.save_state()
    s2 = Solver(op, cfg.dims, full, mode=mode)
    U2 = torch.empty(n, dtype=torch.float64, device=cuda)
    i2 = s2.resume(state, U2)
    torch.cuda.synchronize()
    for k in ("total_iters", "outer_iters", "backtracks", "restarts"):
        assert i2[k] == i_full[k], k
    assert torch.equal(U2, U_full)


def test_resume_rejects_other_shapes(cuda, oracle):
    import torch
    from tval3_gb300 import PREC_FP64, Operator, Solver, SparseMatrix, Tval3Error
    cfg, op, b, n = _setup(oracle)
    s1 = Solver(op, cfg.dims, dict(cfg.opts, maxit=3), mode=1)
    U1 = torch.empty(n, dtype=torch.float64, device=cuda)
    s1.solve(torch.tensor(b, device=cuda), U1)
    state = s1.save_state()
    s2 = Solver(op, cfg.dims, dict(cfg.opts, maxit=3), mode=1, layers=2)
    with pytest.raises(Tval3Error):
        s2.resume(state, torch.empty(2 * n, dtype=torch.float64, device=cuda))
    with pytest.raises(Tval3Error):
        s1.resume(b"not a state" + bytes(64), U1)
