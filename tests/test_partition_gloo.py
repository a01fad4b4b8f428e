"""The row-slab partition and its one exchange step (the sum-reduce of
partial A^T y volumes), run as world_size-2 gloo ranks on the CPU, equal the
unpartitioned products; the b-space inner products reduce as scalars."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _problem():
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parents[1]
    for p in (str(root / "tval3-gpu_gb300"), str(root)):
        if p not in sys.path:
            sys.path.insert(0, p)
    from oracle import oracle as O
    from tval3_gb300 import workloads as W
    cfg, geo, x = W.config_3d(16, 12, 12, seed=3)
    ptr, ind, val = O.siddon_csr(geo)
    return ptr, ind, val, x.reshape(-1).astype(np.float64)


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from tval3_gb300 import partition as P
        ptr, ind, val, x = _problem()
        m, n = ptr.size - 1, x.size
        rng = np.random.default_rng(7)
        y = rng.standard_normal(m)
        bounds = P.slab_bounds(ptr, world, group=12)
        r0, r1 = bounds[rank]
        sp, si, sv = P.slab(ptr, ind, val, r0, r1)
        Ax_slab = P.local_matvec(sp, si, sv, x)
        Aty = P.allreduce_sum(P.local_rmatvec(sp, si, sv, y[r0:r1], n))
        lam = P.allreduce_sum(np.array([np.dot(Ax_slab, y[r0:r1])]))
        q.put((rank, r0, r1, Ax_slab, Aty, float(lam[0])))
    finally:
        dist.destroy_process_group()


def test_slab_bounds_balance_and_groups():
    from tval3_gb300 import partition as P
    ptr, ind, val, x = _problem()
    for world in (1, 2, 3, 4):
        b = P.slab_bounds(ptr, world, group=12)
        assert b[0][0] == 0 and b[-1][1] == ptr.size - 1
        assert all(b[i][1] == b[i + 1][0] for i in range(world - 1))
        assert all(r1 % 12 == 0 for _, r1 in b[:-1])
        loads = [ptr[r1] - ptr[r0] for r0, r1 in b]
        assert max(loads) <= ptr[-1] / world + 12 * np.diff(ptr).max() + 1


def test_partitioned_products_gloo_world2():
    import multiprocessing as mp
    import scipy.sparse as sp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    ptr, ind, val, x = _problem()
    A = sp.csr_matrix((val.astype(np.float64), ind, ptr), shape=(ptr.size - 1, x.size))
    y = np.random.default_rng(7).standard_normal(A.shape[0])
    Ax = np.concatenate([r[3] for r in res])
    assert np.allclose(Ax, A @ x, rtol=1e-12, atol=1e-12)
    for r in res:
        assert np.allclose(r[4], A.T @ y, rtol=1e-10, atol=1e-10)
        assert abs(r[5] - float(np.dot(A @ x, y))) <= 1e-9 * abs(float(np.dot(A @ x, y)))


OPTS = dict(mu=256., mu0=64., beta=32., beta0=8., rate_cnt=2., tol=1e-4, tol_inn=1e-3, maxcnt=10, maxit=40,
            c=1e-5, gamma=0.6, gam=0.9995, rate_gam=0.9, nonneg=1)


def _solve_rank(rank, world, port, q, iso):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle as O
        from tval3_gb300 import partition as P
        ptr, ind, val, x = _problem()
        b = O.spmv(ptr, ind, val, x) * (1.0 + 0.01 * np.random.default_rng(1).standard_normal(ptr.size - 1))
        r0, r1 = P.slab_bounds(ptr, world, group=12)[rank]
        U, info = P.partitioned_tval3(P.slab(ptr, ind, val, r0, r1), r0, b[r0:r1], (16, 16, 16), OPTS, iso=iso,
                                      comm=P.SlabComm())
        q.put((rank, U, info))
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("iso", [False, True])
def test_partitioned_solve_gloo_world2(iso):
    """The whole TVAL3 loop on two gloo ranks, each holding a row slab of A
    (A^T y all-reduced, lam3 / lam5 / ||Ad||^2 reduced as scalars), follows
    the unpartitioned FP64 oracle solve: identical iteration, outer,
    backtracking and restart counts, and a result within 1e-9."""
    import multiprocessing as mp
    from oracle import oracle as O
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_solve_rank, args=(r, 2, port, q, iso)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted([q.get(timeout=300) for _ in procs], key=lambda t: t[0])
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    ptr, ind, val, x = _problem()
    b = O.spmv(ptr, ind, val, x) * (1.0 + 0.01 * np.random.default_rng(1).standard_normal(ptr.size - 1))
    Uo, io = O.tval3_csr((16, 16, 16), ptr, ind, val, b, dict(OPTS, tv_type=int(iso)), prec=0)
    Uo = Uo.reshape(-1)
    for _, U, info in res:
        assert (info["total_iters"], info["outer_iters"], info["backtracks"], info["restarts"]) == \
            (io["total_iters"], io["outer_iters"], io["backtracks"], io["restarts"])
        assert np.linalg.norm(U - Uo) <= 1e-9 * np.linalg.norm(Uo)
    assert np.array_equal(res[0][1], res[1][1])
