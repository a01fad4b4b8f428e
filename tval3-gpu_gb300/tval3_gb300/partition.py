"""Row-slab partition of the ray matrix over ranks (host logic).

The reference splits A by rays across the GPUs of one process
(3d/mat_vec_mul_sparse.h:419-499 for CSR row slabs; 3d/mat_vec_mul_dynamic.h:
451-556 cuts the ray list only on transducer-group boundaries, emitterPerTas =
4 emitters).  With rays partitioned:

- A*x needs x on every rank and produces each rank's slab of b-space values
  (no exchange; b, Au and delta stay local);
- A^T*y is a sum over ranks of the slabs' partial volumes: the one exchange
  step (the reference's horizontal cut + mulChain, :863-866, :934-957);
- inner products over b-space vectors (lam3, lam5, ||Ad||^2) are sums of
  per-rank scalars.

Each box in this deployment has one GPU, so the library runs replicas; this
module is the partition and reduce logic, exercised with torch.distributed
(gloo) ranks on the CPU by tests/test_partition_gloo.py.
"""
from __future__ import annotations

import numpy as np


def slab_bounds(ptr: np.ndarray, nranks: int, group: int = 1) -> list[tuple[int, int]]:
    """Contiguous row ranges with balanced nonzeros.  Cuts fall on multiples
    of `group` rows (a transducer group of rays) unless that leaves a rank
    empty; the last range ends at the last row."""
    ptr = np.asarray(ptr, dtype=np.int64)
    m = ptr.size - 1
    nnz = int(ptr[-1])
    cuts = [0]
    for k in range(1, nranks):
        target = nnz * k / nranks
        r = int(np.searchsorted(ptr, target, side="left"))
        if group > 1:
            r = int(round(r / group)) * group
        r = min(max(r, cuts[-1]), m)
        cuts.append(r)
    cuts.append(m)
    return [(cuts[i], cuts[i + 1]) for i in range(nranks)]


def slab(ptr, ind, val, r0: int, r1: int):
    """The CSR of rows [r0, r1) (row pointers rebased to 0)."""
    ptr = np.asarray(ptr)
    lo, hi = int(ptr[r0]), int(ptr[r1])
    return (ptr[r0:r1 + 1] - lo).astype(np.int32), np.asarray(ind[lo:hi]), np.asarray(val[lo:hi])


def local_matvec(ptr, ind, val, x):
    """Rows of this slab times x (x replicated on every rank)."""
    out = np.zeros(ptr.size - 1, dtype=np.float64)
    for r in range(ptr.size - 1):
        s = slice(ptr[r], ptr[r + 1])
        out[r] = np.dot(val[s].astype(np.float64), x[ind[s]])
    return out


def local_rmatvec(ptr, ind, val, y_slab, n):
    """This slab's partial volume A_slab^T y_slab (to be sum-reduced)."""
    out = np.zeros(n, dtype=np.float64)
    rows = np.repeat(np.arange(ptr.size - 1), np.diff(ptr))
    np.add.at(out, ind, val.astype(np.float64) * y_slab[rows])
    return out


def allreduce_sum(t, group=None):
    """Sum over ranks (torch.distributed); the exchange step of A^T y."""
    import torch
    import torch.distributed as dist
    tt = torch.as_tensor(t)
    dist.all_reduce(tt, op=dist.ReduceOp.SUM, group=group)
    return tt.numpy() if isinstance(t, np.ndarray) else tt


class SlabComm:
    """The exchange steps of a row-slab partition: a sum over ranks of
    arrays (partial A^T y volumes, b-space inner products) and an all-gather
    of small host objects.  Without a process group (one rank) both are the
    identity."""

    def __init__(self, group=None, distributed: bool | None = None):
        import torch.distributed as dist
        self.group = group
        self.dist = dist.is_available() and dist.is_initialized() if distributed is None else distributed

    def sum(self, a):
        a = np.asarray(a, dtype=np.float64)
        if not self.dist:
            return a
        return np.asarray(allreduce_sum(a.copy(), self.group), dtype=np.float64)

    def gather(self, obj):
        if not self.dist:
            return [obj]
        import torch.distributed as dist
        out = [None] * dist.get_world_size(self.group)
        dist.all_gather_object(out, obj, group=self.group)
        return out


def _D(U, dims):
    p, q, r = dims
    V = U.reshape(r, q, p)
    return np.stack([np.roll(V, -1, axis=2) - V, np.roll(V, -1, axis=1) - V, np.roll(V, -1, axis=0) - V]).reshape(3, -1)


def _Dt(X, dims):
    p, q, r = dims
    X = X.reshape(3, r, q, p)
    return ((np.roll(X[0], 1, axis=2) - X[0]) + (np.roll(X[1], 1, axis=1) - X[1]) +
            (np.roll(X[2], 1, axis=0) - X[2])).reshape(-1)


def partitioned_tval3(slab_csr, row0: int, b_slab, dims, opts: dict, iso: bool = False, comm: SlabComm | None = None):
    """The TVAL3 loop of 3d/tval3_gpu_3d.cpp:1089-1345 (anisotropic or
    isotropic TV, nonnegativity, continuation, nonmonotone line search with
    Barzilai-Borwein steps and at most five backtracking steps, then a
    restart) with A partitioned by rays: this rank holds the rows
    [row0, row0 + len(b_slab)) of A (slab_csr = (ptr, ind, val)) and the
    matching slab of b.  As in the reference's multi-GPU operator
    (3d/mat_vec_mul_sparse.h:419-499, :863-866, :934-957):

    - A*x is the slab's rows (x, a volume, is the same on every rank);
    - A^T*y is the sum over ranks of the slabs' partial volumes (comm.sum);
    - the b-space terms lam3 = ||Au - b||^2, lam5 = <delta, Au - b> and
      ||Ad||^2 of the first step size are sums of per-rank scalars;
    - the b scaling takes the entries of smallest and largest magnitude over
      all ranks (first occurrence in ray order, 3d/tval3_gpu_3d.cpp:226-266).

    Every volume-space operation is repeated on every rank with the same
    reduced inputs, so all ranks take the same control flow and return the
    same U.  Returns (U, info) with U unscaled as in the reference."""
    comm = comm or SlabComm(distributed=False)
    ptr, ind, val = slab_csr
    ptr = np.asarray(ptr)
    n = int(np.prod(dims))
    bl = np.asarray(b_slab, dtype=np.float64)
    o = dict(opts)
    # b scaling over all rays
    loc = []
    if bl.size:
        i0, i1 = int(np.argmin(np.abs(bl))), int(np.argmax(np.abs(bl)))
        loc = [(abs(bl[i0]), row0 + i0, bl[i0], abs(bl[i1]), row0 + i1, bl[i1])]
    allv = [t for part in comm.gather(loc) for t in part]
    bmin = min(allv, key=lambda t: (t[0], t[1]))[2]
    bmax = max(allv, key=lambda t: (t[3], -t[4]))[5]
    dif = abs(bmax - bmin)
    scl = 0.5 / dif if dif < 0.5 else (1.5 / dif if dif > 1.5 else 1.0)
    if dif == 0.0:
        scl = 1.0
    bl = bl * scl

    def Ax(x):
        return local_matvec(ptr, ind, val, x)

    def Aty(y):
        return comm.sum(local_rmatvec(ptr, ind, val, y, n))

    def bdot(u, v):
        return float(comm.sum(np.array([float(np.dot(u, v))]))[0])

    Atb = Aty(bl)
    U = Atb.copy()
    mu, beta = min(o["mu0"], o["mu"]), min(o["beta0"], o["beta"])
    gam = o["gam"]
    sig = np.zeros((3, n))
    delta = np.zeros(bl.size)
    DtsAtd = np.zeros(n)

    def shrink(DU):
        ub = DU - sig / beta
        if not iso:
            t = np.maximum(np.abs(ub) - 1 / beta, 0)
            return np.where(ub >= 0, t, -t), t.sum()
        nv = np.sqrt((ub ** 2).sum(0))
        t = np.maximum(nv - 1 / beta, 0)
        sc = np.where(nv > 0, t / np.where(nv > 0, nv, 1), 0)
        return ub * sc, t.sum()

    def getg(U, DU, W):
        Au = Ax(U)
        g = Aty(Au) - Atb
        V = DU - W
        r = Au - bl
        return Au, g, _Dt(V, dims), (V ** 2).sum(), bdot(r, r), (sig * V).sum(), bdot(delta, r)

    def first_tau(d):
        Dd = _D(d, dims)
        Ad = Ax(d)
        return abs((d @ d) / ((Dd ** 2).sum() + mu / beta * bdot(Ad, Ad)))

    DU = _D(U, dims)
    W, lam1 = shrink(DU)
    Au, g, g2, lam2, lam3, lam4, lam5 = getg(U, DU, W)

    def F():
        return lam1 + beta / 2 * lam2 + mu / 2 * lam3 - lam4 - lam5

    f = F()
    d = g2 + mu / beta * g + DtsAtd
    rcdU = U.copy()
    Q, C = 1.0, f
    outer = total = nbt = nrs = 0
    uup = gp = g2p = None
    while outer < o["maxcnt"] and total < o["maxit"]:
        fst = True
        while total < o["maxit"]:
            if fst:
                tau = first_tau(d)
            else:
                tau = abs((uup @ uup) / (uup @ ((g2 - g2p) + mu / beta * (g - gp))))
            Up, gp, g2p, Aup, DUp = U, g, g2, Au, DU
            U = U - tau * d
            if o["nonneg"]:
                U = np.maximum(U, 0)
            DU = _D(U, dims)
            Au, g, g2, lam2, lam3, lam4, lam5 = getg(U, DU, W)
            f = F()
            alpha = 1.0
            dU = U - Up
            carm = (d @ d) * tau * o["c"] * beta
            if abs(f) > abs(C - alpha * carm):
                dg, dg2, dAu, dDU = g - gp, g2 - g2p, Au - Aup, DU - DUp
                cnt = 0
                while abs(f) > abs(C - alpha * carm):
                    if cnt == 5:
                        gam *= o["rate_gam"]
                        tau = first_tau(d)
                        U = np.maximum(Up - tau * d, 0) if o["nonneg"] else Up - tau * d
                        DU = _D(U, dims)
                        Au, g, g2, lam2, lam3, lam4, lam5 = getg(U, DU, W)
                        f = F()
                        nrs += 1
                        break
                    alpha *= o["gamma"]
                    g, g2, U, Au, DU = gp + alpha * dg, g2p + alpha * dg2, Up + alpha * dU, Aup + alpha * dAu, \
                        DUp + alpha * dDU
                    V = DU - W
                    r = Au - bl
                    lam2, lam4 = (V ** 2).sum(), (sig * V).sum()
                    lam3, lam5 = bdot(r, r), bdot(delta, r)
                    f = F()
                    cnt += 1
                    nbt += 1
            f -= lam1 + beta / 2 * lam2 - lam4
            W, lam1 = shrink(DU)
            V = DU - W
            lam2, lam4 = (V ** 2).sum(), (sig * V).sum()
            g2 = _Dt(V, dims)
            f += lam1 + beta / 2 * lam2 - lam4
            Qp = Q
            Q = gam * Qp + 1
            C = (gam * Qp * C + f) / Q
            uup = U - Up
            d = g2 + mu / beta * g + DtsAtd
            total += 1
            nrmup = np.linalg.norm(Up)
            if np.linalg.norm(uup) / nrmup < o["tol_inn"] and not fst:
                break
            fst = False
        outer += 1
        relout = np.linalg.norm(U - rcdU) / nrmup
        rcdU = U.copy()
        if relout < o["tol"]:
            break
        f += lam4 + lam5
        V = DU - W
        sig = sig - beta * V
        lam4 = (sig * V).sum()
        r = Au - bl
        delta = delta - mu * r
        lam5 = bdot(delta, r)
        f -= lam4 + lam5
        beta0 = beta
        beta = min(beta * o["rate_cnt"], o["beta"])
        mu = min(mu * o["rate_cnt"], o["mu"])
        f = F()
        DtsAtd = beta0 / beta * d
        d = g2 + mu / beta * g + DtsAtd
        gam = o["gam"]
        Q, C = 1.0, f
    return U / scl, dict(total_iters=total, outer_iters=outer, backtracks=nbt, restarts=nrs)
