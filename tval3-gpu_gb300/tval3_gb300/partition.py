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
