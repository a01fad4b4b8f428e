"""The bounded device waits of the pipelined kernels (mbar.cuh) give up and
report it.  One warp waits on an mbarrier phase that nothing completes, with
a limit of 2,000,000 SM cycles (about a millisecond) instead of the kernels'
4e9: the call reports the timeout after at least the limit, and the context
keeps working (a product afterwards matches the oracle's).  The wait is
bounded by construction, so nothing faults or hangs."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_bounded_wait_gives_up_and_context_survives(cuda, oracle):
    import torch
    from tval3_gb300 import Operator, capi
    from tval3_gb300 import workloads as W
    lib = capi.load()
    t, w = C.c_int(-1), C.c_int64(0)
    capi.check(lib.tval3_selftest_bounded_wait(2_000_000, C.byref(t), C.byref(w)))
    assert t.value == 1
    # at least the limit; the try_wait suspend hint (about a microsecond)
    # bounds the overshoot far below the generous upper bound here
    assert 2_000_000 <= w.value < 200_000_000
    # a phase that nothing completes and a limit of 0: gives up at once
    capi.check(lib.tval3_selftest_bounded_wait(0, C.byref(t), C.byref(w)))
    assert t.value == 1
    # the context is intact: a product matches the oracle's
    geo = W.ring_geometry(32, 48)
    op = Operator.from_geometry(geo, mode=0)
    ptr, ind, val = oracle.siddon_csr(geo)
    x = np.random.default_rng(3).uniform(0.0, 1.0, op.cols)
    y = torch.empty(op.rows, device=cuda)
    op.mat_vec_mul(0, torch.tensor(x, dtype=torch.float32, device=cuda), y)
    torch.cuda.synchronize()
    ref = oracle.spmv(ptr, ind, val, x.astype(np.float32))
    assert np.allclose(y.cpu().numpy(), ref, rtol=1e-5, atol=1e-5 * float(np.abs(ref).max()))
