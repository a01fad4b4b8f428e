"""Dense A^T*y without device allocation (tval3_dense_rmatvec_f32_noalloc)
against the operator-handle path (tval3_op_create_dense + tval3_mat_vec_mul
with trans = 1), both through the C ABI, and against an independent FP64
product on the host.  The paths sum the rows in different orders, so they
agree to FP32 rounding: |x - x_ref| <= 1e-5 * sum|A||y| per column.  Two calls
in a row check that the static scratch is reused cleanly; a call recorded
inside a CUDA graph capture (where any device allocation would invalidate
the capture) and replayed gives the same result; rows = 0 writes zeros; the
size limit is rejected with TVAL3_ERR_SHAPE."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _dense_ref(lib, A, y):
    import torch
    from tval3_gb300 import capi
    rows, cols = A.shape
    h = capi.DenseHost(rows, cols, 1, capi.PREC_FP32, A.ctypes.data)
    op = C.c_void_p()
    capi.check(lib.tval3_op_create_dense(C.byref(op), C.byref(h), capi.PREC_FP32))
    try:
        yd = torch.from_numpy(y).cuda()
        xd = torch.empty(cols, dtype=torch.float32, device="cuda")
        capi.check(lib.tval3_mat_vec_mul(op, 1, yd.data_ptr(), xd.data_ptr(), None))
        torch.cuda.synchronize()
        return xd.cpu().numpy()
    finally:
        lib.tval3_op_destroy(op)


@pytest.mark.parametrize("rows,cols", [(1000, 3000), (32640, 4096), (7, 1 << 20)])
def test_noalloc_matches_operator_path(cuda, rows, cols):
    import torch
    from tval3_gb300 import capi
    lib = capi.load()
    rng = np.random.default_rng(rows + cols)
    A = rng.standard_normal((rows, cols), dtype=np.float32)
    y = rng.standard_normal(rows, dtype=np.float32)
    ref = _dense_ref(lib, A, y)
    exact = A.T.astype(np.float64) @ y.astype(np.float64)
    bound = 1e-5 * (np.abs(A).T @ np.abs(y)) + 1e-30
    assert np.all(np.abs(ref - exact) <= bound)
    Ad = torch.from_numpy(A).cuda()
    yd = torch.from_numpy(y).cuda()
    for _ in range(2):
        xd = torch.full((cols,), float("nan"), dtype=torch.float32, device="cuda")
        capi.check(lib.tval3_dense_rmatvec_f32_noalloc(rows, cols, Ad.data_ptr(), yd.data_ptr(), xd.data_ptr(),
                                                        None))
        torch.cuda.synchronize()
        x = xd.cpu().numpy()
        assert np.all(np.abs(x - ref) <= bound)
        assert np.all(np.abs(x - exact) <= bound)


def test_noalloc_inside_graph_capture(cuda):
    """After one ordinary call, a call made while a stream is captured (where
    a cudaMalloc would break the capture) records into the graph; replaying
    the graph gives the same x as the ordinary call."""
    import torch
    from tval3_gb300 import capi
    lib = capi.load()
    rows, cols = 2048, 5000
    rng = np.random.default_rng(5)
    A = torch.from_numpy(rng.standard_normal((rows, cols), dtype=np.float32)).cuda()
    y = torch.from_numpy(rng.standard_normal(rows, dtype=np.float32)).cuda()
    x0 = torch.empty(cols, dtype=torch.float32, device="cuda")
    capi.check(lib.tval3_dense_rmatvec_f32_noalloc(rows, cols, A.data_ptr(), y.data_ptr(), x0.data_ptr(), None))
    torch.cuda.synchronize()
    x1 = torch.full((cols,), float("nan"), dtype=torch.float32, device="cuda")
    g = torch.cuda.CUDAGraph()
    st = []
    with torch.cuda.graph(g):
        s = torch.cuda.current_stream().cuda_stream
        st.append(lib.tval3_dense_rmatvec_f32_noalloc(rows, cols, A.data_ptr(), y.data_ptr(), x1.data_ptr(), s))
    assert st == [0], lib.tval3_last_error_message()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(x0, x1)


def test_noalloc_zero_rows(cuda):
    """rows = 0: A^T y is the zero vector."""
    import torch
    from tval3_gb300 import capi
    lib = capi.load()
    cols = 777
    A = torch.zeros(1, dtype=torch.float32, device="cuda")
    y = torch.zeros(1, dtype=torch.float32, device="cuda")
    x = torch.full((cols,), float("nan"), dtype=torch.float32, device="cuda")
    capi.check(lib.tval3_dense_rmatvec_f32_noalloc(0, cols, A.data_ptr(), y.data_ptr(), x.data_ptr(), None))
    torch.cuda.synchronize()
    assert torch.count_nonzero(x).item() == 0 and not torch.isnan(x).any()


def test_noalloc_rejects_oversize(cuda):
    import torch
    from tval3_gb300 import capi
    lib = capi.load()
    cols = (1 << 20) + 1
    Ad = torch.zeros(cols, dtype=torch.float32, device="cuda")
    yd = torch.zeros(1, dtype=torch.float32, device="cuda")
    xd = torch.zeros(cols, dtype=torch.float32, device="cuda")
    st = lib.tval3_dense_rmatvec_f32_noalloc(1, cols, Ad.data_ptr(), yd.data_ptr(), xd.data_ptr(), None)
    assert st == 2  # TVAL3_ERR_SHAPE
    assert b"exceeds the static scratch" in lib.tval3_last_error_message()
