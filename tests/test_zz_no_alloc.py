"""Dense A^T*y without device allocation (tval3_dense_rmatvec_f32_noalloc)
against the operator-handle path (tval3_op_create_dense + tval3_mat_vec_mul
with trans = 1), both through the C ABI.  The two sum the rows in different
slab orders, so they agree to FP32 rounding: |x - x_ref| <= 1e-5 * sum|A||y|
per column.  Two calls in a row check that the static scratch is reused
cleanly; the size limit is rejected with TVAL3_ERR_SHAPE."""
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
    bound = 1e-5 * (np.abs(A).T @ np.abs(y)) + 1e-30
    Ad = torch.from_numpy(A).cuda()
    yd = torch.from_numpy(y).cuda()
    for _ in range(2):
        xd = torch.full((cols,), float("nan"), dtype=torch.float32, device="cuda")
        capi.check(lib.tval3_dense_rmatvec_f32_noalloc(rows, cols, Ad.data_ptr(), yd.data_ptr(), xd.data_ptr(),
                                                        None))
        torch.cuda.synchronize()
        x = xd.cpu().numpy()
        assert np.all(np.abs(x - ref) <= bound)


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
