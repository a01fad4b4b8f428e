"""GPU parity of the operators (A, A^T, D, D^T) and of the device ray-matrix
builders against the CPU oracle, through the C ABI."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _torch():
    import torch
    return torch


def _small_3d(n=24, ne=20, seed=0):
    from tval3_gb300 import workloads as W
    return W.config_3d(n, ne, ne, seed=seed)


@pytest.mark.parametrize("which", ["ring", "hemi"])
@pytest.mark.parametrize("traversal", [0, 1])
def test_device_ray_matrix_bitexact(cuda, oracle, which, traversal):
    """The device-built CSR (row pointers, voxel indices, values) equals the
    oracle's construction bit for bit (Bresenham: dyn_calc_kernel's walk)."""
    from tval3_gb300 import Operator
    from tval3_gb300 import workloads as W
    geo = W.ring_geometry(64, 128) if which == "ring" else _small_3d(40, 48)[1]
    geo = geo.with_traversal(traversal)
    ref = oracle.bresenham_csr(geo) if traversal == 0 else oracle.siddon_csr(geo)
    op = Operator.from_geometry(geo, mode=0)
    ptr, ind, val, tptr, tind, tval = op.export_csr()
    assert np.array_equal(ptr, ref[0])
    assert np.array_equal(ind, ref[1])
    assert np.array_equal(val.view(np.uint32), ref[2].view(np.uint32))
    rt = oracle.transpose(ptr.size - 1, op.cols, *ref)
    assert np.array_equal(tptr, rt[0]) and np.array_equal(tind, rt[1]) and np.array_equal(tval, rt[2])


def _vecs(torch, op, dtype, seed=0):
    g = torch.Generator(device="cpu").manual_seed(seed)
    x = torch.randn(op.cols, generator=g, dtype=torch.float64)
    y = torch.randn(op.rows, generator=g, dtype=torch.float64)
    return x, y


@pytest.mark.parametrize("prec", [0, 1, 2, 3])
def test_spmv_parity_and_adjoint(cuda, oracle, prec):
    """A x and A^T y against the oracle's FP64 products (FP32 storage:
    1e-5 relative; FP64: 1e-12; BF16/FP16: against the dequantised matrix),
    and the dot-product test <Ax, y> = <x, A^T y>."""
    torch = _torch()
    from tval3_gb300 import Operator, SparseMatrix
    cfg, geo, x0 = _small_3d()
    ptr, ind, val = oracle.siddon_csr(geo)
    m, n = ptr.size - 1, x0.size
    tptr, tind, tval = oracle.transpose(m, n, ptr, ind, val)
    A = SparseMatrix(m, n, ptr, ind, val.astype(np.float64) if prec == 1 else val,
                     tptr, tind, tval.astype(np.float64) if prec == 1 else tval)
    op = Operator.from_sparse(A, precision=prec)
    vt = torch.float64 if prec == 1 else torch.float32
    x, y = _vecs(torch, op, vt)
    xd, yd = x.to(cuda, vt), y.to(cuda, vt)
    Ax = torch.empty(m, device=cuda, dtype=vt)
    Aty = torch.empty(n, device=cuda, dtype=vt)
    op.mat_vec_mul(0, xd, Ax)
    op.mat_vec_mul(1, yd, Aty)
    torch.cuda.synchronize()
    if prec in (2, 3):
        qptr, qind, qval, qtptr, qtind, qtval = op.export_csr()
        assert np.array_equal(qind, ind) and np.array_equal(qtind, tind)
        ref_val, ref_tval = qval, qtval
        # round-to-nearest of v / rowmax: half an ulp relative (2^-8 BF16, 2^-11
        # FP16), plus FP16's subnormal spacing 2^-24 of the row maximum
        rowmax = np.maximum.reduceat(np.abs(val), ptr[:-1])[np.repeat(np.arange(m), np.diff(ptr))] \
            if val.size else val
        bound = (2.0 ** -8 if prec == 2 else 2.0 ** -11) * np.abs(val) + (0 if prec == 2 else 2.0 ** -24) * rowmax
        assert np.all(np.abs(qval.astype(np.float64) - val) <= bound * 1.001 + 1e-30)
        tol = 1e-5
    else:
        ref_val, ref_tval = val, tval
        tol = 1e-12 if prec == 1 else 1e-5
    ref_Ax = oracle.spmv(ptr, ind, ref_val, x.numpy())
    ref_Aty = oracle.spmv(tptr, tind, ref_tval, y.numpy())
    got_Ax = Ax.double().cpu().numpy()
    got_Aty = Aty.double().cpu().numpy()
    assert np.linalg.norm(got_Ax - ref_Ax) <= tol * np.linalg.norm(ref_Ax)
    assert np.linalg.norm(got_Aty - ref_Aty) <= tol * np.linalg.norm(ref_Aty)
    lhs = float(np.dot(got_Ax, y.numpy()))
    rhs = float(np.dot(x.numpy(), got_Aty))
    assert abs(lhs - rhs) <= (1e-12 if prec == 1 else 1e-5) * max(abs(lhs), 1.0)


def test_double_float_products(cuda, oracle):
    """FP32_DF64 operators take {hi, lo} FP32 pairs; their products agree with
    the FP64 oracle to double-float accuracy (~1e-13), far below FP32."""
    import ctypes as C
    torch = _torch()
    from tval3_gb300 import PREC_FP32_DF64, Operator, SparseMatrix, capi
    cfg, geo, x0 = _small_3d()
    ptr, ind, val = oracle.siddon_csr(geo)
    m, n = ptr.size - 1, x0.size
    op = Operator.from_sparse(SparseMatrix(m, n, ptr, ind, val), precision=PREC_FP32_DF64)
    x, y = _vecs(torch, op, torch.float64, seed=2)
    lib = capi.load()
    def to_pairs(v):
        out = torch.empty(2 * v.numel(), dtype=torch.float32, device=cuda)
        capi.check(lib.tval3_df64_from_f64(v.to(cuda).data_ptr(), out.data_ptr(), v.numel(), None))
        return out
    def from_pairs(p, k):
        out = torch.empty(k, dtype=torch.float64, device=cuda)
        capi.check(lib.tval3_df64_to_f64(p.data_ptr(), out.data_ptr(), k, None))
        return out
    xp, yp = to_pairs(x), to_pairs(y)
    Axp = torch.empty(2 * m, dtype=torch.float32, device=cuda)
    Atyp = torch.empty(2 * n, dtype=torch.float32, device=cuda)
    op.mat_vec_mul(0, xp, Axp)
    op.mat_vec_mul(1, yp, Atyp)
    torch.cuda.synchronize()
    Ax = from_pairs(Axp, m).cpu().numpy()
    Aty = from_pairs(Atyp, n).cpu().numpy()
    torch.cuda.synchronize()
    tptr, tind, tval = oracle.transpose(m, n, ptr, ind, val)
    ref_Ax = oracle.spmv(ptr, ind, val, x.numpy())
    ref_Aty = oracle.spmv(tptr, tind, tval, y.numpy())
    assert np.linalg.norm(Ax - ref_Ax) <= 1e-12 * np.linalg.norm(ref_Ax)
    assert np.linalg.norm(Aty - ref_Aty) <= 1e-12 * np.linalg.norm(ref_Aty)


def _box_geometry(nx, ny, nz, ne, nr, seed):
    """Transducers on the ellipsoid inscribed in an nx x ny x nz box, 80 % of
    the pairs in use, scale factor 0.5."""
    from tval3_gb300.api import Geometry
    rng = np.random.default_rng(seed)
    half = np.array([nx, ny, nz], dtype=np.float64) / 2.0

    def pts(k):
        u = rng.normal(size=(k, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        return half + 0.98 * half * u

    em, rc = pts(ne), pts(nr)
    dims = (nx, ny, nz)
    ie = [np.clip(np.floor(em[:, a]), 0, dims[a] - 1).astype(np.int32) for a in range(3)]
    ir = [np.clip(np.floor(rc[:, a]), 0, dims[a] - 1).astype(np.int32) for a in range(3)]
    use = (rng.random(ne * nr) < 0.8).astype(np.uint32)
    return Geometry(rv_x=nx, rv_y=ny, rv_z=nz, x_emitters=ie[0], y_emitters=ie[1], z_emitters=ie[2],
                    x_receivers=ir[0], y_receivers=ir[1], z_receivers=ir[2], num_emitters=ne, num_receivers=nr,
                    numMPs=1, use_path=use, scale_factor=0.5, traversal=1,
                    pos=tuple(em[:, a].copy() for a in range(3)) + tuple(rc[:, a].copy() for a in range(3)))


@pytest.mark.parametrize("which", ["hemi", "ring", "odd"])
@pytest.mark.parametrize("traversal", [0, 1])
def test_on_the_fly_matches_oracle(cuda, oracle, which, traversal):
    """On-the-fly traversal (Bresenham: dyn_calc_kernel's mode; Siddon: the
    builder's FP64 walk per ray) against the oracle's products of its CSR:
    A x and A^T y within FP32 summation order, the adjoint identity
    <Ax, y> = <x, A^T y>, the implied matrix's nonzero count, the stored CSR
    operator's products, and A^T y (tile runs summed in a fixed order)
    bit-identical over repeats.  Volumes: 40^3 hemisphere (8^3 tiles, partial
    edge tiles), 64^2 ring (16^2 tiles) and 33 x 17 x 9 (ragged tiles)."""
    torch = _torch()
    from tval3_gb300 import Operator
    from tval3_gb300 import workloads as W
    if which == "hemi":
        geo = _small_3d(40, 48)[1]
    elif which == "ring":
        geo = W.ring_geometry(64, 128)
    else:
        geo = _box_geometry(33, 17, 9, 24, 20, seed=2)
    geo = geo.with_traversal(traversal)
    ptr, ind, val = oracle.bresenham_csr(geo) if traversal == 0 else oracle.siddon_csr(geo)
    op = Operator.from_geometry(geo, mode=1)
    n = op.cols
    assert op.nnz == ind.size
    tptr, tind, tval = oracle.transpose(ptr.size - 1, n, ptr, ind, val)
    x, y = _vecs(torch, op, torch.float32)
    x32, y32 = x.float(), y.float()
    Ax = torch.empty(op.rows, device=cuda)
    Aty = torch.empty(n, device=cuda)
    op.mat_vec_mul(0, x32.to(cuda), Ax)
    op.mat_vec_mul(1, y32.to(cuda), Aty)
    torch.cuda.synchronize()
    ref_Ax = oracle.spmv(ptr, ind, val, x32.double().numpy())
    ref_Aty = oracle.spmv(tptr, tind, tval, y32.double().numpy())
    Axn, Atyn = Ax.double().cpu().numpy(), Aty.double().cpu().numpy()
    assert np.linalg.norm(Axn - ref_Ax) <= 1e-5 * np.linalg.norm(ref_Ax)
    assert np.linalg.norm(Atyn - ref_Aty) <= 1e-5 * np.linalg.norm(ref_Aty)
    # empty rows and columns are exact zeros
    assert np.all(Axn[np.diff(ptr) == 0] == 0) and np.all(Atyn[np.diff(tptr) == 0] == 0)
    lhs, rhs = float(np.dot(Axn, y32.double().numpy())), float(np.dot(x32.double().numpy(), Atyn))
    assert abs(lhs - rhs) <= 1e-5 * np.linalg.norm(Axn) * np.linalg.norm(y32.double().numpy())
    # the stored CSR operator of the same geometry gives the same products
    st = Operator.from_geometry(geo, mode=0)
    Ax2 = torch.empty_like(Ax)
    Aty2 = torch.empty_like(Aty)
    st.mat_vec_mul(0, x32.to(cuda), Ax2)
    st.mat_vec_mul(1, y32.to(cuda), Aty2)
    for _ in range(3):
        again = torch.empty_like(Aty)
        op.mat_vec_mul(1, y32.to(cuda), again)
        torch.cuda.synchronize()
        assert torch.equal(again, Aty)
    assert torch.allclose(Ax2, Ax, rtol=1e-5, atol=1e-5 * float(Ax.abs().max()))
    assert torch.allclose(Aty2, Aty, rtol=1e-5, atol=1e-5 * float(Aty.abs().max()))


@pytest.mark.parametrize("dims", [(7, 5, 3), (64, 64, 1), (33, 17, 9)])
@pytest.mark.parametrize("f64", [False, True])
def test_D_Dt_parity(cuda, oracle, dims, f64):
    torch = _torch()
    from tval3_gb300 import D, Dt
    p, q, r = dims
    n = p * q * r
    dt = torch.float64 if f64 else torch.float32
    g = torch.Generator().manual_seed(3)
    U = torch.randn(n, generator=g, dtype=torch.float64)
    P = torch.randn(3 * n, generator=g, dtype=torch.float64)
    DU = torch.empty(3 * n, device=cuda, dtype=dt)
    DtP = torch.empty(n, device=cuda, dtype=dt)
    D(U.to(cuda, dt), dims, DU)
    Dt(P.to(cuda, dt), dims, DtP)
    torch.cuda.synchronize()
    tol = 1e-15 if f64 else 1e-6
    ref = oracle.D(U.numpy(), dims).reshape(-1)
    assert np.abs(DU.double().cpu().numpy() - ref).max() <= tol * 10
    ref_t = oracle.Dt(P.numpy(), dims)
    assert np.abs(DtP.double().cpu().numpy() - ref_t).max() <= tol * 20
    lhs = float((DU.double().cpu() * P).sum())
    rhs = float((U * DtP.double().cpu()).sum())
    assert abs(lhs - rhs) <= (1e-12 if f64 else 1e-5) * max(abs(lhs), 1.0)


def test_dense_operator_parity(cuda):
    torch = _torch()
    from tval3_gb300 import DenseMatrix, Operator
    rng = np.random.default_rng(0)
    A = rng.normal(size=(300, 200)).astype(np.float32)
    x = rng.normal(size=200)
    y = rng.normal(size=300)
    for prec, tol in ((0, 1e-5), (2, 1e-2)):
        op = Operator.from_dense(DenseMatrix(A), precision=prec)
        Ax = torch.empty(300, device=cuda)
        Aty = torch.empty(200, device=cuda)
        op.mat_vec_mul(0, torch.tensor(x, dtype=torch.float32, device=cuda), Ax)
        op.mat_vec_mul(1, torch.tensor(y, dtype=torch.float32, device=cuda), Aty)
        torch.cuda.synchronize()
        assert np.linalg.norm(Ax.cpu().numpy() - A @ x) <= tol * np.linalg.norm(A @ x)
        assert np.linalg.norm(Aty.cpu().numpy() - A.T @ y) <= tol * np.linalg.norm(A.T @ y)


def test_empty_rays_and_empty_matrix(cuda, oracle):
    """Rays that miss the grid give empty rows; a matrix with no nonzeros is valid."""
    torch = _torch()
    from tval3_gb300 import Geometry, Operator
    geo = Geometry(rv_x=8, rv_y=8, rv_z=1, x_emitters=[0, 0], y_emitters=[0, 0], z_emitters=[0, 0],
                   x_receivers=[0, 0], y_receivers=[0, 0], z_receivers=[0, 0], traversal=1,
                   pos=(np.array([-2.0, 1.0]), np.array([-2.0, 1.0]), np.array([0.5, 0.5]),
                        np.array([-2.0, 7.0]), np.array([9.0, 7.0]), np.array([0.5, 0.5])))
    op = Operator.from_geometry(geo, mode=0)
    ref = oracle.siddon_csr(geo)
    ptr, ind, val, *_ = op.export_csr()
    assert np.array_equal(ptr, ref[0]) and np.array_equal(ind, ref[1])
    assert ptr[1] == ptr[0]  # the ray outside the grid is an empty row
    y = torch.zeros(op.rows, device=cuda)
    op.mat_vec_mul(0, torch.ones(op.cols, device=cuda), y)
    torch.cuda.synchronize()
    assert float(y[0]) == 0.0
    # the on-the-fly operator of the same rays: the missing ray's row is 0,
    # the other one's sum is the stored row's, A^T of a one-hot y is its column
    fly = Operator.from_geometry(geo, mode=1)
    assert fly.nnz == ind.size
    yf = torch.full((op.rows,), 7.0, device=cuda)
    fly.mat_vec_mul(0, torch.ones(op.cols, device=cuda), yf)
    xt = torch.full((op.cols,), 7.0, device=cuda)
    onehot = torch.zeros(op.rows, device=cuda)
    onehot[1] = 1.0
    fly.mat_vec_mul(1, onehot, xt)
    torch.cuda.synchronize()
    assert float(yf[0]) == 0.0 and abs(float(yf[1]) - float(y[1])) <= 1e-6 * abs(float(y[1]))
    col = np.zeros(op.cols)
    col[ind[ptr[1]:ptr[2]]] = val[ptr[1]:ptr[2]]
    assert np.allclose(xt.cpu().numpy(), col, rtol=0, atol=1e-7)
    # every ray misses: no tile runs at all, both products are zeros
    miss = Geometry(rv_x=8, rv_y=8, rv_z=1, x_emitters=[0], y_emitters=[0], z_emitters=[0],
                    x_receivers=[0], y_receivers=[0], z_receivers=[0], traversal=1,
                    pos=(np.array([-2.0]), np.array([-2.0]), np.array([0.5]),
                         np.array([-2.0]), np.array([9.0]), np.array([0.5])))
    fm = Operator.from_geometry(miss, mode=1)
    assert fm.nnz == 0
    ym = torch.full((1,), 3.0, device=cuda)
    xm = torch.full((64,), 3.0, device=cuda)
    fm.mat_vec_mul(0, torch.ones(64, device=cuda), ym)
    fm.mat_vec_mul(1, torch.ones(1, device=cuda), xm)
    torch.cuda.synchronize()
    assert float(ym[0]) == 0.0 and float(xm.abs().sum()) == 0.0


@pytest.mark.parametrize("traversal", [0, 1])
def test_multi_mp_geometry_bitexact(cuda, oracle, traversal):
    """Two measurement positions (numMPs = 2: the transducer coordinates of
    each position one after the other) and a partial use_path mask: the ray
    list follows 3d/mat_vec_mul_dynamic.h:477-556 (signal i of position k:
    emitter k*E + i/R, receiver k*R + i%R, only flagged pairs), and the
    device-built CSR equals the oracle's bit for bit (Bresenham and Siddon)."""
    from tval3_gb300 import Geometry, Operator
    from tval3_gb300 import workloads as W
    g1 = W.hemisphere_geometry(24, 20, 16, seed=3)
    g2 = W.hemisphere_geometry(24, 20, 16, seed=9)  # the second position: a rotated lattice
    cat = lambda a, b: np.concatenate([a, b])
    use = (np.random.default_rng(5).random(20 * 16) < 0.6).astype(np.uint32)
    pos = tuple(cat(a, b) for a, b in zip(g1.pos, g2.pos))
    geo = Geometry(rv_x=24, rv_y=24, rv_z=24,
                   x_emitters=cat(g1.x_emitters, g2.x_emitters), y_emitters=cat(g1.y_emitters, g2.y_emitters),
                   z_emitters=cat(g1.z_emitters, g2.z_emitters), x_receivers=cat(g1.x_receivers, g2.x_receivers),
                   y_receivers=cat(g1.y_receivers, g2.y_receivers), z_receivers=cat(g1.z_receivers, g2.z_receivers),
                   num_emitters=20, num_receivers=16, numMPs=2, use_path=use, scale_factor=1.0,
                   traversal=traversal, pos=pos)
    assert geo.nrays == 2 * int(use.sum())
    pairs = oracle.ray_list(2, 20, 16, use)
    assert np.array_equal(pairs, geo.ray_pairs())
    ref = oracle.bresenham_csr(geo) if traversal == 0 else oracle.siddon_csr(geo)
    op = Operator.from_geometry(geo, mode=0)
    ptr, ind, val, tptr, tind, tval = op.export_csr()
    assert op.rows == geo.nrays
    assert np.array_equal(ptr, ref[0]) and np.array_equal(ind, ref[1])
    assert np.array_equal(val.view(np.uint32), ref[2].view(np.uint32))
