"""Tile-staged products (tiled.cu): operators built from a geometry know
their volume and regroup A^T by voxel tiles (each tile's y values staged in
shared memory) and A into per-tile ray segments (each tile's x values staged,
per-ray partials added in tile order); operators built from a bare sparse
matrix use the plain CSR kernels.  Both must give the same products:
double-float to 1e-12, FP32 and BF16 to 1e-5 (relative to sum |a||v| per
output)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _geo(kind):
    from tval3_gb300 import workloads as W
    if kind == "ring":
        return W.ring_geometry(64, 96)
    if kind == "dense_ring":
        # ~16,000 rays through each 16 x 16 tile: beyond the shared memory of
        # a double-float ray list, so A^T falls back to smaller tiles
        return W.ring_geometry(64, 320)
    if kind == "big":
        # 160^3 voxels (8,000 tiles of 8^3): A*x takes 16 x 8 x 8 tiles
        return W.hemisphere_geometry(160, 24, 24, seed=2)
    if kind == "mixed":
        return _mixed_geometry()
    return W.hemisphere_geometry(40, 48, 48, seed=1)


def _mixed_geometry(nv=96, ne=25, nr=28, seed=3):
    """Transducers on a sphere of radius 0.95 nv around a 96^3 volume: 700
    rays (not a multiple of the reduction's 32-ray groups or 256-ray windows),
    333 of them missing the grid (empty rows), 110 crossing more than 16 of
    the 8^3 tiles (the per-ray reduction's loads past its staged partials)."""
    from tval3_gb300.api import Geometry
    rng = np.random.default_rng(seed)
    c = nv / 2.0

    def pts(k):
        u = rng.normal(size=(k, 3))
        u /= np.linalg.norm(u, axis=1, keepdims=True)
        return c + 0.95 * nv * u

    em, rc = pts(ne), pts(nr)
    ie, ir = ([np.clip(np.floor(P[:, a]), 0, nv - 1).astype(np.int32) for a in range(3)] for P in (em, rc))
    return Geometry(rv_x=nv, rv_y=nv, rv_z=nv, x_emitters=ie[0], y_emitters=ie[1], z_emitters=ie[2],
                    x_receivers=ir[0], y_receivers=ir[1], z_receivers=ir[2], num_emitters=ne, num_receivers=nr,
                    traversal=1, pos=tuple(em[:, a].copy() for a in range(3)) + tuple(rc[:, a].copy() for a in range(3)))


@pytest.mark.parametrize("kind", ["ring", "hemi", "dense_ring", "big", "mixed"])
@pytest.mark.parametrize("prec", ["fp32", "df64", "bf16"])
@pytest.mark.parametrize("trans", [1, 0])
def test_tiled_products_match_plain_csr(cuda, kind, prec, trans):
    import torch
    from tval3_gb300 import PREC_BF16, PREC_FP32, PREC_FP32_DF64, Operator, SparseMatrix
    geo = _geo(kind)
    p = {"fp32": PREC_FP32, "df64": PREC_FP32_DF64, "bf16": PREC_BF16}[prec]
    tiled = Operator.from_geometry(geo, mode=0, precision=p)
    ptr, ind, val, tptr, tind, tval = Operator.from_geometry(geo, mode=0, precision=PREC_FP32).export_csr()
    m, n = ptr.size - 1, tptr.size - 1
    plain = Operator.from_sparse(SparseMatrix(m, n, ptr, ind, val, tptr, tind, tval), precision=p)
    # small operators keep the tile-staged form without a timing contest
    assert tiled.variant(trans) == 1 and plain.variant(trans) == 0
    g = torch.Generator().manual_seed(7 + trans)
    lin, lout = (m, n) if trans else (n, m)
    yh = torch.randn(lin, dtype=torch.float64, generator=g)
    absA = np.zeros(lout)
    if trans:
        np.add.at(absA, np.repeat(np.arange(n), np.diff(tptr)), np.abs(tval.astype(np.float64)) * np.abs(yh.numpy()[tind]))
    else:
        np.add.at(absA, np.repeat(np.arange(m), np.diff(ptr)), np.abs(val.astype(np.float64)) * np.abs(yh.numpy()[ind]))
    if prec == "df64":
        from tval3_gb300 import capi
        lib = capi.load()
        yd = torch.empty(2 * lin, dtype=torch.float32, device=cuda)
        capi.check(lib.tval3_df64_from_f64(yh.to(cuda).data_ptr(), yd.data_ptr(), lin, None))
        outs = []
        for op in (tiled, plain):
            xd = torch.empty(2 * lout, dtype=torch.float32, device=cuda)
            op.mat_vec_mul(trans, yd, xd)
            xo = torch.empty(lout, dtype=torch.float64, device=cuda)
            capi.check(lib.tval3_df64_to_f64(xd.data_ptr(), xo.data_ptr(), lout, None))
            outs.append(xo.cpu().numpy())
        tol = 1e-12
    else:
        yd = yh.float().to(cuda)
        outs = []
        for op in (tiled, plain):
            xd = torch.empty(lout, dtype=torch.float32, device=cuda)
            op.mat_vec_mul(trans, yd, xd)
            outs.append(xd.cpu().numpy().astype(np.float64))
        tol = 1e-5
    torch.cuda.synchronize()
    assert np.all(np.abs(outs[0] - outs[1]) <= tol * absA + 1e-30)


def test_tiled_solve_matches_oracle_fp64(cuda, oracle):
    """A full FP64 3D solve through a solver (which gives its operator the
    volume, so A^T is tiled) keeps the oracle's control flow and result."""
    import torch
    from tval3_gb300 import PREC_FP64, Operator, Solver, SparseMatrix
    from tval3_gb300 import workloads as W
    cfg, geo, x = W.config_3d(24, 32, 32, seed=2)
    ptr, ind, val = oracle.siddon_csr(geo)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), cfg.noise, 2).astype(np.float64)
    o = dict(cfg.opts, maxit=60)
    Uo, io = oracle.tval3_csr(cfg.dims, ptr, ind, val, b, o)
    op = Operator.from_sparse(SparseMatrix(ptr.size - 1, x.size, ptr, ind, val.astype(np.float64)),
                              precision=PREC_FP64)
    s = Solver(op, cfg.dims, o, mode=1)
    U = torch.empty(x.size, dtype=torch.float64, device=cuda)
    ig = s.solve(torch.tensor(b, device=cuda), U)
    assert (ig["total_iters"], ig["outer_iters"], ig["backtracks"], ig["restarts"]) == \
        (io["total_iters"], io["outer_iters"], io["backtracks"], io["restarts"])
    assert np.linalg.norm(U.cpu().numpy() - Uo.reshape(-1)) <= 1e-7 * np.linalg.norm(Uo)


@pytest.mark.parametrize("kind", ["ring", "hemi"])
@pytest.mark.parametrize("prec", ["fp32", "df64", "fp64vec"])
def test_pipelined_AT_is_bit_identical_to_tiled(cuda, kind, prec):
    """Variant 2 of A^T*y (producer warp streaming the units through a
    shared-memory ring) forms exactly the sums of variant 1, in the same
    order: the outputs agree bit for bit, rows without nonzeros included."""
    import torch
    from tval3_gb300 import PREC_FP32, PREC_FP32_DF64, PREC_FP32_F64VEC, Operator
    geo = _geo(kind)
    p = {"fp32": PREC_FP32, "df64": PREC_FP32_DF64, "fp64vec": PREC_FP32_F64VEC}[prec]
    op = Operator.from_geometry(geo, mode=0, precision=p)
    g = torch.Generator().manual_seed(11)
    words = 2 if prec == "df64" else 1
    dt = torch.float64 if prec == "fp64vec" else torch.float32
    y = torch.randn(words * op.rows, generator=g, dtype=torch.float64).to(dt).to(cuda)
    if prec == "df64":
        y[1::2] = y[0::2] * 1e-8  # a nonzero low word in every element
    outs = []
    for v in (1, 2):
        op.set_variant(1, v)
        assert op.variant(1) == v
        x = torch.full((words * op.cols,), float("nan"), dtype=dt, device=cuda)
        for _ in range(2):  # twice: the second launch starts from a used ring
            op.mat_vec_mul(1, y, x)
        outs.append(x.cpu())
    torch.cuda.synchronize()
    assert not torch.isnan(outs[1]).any()
    assert torch.equal(outs[0], outs[1])


def test_pipelined_AT_in_a_solve(cuda, oracle):
    """A double-float 3D solve with A^T pinned to the pipelined kernel (its
    SUB epilogue, g = A^T Au - Atb) takes the same path to the same result,
    bit for bit, as with the tile-staged kernel."""
    import torch
    from tval3_gb300 import PREC_FP32_DF64, Operator, Solver
    from tval3_gb300 import workloads as W
    cfg, geo, x = W.config_3d(24, 32, 32, seed=4)
    ptr, ind, val = oracle.siddon_csr(geo)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), cfg.noise, 4).astype(np.float64)
    o = dict(cfg.opts, maxit=40)
    res = []
    for v in (1, 2):
        op = Operator.from_geometry(geo, mode=0, precision=PREC_FP32_DF64)
        op.set_variant(1, v)
        s = Solver(op, cfg.dims, o, mode=1)
        U = torch.empty(x.size, dtype=torch.float64, device=cuda)
        info = s.solve(torch.tensor(b, device=cuda), U)
        torch.cuda.synchronize()
        assert op.variant(1) == v
        res.append((info["total_iters"], info["backtracks"], info["restarts"], U.cpu()))
        s.close()
    assert res[0][:3] == res[1][:3]
    assert torch.equal(res[0][3], res[1][3])


def test_variant_pinning(cuda):
    """tval3_op_set_variant pins the kernel of each product; the two kernels
    of one operator agree, and an operator without a volume has no tiled form."""
    import torch
    from tval3_gb300 import PREC_FP32, Operator, SparseMatrix, Tval3Error
    geo = _geo("hemi")
    op = Operator.from_geometry(geo, mode=0, precision=PREC_FP32)
    g = torch.Generator().manual_seed(3)
    y = torch.randn(op.rows, generator=g).to(cuda)
    outs = []
    for v in (0, 1, 2):
        op.set_variant(1, v)
        assert op.variant(1) == v
        x = torch.empty(op.cols, device=cuda)
        op.mat_vec_mul(1, y, x)
        outs.append(x)
    torch.cuda.synchronize()
    assert torch.allclose(outs[0], outs[1], rtol=1e-5, atol=1e-5 * float(outs[0].abs().max()))
    assert torch.equal(outs[1], outs[2])
    with pytest.raises(Tval3Error):
        op.set_variant(0, 2)  # A*x has no pipelined form
    ptr, ind, val, tptr, tind, tval = op.export_csr()
    bare = Operator.from_sparse(SparseMatrix(ptr.size - 1, tptr.size - 1, ptr, ind, val), precision=PREC_FP32)
    with pytest.raises(Tval3Error):
        bare.set_variant(0, 1)
