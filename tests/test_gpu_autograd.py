"""Autograd binding: the hand-written adjoints (A^T, D^T, shrinkage
subgradient, and the whole inner step's tval3_unroll_step_adjoint) pass
torch.autograd.gradcheck and dot-product tests in FP64; the gradient of a
loss through K unrolled TVAL3 iterations (each one fused _InnerStep) with
respect to b, mu and beta agrees with central finite differences (h = 1e-5,
FP64) and with the same map composed from the single-operator Functions
(the eager reference below, kept only here)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _op64(oracle, n=8, ne=6, seed=0):
    from tval3_gb300 import PREC_FP64, Operator, SparseMatrix
    from tval3_gb300 import workloads as W
    cfg, geo, x = W.config_3d(n, ne, ne, seed=seed)
    ptr, ind, val = oracle.siddon_csr(geo)
    op = Operator.from_sparse(SparseMatrix(ptr.size - 1, x.size, ptr, ind, val.astype(np.float64)),
                              precision=PREC_FP64)
    return cfg, geo, x, op


def test_gradcheck_operators(cuda, oracle):
    import torch
    from tval3_gb300 import autograd as AG
    cfg, geo, x, op = _op64(oracle)
    dims = cfg.dims
    n = x.size
    g = torch.Generator().manual_seed(0)
    xv = torch.randn(n, dtype=torch.float64, generator=g).to(cuda).requires_grad_()
    yv = torch.randn(op.rows, dtype=torch.float64, generator=g).to(cuda).requires_grad_()
    assert torch.autograd.gradcheck(lambda t: AG.A(op, t), (xv,), eps=1e-6, atol=1e-8)
    assert torch.autograd.gradcheck(lambda t: AG.At(op, t), (yv,), eps=1e-6, atol=1e-8)
    assert torch.autograd.gradcheck(lambda t: AG.D(t, dims), (xv,), eps=1e-6, atol=1e-8)
    v3 = torch.randn(3 * n, dtype=torch.float64, generator=g).to(cuda).requires_grad_()
    assert torch.autograd.gradcheck(lambda t: AG.Dt(t, dims), (v3,), eps=1e-6, atol=1e-8)


@pytest.mark.parametrize("iso", [True, False])
def test_shrink_adjoint_gradcheck(cuda, iso):
    import torch
    from tval3_gb300 import autograd as AG
    g = torch.Generator().manual_seed(1)
    v = (torch.randn(3 * 50, dtype=torch.float64, generator=g) * 0.5).to(cuda)
    # keep away from the kinks |v| = t, where the subgradient is not a derivative
    t = torch.tensor(0.3, dtype=torch.float64, device=cuda, requires_grad=True)
    if iso:
        nv = v.reshape(3, -1).norm(dim=0)
        keep = ((nv - 0.3).abs() > 0.05).repeat(3)
    else:
        keep = ((v.abs() - 0.3).abs() > 0.05)
    v = torch.where(keep, v, torch.full_like(v, 0.9)).requires_grad_()
    assert torch.autograd.gradcheck(lambda a, b: AG.shrink(a, b, iso), (v, t), eps=1e-7, atol=1e-7)


def test_dot_product_adjoints(cuda, oracle):
    import torch
    from tval3_gb300 import autograd as AG
    cfg, geo, x, op = _op64(oracle, 12, 8)
    dims = cfg.dims
    g = torch.Generator().manual_seed(2)
    u = torch.randn(x.size, dtype=torch.float64, generator=g).to(cuda)
    y = torch.randn(op.rows, dtype=torch.float64, generator=g).to(cuda)
    p = torch.randn(3 * x.size, dtype=torch.float64, generator=g).to(cuda)
    assert abs(float((AG.A(op, u) * y).sum() - (u * AG.At(op, y)).sum())) < 1e-10 * float(y.norm() * u.norm())
    assert abs(float((AG.D(u, dims) * p).sum() - (u * AG.Dt(p, dims)).sum())) < 1e-10 * float(p.norm() * u.norm())


def _loss_setup(oracle, n, ne, iters, cuda):
    import torch
    from tval3_gb300 import workloads as W
    cfg, geo, x, op = _op64(oracle, n, ne, seed=3)
    ptr, ind, val = oracle.siddon_csr(geo)
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), 0.01, 3).astype(np.float64)
    # scale as the reference does (scaleb_gpu), so mu and beta have their usual meaning
    bmin, bmax = b[np.argmin(np.abs(b))], b[np.argmax(np.abs(b))]
    scl = 1.5 / abs(bmax - bmin)
    bt = torch.tensor(b * scl, device=cuda)
    xt = torch.tensor(x.reshape(-1) * scl, dtype=torch.float64, device=cuda)
    return cfg, op, bt, xt


@pytest.mark.parametrize("size,rays,iters", [(16, 12, 8), (96, 256, 20)])
def test_unrolled_gradient_vs_finite_differences(cuda, oracle, size, rays, iters):
    """loss = ||U_K - x_true||^2 through K unrolled iterations; gradients wrt
    b (random direction), mu and beta vs central differences with h = 1e-5
    (relative to mu and beta, absolute along the unit direction for b).  The
    96^3, 256 x 256-ray, 20-iteration case is the differentiable workload.
    The map is piecewise smooth: every voxel's shrinkage threshold and
    nonnegativity clamp is a kink, and at 96^3 a step of 1e-3 along b crosses
    enough of them that the difference quotient is an average slope (0.346
    against the local derivative 0.444 here); at 1e-5 the two agree to 1e-6."""
    import torch
    from tval3_gb300 import autograd as AG
    cfg, op, b, xt = _loss_setup(oracle, size, rays, iters, cuda)
    dims = cfg.dims
    mu0, beta0 = 2.0 ** 9, 2.0 ** 6

    def loss(bb, mu, beta):
        U = AG.unrolled_tval3(op, bb, dims, mu, beta, iters=iters, iso=True)
        return ((U - xt) ** 2).sum()

    bb = b.clone().requires_grad_()
    mu = torch.tensor(mu0, dtype=torch.float64, device=cuda, requires_grad=True)
    beta = torch.tensor(beta0, dtype=torch.float64, device=cuda, requires_grad=True)
    L = loss(bb, mu, beta)
    L.backward()
    g = torch.Generator().manual_seed(5)
    v = torch.randn(b.numel(), dtype=torch.float64, generator=g).to(cuda)
    v /= v.norm()
    h = 1e-5
    with torch.no_grad():
        fd_b = (loss(b + h * v, mu0, beta0) - loss(b - h * v, mu0, beta0)) / (2 * h)
        fd_mu = (loss(b, mu0 * (1 + h), beta0) - loss(b, mu0 * (1 - h), beta0)) / (2 * h * mu0)
        fd_beta = (loss(b, mu0, beta0 * (1 + h)) - loss(b, mu0, beta0 * (1 - h))) / (2 * h * beta0)
    an_b = float((bb.grad * v).sum())
    for an, fd in ((an_b, float(fd_b)), (float(mu.grad), float(fd_mu)), (float(beta.grad), float(fd_beta))):
        assert abs(an - fd) <= 2e-3 * max(abs(fd), 1e-8 * float(L.detach())), (an, fd)


def _eager_unrolled(op, b, dims, mu, beta, iters, iso=True, nonneg=True, sigma=None, delta=None):
    """The unrolled map composed from the single-operator Functions (A, At,
    D, Dt, shrink) and PyTorch elementwise ops: the reference the fused
    _InnerStep is checked against."""
    import torch
    from tval3_gb300 import autograd as AG
    dt = b.dtype
    n = dims[0] * dims[1] * dims[2]
    sig = sigma if sigma is not None else torch.zeros(3 * n, dtype=dt, device=b.device)
    dl = delta if delta is not None else torch.zeros(b.numel(), dtype=dt, device=b.device)
    dot = lambda x, y: (x * y).sum()

    def grad_dir(U):
        DU = AG.D(U, dims)
        W = AG.shrink(DU - sig / beta, 1.0 / beta, iso)
        g = AG.At(op, AG.A(op, U) - b) - AG.At(op, dl) / mu
        g2 = AG.Dt(DU - W, dims) - AG.Dt(sig, dims) / beta
        return g2 + (mu / beta) * g, g, g2

    U = AG.At(op, b)
    Up = gp = g2p = None
    for k in range(iters):
        d, g, g2 = grad_dir(U)
        if k == 0:
            Dd, Ad = AG.D(d, dims), AG.A(op, d)
            tau = torch.abs(dot(d, d) / (dot(Dd, Dd) + (mu / beta) * dot(Ad, Ad)))
        else:
            s_ = U - Up
            tau = torch.abs(dot(s_, s_) / dot(s_, (g2 - g2p) + (mu / beta) * (g - gp)))
        Un = U - tau * d
        if nonneg:
            Un = torch.relu(Un)
        Up, gp, g2p, U = U, g, g2, Un
    return U


@pytest.mark.parametrize("iso", [True, False])
def test_fused_step_matches_eager_reference(cuda, oracle, iso):
    """U_K and the gradients wrt b, mu, beta of the fused map equal those of
    the eager composition (FP64; only summation orders differ), with nonzero
    multipliers sigma and delta."""
    import torch
    from tval3_gb300 import autograd as AG
    cfg, op, b, xt = _loss_setup(oracle, 12, 8, 6, cuda)
    g = torch.Generator().manual_seed(7)
    n = xt.numel()
    sig = (0.05 * torch.randn(3 * n, dtype=torch.float64, generator=g)).to(cuda)
    dl = (0.05 * torch.randn(b.numel(), dtype=torch.float64, generator=g)).to(cuda)
    outs = []
    for fn in (AG.unrolled_tval3, _eager_unrolled):
        bb = b.clone().requires_grad_()
        mu = torch.tensor(512.0, dtype=torch.float64, device=cuda, requires_grad=True)
        beta = torch.tensor(64.0, dtype=torch.float64, device=cuda, requires_grad=True)
        U = fn(op, bb, cfg.dims, mu, beta, iters=6, iso=iso, sigma=sig, delta=dl)
        ((U - xt) ** 2).sum().backward()
        outs.append((U.detach(), bb.grad, mu.grad, beta.grad))
    (U1, gb1, gm1, gbt1), (U2, gb2, gm2, gbt2) = outs
    assert torch.allclose(U1, U2, rtol=1e-10, atol=1e-12 * float(U2.abs().max()))
    assert torch.allclose(gb1, gb2, rtol=1e-8, atol=1e-10 * float(gb2.abs().max()))
    assert abs(float(gm1) - float(gm2)) <= 1e-8 * abs(float(gm2)) + 1e-14
    assert abs(float(gbt1) - float(gbt2)) <= 1e-8 * abs(float(gbt2)) + 1e-14


def _numpy_unrolled(ptr, ind, val, b, dims, mu, beta, iters, iso=True, nonneg=True):
    """The unrolled map in numpy (FP64, CPU), from the formulas alone:
    periodic forward differences on the [z, x, y] volume, isotropic or
    anisotropic shrinkage, the Barzilai-Borwein step and the projection."""
    import scipy.sparse as sp
    p, q, r = dims
    n = p * q * r
    A = sp.csr_matrix((val.astype(np.float64), ind, ptr), shape=(ptr.size - 1, n))

    def D(u):
        v = u.reshape(r, q, p)
        return np.concatenate([(np.roll(v, -1, 2) - v).ravel(), (np.roll(v, -1, 1) - v).ravel(),
                               (np.roll(v, -1, 0) - v).ravel()])

    def Dt(w):
        a, c, e = (w[k * n:(k + 1) * n].reshape(r, q, p) for k in range(3))
        return ((np.roll(a, 1, 2) - a) + (np.roll(c, 1, 1) - c) + (np.roll(e, 1, 0) - e)).ravel()

    def shrink(v, t):
        v3 = v.reshape(3, n)
        if iso:
            nv = np.sqrt((v3 * v3).sum(0))
            sc = np.where(nv > t, (nv - t) / np.where(nv > 0, nv, 1.0), 0.0)
            return (v3 * sc).ravel()
        return (np.sign(v3) * np.maximum(np.abs(v3) - t, 0.0)).ravel()

    kap = mu / beta
    U = A.T @ b
    Up = gp = g2p = None
    for k in range(iters):
        DU = D(U)
        W = shrink(DU, 1.0 / beta)
        g2 = Dt(DU - W)
        g = A.T @ (A @ U - b)
        d = g2 + kap * g
        if k == 0:
            Dd, Ad = D(d), A @ d
            tau = abs(d @ d / (Dd @ Dd + kap * (Ad @ Ad)))
        else:
            s_ = U - Up
            tau = abs(s_ @ s_ / (s_ @ ((g2 - g2p) + kap * (g - gp))))
        Un = U - tau * d
        if nonneg:
            Un = np.maximum(Un, 0.0)
        Up, gp, g2p, U = U, g, g2, Un
    return U


@pytest.mark.parametrize("iso", [True, False])
def test_fused_forward_matches_numpy(cuda, oracle, iso):
    """The fused unrolled map's U_K against a numpy evaluation of the same
    formulas on the CPU (FP64; only summation orders differ): 8 steps on a
    12^3 hemisphere problem."""
    import torch
    from tval3_gb300 import autograd as AG
    cfg, geo, x, op = _op64(oracle, 12, 8, seed=5)
    ptr, ind, val = oracle.siddon_csr(geo)
    from tval3_gb300 import workloads as W
    b = W.add_noise(oracle.spmv(ptr, ind, val, x), 0.01, 5).astype(np.float64)
    b *= 1.5 / abs(b.max() - b.min())
    U = AG.unrolled_tval3(op, torch.tensor(b, device=cuda), cfg.dims, 512.0, 64.0, iters=8, iso=iso)
    Un = _numpy_unrolled(ptr, ind, val, b, cfg.dims, 512.0, 64.0, 8, iso=iso)
    assert np.linalg.norm(U.cpu().numpy() - Un) <= 1e-10 * np.linalg.norm(Un)


@pytest.mark.parametrize("first", [True, False])
def test_inner_step_gradcheck(cuda, oracle, first):
    """torch.autograd.gradcheck of one fused step wrt U, Up, gp, g2p, b and
    (mu, beta) (FP64, no projection so the map is smooth away from the
    shrinkage kinks, which random inputs at eps = 1e-6 do not cross)."""
    import torch
    from tval3_gb300 import autograd as AG
    cfg, geo, x, op = _op64(oracle, 6, 5, seed=4)
    dims = cfg.dims
    n, m = x.size, op.rows
    g = torch.Generator().manual_seed(11)
    mk = lambda k, sc=1.0: (sc * torch.randn(k, dtype=torch.float64, generator=g)).to(cuda).requires_grad_()
    U, Up, gp, g2p = mk(n), mk(n), mk(n), mk(n)
    b = mk(m)
    mub = torch.tensor([4.0, 2.0], dtype=torch.float64, device=cuda, requires_grad=True)
    sig = (0.1 * torch.randn(3 * n, dtype=torch.float64, generator=g)).to(cuda)

    def f(U_, Up_, gp_, g2p_, b_, mub_):
        if first:
            outs = AG._InnerStep.apply(U_, None, None, None, b_, mub_, op, dims, True, True, False, sig, None)
        else:
            outs = AG._InnerStep.apply(U_, Up_, gp_, g2p_, b_, mub_, op, dims, False, True, False, sig, None)
        return outs

    assert torch.autograd.gradcheck(f, (U, Up, gp, g2p, b, mub), eps=1e-6, atol=1e-6, rtol=1e-5)
