"""PyTorch autograd binding of the TVAL3 operators (the only PyTorch-facing part).

Every forward and backward runs a kernel of libtval3_gb300.so through the C
ABI on the caller's current stream; the backward of each map is its
hand-written adjoint kernel:

    A      forward CSR A*x                  backward A^T*g   (mat_vec_mul, trans)
    At     forward A^T*y                    backward A*g
    D      forward periodic differences     backward D^T     (3d/tval3_gpu_3d.cpp:271-361)
    Dt     forward D^T                      backward D
    shrink forward shrinkage W(v, t)        backward subgradient (tval3_shrink_adjoint)

`unrolled_tval3` composes them into K inner iterations of the TVAL3
u-subproblem (3d/tval3_gpu_3d.cpp:823-1029): W = shrink(DU - sigma/beta,
1/beta), d = D^T(DU - W) + mu/beta A^T(AU - b), Barzilai-Borwein step tau
(first step |<d,d> / (||Dd||^2 + mu/beta ||Ad||^2)|), U <- max(U - tau d, 0).
The nonmonotone Armijo test of the reference is a discrete decision and is
not part of the differentiable map; everything else, including tau, is
differentiated.  Each iteration is checkpointed (recomputed in the backward
pass) so memory stays at one iteration's state.
"""
from __future__ import annotations

import torch
from torch.utils.checkpoint import checkpoint

from . import capi
from .api import Operator


def _stream():
    return torch.cuda.current_stream().cuda_stream


class _MatVec(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, op, trans):
        x = x.contiguous()
        out = torch.empty(op.cols if trans else op.rows, dtype=x.dtype, device=x.device)
        op.mat_vec_mul(trans, x, out, stream=_stream())
        ctx.op, ctx.trans = op, trans
        return out

    @staticmethod
    def backward(ctx, g):
        g = g.contiguous()
        op, trans = ctx.op, ctx.trans
        gx = torch.empty(op.rows if trans else op.cols, dtype=g.dtype, device=g.device)
        op.mat_vec_mul(1 - trans, g, gx, stream=_stream())
        return gx, None, None


def A(op: Operator, x: torch.Tensor) -> torch.Tensor:
    """y = A x (differentiable; backward A^T)."""
    return _MatVec.apply(x, op, 0)


def At(op: Operator, y: torch.Tensor) -> torch.Tensor:
    """x = A^T y (differentiable; backward A)."""
    return _MatVec.apply(y, op, 1)


def _dfun(x, dims, out_n, adjoint):
    lib = capi.load()
    out = torch.empty(out_n, dtype=x.dtype, device=x.device)
    if x.dtype == torch.float64:
        f = lib.tval3_Dt_f64 if adjoint else lib.tval3_D_f64
    else:
        f = lib.tval3_Dt_f32 if adjoint else lib.tval3_D_f32
    capi.check(f(*dims, x.data_ptr(), out.data_ptr(), _stream()))
    return out


class _D(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, dims, adjoint):
        u = u.contiguous()
        n = dims[0] * dims[1] * dims[2]
        ctx.dims, ctx.adjoint = dims, adjoint
        return _dfun(u, dims, n if adjoint else 3 * n, adjoint)

    @staticmethod
    def backward(ctx, g):
        n = ctx.dims[0] * ctx.dims[1] * ctx.dims[2]
        return _dfun(g.contiguous(), ctx.dims, 3 * n if ctx.adjoint else n, not ctx.adjoint), None, None


def D(u: torch.Tensor, dims) -> torch.Tensor:
    """Periodic forward differences (3 n-vectors: along y, x, z)."""
    return _D.apply(u, tuple(dims), False)


def Dt(v: torch.Tensor, dims) -> torch.Tensor:
    """Adjoint of D."""
    return _D.apply(v, tuple(dims), True)


class _Shrink(torch.autograd.Function):
    @staticmethod
    def forward(ctx, v, t, iso):
        v = v.contiguous()
        n = v.numel() // 3
        lib = capi.load()
        W = torch.empty_like(v)
        f = lib.tval3_shrink_f64 if v.dtype == torch.float64 else lib.tval3_shrink_f32
        capi.check(f(n, v.data_ptr(), float(t), int(iso), W.data_ptr(), _stream()))
        ctx.save_for_backward(v, t if torch.is_tensor(t) else torch.tensor(float(t)))
        ctx.iso = iso
        return W

    @staticmethod
    def backward(ctx, gW):
        v, t = ctx.saved_tensors
        n = v.numel() // 3
        lib = capi.load()
        gv = torch.empty_like(v)
        gt = torch.empty(n, dtype=v.dtype, device=v.device)
        f = lib.tval3_shrink_adjoint_f64 if v.dtype == torch.float64 else lib.tval3_shrink_adjoint_f32
        capi.check(f(n, v.data_ptr(), float(t), int(ctx.iso), gW.contiguous().data_ptr(), gv.data_ptr(),
                     gt.data_ptr(), _stream()))
        return gv, gt.sum().to(t.dtype).reshape(t.shape), None


def shrink(v: torch.Tensor, t, iso: bool = True) -> torch.Tensor:
    """W = shrink(v, t): isotropic (per voxel) or anisotropic (per component)."""
    if not torch.is_tensor(t):
        t = torch.tensor(float(t), dtype=v.dtype, device=v.device)
    return _Shrink.apply(v, t, iso)


def _dot(a, b):
    return (a * b).sum()


def unrolled_tval3(op: Operator, b: torch.Tensor, dims, mu, beta, iters: int = 20, iso: bool = True,
                   nonneg: bool = True, sigma=None, delta=None, use_checkpoint: bool = True) -> torch.Tensor:
    """K differentiable inner iterations of the TVAL3 u-subproblem from U = A^T b.
    mu and beta may be tensors requiring grad; returns U_K (n-vector)."""
    dt = b.dtype
    mu = mu if torch.is_tensor(mu) else torch.tensor(float(mu), dtype=dt, device=b.device)
    beta = beta if torch.is_tensor(beta) else torch.tensor(float(beta), dtype=dt, device=b.device)
    n = dims[0] * dims[1] * dims[2]
    sig = sigma if sigma is not None else torch.zeros(3 * n, dtype=dt, device=b.device)
    dl = delta if delta is not None else torch.zeros(b.numel(), dtype=dt, device=b.device)
    Atb = At(op, b)

    def grad_dir(U, mu, beta):
        DU = D(U, dims)
        W = shrink(DU - sig / beta, 1.0 / beta, iso)
        g = At(op, A(op, U) - b) - At(op, dl) / mu
        g2 = Dt(DU - W, dims) - Dt(sig, dims) / beta
        return g2 + (mu / beta) * g, g, g2

    def step(U, Up, gp, g2p, first, mu, beta):
        d, g, g2 = grad_dir(U, mu, beta)
        if first:
            Dd = D(d, dims)
            Ad = A(op, d)
            tau = torch.abs(_dot(d, d) / (_dot(Dd, Dd) + (mu / beta) * _dot(Ad, Ad)))
        else:
            s = U - Up
            tau = torch.abs(_dot(s, s) / _dot(s, (g2 - g2p) + (mu / beta) * (g - gp)))
        Un = U - tau * d
        if nonneg:
            Un = torch.relu(Un)
        return Un, g, g2

    U = Atb
    Up = gp = g2p = None
    for k in range(iters):
        first = k == 0
        if first:
            def fn(U_, mu_, beta_):
                return step(U_, None, None, None, True, mu_, beta_)
            args = (U, mu, beta)
        else:
            def fn(U_, Up_, gp_, g2p_, mu_, beta_):
                return step(U_, Up_, gp_, g2p_, False, mu_, beta_)
            args = (U, Up, gp, g2p, mu, beta)
        if use_checkpoint:
            Un, g, g2 = checkpoint(fn, *args, use_reentrant=False)
        else:
            Un, g, g2 = fn(*args)
        Up, gp, g2p, U = U, g, g2, Un
    return U
