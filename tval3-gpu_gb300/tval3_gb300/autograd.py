"""PyTorch autograd binding of the TVAL3 operators (the only PyTorch-facing part).

Every forward and backward runs a kernel of libtval3_gb300.so through the C
ABI on the caller's current stream; the backward of each map is its
hand-written adjoint kernel:

    A      forward CSR A*x                  backward A^T*g   (mat_vec_mul, trans)
    At     forward A^T*y                    backward A*g
    D      forward periodic differences     backward D^T     (3d/tval3_gpu_3d.cpp:271-361)
    Dt     forward D^T                      backward D
    shrink forward shrinkage W(v, t)        backward subgradient (tval3_shrink_adjoint)

`unrolled_tval3` runs K inner iterations of the TVAL3 u-subproblem
(3d/tval3_gpu_3d.cpp:823-1029), each one `_InnerStep` Function: W =
shrink(DU - sigma/beta, 1/beta), d = D^T(DU - W - sigma/beta) + mu/beta
A^T(AU - b - delta/mu), Barzilai-Borwein step tau (first step |<d,d> /
(||Dd||^2 + mu/beta ||Ad||^2)|), U <- max(U - tau d, 0).  Its forward is one
C call of fused kernels (tval3_unroll_step_*) and its backward one C call of
hand-written adjoint kernels (tval3_unroll_step_adjoint_*: projection mask,
BB quotient, transposed products, shrinkage subgradient).  The nonmonotone
Armijo test of the reference is a discrete decision and is not part of the
differentiable map; everything else, including tau, is differentiated.  A
step keeps only its inputs and recomputes its intermediates in the backward
pass (per-iteration checkpointing), so memory stays at U, g, g2 per step.
"""
from __future__ import annotations

import torch

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


def _ptr(t):
    return t.data_ptr() if t is not None else None


class _InnerStep(torch.autograd.Function):
    """One inner step of the TVAL3 u-subproblem as a single Function: the
    forward is tval3_unroll_step_* (fused kernels), the backward
    tval3_unroll_step_adjoint_* (hand-written adjoint kernels: projection
    mask, BB quotient, the transposed products, shrinkage subgradient).  Only
    the inputs are kept; the backward recomputes the step's intermediates, so
    each step is its own checkpoint."""

    @staticmethod
    def forward(ctx, U, Up, gp, g2p, b, mub, op, dims, first, iso, nonneg, sigma, delta):
        lib = capi.load()
        f = lib.tval3_unroll_step_f64 if U.dtype == torch.float64 else lib.tval3_unroll_step_f32
        U = U.contiguous()
        b = b.contiguous()
        mub = mub.detach().to(torch.float64).contiguous()
        Un, g, g2 = torch.empty_like(U), torch.empty_like(U), torch.empty_like(U)
        ins = [None, None, None] if first else [Up.contiguous(), gp.contiguous(), g2p.contiguous()]
        capi.check(f(op.handle, *dims, int(first), int(iso), int(nonneg), mub.data_ptr(), U.data_ptr(),
                     *[_ptr(t) for t in ins], b.data_ptr(), _ptr(sigma), _ptr(delta), Un.data_ptr(), g.data_ptr(),
                     g2.data_ptr(), _stream()))
        ctx.save_for_backward(U, *(t if t is not None else torch.empty(0, device=U.device) for t in ins), b, mub)
        ctx.op, ctx.dims, ctx.first, ctx.iso, ctx.nonneg = op, dims, first, iso, nonneg
        ctx.sigma, ctx.delta = sigma, delta
        return Un, g, g2

    @staticmethod
    def backward(ctx, gUn, gg, gg2):
        U, Up, gp, g2p, b, mub = ctx.saved_tensors
        first = ctx.first
        lib = capi.load()
        f = lib.tval3_unroll_step_adjoint_f64 if U.dtype == torch.float64 else lib.tval3_unroll_step_adjoint_f32
        gU = torch.empty_like(U)
        gUp = ggp = gg2p = None
        if not first:
            gUp, ggp, gg2p = torch.empty_like(U), torch.empty_like(U), torch.empty_like(U)
        gb = torch.empty_like(b)
        gmub = torch.empty(2, dtype=torch.float64, device=U.device)
        cont = lambda t: t.contiguous() if t is not None else None
        ins = [None, None, None] if first else [Up, gp, g2p]
        capi.check(f(ctx.op.handle, *ctx.dims, int(first), int(ctx.iso), int(ctx.nonneg), mub.data_ptr(),
                     U.data_ptr(), *[_ptr(t) for t in ins], b.data_ptr(), _ptr(ctx.sigma), _ptr(ctx.delta),
                     _ptr(cont(gUn)), _ptr(cont(gg)), _ptr(cont(gg2)), gU.data_ptr(), _ptr(gUp), _ptr(ggp),
                     _ptr(gg2p), gb.data_ptr(), gmub.data_ptr(), _stream()))
        return (gU, gUp, ggp, gg2p, gb, gmub, None, None, None, None, None, None, None)


def unrolled_tval3(op: Operator, b: torch.Tensor, dims, mu, beta, iters: int = 20, iso: bool = True,
                   nonneg: bool = True, sigma=None, delta=None) -> torch.Tensor:
    """K differentiable inner iterations of the TVAL3 u-subproblem from
    U = A^T b, each one _InnerStep (fused forward kernels, hand-written
    adjoint kernels, recomputation in the backward pass as per-iteration
    checkpointing).  mu and beta may be tensors requiring grad; b may require
    grad; returns U_K (n-vector).  sigma (3n) and delta (m) are the fixed
    multipliers (zero when None)."""
    dt = b.dtype
    mu = mu if torch.is_tensor(mu) else torch.tensor(float(mu), dtype=torch.float64, device=b.device)
    beta = beta if torch.is_tensor(beta) else torch.tensor(float(beta), dtype=torch.float64, device=b.device)
    mub = torch.stack([mu.to(torch.float64).reshape(()), beta.to(torch.float64).reshape(())])
    sig = sigma.to(dt).contiguous() if sigma is not None else None
    dl = delta.to(dt).contiguous() if delta is not None else None
    dims = tuple(int(v) for v in dims)
    U = At(op, b)
    Up = gp = g2p = None
    for k in range(iters):
        Un, g, g2 = _InnerStep.apply(U, Up, gp, g2p, b, mub, op, dims, k == 0, iso, nonneg, sig, dl)
        Up, gp, g2p, U = U, g, g2, Un
    return U
