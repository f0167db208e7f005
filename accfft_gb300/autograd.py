"""Differentiable spectral transforms and operators (torch.autograd).

Forward passes run the plan's kernels; backward passes run the adjoint
kernels of the C ABI (no framework FFT anywhere):

    rfft3        u -> X = R u                 backward: R^T g  = accfft_c_r2c_adjoint
    irfft3       X -> x = c2r(X) (unnormalised) backward: w * R g = accfft_c_c2r_adjoint
    grad         u -> (du/dx, du/dy, du/dz)   backward: -div g   = accfft_c_grad_adjoint
    divergence   (a_x, a_y, a_z) -> div a      backward: -grad g  = accfft_c_divergence_adjoint
    laplace, biharmonic, inv_laplace, inv_biharmonic
                 c2r . S . r2c with a real diagonal symbol S: self-adjoint
                 (the half-spectrum weights of r2c^T and c2r^T cancel), so the
                 backward is the same operator.

R is the plan's unnormalised r2c and w the half-spectrum weights (1 on the
kz = 0 and kz = N2/2 planes, 2 elsewhere).  Gradients follow PyTorch's
convention for real inputs of complex-valued functions (the same as
torch.fft.rfftn / irfftn with norm="backward" / "forward").

Every call enqueues on PyTorch's current CUDA stream (the plan is switched to
that stream in non-blocking mode).  Plans must be out-of-place r2c plans
(PlanR2C) with the tensors' shape and dtype.
"""
from __future__ import annotations

import torch

from . import PlanR2C

_COMPLEX = {torch.float32: torch.complex64, torch.float64: torch.complex128}


def _bind(plan: PlanR2C, *tensors):
    for t in tensors:
        if t is None:
            continue
        if not (t.is_cuda and (t.dtype in _COMPLEX or t.dtype in _COMPLEX.values())):
            raise ValueError("expected CUDA float32/float64 (or complex64/128) tensors")
    plan.set_stream(torch.cuda.current_stream().cuda_stream, blocking=False)


def _real(plan, like):
    return torch.empty(plan.n, dtype=like.dtype if not like.is_complex() else like.real.dtype, device=like.device)


def _spec(plan, like):
    n0, n1, n2 = plan.n
    return torch.empty((n0, n1, n2 // 2 + 1), dtype=_COMPLEX[like.dtype], device=like.device)


class RFFT3(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, plan):
        u = u.contiguous()
        _bind(plan, u)
        X = _spec(plan, u)
        plan.r2c(u, torch.view_as_real(X))
        ctx.plan = plan
        return X

    @staticmethod
    def backward(ctx, g):
        plan = ctx.plan
        g = g.contiguous()
        _bind(plan, g)
        du = _real(plan, g)
        plan.r2c_adjoint(torch.view_as_real(g), du)
        return du, None


class IRFFT3(torch.autograd.Function):
    @staticmethod
    def forward(ctx, X, plan):
        X = X.contiguous()
        _bind(plan, X)
        x = _real(plan, X)
        plan.c2r(torch.view_as_real(X), x)
        ctx.plan = plan
        return x

    @staticmethod
    def backward(ctx, g):
        plan = ctx.plan
        g = g.contiguous()
        _bind(plan, g)
        dX = _spec(plan, g)
        plan.c2r_adjoint(g, torch.view_as_real(dX))
        return dX, None


class Grad(torch.autograd.Function):
    @staticmethod
    def forward(ctx, u, plan):
        u = u.contiguous()
        _bind(plan, u)
        gx, gy, gz = (torch.empty_like(u) for _ in range(3))
        plan.grad(gx, gy, gz, u)
        ctx.plan = plan
        return gx, gy, gz

    @staticmethod
    def backward(ctx, dgx, dgy, dgz):
        plan = ctx.plan
        ref = next(t for t in (dgx, dgy, dgz) if t is not None)
        zeros = torch.zeros_like(ref)
        gs = [(t if t is not None else zeros).contiguous() for t in (dgx, dgy, dgz)]
        _bind(plan, *gs)
        out = torch.empty_like(ref)
        plan.grad_adjoint(out, *gs)
        return out, None


class Divergence(torch.autograd.Function):
    @staticmethod
    def forward(ctx, ax, ay, az, plan):
        ax, ay, az = ax.contiguous(), ay.contiguous(), az.contiguous()
        _bind(plan, ax, ay, az)
        d = torch.empty_like(ax)
        plan.divergence(d, ax, ay, az)
        ctx.plan = plan
        return d

    @staticmethod
    def backward(ctx, g):
        plan = ctx.plan
        g = g.contiguous()
        _bind(plan, g)
        outs = [torch.empty_like(g) for _ in range(3)]
        plan.divergence_adjoint(*outs, g)
        return outs[0], outs[1], outs[2], None


def _apply_op(name, plan, u):
    u = u.contiguous()
    _bind(plan, u)
    out = torch.empty_like(u)
    getattr(plan, name)(out, u)
    return out


def _self_adjoint(name):
    """autograd Function of a self-adjoint operator of the plan"""

    def forward(ctx, u, plan):
        ctx.plan = plan
        return _apply_op(name, plan, u)

    def backward(ctx, g):
        return _apply_op(name, ctx.plan, g), None

    return type(name.title().replace("_", ""), (torch.autograd.Function,),
                {"forward": staticmethod(forward), "backward": staticmethod(backward)})


Laplace = _self_adjoint("laplace")
Biharmonic = _self_adjoint("biharmonic")
InvLaplace = _self_adjoint("inv_laplace")
InvBiharmonic = _self_adjoint("inv_biharmonic")


def rfft3(u, plan):
    return RFFT3.apply(u, plan)


def irfft3(X, plan):
    return IRFFT3.apply(X, plan)


def grad(u, plan):
    return Grad.apply(u, plan)


def divergence(ax, ay, az, plan):
    return Divergence.apply(ax, ay, az, plan)


def laplace(u, plan):
    return Laplace.apply(u, plan)


def biharmonic(u, plan):
    return Biharmonic.apply(u, plan)


def inv_laplace(u, plan):
    return InvLaplace.apply(u, plan)


def inv_biharmonic(u, plan):
    return InvBiharmonic.apply(u, plan)
