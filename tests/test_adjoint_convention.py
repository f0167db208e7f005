"""The adjoint formulas implemented by accfft_c_r2c_adjoint / c2r_adjoint,
restated with the oracle, against PyTorch's own autograd of torch.fft (CPU):
  VJP of rfftn  with cotangent g (half spectrum) = c2r(g / w)
  VJP of irfftn (unnormalised) with cotangent r  = w * r2c(r)
w = 1 on the kz = 0 and kz = N2/2 planes, 2 elsewhere."""
import numpy as np
import pytest
import torch

from conftest import rng


def weights(n):
    h = n[2] // 2 + 1
    w = np.full(h, 2.0)
    w[0] = 1.0
    if n[2] % 2 == 0:
        w[-1] = 1.0
    return w[None, None, :]


@pytest.mark.parametrize("n", [(4, 6, 8), (5, 7, 6), (8, 8, 10)])
def test_rfftn_vjp_is_weighted_c2r(oracle, n):
    r = rng(7)
    u = torch.tensor(r.standard_normal(n), requires_grad=True)
    h = (n[0], n[1], n[2] // 2 + 1)
    g = r.standard_normal(h) + 1j * r.standard_normal(h)
    X = torch.fft.rfftn(u)
    (du,) = torch.autograd.grad(X, u, grad_outputs=torch.tensor(g))
    ours = oracle.c2r(g / weights(n), n[2])
    assert oracle.rel_l2(ours, du.numpy()) < 1e-13


@pytest.mark.parametrize("n", [(4, 6, 8), (5, 7, 6), (8, 8, 10)])
def test_irfftn_vjp_is_weighted_r2c(oracle, n):
    r = rng(8)
    h = (n[0], n[1], n[2] // 2 + 1)
    X = torch.tensor(r.standard_normal(h) + 1j * r.standard_normal(h), requires_grad=True)
    x = torch.fft.irfftn(X, s=n, norm="forward")
    g = r.standard_normal(n)
    (dX,) = torch.autograd.grad(x, X, grad_outputs=torch.tensor(g))
    ours = weights(n) * oracle.r2c(g)
    assert oracle.rel_l2(ours, dX.numpy()) < 1e-13
