"""Backward passes (adjoint kernels behind torch.autograd.Function) against
finite differences (torch.autograd.gradcheck in double), against PyTorch's
own torch.fft gradients, and on the 256^3 float32 differentiation workload
against FP64 central differences along random directions."""
import numpy as np
import pytest

from conftest import rng

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ag(cuda):
    import accfft_gb300.autograd as m

    return m


def test_gradcheck_transforms_and_operators(cuda, native, ag):
    torch = cuda
    n = (6, 4, 8)
    plan = native.PlanR2C(n, "float64")
    u = torch.randn(n, dtype=torch.float64, device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(lambda x: ag.rfft3(x, plan), (u,))
    X = torch.randn((6, 4, 5), dtype=torch.complex128, device="cuda", requires_grad=True)
    assert torch.autograd.gradcheck(lambda y: ag.irfft3(y, plan), (X,))
    assert torch.autograd.gradcheck(lambda x: ag.grad(x, plan), (u,))
    a = [torch.randn(n, dtype=torch.float64, device="cuda", requires_grad=True) for _ in range(3)]
    assert torch.autograd.gradcheck(lambda x, y, z: ag.divergence(x, y, z, plan), tuple(a))
    for f in (ag.laplace, ag.biharmonic, ag.inv_laplace, ag.inv_biharmonic):
        assert torch.autograd.gradcheck(lambda x: f(x, plan), (u,))


def torch_fft_loss(torch, u, f):
    """The differentiation workload with torch.fft (float64): spectral gradient
    and inverse Laplacian with the reference's wave numbers (Nyquist -> 0)."""
    n0, n1, n2 = u.shape

    def fold(m, n):
        k = torch.arange(m, device=u.device, dtype=torch.float64)
        w = torch.where(k > n // 2, k - n, k)
        return torch.where(k == n // 2, torch.zeros_like(w), w)

    wx = fold(n0, n0)[:, None, None]
    wy = fold(n1, n1)[None, :, None]
    wz = fold(n2 // 2 + 1, n2)[None, None, :]
    U = torch.fft.rfftn(u)
    g = [torch.fft.irfftn(1j * w * U, s=u.shape) for w in (wx, wy, wz)]
    k2 = wx * wx + wy * wy + wz * wz
    inv = torch.where(k2 > 0, -1.0 / torch.where(k2 > 0, k2, torch.ones_like(k2)), torch.zeros_like(k2))
    il = torch.fft.irfftn(inv * U, s=u.shape)
    return 0.5 * sum((t * t).sum() for t in g) + (f * il).sum()


def ours_loss(ag, plan, u, f):
    gx, gy, gz = ag.grad(u, plan)
    return 0.5 * ((gx * gx).sum() + (gy * gy).sum() + (gz * gz).sum()) + (f * ag.inv_laplace(u, plan)).sum()


@pytest.mark.parametrize("n", [(32, 24, 40), (64, 64, 64)])
def test_loss_gradient_matches_torch_fft(cuda, native, ag, n):
    torch = cuda
    plan = native.PlanR2C(n, "float64")
    u = torch.randn(n, dtype=torch.float64, device="cuda")
    f = torch.randn(n, dtype=torch.float64, device="cuda")
    u1 = u.clone().requires_grad_(True)
    L1 = ours_loss(ag, plan, u1, f)
    (g1,) = torch.autograd.grad(L1, u1)
    u2 = u.clone().requires_grad_(True)
    L2 = torch_fft_loss(torch, u2, f)
    (g2,) = torch.autograd.grad(L2, u2)
    assert abs(L1.item() - L2.item()) <= 1e-12 * abs(L2.item())
    assert ((g1 - g2).norm() / g2.norm()).item() < 1e-12


def smooth_field(n, sigma, seed):
    """N(0,1) field smoothed by a Gaussian of width sigma cells (spectral filter)."""
    r = np.random.default_rng(seed)
    u = r.standard_normal(n)
    U = np.fft.rfftn(u)
    k = [np.fft.fftfreq(m) for m in n[:2]] + [np.fft.rfftfreq(n[2])]
    kk = k[0][:, None, None] ** 2 + k[1][None, :, None] ** 2 + k[2][None, None, :] ** 2
    return np.fft.irfftn(U * np.exp(-2 * np.pi ** 2 * sigma ** 2 * kk), s=n, axes=(0, 1, 2))


def test_differentiation_workload_256_fd64(cuda, native, ag):
    """256^3, L(u) = 0.5 |grad u|^2 + <f, inv_laplace u>, u Gaussian-smoothed
    (4 cells), f ~ N(0,1).  Against FP64 central differences (eps = 1e-6)
    along 16 random N(0,1) directions v:
      - the FP64 backward agrees to <= 1e-6 relative;
      - the float32 backward agrees to float32 accuracy: <g, v> cancels by
        about sqrt(N) = 4096 for a random v, so its relative error is bounded
        by ~eps32 * sqrt(N) (about 2.4e-4), not by 1e-6.
    The float32 gradient field is also compared with the torch.fft float64
    gradient (relative L2)."""
    torch = cuda
    n = (256, 256, 256)
    u64 = torch.tensor(smooth_field(n, 4.0, 11), device="cuda")
    f64 = torch.tensor(np.random.default_rng(12).standard_normal(n), device="cuda")
    p32 = native.PlanR2C(n, "float32")
    p64 = native.PlanR2C(n, "float64")
    u32 = u64.float().requires_grad_(True)
    (g32,) = torch.autograd.grad(ours_loss(ag, p32, u32, f64.float()), u32)
    ud = u64.clone().requires_grad_(True)
    (g64,) = torch.autograd.grad(ours_loss(ag, p64, ud, f64), ud)
    gen = torch.Generator(device="cuda").manual_seed(13)
    eps = 1e-6
    worst64 = worst32 = 0.0
    with torch.no_grad():
        for _ in range(16):
            v = torch.randn(n, dtype=torch.float64, device="cuda", generator=gen)
            lp = ours_loss(ag, p64, u64 + eps * v, f64).item()
            lm = ours_loss(ag, p64, u64 - eps * v, f64).item()
            fd = (lp - lm) / (2 * eps)
            worst64 = max(worst64, abs((g64 * v).sum().item() - fd) / abs(fd))
            worst32 = max(worst32, abs((g32.double() * v).sum().item() - fd) / abs(fd))
    print(f"FD64 vs backward: fp64 worst {worst64:.2e}, fp32 worst {worst32:.2e}")
    assert worst64 < 1e-6, worst64
    assert worst32 < 2.4e-4, worst32
    ut = u64.clone().requires_grad_(True)
    (gt,) = torch.autograd.grad(torch_fft_loss(torch, ut, f64), ut)
    rel32 = ((g32.double() - gt).norm() / gt.norm()).item()
    rel64 = ((g64 - gt).norm() / gt.norm()).item()
    print(f"vs torch.fft fp64 gradient: fp32 {rel32:.2e}, fp64 {rel64:.2e}")
    assert rel32 < 1e-5 and rel64 < 1e-12


def test_fp32_backward_fd_along_smooth_directions(cuda, native, ag):
    """The 1e-6 bound for the spectral-gradient backward, in float32:
    256^3, the same loss as above, against FP64 central differences along 16
    smooth directions (N(0,1) fields smoothed by a Gaussian of 4 cells, like
    u itself).  Along such directions <g, v> does not cancel, so the float32
    backward is held to <= 1e-6 relative."""
    torch = cuda
    n = (256, 256, 256)
    u64 = torch.tensor(smooth_field(n, 4.0, 11), device="cuda")
    f64 = torch.tensor(np.random.default_rng(12).standard_normal(n), device="cuda")
    p32 = native.PlanR2C(n, "float32")
    p64 = native.PlanR2C(n, "float64")
    u32 = u64.float().requires_grad_(True)
    (g32,) = torch.autograd.grad(ours_loss(ag, p32, u32, f64.float()), u32)
    eps = 1e-6
    worst = 0.0
    with torch.no_grad():
        for k in range(16):
            v = torch.tensor(smooth_field(n, 4.0, 100 + k), device="cuda")
            lp = ours_loss(ag, p64, u64 + eps * v, f64).item()
            lm = ours_loss(ag, p64, u64 - eps * v, f64).item()
            fd = (lp - lm) / (2 * eps)
            worst = max(worst, abs((g32.double() * v).sum().item() - fd) / abs(fd))
    print(f"FD64 vs float32 backward along smooth directions: worst {worst:.2e}")
    assert worst < 1e-6, worst
