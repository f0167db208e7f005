"""Properties that hold at any size, checked at the workload sizes (512^3 in
float and double, 1024^3 in float) where the oracle would take minutes:
linearity of r2c, Parseval's identity over the half spectrum, the round trip,
and the exact spectrum of u = sin x + sin y cos 2z (configuration 1's field
without its noise term: four stored modes)."""
import math

import pytest

pytestmark = pytest.mark.gpu

TOL = {"float64": 1e-12, "float32": 1e-5}


def half_energy(torch, X, n):
    """sum |u|^2 from the half spectrum: (1/N) (planes kz = 0 and N2/2 once,
    the others twice)"""
    N = n[0] * n[1] * n[2]
    a = (X.double() ** 2).sum(dim=-1)         # |X|^2 per entry, shape (N0, N1, N2/2+1)
    w = torch.full((n[2] // 2 + 1,), 2.0, dtype=torch.float64, device=X.device)
    w[0] = 1.0
    w[-1] = 1.0
    return (a * w).sum().item() / N


@pytest.mark.parametrize("dtype,n", [("float32", (512, 512, 512)), ("float64", (512, 512, 512)),
                                     ("float32", (1024, 1024, 1024))])
def test_full_size_properties(cuda, native, dtype, n):
    torch = cuda
    tdt = getattr(torch, dtype)
    g = torch.Generator(device="cuda").manual_seed(17)
    u = torch.randn(n, generator=g, device="cuda", dtype=tdt)
    plan = native.PlanR2C(n, dtype)
    X = torch.empty((n[0], n[1], n[2] // 2 + 1, 2), dtype=tdt, device="cuda")
    plan.r2c(u, X)
    # Parseval
    e_u = (u.double() ** 2).sum().item()
    assert abs(half_energy(torch, X, n) - e_u) / e_u < TOL[dtype]
    # round trip
    back = torch.empty_like(u)
    plan.c2r(X, back)
    N = n[0] * n[1] * n[2]
    assert ((back.double() / N - u.double()).norm() / u.double().norm()).item() < TOL[dtype]
    del back
    if n[0] > 512:
        return
    # linearity: r2c(2u - 3v) = 2 r2c(u) - 3 r2c(v)
    v = torch.randn(n, generator=g, device="cuda", dtype=tdt)
    Y = torch.empty_like(X)
    Z = torch.empty_like(X)
    plan.r2c(v, Y)
    w = 2 * u - 3 * v
    plan.r2c(w, Z)
    ref = 2 * X.double() - 3 * Y.double()
    assert ((Z.double() - ref).norm() / ref.norm()).item() < TOL[dtype]


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_full_size_analytic_modes(cuda, native, dtype):
    torch = cuda
    n = (512, 512, 512)
    tdt = getattr(torch, dtype)
    ax = [torch.arange(m, device="cuda", dtype=torch.float64) * (2 * math.pi / m) for m in n]
    x, y, z = ax[0][:, None, None], ax[1][None, :, None], ax[2][None, None, :]
    u = (torch.sin(x) + torch.sin(y) * torch.cos(2 * z)).to(tdt)
    plan = native.PlanR2C(n, dtype)
    X = torch.empty((n[0], n[1], n[2] // 2 + 1, 2), dtype=tdt, device="cuda")
    plan.r2c(u, X)
    N = n[0] * n[1] * n[2]
    Xc = torch.complex(X[..., 0].double(), X[..., 1].double())
    expect = {(1, 0, 0): -0.5j * N, (n[0] - 1, 0, 0): 0.5j * N, (0, 1, 2): -0.25j * N, (0, n[1] - 1, 2): 0.25j * N}
    scale = N / 2
    for (i, j, k), val in expect.items():
        assert abs(Xc[i, j, k].item() - val) < TOL[dtype] * scale * 10
        Xc[i, j, k] = 0
    # everything else is rounding noise
    assert Xc.abs().max().item() < TOL[dtype] * scale * 10


def test_full_size_c2c(cuda, native):
    torch = cuda
    n = (512, 512, 512)
    g = torch.Generator(device="cuda").manual_seed(19)
    a = torch.randn((*n, 2), generator=g, device="cuda")
    plan = native.PlanC2C(n, "float32")
    A = torch.empty_like(a)
    plan.c2c(-1, a, A)
    N = n[0] * n[1] * n[2]
    e_a = (a.double() ** 2).sum().item()
    assert abs((A.double() ** 2).sum().item() / N - e_a) / e_a < TOL["float32"]
    back = torch.empty_like(a)
    plan.c2c(1, A, back)
    assert ((back.double() / N - a.double()).norm() / a.double().norm()).item() < TOL["float32"]


def test_full_size_operators_fp64(cuda, native):
    """512^3 double: laplace, inv_laplace and grad of
    u = sin x cos 2y sin 3z + 0.5 cos 5x against their exact values."""
    torch = cuda
    n = (512, 512, 512)
    ax = [torch.arange(m, device="cuda", dtype=torch.float64) * (2 * math.pi / m) for m in n]
    x, y, z = ax[0][:, None, None], ax[1][None, :, None], ax[2][None, None, :]
    s = torch.sin(x) * torch.cos(2 * y) * torch.sin(3 * z)
    c5 = torch.cos(5 * x) + 0 * y * z
    u = s + 0.5 * c5
    plan = native.PlanR2C(n, "float64")
    out = torch.empty_like(u)
    plan.laplace(out, u)
    ref = -14 * s - 12.5 * c5
    assert ((out - ref).norm() / ref.norm()).item() < 1e-10
    plan.inv_laplace(out, u)
    ref = -s / 14 - 0.02 * c5
    assert ((out - ref).norm() / ref.norm()).item() < 1e-12
    gx, gy, gz = (torch.empty_like(u) for _ in range(3))
    plan.grad(gx, gy, gz, u)
    refs = (torch.cos(x) * torch.cos(2 * y) * torch.sin(3 * z) - 2.5 * torch.sin(5 * x) + 0 * y * z,
            -2 * torch.sin(x) * torch.sin(2 * y) * torch.sin(3 * z),
            3 * torch.sin(x) * torch.cos(2 * y) * torch.cos(3 * z))
    for got, r in zip((gx, gy, gz), refs):
        assert ((got - r).norm() / r.norm()).item() < 1e-11
