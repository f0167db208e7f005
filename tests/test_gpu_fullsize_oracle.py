"""The workload sizes against the oracle, on the GPU machine.

The oracle runs on every host thread (a 512^3 double r2c + c2r takes about a
second on 16 cores), so the sizes the benchmarks use are checked directly:
  - 512^3 r2c and c2r, float and double, N(0,1) field / N(0,1) half spectrum;
  - 256^3 and 512^3 c2c, both directions, float and double;
  - 512^3 float laplace, biharmonic, grad and divergence, and double
    divergence and biharmonic, on N(0,1) fields;
  - 1024^3 float r2c of the turbulence-spectrum field (amplitudes
    N(0,1) |k|^(-5/3) for 0 < |k| <= 256, uniform phases), for the CUDA-core
    form, both tensor-core forms and the double drop-in, each against the same
    oracle spectrum.
Bounds: rel-L2 <= 1e-12 (double) and <= 1e-5 (float, float inputs against
the double oracle); the tensor-core forms' bound is stated in test_gpu_tc.py.
Inputs are generated on the GPU with seeded torch generators (plumbing, not
the product path) and copied to the host for the oracle.
"""
import numpy as np
import pytest

from test_gpu_tc import TOL as TC_TOL

pytestmark = pytest.mark.gpu

TOL = {"float64": 1e-12, "float32": 1e-5}


def rel_l2_chunked(a_dev, ref, cplx):
    """rel-L2 of a device array against a host reference, slab by slab along
    axis 0 (bounded host temporaries at 1024^3)."""
    num = den = 0.0
    for i0 in range(0, ref.shape[0], 64):
        a = a_dev[i0:i0 + 64].cpu().numpy().astype(np.float64)
        if cplx:
            a = a[..., 0] + 1j * a[..., 1]
        r = ref[i0:i0 + 64]
        num += float(np.sum(np.abs(a - r) ** 2))
        den += float(np.sum(np.abs(r) ** 2))
    return (num / den) ** 0.5


def host(t):
    return t.cpu().numpy().astype(np.float64)


def host_c(t):
    a = t.cpu().numpy().astype(np.float64)
    return a[..., 0] + 1j * a[..., 1]


def randn(torch, shape, dtype, seed):
    g = torch.Generator(device="cuda").manual_seed(seed)
    return torch.randn(shape, generator=g, device="cuda", dtype=getattr(torch, dtype))


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_512_r2c_c2r_vs_oracle(cuda, native, oracle, dtype):
    torch = cuda
    n = (512, 512, 512)
    h = (n[0], n[1], n[2] // 2 + 1)
    plan = native.PlanR2C(n, dtype)
    u = randn(torch, n, dtype, 101)
    X = torch.empty(h + (2,), dtype=u.dtype, device="cuda")
    plan.r2c(u, X)
    ref = oracle.r2c(host(u))
    assert rel_l2_chunked(X, ref, True) < TOL[dtype]
    del ref
    S = randn(torch, h + (2,), dtype, 102)
    back = torch.empty_like(u)
    plan.c2r(S, back)
    refb = oracle.c2r(host_c(S), n[2])
    assert rel_l2_chunked(back, refb, False) < TOL[dtype]


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("m", [256, 512])
def test_c2c_vs_oracle(cuda, native, oracle, dtype, m):
    torch = cuda
    n = (m, m, m)
    plan = native.PlanC2C(n, dtype)
    a = randn(torch, n + (2,), dtype, 103)
    aq = host_c(a)
    out = torch.empty_like(a)
    for direction in (-1, 1):
        plan.c2c(direction, a, out)
        assert rel_l2_chunked(out, oracle.c2c(aq, direction), True) < TOL[dtype], direction


@pytest.mark.parametrize("dtype,ops", [("float32", ("laplace", "biharmonic", "grad", "divergence")),
                                       ("float64", ("biharmonic", "divergence"))])
def test_512_operators_vs_oracle(cuda, native, oracle, dtype, ops):
    torch = cuda
    n = (512, 512, 512)
    plan = native.PlanR2C(n, dtype)
    u = randn(torch, n, dtype, 104)
    uq = host(u)
    out = torch.empty_like(u)
    for op in ops:
        if op in ("laplace", "biharmonic"):
            getattr(plan, op)(out, u)
            assert rel_l2_chunked(out, oracle.spectral_op(uq, op), False) < TOL[dtype], op
        elif op == "grad":
            g = [torch.empty_like(u) for _ in range(3)]
            plan.grad(*g, u)
            for j, r in enumerate(oracle.grad(uq)):
                assert rel_l2_chunked(g[j], r, False) < TOL[dtype], ("grad", j)
            del g
        else:
            v = [randn(torch, n, dtype, 105 + j) for j in range(3)]
            plan.divergence(out, *v)
            assert rel_l2_chunked(out, oracle.divergence(*[host(t) for t in v]), False) < TOL[dtype], op


def turbulence_field(torch, n, seed, kmax=256):
    """Real field whose spectrum has amplitudes N(0,1) |k|^(-5/3) for
    0 < |k| <= kmax and uniform phases (Hermitian completion by the inverse
    real transform)."""
    g = torch.Generator(device="cuda").manual_seed(seed)
    h2 = n[2] // 2 + 1
    kx = torch.fft.fftfreq(n[0], d=1.0 / n[0], device="cuda")[:, None, None]
    ky = torch.fft.fftfreq(n[1], d=1.0 / n[1], device="cuda")[None, :, None]
    kz = torch.arange(h2, device="cuda", dtype=torch.float32)[None, None, :]
    k = torch.sqrt(kx * kx + ky * ky + kz * kz)
    amp = torch.randn((n[0], n[1], h2), generator=g, device="cuda") * torch.where(
        (k > 0) & (k <= kmax), k.clamp(min=1.0) ** (-5.0 / 3.0), torch.zeros_like(k))
    del k
    phase = torch.rand((n[0], n[1], h2), generator=g, device="cuda") * (2 * np.pi)
    spec = torch.polar(amp, phase)
    del amp, phase
    u = torch.fft.irfftn(spec, s=n, norm="forward")
    return u.contiguous()


def test_1024_turbulence_all_forms_vs_oracle(cuda, native, oracle):
    torch = cuda
    n = (1024, 1024, 1024)
    h = (n[0], n[1], n[2] // 2 + 1)
    u = turbulence_field(torch, n, 106)
    ref = oracle.r2c(host(u))
    X = torch.empty(h + (2,), device="cuda")
    errs = {}
    for name, flags in (("float32", 0), ("tf32", native.TC_TF32), ("bf16", native.TC_BF16)):
        plan = native.PlanR2C(n, "float32", flags=flags)
        plan.r2c(u, X)
        errs[name] = rel_l2_chunked(X, ref, True)
        if name == "float32":
            back = torch.empty_like(u)
            plan.c2r(X, back)
            rt = ((back.double() / (n[0] * n[1] * n[2]) - u.double()).norm() / u.double().norm()).item()
            assert rt < TOL["float32"]
            del back
        plan.destroy()
    del X
    ud = u.double()
    del u
    Xd = torch.empty(h + (2,), dtype=torch.float64, device="cuda")
    plan = native.PlanR2C(n, "float64")
    plan.r2c(ud, Xd)
    errs["float64"] = rel_l2_chunked(Xd, ref, True)
    print("1024^3 turbulence r2c rel-L2 vs oracle:", errs)
    assert errs["float32"] < TOL["float32"]
    assert errs["float64"] < TOL["float64"]
    assert errs["tf32"] < TC_TOL["tf32"] and errs["bf16"] < TC_TOL["bf16"]
