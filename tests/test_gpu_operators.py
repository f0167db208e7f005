"""Parity of the CUDA spectral operators with the oracle (the reference's
operator semantics), through the C ABI."""
import numpy as np
import pytest

from conftest import rng
from test_gpu_transforms import empty, from_dev, to_dev
from test_oracle import step5_biharmonic, step5_field, step5_grad, step5_laplace, rel_l1

pytestmark = pytest.mark.gpu

TOL = {"float64": 1e-12, "float32": 1e-5}
SHAPES = [(8, 8, 8), (16, 12, 10), (5, 9, 4), (48, 96, 64), (128, 128, 128), (160, 180, 200)]


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", SHAPES)
@pytest.mark.parametrize("op", ["laplace", "biharmonic", "inv_laplace", "inv_biharmonic"])
def test_spectral_ops(cuda, native, oracle, n, dtype, op):
    torch = cuda
    u = rng(50).standard_normal(n)
    plan = native.PlanR2C(n, dtype)
    du = to_dev(torch, u, dtype)
    keep = du.clone()
    do = empty(torch, n, dtype)
    getattr(plan, op)(do, du)
    ref = oracle.spectral_op(u.astype(dtype).astype(np.float64), op)
    assert oracle.rel_l2(from_dev(do), ref) < TOL[dtype]
    assert torch.equal(du, keep)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", SHAPES)
def test_grad_divergence(cuda, native, oracle, n, dtype):
    torch = cuda
    u = rng(51).standard_normal(n)
    uq = u.astype(dtype).astype(np.float64)
    plan = native.PlanR2C(n, dtype)
    du = to_dev(torch, u, dtype)
    g = [empty(torch, n, dtype) for _ in range(3)]
    plan.grad(*g, du)
    ref = oracle.grad(uq)
    for j in range(3):
        assert oracle.rel_l2(from_dev(g[j]), ref[j]) < TOL[dtype], j
    gs = [empty(torch, n, dtype) for _ in range(3)]
    plan.grad(*gs, du, slow=True)
    refs = oracle.grad_slow(uq)
    for j in range(3):
        assert oracle.rel_l2(from_dev(gs[j]), refs[j]) < TOL[dtype], j
    a = [rng(52 + j).standard_normal(n) for j in range(3)]
    da = [to_dev(torch, x, dtype) for x in a]
    div = empty(torch, n, dtype)
    plan.divergence(div, *da)
    aq = [x.astype(dtype).astype(np.float64) for x in a]
    refd = oracle.divergence(*aq)
    assert oracle.rel_l2(from_dev(div), refd) < TOL[dtype]
    # the slow form keeps the reference's partial-axis transforms, which on odd
    # axes give a different result from the fast form
    plan.divergence(div, *da, slow=True)
    assert oracle.rel_l2(from_dev(div), oracle.divergence_slow(*aq)) < TOL[dtype]


@pytest.mark.parametrize("xyz", [1, 2, 4, 5])
def test_grad_component_selection(cuda, native, oracle, xyz):
    torch = cuda
    n = (16, 24, 32)
    u = rng(53).standard_normal(n)
    plan = native.PlanR2C(n, "float64")
    du = to_dev(torch, u, "float64")
    outs = [empty(torch, n, "float64") if xyz & (1 << j) else None for j in range(3)]
    plan.grad(*outs, du, xyz=xyz)
    ref = oracle.grad(u)
    for j in range(3):
        if outs[j] is not None:
            assert oracle.rel_l2(from_dev(outs[j]), ref[j]) < 1e-12


def test_step5_closed_forms_on_gpu(cuda, native):
    """steps/step5/step5_gpu.cpp:559-699 on the GPU in double: every operator
    against its closed form, relative L1 below 1e-10 (biharmonic 1e-8: the
    reference's 1e-10 is out of reach for any double-precision FFT at this
    size -- numpy.fft gives 2.8e-10 -- because |k|^4 amplifies the rounding
    noise of the forward transform)."""
    torch = cuda
    n = (128, 128, 128)
    u, _ = step5_field(n)
    plan = native.PlanR2C(n, "float64")
    du = to_dev(torch, u, "float64")
    g = [empty(torch, n, "float64") for _ in range(3)]
    plan.grad(*g, du)
    for j, ref in enumerate(step5_grad(n)):
        assert rel_l1(from_dev(g[j]), ref) < 1e-10
    lap = empty(torch, n, "float64")
    plan.laplace(lap, du)
    assert rel_l1(from_dev(lap), step5_laplace(n)) < 1e-10
    bih = empty(torch, n, "float64")
    plan.biharmonic(bih, du)
    assert rel_l1(from_dev(bih), step5_biharmonic(n)) < 1e-8
    div = empty(torch, n, "float64")
    plan.divergence(div, *g)
    assert rel_l1(from_dev(div), step5_laplace(n)) < 1e-10


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", [(16, 12, 10), (48, 96, 64), (128, 128, 128)])
def test_heat_and_helmholtz(cuda, native, oracle, n, dtype):
    torch = cuda
    u = rng(55).standard_normal(n)
    uq = u.astype(dtype).astype(np.float64)
    plan = native.PlanR2C(n, dtype)
    du = to_dev(torch, u, dtype)
    out = empty(torch, n, dtype)
    for t in (0.0, 1e-3, 0.1):
        plan.heat(out, du, t)
        assert oracle.rel_l2(from_dev(out), oracle.spectral_op(uq, "heat", param=t)) < TOL[dtype]
    for alpha in (0.0, 1.0, 7.5):
        plan.helmholtz(out, du, alpha)
        assert oracle.rel_l2(from_dev(out), oracle.spectral_op(uq, "helmholtz", param=alpha)) < TOL[dtype]


def test_heat_exact_solution_and_poisson(cuda, native, oracle):
    """sin x sin y sin z decays as exp(-3t) under the heat propagator
    (steps/step6/step6.cpp:31-97 checks the same kind of exact solution), and
    solves (alpha - laplace) v = (alpha + 3) sin x sin y sin z."""
    torch = cuda
    n = (64, 64, 64)
    X, Y, Z = np.meshgrid(*[2 * np.pi * np.arange(k) / k for k in n], indexing="ij")
    s = np.sin(X) * np.sin(Y) * np.sin(Z)
    plan = native.PlanR2C(n, "float64")
    ds = to_dev(torch, s, "float64")
    out = empty(torch, n, "float64")
    plan.heat(out, ds, 0.25)
    assert np.abs(from_dev(out) - np.exp(-0.75) * s).max() < 1e-13
    plan.helmholtz(out, to_dev(torch, (2.0 + 3.0) * s, "float64"), 2.0)
    assert np.abs(from_dev(out) - s).max() < 1e-13
    plan.helmholtz(out, to_dev(torch, -3.0 * s, "float64"), 0.0)   # Poisson: -laplace v = -3 s -> v = -s
    assert np.abs(from_dev(out) + s).max() < 1e-13


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", [(16, 12, 10), (48, 96, 64), (128, 128, 128), (160, 180, 200)])
@pytest.mark.parametrize("method", [0, 1])
def test_poisson_step4(cuda, native, oracle, n, dtype, method):
    torch = cuda
    u = rng(57).standard_normal(n)
    plan = native.PlanR2C(n, dtype)
    du = to_dev(torch, u, dtype)
    out = empty(torch, n, dtype)
    plan.poisson(out, du, method)
    ref = oracle.spectral_op(u.astype(dtype).astype(np.float64), "poisson_fd" if method == 0 else "poisson_spec")
    assert oracle.rel_l2(from_dev(out), ref) < TOL[dtype]
