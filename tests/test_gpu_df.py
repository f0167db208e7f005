"""Double plans computing in double-float (ACCFFT_C_F64_DF): parity with the
FP64 oracle through the C ABI.

Tolerance: rel-L2 1e-13 against the oracle in double (a 48-bit significand
through the passes; measured about 1e-14), inside the 1e-12 bar of the
double drop-in."""
import numpy as np
import pytest

from conftest import rng
from test_gpu_transforms import empty, from_dev, to_dev

pytestmark = pytest.mark.gpu

TOL = 1e-13
SHAPES = [(4, 6, 8), (8, 8, 8), (16, 12, 10), (5, 9, 4), (48, 96, 64), (64, 32, 128), (90, 100, 180),
          (128, 128, 128), (160, 180, 200), (256, 256, 256), (200, 192, 96), (2, 1024, 512)]
C2C_SHAPES = [(4, 6, 8), (9, 5, 6), (16, 12, 10), (48, 96, 64), (160, 180, 200), (256, 128, 64)]


@pytest.mark.parametrize("n", SHAPES)
def test_df_r2c_c2r(cuda, native, oracle, n):
    torch = cuda
    u = rng(30).standard_normal(n)
    plan = native.PlanR2C(n, "float64", flags=native.F64_DF)
    du = to_dev(torch, u, "float64")
    dh = empty(torch, (n[0], n[1], n[2] // 2 + 1, 2), "float64")
    plan.r2c(du, dh)
    ref = oracle.r2c(u)
    assert oracle.rel_l2(from_dev(dh, True), ref) < TOL
    h = rng(31).standard_normal(ref.shape) + 1j * rng(32).standard_normal(ref.shape)
    dh2 = to_dev(torch, h, "float64")
    keep = dh2.clone()
    db = empty(torch, n, "float64")
    plan.c2r(dh2, db)
    assert oracle.rel_l2(from_dev(db), oracle.c2r(h, n[2])) < TOL
    assert torch.equal(dh2, keep)
    plan.destroy()


@pytest.mark.parametrize("n", C2C_SHAPES)
def test_df_c2c(cuda, native, oracle, n):
    torch = cuda
    a = rng(33).standard_normal(n) + 1j * rng(34).standard_normal(n)
    plan = native.PlanC2C(n, "float64", flags=native.F64_DF)
    da = to_dev(torch, a, "float64")
    out = empty(torch, n + (2,), "float64")
    plan.c2c(-1, da, out)
    assert oracle.rel_l2(from_dev(out, True), oracle.c2c(a, -1)) < TOL
    back = empty(torch, n + (2,), "float64")
    plan.c2c(1, out, back)
    assert oracle.rel_l2(from_dev(back, True) / np.prod(n), a) < TOL
    plan.destroy()


@pytest.mark.parametrize("xyz", [1, 2, 3, 4, 5, 6])
def test_df_partial_axes(cuda, native, oracle, xyz):
    """xyz bitsets on a double-float plan, against the oracle (with z skipped
    the remaining passes transform the input array in place, as the
    reference does)."""
    torch = cuda
    n = (16, 12, 20)
    h = (n[0], n[1], n[2] // 2 + 1)
    plan = native.PlanR2C(n, "float64", flags=native.F64_DF)
    if xyz & 4:
        u = rng(40).standard_normal(n)
        dh = empty(torch, h + (2,), "float64")
        plan.r2c(to_dev(torch, u, "float64"), dh, xyz=xyz)
        got, ref = from_dev(dh, True), oracle.r2c(u, xyz)
    else:
        c = rng(41).standard_normal(h) + 1j * rng(42).standard_normal(h)
        dc = to_dev(torch, c, "float64")
        plan.r2c(dc, empty(torch, h + (2,), "float64"), xyz=xyz)
        got, ref = from_dev(dc, True), oracle.r2c(c, xyz)
    assert oracle.rel_l2(got, ref) < TOL
    plan.destroy()


def test_df_plans_reject_derivatives_and_float(cuda, native):
    """Double-float plans run the transforms and the 3-D spectral operators;
    the derivative operators (grad, divergence, single-axis transforms) stay
    with plain double plans."""
    torch = cuda
    n = (16, 16, 16)
    p = native.PlanR2C(n, "float64", flags=native.F64_DF)
    u = torch.zeros(n, dtype=torch.float64, device="cuda")
    with pytest.raises(native.AccfftError) as e:
        p.grad(torch.empty_like(u), torch.empty_like(u), torch.empty_like(u), u)
    assert e.value.code == native.EUNSUPPORTED
    p.destroy()
    with pytest.raises(native.AccfftError) as e:
        native.PlanR2C(n, "float32", flags=native.F64_DF)
    assert e.value.code == native.EUNSUPPORTED


def test_df_512_round_trip(cuda, native):
    """512^3 in double-float against the plain double plan (the oracle's
    accuracy at this size is pinned by the double plan's own tests)."""
    torch = cuda
    n = (512, 512, 512)
    g = torch.Generator(device="cuda").manual_seed(36)
    u = torch.randn(n, dtype=torch.float64, device="cuda", generator=g)
    h = (n[0], n[1], n[2] // 2 + 1, 2)
    pd = native.PlanR2C(n, "float64")
    spec = torch.empty(h, dtype=torch.float64, device="cuda")
    pd.r2c(u, spec)
    pf = native.PlanR2C(n, "float64", flags=native.F64_DF)
    s2 = torch.empty(h, dtype=torch.float64, device="cuda")
    pf.r2c(u, s2)
    assert ((s2 - spec).norm() / spec.norm()).item() < TOL
    del spec
    back = torch.empty_like(u)
    pf.c2r(s2, back)
    assert ((back / u.numel() - u).norm() / u.norm()).item() < TOL
    pd.destroy()
    pf.destroy()


@pytest.mark.parametrize("scale_exp", [-900, -400, -60, 60, 400, 900])
def test_df_scale_invariance(cuda, native, scale_exp):
    """Each transform scales by the exact power of two that puts its input's
    largest magnitude in [1, 2): data far outside float's exponent range
    transforms to the same bits times the same power of two."""
    torch = cuda
    n = (32, 24, 40)
    u = torch.from_numpy(rng(37).standard_normal(n)).cuda()
    f = 2.0 ** scale_exp
    plan = native.PlanR2C(n, "float64", flags=native.F64_DF)
    h = (n[0], n[1], n[2] // 2 + 1, 2)
    a, b = torch.empty(h, dtype=torch.float64, device="cuda"), torch.empty(h, dtype=torch.float64, device="cuda")
    plan.r2c(u, a)
    plan.r2c(u * f, b)
    assert torch.equal(b, a * f)
    ra, rb = torch.empty_like(u), torch.empty_like(u)
    plan.c2r(a, ra)
    plan.c2r(b, rb)
    assert torch.equal(rb, ra * f)
    c = torch.from_numpy(rng(38).standard_normal(n + (2,))).cuda()
    pc = native.PlanC2C(n, "float64", flags=native.F64_DF)
    ca, cb = torch.empty_like(c), torch.empty_like(c)
    pc.c2c(-1, c, ca)
    pc.c2c(-1, c * f, cb)
    assert torch.equal(cb, ca * f)
    plan.destroy()
    pc.destroy()


def test_df_wide_dynamic_range(cuda, native, oracle):
    """Entries spanning 2^-300 .. 2^300 in one field: normwise accuracy is
    set by the largest ones, as in IEEE double."""
    torch = cuda
    n = (16, 20, 24)
    r = rng(39)
    u = r.standard_normal(n) * np.exp2(r.integers(-300, 300, size=n))
    plan = native.PlanR2C(n, "float64", flags=native.F64_DF)
    dh = empty(torch, (n[0], n[1], n[2] // 2 + 1, 2), "float64")
    plan.r2c(to_dev(torch, u, "float64"), dh)
    assert oracle.rel_l2(from_dev(dh, True), oracle.r2c(u)) < TOL
    z = torch.zeros(n, dtype=torch.float64, device="cuda")
    plan.r2c(z, dh)
    assert not dh.any()
    plan.destroy()


def test_df_plans_reject_host_arrays(cuda, native):
    torch = cuda
    n = (8, 8, 8)
    plan = native.PlanR2C(n, "float64", flags=native.F64_DF)
    hu = torch.zeros(n, dtype=torch.float64).pin_memory()
    with pytest.raises(native.AccfftError) as e:
        plan.r2c(hu, torch.empty((8, 8, 5, 2), dtype=torch.float64, device="cuda"))
    assert e.value.code == native.EUNSUPPORTED
    plan.destroy()


OPS_DF = ("laplace", "biharmonic", "inv_laplace", "inv_biharmonic")


@pytest.mark.parametrize("n", [(8, 8, 8), (5, 9, 4), (16, 12, 10), (48, 96, 64), (90, 100, 180), (128, 128, 128)])
def test_df_operators_vs_oracle(cuda, native, oracle, n):
    """The 3-D operators of double-float plans (the plan's r2c, the symbol in
    double, the plan's c2r) against the oracle, and the spectral Poisson
    solve, heat and Helmholtz against the plain double plan (itself pinned to
    the oracle); odd and even axes."""
    torch = cuda
    u = rng(33).standard_normal(n)
    du = to_dev(torch, u, "float64")
    df = native.PlanR2C(n, "float64", flags=native.F64_DF)
    dp = native.PlanR2C(n, "float64")
    out = empty(torch, n, "float64")
    for op in OPS_DF:
        getattr(df, op)(out, du)
        assert oracle.rel_l2(from_dev(out), oracle.spectral_op(u, op)) < 1e-12, op
    ref = empty(torch, n, "float64")
    for name, call in (("poisson", lambda p, o: p.poisson(o, du, method=1)),
                       ("heat", lambda p, o: p.heat(o, du, 0.01)),
                       ("helmholtz", lambda p, o: p.helmholtz(o, du, 2.5))):
        call(df, out)
        call(dp, ref)
        assert ((out - ref).norm() / ref.norm()).item() < 1e-12, name
    with pytest.raises(native.AccfftError) as e:
        df.poisson(out, du, method=0)   # the finite-difference eigenvalues stay with plain double plans
    assert e.value.code == native.EUNSUPPORTED
    df.destroy()
    dp.destroy()
