"""Axis lengths without compiled kernels (the generic kernels of gen.cu)
against the oracle, through the C ABI: r2c / c2r (odd N2 included), c2c,
partial xyz, in-place plans and the 3-D spectral operators (r2c, symbol
pass, c2r), in float (rel-L2 <= 1e-5) and double (<= 1e-12), grids mixing
compiled and generic axes; and the calls such plans refuse."""
import numpy as np
import pytest

from conftest import rng
from test_gpu_transforms import TOL, empty, from_dev, to_dev

pytestmark = pytest.mark.gpu

# every grid has at least one axis outside the compiled lengths
R2C_GRIDS = [(7, 11, 13), (36, 30, 14), (64, 18, 96), (27, 64, 50), (14, 49, 62), (121, 6, 20), (2048, 3, 6),
             (5, 9, 7), (12, 8, 2048), (6, 7, 1)]
C2C_GRIDS = [(7, 11, 13), (36, 30, 14), (64, 18, 96), (4, 20, 18), (13, 1, 31)]


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("n", R2C_GRIDS)
def test_generic_r2c_c2r(cuda, native, oracle, n, dtype):
    torch = cuda
    h = (n[0], n[1], n[2] // 2 + 1)
    plan = native.PlanR2C(n, dtype)
    u = rng(40).standard_normal(n)
    dh = empty(torch, h + (2,), dtype)
    plan.r2c(to_dev(torch, u, dtype), dh)
    assert oracle.rel_l2(from_dev(dh, True), oracle.r2c(u.astype(dtype).astype(np.float64))) < TOL[dtype]
    s = rng(41).standard_normal(h) + 1j * rng(42).standard_normal(h)
    ds = to_dev(torch, s, dtype)
    keep = ds.clone()
    db = empty(torch, n, dtype)
    plan.c2r(ds, db)
    assert oracle.rel_l2(from_dev(db), oracle.c2r(from_dev(keep, True), n[2])) < TOL[dtype]
    assert torch.equal(ds, keep)
    plan.destroy()


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("n", C2C_GRIDS)
def test_generic_c2c(cuda, native, oracle, n, dtype):
    torch = cuda
    plan = native.PlanC2C(n, dtype)
    a = rng(43).standard_normal(n) + 1j * rng(44).standard_normal(n)
    da = to_dev(torch, a, dtype)
    aq = from_dev(da, True)
    out = empty(torch, n + (2,), dtype)
    for direction in (-1, 1):
        plan.c2c(direction, da, out)
        assert oracle.rel_l2(from_dev(out, True), oracle.c2c(aq, direction)) < TOL[dtype], direction
    plan.destroy()


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_generic_partial_xyz_and_in_place(cuda, native, oracle, dtype):
    """Partial transforms (the reference's xyz bitset) and an in-place plan
    (z rows padded to 2*(N2/2+1) reals) on a grid with generic y and z."""
    torch = cuda
    n = (16, 18, 14)
    h = (n[0], n[1], n[2] // 2 + 1)
    u = rng(45).standard_normal(n)
    uq = u.astype(dtype).astype(np.float64)
    plan = native.PlanR2C(n, dtype)
    for xyz in (4, 6, 5):   # z only, z+y, z+x
        dh = empty(torch, h + (2,), dtype)
        plan.r2c(to_dev(torch, u, dtype), dh, xyz=xyz)
        assert oracle.rel_l2(from_dev(dh, True), oracle.r2c(uq, xyz=xyz)) < TOL[dtype], xyz
    plan.destroy()
    buf = torch.zeros((n[0], n[1], 2 * h[2]), dtype=getattr(torch, dtype), device="cuda")
    ip = native.PlanR2C(n, dtype, data=buf, data_out=buf)
    assert ip.inplace
    buf[:, :, :n[2]] = to_dev(torch, u, dtype)
    ip.r2c(buf, buf)
    assert oracle.rel_l2(from_dev(buf.view(h + (2,)), True), oracle.r2c(uq)) < TOL[dtype]
    s = from_dev(buf.view(h + (2,)), True)
    ip.c2r(buf, buf)
    assert oracle.rel_l2(from_dev(buf)[:, :, :n[2]], oracle.c2r(s, n[2])) < TOL[dtype]
    ip.destroy()


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("n", [(7, 11, 13), (36, 30, 14), (64, 18, 96)])
def test_generic_operators(cuda, native, oracle, n, dtype):
    torch = cuda
    u = rng(46).standard_normal(n)
    du = to_dev(torch, u, dtype)
    uq = u.astype(dtype).astype(np.float64)
    plan = native.PlanR2C(n, dtype)
    out = empty(torch, n, dtype)
    for op in ("laplace", "biharmonic", "inv_laplace", "inv_biharmonic"):
        getattr(plan, op)(out, du)
        assert oracle.rel_l2(from_dev(out), oracle.spectral_op(uq, op)) < TOL[dtype], op
    plan.destroy()


def test_generic_plans_refuse_other_calls(cuda, native):
    torch = cuda
    n = (8, 18, 8)
    plan = native.PlanR2C(n, "float32")
    u = torch.zeros(n, device="cuda")
    g = [torch.empty_like(u) for _ in range(3)]
    with pytest.raises(native.AccfftError) as e:
        plan.grad(*g, u)
    assert e.value.code == native.EUNSUPPORTED
    with pytest.raises(native.AccfftError) as e:
        plan.r2c(u.cpu().pin_memory(), torch.empty((8, 18, 5, 2), device="cuda"))
    assert e.value.code == native.EUNSUPPORTED
    with pytest.raises(native.AccfftError) as e:
        native.PlanR2C(n, "float64", flags=native.F64_DF)
    assert e.value.code == native.EUNSUPPORTED
    plan.destroy()
