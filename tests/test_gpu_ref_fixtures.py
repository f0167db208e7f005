"""The CUDA path against results produced by AccFFT's OWN code, through the
C ABI.

tests/golden/ref_cases.npz holds outputs of the reference's unmodified CPU
host code (see tests/test_ref_fixtures.py).  Every case of every grid the
CUDA path supports runs here in double (rel-L2 <= 1e-12) and float (<= 1e-5,
float inputs against the double reference): full and partial-xyz r2c / c2r
/ c2c (with z cleared the passes act in place on the input array, as in
src/accfft_gpu.cpp:486-488), in-place padded plans, single-axis transforms
(the reference CPU path's transposed layouts mapped to the GPU path's), and
every operator, on N(0,1) and Nyquist-dominated fields, even and odd axes.
"""
import numpy as np
import pytest

from test_gpu_transforms import empty, from_dev, to_dev
from test_ref_fixtures import FIX, cpu_to_gpu_axis, fixture, inputs

pytestmark = pytest.mark.gpu

TOL = {"float64": 1e-12, "float32": 1e-5}
GPU_SHAPES = [(8, 6, 10), (5, 9, 4), (6, 5, 12), (2, 4, 6), (16, 12, 10), (9, 10, 8), (4, 20, 18), (1, 6, 8)]
OPS1 = ("laplace", "biharmonic", "inv_laplace", "inv_biharmonic")


def run_case(torch, native, n, dtype, case, inp, order=0):
    """The CUDA path's result for one fixture case (numpy, GPU-path layouts);
    order 0 runs full r2c / c2r in the reference's pass order, 1 in the
    packed order."""
    h = (n[0], n[1], n[2] // 2 + 1)
    dev = lambda a: to_dev(torch, a, dtype)                       # noqa: E731
    new = lambda shape: empty(torch, shape, dtype)                # noqa: E731
    if case == "r2c_ip" or case == "c2r_ip":
        buf = torch.zeros((n[0], n[1], 2 * h[2]), dtype=getattr(torch, dtype), device="cuda")
        plan = native.PlanR2C(n, dtype, data=buf, data_out=buf)
        assert plan.inplace
        if case == "r2c_ip":
            buf[:, :, :n[2]] = dev(inp["u"])
            plan.r2c(buf, buf)
            return from_dev(buf.view(h + (2,)), True)
        buf.view(h + (2,))[:] = dev(inp["h"])
        plan.c2r(buf, buf)
        return from_dev(buf)[:, :, :n[2]]
    if case.startswith("c2c"):
        plan = native.PlanC2C(n, dtype)
        xyz = int(case.split("_")[1])
        d = dev(inp["c"])
        o = new(n + (2,))
        plan.c2c(-1 if case[3] == "f" else 1, d, o, xyz=xyz)
        return from_dev(o if xyz & 4 else d, True)
    plan = native.PlanR2C(n, dtype)
    plan.set_pass_order(order)
    if case.startswith("r2c_"):
        _, f, xyz = case.split("_")
        xyz = int(xyz)
        x = dev(inp[f])
        o = new(h + (2,))
        plan.r2c(x, o, xyz=xyz)
        return from_dev(o if xyz & 4 else x, True)
    if case.startswith("c2r_"):
        xyz = int(case.split("_")[1])
        s = dev(inp["h"])
        o = new(n)
        plan.c2r(s, o, xyz=xyz)
        return from_dev(o) if xyz & 4 else from_dev(s, True)
    if case.startswith("ax"):
        a = int(case[2])
        hs = list(n)
        hs[a] = n[a] // 2 + 1
        if case[3] == "f":
            o = new(tuple(hs) + (2,))
            plan.r2c_axis(a, dev(inp[case.split("_")[1]]), o)
            return from_dev(o, True)
        o = new(n)
        plan.c2r_axis(a, dev(cpu_to_gpu_axis(a, inp[["hx", "hy", "h"][a]])), o)
        return from_dev(o)
    if case.startswith("grad"):
        slow = case.startswith("grad_slow")
        f = case.rsplit("_", 1)[1]
        xyz = 5 if case == "grad_p5_u" else 7
        g = [torch.zeros(n, dtype=getattr(torch, dtype), device="cuda") for _ in range(3)]
        plan.grad(*g, dev(inp[f]), xyz=xyz, slow=slow)
        return np.stack([from_dev(t) for t in g])
    if case.startswith("div"):
        o = new(n)
        plan.divergence(o, *[dev(v) for v in inp["v"]], slow=case.startswith("div_slow"))
        return from_dev(o)
    op, f = case.rsplit("_", 1)
    assert op in OPS1, case
    o = new(n)
    getattr(plan, op)(o, dev(inp[f]))
    return from_dev(o)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", GPU_SHAPES)
def test_cuda_path_matches_reference(cuda, native, oracle, n, dtype):
    z = np.load(FIX)
    t = "x".join(map(str, n))
    inp = inputs(z, t)
    names = [k.split("__")[2] for k in z.files if k.startswith(f"out__{t}__")]
    assert len(names) >= 50
    bad = []
    for case in names:
        got = run_case(cuda, native, n, dtype, case, inp)
        e = oracle.rel_l2(got, fixture(z, t, case))
        if not e <= TOL[dtype]:
            bad.append((case, e))
    assert not bad, bad


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", GPU_SHAPES)
def test_packed_order_matches_reference(cuda, native, oracle, n, dtype):
    """Full r2c / c2r in the packed pass order against the reference's own results."""
    z = np.load(FIX)
    t = "x".join(map(str, n))
    inp = inputs(z, t)
    for case in ("r2c_u_7", "r2c_nyq_7", "c2r_7"):
        got = run_case(cuda, native, n, dtype, case, inp, order=1)
        assert oracle.rel_l2(got, fixture(z, t, case)) <= TOL[dtype], case


# grids the reference's CPU path runs with an odd N2: every axis of the
# CUDA path then goes through the generic kernels (z as the full real line)
ODD_N2_SHAPES = [(7, 5, 9), (3, 11, 7)]
GENERIC_CASES = ("r2c_", "c2r_", "c2c", "laplace_", "biharmonic_", "inv_laplace_", "inv_biharmonic_")


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", ODD_N2_SHAPES)
def test_odd_n2_grids_match_reference(cuda, native, oracle, n, dtype):
    """The reference's own results on its odd-N2 grids: the transforms and
    the 3-D operators (the calls plans with generic-length axes take)."""
    z = np.load(FIX)
    t = "x".join(map(str, n))
    inp = inputs(z, t)
    names = [k.split("__")[2] for k in z.files if k.startswith(f"out__{t}__")]
    names = [c for c in names if c.startswith(GENERIC_CASES)]
    assert len(names) >= 12
    bad = []
    for case in names:
        got = run_case(cuda, native, n, dtype, case, inp)
        e = oracle.rel_l2(got, fixture(z, t, case))
        if not e <= TOL[dtype]:
            bad.append((case, e))
    assert not bad, bad
