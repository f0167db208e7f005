"""Tensor-core forms of the float r2c / c2r path (ACCFFT_C_TC_TF32 and
ACCFFT_C_TC_BF16): radix-16 stages as 32x32 real matrix products with FP32
accumulation, A operands in tensor memory, against the FP64 oracle and
against the CUDA-core form."""
import numpy as np
import pytest

from conftest import rng
from test_gpu_transforms import empty, from_dev, to_dev

pytestmark = pytest.mark.gpu

# rel-L2 bounds vs the FP64 oracle, both 1e-6 (the FP32 form's target): the
# three-way BF16 split (six products) is exact for float data and drops only
# products below 2^-16 relative; 3xTF32 keeps about 22 bits per operand and
# drops the lo*lo product (measured 4.5e-7 at 512^3, 4.4e-7 at 1024^3)
TOL = {"tf32": 1e-6, "bf16": 1e-6}


def flag(native, form):
    return native.TC_TF32 if form == "tf32" else native.TC_BF16


@pytest.mark.parametrize("form", ["tf32", "bf16"])
@pytest.mark.parametrize("n", [(128, 128, 256), (256, 128, 512), (128, 512, 1024), (1024, 128, 256)])
def test_tc_r2c_c2r_vs_oracle(cuda, native, oracle, n, form):
    torch = cuda
    u = rng(70).standard_normal(n)
    plan = native.PlanR2C(n, "float32", flags=flag(native, form))
    du = to_dev(torch, u, "float32")
    spec = empty(torch, (n[0], n[1], n[2] // 2 + 1, 2), "float32")
    plan.r2c(du, spec)
    s = from_dev(spec, True)
    ref = oracle.r2c(u.astype(np.float32).astype(np.float64))
    assert oracle.rel_l2(s, ref) < TOL[form]
    back = empty(torch, n, "float32")
    keep = spec.clone()
    plan.c2r(spec, back)
    assert torch.equal(spec, keep)                   # out-of-place c2r keeps its input
    assert oracle.rel_l2(from_dev(back) / np.prod(n), u.astype(np.float32)) < 2 * TOL[form]


def test_tc_matches_cuda_core_form(cuda, native):
    torch = cuda
    n = (256, 256, 256)
    u = torch.randn(n, device="cuda")
    a = native.PlanR2C(n, "float32")
    b = native.PlanR2C(n, "float32", flags=native.TC_TF32)
    sa = torch.empty((256, 256, 129, 2), device="cuda")
    sb = torch.empty_like(sa)
    a.r2c(u, sa)
    b.r2c(u, sb)
    assert ((sa - sb).norm() / sa.norm()).item() < 2e-6


def test_tc_plan_limits(cuda, native):
    torch = cuda
    with pytest.raises(native.AccfftError):
        native.PlanR2C((96, 128, 256), "float32", flags=native.TC_TF32)    # 96 has no tensor-core kernel
    with pytest.raises(native.AccfftError):
        native.PlanR2C((128, 128, 256), "float64", flags=native.TC_TF32)   # float plans only
    plan = native.PlanR2C((128, 128, 256), "float32", flags=native.TC_TF32)
    u = torch.randn((128, 128, 256), device="cuda")
    out = torch.empty_like(u)
    with pytest.raises(native.AccfftError) as e:
        plan.laplace(out, u)
    assert e.value.code == native.EUNSUPPORTED
    spec = torch.empty((128, 128, 129, 2), device="cuda")
    with pytest.raises(native.AccfftError):
        plan.r2c(u, spec, xyz=4)
