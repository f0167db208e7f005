"""Radix / tile variants of the float r2c / c2r passes and the plan-time
tuner (ACCFFT_MEASURE): every variant against the oracle in both pass orders,
and the tuner's choice cached per grid."""
import numpy as np
import pytest

from conftest import rng
from test_gpu_transforms import empty, from_dev, to_dev

pytestmark = pytest.mark.gpu

TOL = 1e-5


@pytest.mark.parametrize("order", [0, 1])
@pytest.mark.parametrize("n", [(64, 128, 256), (256, 64, 128), (128, 512, 128), (1024, 64, 512), (64, 1024, 256)])
def test_every_variant_matches_oracle(cuda, native, oracle, n, order):
    torch = cuda
    h = (n[0], n[1], n[2] // 2 + 1)
    u = rng(120).standard_normal(n)
    ref = oracle.r2c(u.astype(np.float32).astype(np.float64))
    plan = native.PlanR2C(n, "float32")
    plan.set_pass_order(order)
    du = to_dev(torch, u, "float32")
    spec = empty(torch, h + (2,), "float32")
    back = empty(torch, n, "float32")
    tried = 0
    for w in range(4):
        for v in (1, 2, 3, 4):
            vs = [0, 0, 0, 0]
            vs[w] = v
            try:
                plan.set_variants(*vs)
            except native.AccfftError:
                continue                      # the length has no such variant
            tried += 1
            plan.r2c(du, spec)
            assert oracle.rel_l2(from_dev(spec, True), ref) < TOL, (w, v)
            plan.c2r(spec, back)
            rt = ((back.double() / np.prod(n) - du.double()).norm() / du.double().norm()).item()
            assert rt < TOL, (w, v)
    assert tried >= 3


def test_measure_tunes_and_caches(cuda, native, oracle):
    torch = cuda
    n = (128, 256, 256)
    p1 = native.PlanR2C(n, "float32", flags=native.ACCFFT_MEASURE)
    t1 = p1.tuning()
    assert t1["tuned"]
    for k in ("y", "x", "z_r2c", "z_c2r"):
        assert t1[k]["radix"] > 0 and t1[k]["tile"] > 0 and t1[k]["variant"] in (0, 1, 2, 3, 4)
    p2 = native.PlanR2C(n, "float32", flags=native.ACCFFT_MEASURE)
    assert p2.tuning() == t1                 # one choice per grid in a process
    est = native.PlanR2C(n, "float32")       # ACCFFT_ESTIMATE: the defaults
    te = est.tuning()
    assert not te["tuned"] and all(te[k]["variant"] == 0 for k in ("y", "x", "z_r2c", "z_c2r"))
    u = rng(121).standard_normal(n)
    du = to_dev(torch, u, "float32")
    spec = empty(torch, (n[0], n[1], n[2] // 2 + 1, 2), "float32")
    p1.r2c(du, spec)
    assert oracle.rel_l2(from_dev(spec, True), oracle.r2c(u.astype(np.float32).astype(np.float64))) < TOL
    with pytest.raises(native.AccfftError):
        native.PlanR2C((16, 16, 16), "float64").set_variants(1, 0, 0, 0)
