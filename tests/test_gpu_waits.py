"""Bounded device-side waits report instead of hanging.

The tensor-core forms wait for their matrix products and the persistent z+y
schedule's items wait for the items of their slab.  With the wait limit at 0
polls every such wait gives up at once: the kernel sets the plan's error word
and finishes without the missing data, and the call returns ACCFFT_C_ECUDA
(the reference's execute has no such failure path; this is the library's own
bound on a device-side spin).  Nothing faults: the context stays usable and
the next call with the default limit is correct.
"""
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture
def zero_wait_limit(native):
    prev = native.set_wait_limit(0)
    yield
    native.set_wait_limit(None)
    assert prev == native.set_wait_limit(None)


def half(n):
    return (n[0], n[1], n[2] // 2 + 1, 2)


def test_persistent_zy_wait_gives_up(cuda, native, zero_wait_limit):
    torch = cuda
    n = (16, 256, 256)
    u = torch.randn(n, device="cuda")
    plan = native.PlanR2C(n, "float32")
    plan.set_zy_schedule(2)
    out = torch.empty(half(n), device="cuda")
    with pytest.raises(native.AccfftError) as e:
        plan.r2c(u, out)
    assert e.value.code == native.ECUDA and "gave up" in str(e.value)
    native.set_wait_limit(None)
    ref = native.PlanR2C(n, "float32")
    ref.set_pass_order(0)                 # the reference's order, as the persistent schedule
    a = torch.empty(half(n), device="cuda")
    ref.r2c(u, a)
    plan.r2c(u, out)                      # the error word was cleared by the report
    assert torch.equal(a, out)


def test_tensor_core_wait_gives_up(cuda, native, zero_wait_limit):
    torch = cuda
    n = (128, 128, 256)
    u = torch.randn(n, device="cuda")
    plan = native.PlanR2C(n, "float32", flags=native.TC_TF32)
    out = torch.empty(half(n), device="cuda")
    with pytest.raises(native.AccfftError) as e:
        plan.r2c(u, out)
    assert e.value.code == native.ECUDA and "tensor-core" in str(e.value)
    native.set_wait_limit(None)
    ref = native.PlanR2C(n, "float32")
    a = torch.empty(half(n), device="cuda")
    ref.r2c(u, a)
    plan.r2c(u, out)
    assert ((out - a).norm() / a.norm()).item() < 1e-5


def test_nonblocking_call_reports_through_check(cuda, native, zero_wait_limit):
    """A non-blocking call cannot see its wait give up; the flag stays set
    until the plan's next blocking call or check() reports it."""
    torch = cuda
    n = (128, 128, 256)
    u = torch.randn(n, device="cuda")
    plan = native.PlanR2C(n, "float32", flags=native.TC_BF16)
    s = torch.cuda.Stream()
    plan.set_stream(s, blocking=False)
    out = torch.empty(half(n), device="cuda")
    torch.cuda.synchronize()
    plan.r2c(u, out)                      # returns at once
    with pytest.raises(native.AccfftError) as e:
        plan.check()
    assert e.value.code == native.ECUDA
    plan.check()                          # reported once, then clear
    native.set_wait_limit(None)
    plan.r2c(u, out)
    plan.check()


def test_pipelined_strided_wait_reports(cuda, native, zero_wait_limit):
    """The x pass of 1024 in variant 4 waits for its tensor-copy tile loads.
    With the limit at 0 polls every CTA gives up on its first tile, lets the
    copies it has issued land (a bounded wait of its own) and leaves; the
    call returns ACCFFT_C_ECUDA, and the next call with the default limit is
    correct."""
    torch = cuda
    n = (1024, 64, 512)
    u = torch.randn(n, device="cuda")
    ref = native.PlanR2C(n, "float32")
    a = torch.empty(half(n), device="cuda")
    plan = native.PlanR2C(n, "float32")
    plan.set_variants(0, 4, 0, 0)
    out = torch.empty(half(n), device="cuda")
    with pytest.raises(native.AccfftError) as e:
        plan.r2c(u, out)
    assert e.value.code == native.ECUDA and "tile loads" in str(e.value)
    native.set_wait_limit(None)
    ref.r2c(u, a)
    plan.r2c(u, out)                      # the error word was cleared by the report
    assert ((out - a).norm() / a.norm()).item() < 1e-6
