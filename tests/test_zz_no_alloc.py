"""The Laplacian entry point that allocates no device memory.

Callers that may not call cudaMalloc (a plugin in an application whose memory
manager has reserved the whole device, a latency-bound loop where an
allocation could stall the GPU) cannot create a plan, so
accfft_c_laplace_gpuf_noalloc works from a library-owned device array.  This
file checks, through the C ABI, that two calls in a row give the same result
as the plan-based accfft_c_laplace, and that a grid too large for the array
is refused.  It is named so that pytest collects it last."""
import ctypes
import os
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL = 1e-5   # float tolerance used by the other float parity tests


def _noalloc(native, n, out, a):
    f = native.lib().accfft_c_laplace_gpuf_noalloc
    return f((ctypes.c_int * 3)(*n), out.data_ptr(), a.data_ptr(), None)


def test_noalloc_laplace_matches_plan_laplace(cuda, native):
    torch = cuda
    n = (64, 48, 80)
    g = torch.Generator(device="cuda").manual_seed(5)
    plan = native.PlanR2C(n, "float32")
    for call in range(2):          # two calls in a row share the device array
        a = torch.randn(n, device="cuda", generator=g) * (1 + call)
        got = torch.full(n, float("nan"), device="cuda")
        rc = _noalloc(native, n, got, a)
        assert rc == 0, native.last_error()
        ref = torch.empty(n, device="cuda")
        plan.laplace(ref, a)
        err = ((got - ref).norm() / ref.norm()).item()
        assert err < TOL, (call, err)
    plan.destroy()


def test_noalloc_rejects_grids_beyond_its_array(cuda, native):
    torch = cuda
    n = (256, 256, 256)            # half spectrum of 67.6 MB > 64 MiB
    a = torch.zeros(n, device="cuda")   # full-size buffers: nothing can run out of bounds
    out = torch.zeros(n, device="cuda")
    rc = _noalloc(native, n, out, a)
    assert rc == native.EINVAL
    assert "working memory" in native.last_error()


def test_noalloc_laplace_matches_oracle(cuda, native):
    """The same two-call check against the oracle directly (the CPU
    restatement of the reference's laplace, pinned to the reference's own
    results), not only through the plan-based entry point."""
    torch = cuda
    sys.path.insert(0, os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "oracle"))
    import accfft_oracle as orc

    n = (40, 20, 48)
    r = np.random.default_rng(6)
    for call in range(2):
        a = r.standard_normal(n).astype(np.float32)
        got = torch.full(n, float("nan"), device="cuda")
        rc = _noalloc(native, n, got, torch.from_numpy(a).cuda())
        assert rc == 0, native.last_error()
        torch.cuda.synchronize()
        ref = orc.spectral_op(a.astype(np.float64), "laplace")
        assert orc.rel_l2(got.cpu().numpy().astype(np.float64), ref) < TOL, call
