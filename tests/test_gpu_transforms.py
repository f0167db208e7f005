"""Parity of the CUDA transforms with the oracle, through the C ABI.

Tolerances (relative L2 against the oracle computed in double from the same
inputs): 1e-12 for double plans, 1e-5 for float plans (the float result is
also stated against the double oracle)."""
import numpy as np
import pytest

from conftest import rng

pytestmark = pytest.mark.gpu

TOL = {"float64": 1e-12, "float32": 1e-5}

R2C_SHAPES = [(4, 6, 8), (8, 8, 8), (16, 12, 10), (5, 9, 4), (32, 64, 16), (48, 96, 64), (64, 32, 128),
              (128, 128, 128), (90, 100, 180), (160, 180, 200), (256, 256, 256), (200, 192, 96)]
C2C_SHAPES = [(4, 6, 8), (8, 8, 8), (9, 5, 6), (16, 12, 10), (48, 96, 64), (128, 128, 128), (160, 180, 200),
              (256, 128, 64)]


def to_dev(torch, a, dtype):
    if np.iscomplexobj(a):
        a = np.ascontiguousarray(np.stack([a.real, a.imag], axis=-1))
    return torch.from_numpy(np.ascontiguousarray(a).astype(dtype)).cuda()


def from_dev(t, cplx=False):
    a = t.cpu().numpy().astype(np.float64)
    if cplx:
        a = a[..., 0] + 1j * a[..., 1]
    return a


def empty(torch, shape, dtype):
    return torch.empty(shape, dtype=getattr(torch, dtype), device="cuda")


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", R2C_SHAPES)
def test_r2c_c2r(cuda, native, oracle, n, dtype):
    torch = cuda
    u = rng(10).standard_normal(n)
    plan = native.PlanR2C(n, dtype)
    du = to_dev(torch, u, dtype)
    dh = empty(torch, (n[0], n[1], n[2] // 2 + 1, 2), dtype)
    plan.r2c(du, dh)
    ref = oracle.r2c(u.astype(dtype).astype(np.float64))
    assert oracle.rel_l2(from_dev(dh, True), ref) < TOL[dtype]
    # c2r of an arbitrary (non-Hermitian-consistent) half spectrum
    h = rng(11).standard_normal(ref.shape) + 1j * rng(12).standard_normal(ref.shape)
    dh2 = to_dev(torch, h, dtype)
    keep = dh2.clone()
    db = empty(torch, n, dtype)
    plan.c2r(dh2, db)
    refb = oracle.c2r(from_dev(keep, True), n[2])
    assert oracle.rel_l2(from_dev(db), refb) < TOL[dtype]
    assert torch.equal(dh2, keep), "out-of-place c2r must leave its input unchanged"
    plan.destroy()


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", C2C_SHAPES)
def test_c2c(cuda, native, oracle, n, dtype):
    torch = cuda
    r = rng(20)
    d = r.standard_normal(n) + 1j * r.standard_normal(n)
    plan = native.PlanC2C(n, dtype)
    dd = to_dev(torch, d, dtype)
    keep = dd.clone()
    do = empty(torch, n + (2,), dtype)
    dq = from_dev(keep, True)
    for direction in (-1, 1):
        plan.c2c(direction, dd, do)
        assert oracle.rel_l2(from_dev(do, True), oracle.c2c(dq, direction)) < TOL[dtype]
        assert torch.equal(dd, keep)
    plan.destroy()


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_r2c_inplace_padded(cuda, native, oracle, dtype):
    """In-place plan (data == data_out): rows padded to 2*(N2/2+1) as in
    steps/step2/step2_gpu.cpp:40-72; round trip returns N*u."""
    torch = cuda
    n = (32, 24, 40)
    u = rng(30).standard_normal(n)
    pad = oracle.pad_rows(u)
    d = to_dev(torch, pad, dtype)
    plan = native.PlanR2C(n, dtype, data=d, data_out=d)
    assert plan.inplace
    plan.r2c(d, d)
    s = from_dev(d.view(n[0], n[1], n[2] // 2 + 1, 2), True)
    assert oracle.rel_l2(s, oracle.r2c(u.astype(dtype).astype(np.float64))) < TOL[dtype]
    plan.c2r(d, d)
    back = from_dev(d)[:, :, :n[2]] / np.prod(n)
    assert oracle.rel_l2(back, u) < TOL[dtype]


PACKED_SHAPES = [(1, 6, 8), (2, 4, 6), (5, 9, 4), (9, 10, 8), (16, 12, 10), (32, 64, 16), (48, 96, 64),
                 (128, 128, 128), (90, 100, 180), (160, 180, 200), (256, 256, 256), (512, 512, 512)]


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", PACKED_SHAPES)
def test_packed_pass_order(cuda, native, oracle, n, dtype):
    """The packed order (y and x passes over the real field viewed as complex
    [N0][N1][N2/2], then mirror-paired z lines) against the oracle and the
    reference's order: odd and even N0 / N1, N0 = 1 and 2 (every line its own
    mirror or paired within its slab), non-Hermitian c2r input."""
    torch = cuda
    h = (n[0], n[1], n[2] // 2 + 1)
    u = rng(13).standard_normal(n)
    plan = native.PlanR2C(n, dtype)
    plan.set_pass_order(1)
    ref_plan = native.PlanR2C(n, dtype)
    ref_plan.set_pass_order(0)
    du = to_dev(torch, u, dtype)
    keep = du.clone()
    dh = empty(torch, h + (2,), dtype)
    plan.r2c(du, dh)
    assert torch.equal(du, keep)
    uq = u.astype(dtype).astype(np.float64)
    if np.prod(n) <= 2 ** 22:
        assert oracle.rel_l2(from_dev(dh, True), oracle.r2c(uq)) < TOL[dtype]
    dn = empty(torch, h + (2,), dtype)
    ref_plan.r2c(du, dn)
    assert ((dh.double() - dn.double()).norm() / dn.double().norm()).item() < TOL[dtype]
    s = rng(14).standard_normal(h) + 1j * rng(15).standard_normal(h)
    ds = to_dev(torch, s, dtype)
    keep = ds.clone()
    db = empty(torch, n, dtype)
    plan.c2r(ds, db)
    assert torch.equal(ds, keep)
    if np.prod(n) <= 2 ** 22:
        assert oracle.rel_l2(from_dev(db), oracle.c2r(from_dev(keep, True), n[2])) < TOL[dtype]
    dbn = empty(torch, n, dtype)
    ref_plan.c2r(ds, dbn)
    assert ((db.double() - dbn.double()).norm() / dbn.double().norm()).item() < TOL[dtype]
    before = native.kernel_launches()
    plan.r2c(du, dh)
    plan.c2r(dh, db)
    assert native.kernel_launches() - before == 6
    assert ((db.double() / np.prod(n) - du.double()).norm() / du.double().norm()).item() < TOL[dtype]


def test_packed_pass_order_eligibility(cuda, native):
    torch = cuda
    n = (16, 16, 16)
    buf = torch.zeros((16, 16, 18), device="cuda")
    inplace = native.PlanR2C(n, "float32", data=buf, data_out=buf)
    with pytest.raises(native.AccfftError):
        inplace.set_pass_order(1)
    with pytest.raises(native.AccfftError):
        native.PlanC2C(n, "float32").set_pass_order(1)
    tc = native.PlanR2C((128, 128, 256), "float32", flags=native.TC_TF32)
    with pytest.raises(native.AccfftError):
        tc.set_pass_order(1)


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("xyz", [1, 2, 3, 4, 5, 6])
def test_partial_axes(cuda, native, oracle, dtype, xyz):
    """xyz bitsets: the selected passes only (with z skipped the remaining
    passes transform the input array in place, as the reference does)."""
    torch = cuda
    n = (16, 12, 20)
    h = (n[0], n[1], n[2] // 2 + 1)
    plan = native.PlanR2C(n, dtype)
    if xyz & 4:
        u = rng(40).standard_normal(n)
        du = to_dev(torch, u, dtype)
        dh = empty(torch, h + (2,), dtype)
        plan.r2c(du, dh, xyz=xyz)
        got = from_dev(dh, True)
        ref = oracle.r2c(u.astype(dtype).astype(np.float64), xyz)
    else:
        c = rng(41).standard_normal(h) + 1j * rng(42).standard_normal(h)
        dc = to_dev(torch, c, dtype)
        q = from_dev(dc, True)
        plan.r2c(dc, empty(torch, h + (2,), dtype), xyz=xyz)
        got = from_dev(dc, True)
        ref = oracle.r2c(q, xyz)
    assert oracle.rel_l2(got, ref) < TOL[dtype]


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_timer_slot4_accumulates(cuda, native, dtype):
    torch = cuda
    n = (64, 64, 64)
    plan = native.PlanR2C(n, dtype)
    du = torch.randn(n, dtype=getattr(torch, dtype), device="cuda")
    dh = empty(torch, (64, 64, 33, 2), dtype)
    timer = [0.0] * 5
    plan.r2c(du, dh, timer=timer)
    plan.r2c(du, dh, timer=timer)
    assert timer[4] > 0 and timer[:4] == [0.0] * 4


def test_kernel_launch_counter(cuda, native):
    torch = cuda
    n = (32, 32, 32)
    plan = native.PlanR2C(n, "float32")
    du = torch.randn(n, device="cuda")
    dh = torch.empty((32, 32, 17, 2), device="cuda")
    before = native.kernel_launches()
    plan.r2c(du, dh)
    assert native.kernel_launches() - before == 3      # z, y and x passes
    # a 3-D operator: z r2c, y, fused x (forward, symbol, inverse), y, z c2r;
    # at N2/2 = 16 through the aligned split layout, whose Nyquist plane
    # rides along in the y and x launches
    out = torch.empty_like(du)
    before = native.kernel_launches()
    plan.laplace(out, du)
    assert native.kernel_launches() - before == 5
    plan2 = native.PlanR2C((32, 32, 40), "float32")      # N2/2 = 20: natural layout
    du2 = torch.randn((32, 32, 40), device="cuda")
    before = native.kernel_launches()
    plan2.laplace(torch.empty_like(du2), du2)
    assert native.kernel_launches() - before == 5


AXIS_SHAPES = [(8, 6, 4), (16, 12, 10), (5, 9, 4), (48, 96, 64), (128, 128, 128), (160, 180, 200), (9, 5, 6)]


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", AXIS_SHAPES)
@pytest.mark.parametrize("axis", [0, 1, 2])
def test_single_axis_r2c_c2r(cuda, native, oracle, n, dtype, axis):
    """accfft_execute_{r2c,c2r}_{x,y,z}_gpu_t layouts: x -> [N0/2+1][N1][N2],
    y -> [N0][N1/2+1][N2], z -> [N0][N1][N2/2+1] (src/accfft_gpu.cpp:1212-1604)."""
    torch = cuda
    u = rng(60 + axis).standard_normal(n)
    plan = native.PlanR2C(n, dtype)
    du = to_dev(torch, u, dtype)
    hshape = list(n)
    hshape[axis] = n[axis] // 2 + 1
    dh = empty(torch, tuple(hshape) + (2,), dtype)
    plan.r2c_axis(axis, du, dh)
    ref = oracle.r2c_axis(u.astype(dtype).astype(np.float64), axis)
    assert oracle.rel_l2(from_dev(dh, True), ref) < TOL[dtype]
    # c2r of an arbitrary half spectrum (imaginary DC / Nyquist parts ignored)
    h = rng(70).standard_normal(ref.shape) + 1j * rng(71).standard_normal(ref.shape)
    dh2 = to_dev(torch, h, dtype)
    keep = dh2.clone()
    db = empty(torch, n, dtype)
    plan.c2r_axis(axis, dh2, db)
    refb = oracle.c2r_axis(from_dev(keep, True), axis, n)
    assert oracle.rel_l2(from_dev(db), refb) < TOL[dtype]
    assert torch.equal(dh2, keep)


@pytest.mark.parametrize("n", [(512, 512, 512), (64, 256, 256), (32, 128, 128)])
def test_fused_slab_pass_float(cuda, native, oracle, n, monkeypatch):
    """Grids with a cluster slab kernel (z and y passes fused, selected with
    ACCFFT_GB300_ZY=fused): the full transform against the oracle, and against
    the same plan run pass by pass (xyz = z, then y, then x), which uses the
    separate z and y kernels."""
    torch = cuda
    u = rng(80).standard_normal(n)
    monkeypatch.setenv("ACCFFT_GB300_ZY", "fused")
    plan = native.PlanR2C(n, "float32")
    du = to_dev(torch, u, "float32")
    h = (n[0], n[1], n[2] // 2 + 1, 2)
    fused, split = empty(torch, h, "float32"), empty(torch, h, "float32")
    before = native.kernel_launches()
    plan.r2c(du, fused)
    fused_launches = native.kernel_launches() - before
    plan.r2c(du, split, xyz=4)
    plan.r2c(split, split, xyz=2)
    plan.r2c(split, split, xyz=1)
    assert fused_launches == 2, "expected the z+y slab kernel and the x pass"
    ref = oracle.r2c(u.astype(np.float32).astype(np.float64))
    assert oracle.rel_l2(from_dev(fused, True), ref) < 1e-5
    assert oracle.rel_l2(from_dev(fused, True), from_dev(split, True)) < 1e-6
    back, back2 = empty(torch, n, "float32"), empty(torch, n, "float32")
    keep = fused.clone()
    plan.c2r(fused, back)
    assert torch.equal(fused, keep)
    plan.c2r(split, split, xyz=1)
    plan.c2r(split, split, xyz=2)
    plan.c2r(split, back2, xyz=4)
    assert oracle.rel_l2(from_dev(back) / np.prod(n), u) < 1e-5
    assert oracle.rel_l2(from_dev(back), from_dev(back2)) < 1e-6
    plan.destroy()


@pytest.mark.parametrize("dtype", ["float32", "float64"])
@pytest.mark.parametrize("n", [(64, 48, 80), (128, 128, 128)])
def test_pinned_host_real_arrays(cuda, native, oracle, n, dtype):
    """r2c reading its real input from pinned host memory and c2r writing its
    real output to pinned host memory (slab batches staged through the
    plan's device ring by the copy engines) give the device-path results."""
    torch = cuda
    u = rng(90).standard_normal(n)
    plan = native.PlanR2C(n, dtype)
    hu = torch.from_numpy(u.astype(dtype)).pin_memory()
    du = hu.cuda()
    s_host, s_dev = empty(torch, (n[0], n[1], n[2] // 2 + 1, 2), dtype), empty(torch, (n[0], n[1], n[2] // 2 + 1, 2), dtype)
    plan.r2c(hu, s_host)
    plan.r2c(du, s_dev)
    assert torch.equal(s_host, s_dev)
    hb = torch.empty(n, dtype=getattr(torch, dtype)).pin_memory()
    db = empty(torch, n, dtype)
    plan.c2r(s_dev, hb)
    plan.c2r(s_dev, db)
    assert torch.equal(hb, db.cpu())
    assert oracle.rel_l2(hb.numpy().astype(np.float64) / np.prod(n), u) < TOL[dtype] * 10


def test_pinned_host_pipelines_in_flight(cuda, native):
    """Two plans on two non-blocking streams with pinned host arrays, several
    pairs in flight: every result equals the device path's; the copies show
    up in the profile as 4 slab batches each way (the default count)."""
    torch = cuda
    n = (48, 40, 64)
    hu = [torch.randn(n).pin_memory() for _ in range(4)]
    hb = [torch.empty(n).pin_memory() for _ in range(4)]
    streams = [torch.cuda.Stream() for _ in range(2)]
    plans = [native.PlanR2C(n, "float32") for _ in range(2)]
    specs = [torch.empty((48, 40, 33, 2), device="cuda") for _ in range(2)]
    for p, s in zip(plans, streams):
        p.set_stream(s.cuda_stream, blocking=False)
    plans[0].set_profiling(True)
    for k in range(4):
        p, spec = plans[k % 2], specs[k % 2]
        p.r2c(hu[k], spec)
        p.c2r(spec, hb[k])
    torch.cuda.synchronize()
    prof = plans[0].profile()
    assert prof["h2d"][0] == 2 * 4 and prof["d2h"][0] == 2 * 4
    ref = native.PlanR2C(n, "float32")
    for k in range(4):
        du = hu[k].cuda()
        spec = torch.empty((48, 40, 33, 2), device="cuda")
        back = torch.empty(n, device="cuda")
        ref.r2c(du, spec)
        ref.c2r(spec, back)
        assert torch.equal(hb[k], back.cpu())


def test_unregistered_host_memory_is_refused(cuda, native):
    torch = cuda
    n = (16, 16, 16)
    plan = native.PlanR2C(n, "float32")
    host = np.zeros(n, np.float32)          # ordinary pageable memory
    spec = empty(torch, (16, 16, 9, 2), "float32")
    with pytest.raises(native.AccfftError) as e:
        plan.r2c(host.ctypes.data, spec)
    assert e.value.code == native.EINVAL and "pinned host memory" in str(e.value)


def test_kernel_profiling_labels(cuda, native):
    """accfft_c_set_profiling / accfft_c_profile_read: per-pass event times of
    a full r2c + c2r and of a 3-D operator."""
    torch = cuda
    n = (64, 64, 64)
    plan = native.PlanR2C(n, "float32")
    u = torch.randn(n, device="cuda")
    spec = torch.empty((64, 64, 33, 2), device="cuda")
    back = torch.empty(n, device="cuda")
    plan.set_profiling(True)
    for _ in range(3):
        plan.r2c(u, spec)
        plan.c2r(spec, back)
    prof = plan.profile()
    assert set(prof) == {"z_r2c", "y", "x", "x_inv", "y_inv", "z_c2r"}
    assert all(cnt == 3 and ms > 0 for cnt, ms in prof.values())
    assert plan.profile() == {}
    assert torch.allclose(back / 64 ** 3, u, atol=1e-5)
    plan.laplace(back, u)
    prof = plan.profile()
    assert set(prof) == {"z_r2c", "y", "x_sym", "y_inv", "z_c2r"}
    plan.set_profiling(False)
    assert plan.profile() == {}


@pytest.mark.parametrize("dtype", ["float64", "float32"])
@pytest.mark.parametrize("n", [(1, 1, 2), (2, 1, 2), (1, 3, 4), (3, 1, 6), (1, 1, 16), (16, 1, 1 * 2)])
def test_degenerate_sizes(cuda, native, oracle, n, dtype):
    """Axes of length one and N2 = 2 (a single z pair) through r2c, c2r and
    laplace."""
    torch = cuda
    u = rng(95).standard_normal(n)
    plan = native.PlanR2C(n, dtype)
    du = to_dev(torch, u, dtype)
    spec = empty(torch, (n[0], n[1], n[2] // 2 + 1, 2), dtype)
    plan.r2c(du, spec)
    assert oracle.rel_l2(from_dev(spec, True), oracle.r2c(u.astype(dtype).astype(np.float64))) < TOL[dtype]
    back = empty(torch, n, dtype)
    plan.c2r(spec, back)
    assert oracle.rel_l2(from_dev(back) / np.prod(n), u.astype(dtype)) < TOL[dtype]
    lap = empty(torch, n, dtype)
    plan.laplace(lap, du)
    ref = oracle.spectral_op(u.astype(dtype).astype(np.float64), "laplace")
    assert np.abs(from_dev(lap) - ref).max() <= TOL[dtype] * max(1.0, np.abs(ref).max())


@pytest.mark.parametrize("n", [(256, 256, 256), (128, 512, 512), (4, 512, 512), (512, 512, 512)])
def test_persistent_zy_schedule(cuda, native, monkeypatch, n):
    """ACCFFT_GB300_ZY=persistent: z and y passes in one persistent kernel with
    per-slab dependency counters; results equal the separate passes' bit for bit."""
    torch = cuda
    u = torch.randn(n, device="cuda")
    ref = native.PlanR2C(n, "float32")
    ref.set_pass_order(0)                  # the reference's order, as the persistent schedule
    monkeypatch.setenv("ACCFFT_GB300_ZY", "persistent")
    plan = native.PlanR2C(n, "float32")
    h = (n[0], n[1], n[2] // 2 + 1, 2)
    a, b = torch.empty(h, device="cuda"), torch.empty(h, device="cuda")
    ref.r2c(u, a)
    before = native.kernel_launches()
    plan.r2c(u, b)
    assert native.kernel_launches() - before == 2           # z+y, then x
    assert torch.equal(a, b)
    ra, rb = torch.empty_like(u), torch.empty_like(u)
    ref.c2r(a, ra)
    plan.c2r(b, rb)
    assert torch.equal(ra, rb)
    assert torch.allclose(rb / u.numel(), u, atol=1e-5)


def test_pdl_on_off_bit_identical(cuda, native):
    """Programmatic dependent launch changes only when a pass's CTAs are
    scheduled, never what they compute: transforms and fused operators give
    the same bits with it off and in both release modes, and so does a
    CUDA-graph capture of a round trip made with it on (the graph keeps the
    programmatic edges)."""
    torch = cuda
    n = (64, 96, 128)
    h_shape = (n[0], n[1], n[2] // 2 + 1, 2)
    u = torch.randn(n, device="cuda")
    prev = native.set_pdl(None)
    out = {}
    try:
        for mode in (0, 1, 2):
            native.set_pdl(mode)
            plan = native.PlanR2C(n, "float32")
            h = torch.empty(h_shape, device="cuda")
            b, lap = torch.empty_like(u), torch.empty_like(u)
            gx, gy, gz = (torch.empty_like(u) for _ in range(3))
            div = torch.empty_like(u)
            plan.r2c(u, h)
            plan.c2r(h.clone(), b)
            plan.laplace(lap, u)
            plan.grad(gx, gy, gz, u)
            plan.divergence(div, gx, gy, gz)
            torch.cuda.synchronize()
            out[mode] = [h, b, lap, gx, gy, gz, div]
            plan.destroy()
        for mode in (1, 2):
            for x, y in zip(out[0], out[mode]):
                assert torch.equal(x, y)

        native.set_pdl(2)
        plan = native.PlanR2C(n, "float32")
        s = torch.cuda.Stream()
        plan.set_stream(s)
        h, b = torch.empty(h_shape, device="cuda"), torch.empty_like(u)
        torch.cuda.synchronize()
        with torch.cuda.stream(s):
            plan.r2c(u, h)
            plan.c2r(h, b)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, stream=s, capture_error_mode="relaxed"):
            plan.r2c(u, h)
            plan.c2r(h, b)
        b.zero_()
        h.zero_()
        torch.cuda.synchronize()
        for _ in range(3):
            g.replay()
        torch.cuda.synchronize()
        assert torch.equal(h, out[0][0])
        assert torch.equal(b, out[0][1])
        plan.destroy()
    finally:
        native.set_pdl(prev)


def test_host_staging_keeps_persistent_control_words(cuda, native, monkeypatch):
    """The staging ring for host arrays is allocated on a plan's first host
    call without releasing the plan's other device words: a persistent-
    schedule plan still matches the separate passes after a host call."""
    torch = cuda
    n = (64, 256, 256)
    h = (n[0], n[1], n[2] // 2 + 1, 2)
    ref = native.PlanR2C(n, "float32")
    ref.set_pass_order(0)
    monkeypatch.setenv("ACCFFT_GB300_ZY", "persistent")
    plan = native.PlanR2C(n, "float32")
    u = torch.randn(n, device="cuda")
    a, b, c = (torch.empty(h, device="cuda") for _ in range(3))
    ref.r2c(u, a)
    plan.r2c(u.cpu().pin_memory(), b)        # host input: staged through the ring
    torch.cuda.synchronize()
    plan.r2c(u, c)                           # device input: persistent z+y kernel
    torch.cuda.synchronize()
    assert torch.allclose(b, a, rtol=0, atol=1e-3 * a.abs().max().item())
    assert torch.equal(c, a)
    plan.destroy()
    ref.destroy()
