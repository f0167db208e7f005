"""Batched uneven-size transforms as one CUDA-graph launch: every instance
against the FP64 oracle."""
import numpy as np
import pytest

from conftest import rng

pytestmark = pytest.mark.gpu


def oracle_result(oracle, u, op):
    if op == "r2c_c2r":
        return oracle.c2r(oracle.r2c(u), u.shape[2])
    if op == "lap_invlap":
        return oracle.spectral_op(oracle.spectral_op(u, "laplace"), "inv_laplace")
    return oracle.spectral_op(u, op)


def test_batch_graph_matches_oracle(cuda, native, oracle, tmp_path):
    torch = cuda
    from accfft_gb300.batch import BatchPlan

    specs = [((32, 32, 32), "r2c_c2r"), ((48, 48, 48), "lap_invlap"), ((160, 180, 200), "r2c_c2r"),
             ((64, 64, 64), "laplace"), ((96, 96, 96), "inv_laplace"), ((128, 128, 128), "r2c_c2r"),
             ((192, 192, 192), "lap_invlap"), ((32, 32, 32), "laplace")]
    bp = BatchPlan(specs, "float32", cache=str(tmp_path / "tune.json"))
    r = rng(99)
    host = [r.uniform(-1, 1, s) for s, _ in specs]
    bp.set_inputs([torch.from_numpy(h.astype(np.float32)).cuda() for h in host])
    info = bp.tune(stream_choices=(1, 4))
    assert info["streams"] in (1, 4)
    bp.capture()
    for o in bp.outputs:
        o.zero_()
    bp.run()
    torch.cuda.synchronize()
    for (shape, op), h, out in zip(specs, host, bp.outputs):
        ref = oracle_result(oracle, h.astype(np.float32).astype(np.float64), op)
        err = oracle.rel_l2(out.cpu().numpy().astype(np.float64), ref)
        assert err < 1e-5, (shape, op, err)
    rep = bp.report()
    assert {tuple(r["grid"]) for r in rep} == {s for s, _ in specs}
    # the cached schedule is reused by a second plan
    bp2 = BatchPlan(specs[:2], "float32", cache=str(tmp_path / "tune.json"))
    bp2.tune(stream_choices=(1,))
    assert set(bp2.schedule) == {(32, 32, 32), (48, 48, 48)}


@pytest.mark.parametrize("order", [0, 1])
def test_grouped_batch_matches_streams_and_oracle(cuda, native, oracle, order):
    """The recorded, level-by-level form (one grouped kernel per pass kind,
    line length and level) gives the per-instance kernels' results bit for
    bit, in the reference's and in the packed pass order, with far fewer
    launches."""
    torch = cuda
    from accfft_gb300.batch import BatchPlan

    specs = [((32, 32, 32), "r2c_c2r"), ((48, 48, 48), "lap_invlap"), ((160, 180, 200), "r2c_c2r"),
             ((64, 64, 64), "laplace"), ((96, 96, 96), "inv_laplace"), ((32, 32, 32), "r2c_c2r"),
             ((192, 192, 192), "lap_invlap"), ((256, 256, 256), "r2c_c2r"), ((32, 48, 64), "laplace")]
    r = rng(98)
    host = [r.uniform(-1, 1, s) for s, _ in specs]
    ins = [torch.from_numpy(h.astype(np.float32)).cuda() for h in host]
    a = BatchPlan(specs, "float32", form="streams")
    g = BatchPlan(specs, "float32", form="grouped")
    for bp in (a, g):
        for inst in bp.instances:
            inst.plan.set_pass_order(order)
        bp.set_inputs(ins)
    a.run()
    before = native.kernel_launches()
    g.run()
    torch.cuda.synchronize()
    launched = native.kernel_launches() - before
    info = g.grouped().info()
    assert info["instances"] == len(specs) and info["tasks"] > info["launches"]
    assert launched <= info["launches"] * 2          # the capture's eager run and nothing per instance
    for (shape, op), h, x, y in zip(specs, host, a.outputs, g.outputs):
        assert torch.equal(x, y), (shape, op)
        ref = oracle_result(oracle, h.astype(np.float32).astype(np.float64), op)
        assert oracle.rel_l2(y.cpu().numpy().astype(np.float64), ref) < 1e-5, (shape, op)


def test_batch_record_rejects(cuda, native):
    torch = cuda
    b = native.Batch()
    p64 = native.PlanR2C((16, 16, 16), "float64")
    with pytest.raises(native.AccfftError):
        b.record(p64)                                    # float plans only
    p = native.PlanR2C((16, 16, 16), "float32")
    u = torch.randn((16, 16, 16), device="cuda")
    g = [torch.empty_like(u) for _ in range(3)]
    with pytest.raises(native.AccfftError):
        with b.recording(p):
            p.grad(*g, u)                                # z derivative pass: not recordable
    q = native.PlanR2C((512, 16, 16), "float32")
    with pytest.raises(native.AccfftError):
        with b.recording(q):
            q.laplace(torch.empty((512, 16, 16), device="cuda"), torch.randn((512, 16, 16), device="cuda"))
