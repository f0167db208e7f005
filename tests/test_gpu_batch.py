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
