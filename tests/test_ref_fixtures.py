"""The oracle against results produced by AccFFT's OWN code.

tests/golden/ref_cases.npz holds outputs of the reference's unmodified CPU
host code (src/accfft.cpp, src/operators.txx, src/transpose.cpp), built by
oracle/build_ref.py against a one-rank MPI and an FFTW-API shim whose DFT is
the oracle's long-double transform (script: tests/golden/gen_ref_cases.py).
These tests pin the oracle's layouts, pass order, xyz handling, single-axis
layouts, Nyquist folding on even and odd lengths and every operator's
multipliers to the reference itself.  Where the reference tree is present
the fixtures are also regenerated and compared bit for bit.
"""
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
FIX = os.path.join(HERE, "golden", "ref_cases.npz")

# rel-L2 of the double oracle against the fixtures: the inverse operators
# divide by |k|^2 or |k|^4 and so weight the lowest modes, whose rounding the
# division does not shrink; everything else within 1e-14
TOL_D = {"inv_laplace": 5e-14, "inv_biharmonic": 5e-14}
TOL_LD = 2e-15     # the long-double oracle computes the same DFT as the shim


def cases():
    z = np.load(FIX)
    shapes = sorted({k.split("__")[1] for k in z.files})
    out = []
    for t in shapes:
        for k in z.files:
            if k.startswith(f"out__{t}__"):
                out.append((t, k.split("__")[2]))
    return out


def cpu_to_gpu_axis(a, s):
    """The reference's CPU single-axis layouts -> the GPU path's
    (y: [n0][n2][n1/2+1] -> [n0][n1/2+1][n2]; x: [n1][n2][n0/2+1] -> [n0/2+1][n1][n2])."""
    if a == 2:
        return s
    return np.ascontiguousarray(s.transpose(0, 2, 1) if a == 1 else s.transpose(2, 0, 1))


def oracle_case(o, n, case, inp, prec):
    """The oracle's result for one fixture case (GPU-path layouts)."""
    if case == "r2c_ip":
        return o.r2c(inp["u"], prec=prec)
    if case.startswith("r2c_"):
        _, f, xyz = case.split("_")
        return o.r2c(inp[f], int(xyz), prec=prec)
    if case == "c2r_ip":
        return o.c2r(inp["h"], n[2], prec=prec)
    if case.startswith("c2r_"):
        return o.c2r(inp["h"], n[2], int(case.split("_")[1]), prec=prec)
    if case.startswith("c2c"):
        return o.c2c(inp["c"], -1 if case[3] == "f" else 1, int(case.split("_")[1]), prec=prec)
    if case.startswith("ax") and case[3] == "f":
        return o.r2c_axis(inp[case.split("_")[1]], int(case[2]), prec=prec)
    if case.startswith("ax") and case[3] == "b":
        a = int(case[2])
        return o.c2r_axis(cpu_to_gpu_axis(a, inp[["hx", "hy", "h"][a]]), a, n, prec=prec)
    if case == "grad_p5_u":
        g = np.stack(o.grad(inp["u"], prec=prec))
        g[1] = 0
        return g
    if case.startswith("grad_slow_"):
        return np.stack(o.grad_slow(inp[case.split("_")[2]], prec=prec))
    if case.startswith("grad_"):
        return np.stack(o.grad(inp[case.split("_")[1]], prec=prec))
    if case == "div_slow_v":
        return o.divergence_slow(*inp["v"], prec=prec)
    if case == "div_v":
        return o.divergence(*inp["v"], prec=prec)
    op, f = case.rsplit("_", 1)
    return o.spectral_op(inp[f], op, prec=prec)


def fixture(z, t, case):
    ref = z[f"out__{t}__{case}"]
    if case.startswith("ax") and case[3] == "f":
        ref = cpu_to_gpu_axis(int(case[2]), ref)
    return ref


def inputs(z, t):
    return {k.split("__")[2]: z[k] for k in z.files if k.startswith(f"in__{t}__")}


def test_fixture_inventory():
    """Every kind of case the reference runs is present, on even, odd and
    length-2 axes."""
    cs = cases()
    kinds = {c.rsplit("_", 1)[0] if not c.startswith(("r2c", "c2r", "c2c")) else c.split("_")[0] for _, c in cs}
    for k in ("r2c", "c2r", "c2cf", "c2cb", "ax0f", "ax1f", "ax2f", "ax0b", "ax1b", "ax2b", "grad", "grad_slow",
              "laplace", "biharmonic", "inv_laplace", "inv_biharmonic", "div", "div_slow"):
        assert k in kinds, k
    shapes = {tuple(map(int, t.split("x"))) for t, _ in cs}
    assert any(m % 2 for s in shapes for m in s) and any(2 in s for s in shapes)


@pytest.mark.parametrize("prec", ["d", "ld"])
def test_oracle_matches_reference(oracle, prec):
    z = np.load(FIX)
    bad = []
    for t, case in cases():
        n = tuple(map(int, t.split("x")))
        got = oracle_case(oracle, n, case, inputs(z, t), prec)
        ref = fixture(z, t, case)
        tol = TOL_LD if prec == "ld" else TOL_D.get(case.rsplit("_", 1)[0], 1e-14)
        e = oracle.rel_l2(got, ref)
        if not e <= tol:
            bad.append((t, case, e))
    assert not bad, bad[:10]


def test_fixtures_regenerate_bit_exact():
    """Where the reference tree is present, oracle/_ref is rebuilt from it and a
    few fixture cases are recomputed: identical bits to the committed file."""
    sys.path.insert(0, os.path.join(HERE, "golden"))
    sys.path.insert(0, os.path.join(os.path.dirname(HERE), "oracle"))
    import build_ref
    import gen_ref_cases as g

    path = build_ref.build()
    if path is None:
        pytest.skip("reference tree not present: the committed fixtures stand")
    ref = g.Ref(path)
    z = np.load(FIX)
    for n in (g.GPU_SHAPES[1], g.ORACLE_SHAPES[0]):
        t = g.tag(n)
        inp = inputs(z, t)
        assert np.array_equal(ref.r2c(n, 7, inp["u"]), z[f"out__{t}__r2c_u_7"])
        assert np.array_equal(ref.op(n, g.OPS["div_slow"], inp["v"]), z[f"out__{t}__div_slow_v"])
        assert np.array_equal(ref.axis(n, 0, -1, inp["nyq"]), z[f"out__{t}__ax0f_nyq"])
        assert np.array_equal(ref.op(n, g.OPS["inv_biharmonic"], inp["nyq"]), z[f"out__{t}__inv_biharmonic_nyq"])
