"""Seeded random grids through the default (packed) pass order against the
oracle, through the C ABI: the mirror-pair z passes (warp-shuffle merge
where the two lines of a pair share a warp, shared-memory staging
elsewhere), the dense y pass and the x pass over odd, even, 1- and 2-long x
and y axes and many z lengths.  Each grid runs a float and a double plan,
r2c of an N(0,1) field and c2r of an arbitrary half spectrum.  Bounds as in
test_gpu_transforms.py: rel-L2 <= 1e-5 (float) and <= 1e-12 (double)
against the double oracle."""
import numpy as np
import pytest

from test_gpu_transforms import TOL, empty, from_dev, to_dev

pytestmark = pytest.mark.gpu


def sweep_grids(native, count=24, seed=2024):
    """`count` grids with every axis supported by the CUDA path (the z axis
    through its half length), drawn with a fixed seed."""
    lib = native.lib()
    r = np.random.default_rng(seed)
    xy = [m for m in range(1, 97) if lib.accfft_c_length_supported(m)]
    zs = [m for m in range(1, 257) if lib.accfft_c_length_supported(m)]
    out = []
    while len(out) < count:
        n = (int(r.choice(xy)), int(r.choice(xy)), 2 * int(r.choice(zs)))
        if n[0] * n[1] * n[2] <= (1 << 21) and n not in out:
            out.append(n)
    return out


@pytest.mark.parametrize("dtype", ["float32", "float64"])
def test_random_grids_packed_order_vs_oracle(cuda, native, oracle, dtype):
    torch = cuda
    bad = []
    for i, n in enumerate(sweep_grids(native)):
        plan = native.PlanR2C(n, dtype)
        h = (n[0], n[1], n[2] // 2 + 1)
        r = np.random.default_rng(100 + i)
        u = r.standard_normal(n)
        dh = empty(torch, h + (2,), dtype)
        plan.r2c(to_dev(torch, u, dtype), dh)
        e1 = oracle.rel_l2(from_dev(dh, True), oracle.r2c(u.astype(dtype).astype(np.float64)))
        s = r.standard_normal(h) + 1j * r.standard_normal(h)
        ds = to_dev(torch, s, dtype)
        db = empty(torch, n, dtype)
        plan.c2r(ds, db)
        e2 = oracle.rel_l2(from_dev(db), oracle.c2r(from_dev(ds, True), n[2]))
        if not (e1 <= TOL[dtype] and e2 <= TOL[dtype]):
            bad.append((n, e1, e2))
        plan.destroy()
    assert not bad, bad
