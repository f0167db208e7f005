"""Generate tests/golden/small_cases.npz: small seeded inputs and their
transforms computed by the oracle in long double and cross-checked against
numpy.fft (pocketfft, an independent implementation of the same DFT).

    python tests/golden/gen_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "..", "..", "oracle"))
import accfft_oracle as o  # noqa: E402

SHAPES = [(4, 6, 8), (8, 8, 8), (6, 10, 12), (5, 9, 4), (16, 12, 10)]


def main():
    rng = np.random.default_rng(20261203)
    out = {}
    for n in SHAPES:
        tag = "x".join(map(str, n))
        u = rng.standard_normal(n)
        s = o.r2c(u, prec="ld")
        assert o.rel_l2(s, o.np_r2c(u)) < 1e-14
        out[f"r2c__{tag}_in"], out[f"r2c__{tag}_out"] = u, s
        h = rng.standard_normal(s.shape) + 1j * rng.standard_normal(s.shape)
        b = o.c2r(h, n[2], prec="ld")
        assert o.rel_l2(b, o.np_c2r(h, n[2])) < 1e-14
        out[f"c2r__{tag}_in"], out[f"c2r__{tag}_out"] = h, b
        d = rng.standard_normal(n) + 1j * rng.standard_normal(n)
        out[f"c2cf__{tag}_in"], out[f"c2cf__{tag}_out"] = d, o.c2c(d, -1, prec="ld")
        out[f"c2cb__{tag}_in"], out[f"c2cb__{tag}_out"] = d, o.c2c(d, 1, prec="ld")
        for op in ("laplace", "biharmonic", "inv_laplace", "inv_biharmonic"):
            out[f"{op}__{tag}_in"], out[f"{op}__{tag}_out"] = u, o.spectral_op(u, op, prec="ld")
    np.savez_compressed(os.path.join(HERE, "small_cases.npz"), **out)
    print(f"wrote {len(out) // 2} cases")


if __name__ == "__main__":
    main()
