"""Generate tests/golden/ref_cases.npz: outputs of AccFFT's OWN CPU code.

The reference's host sources are compiled unmodified by oracle/build_ref.py
(one-rank MPI and FFTW shims; the FFTW calls computed by the oracle's
long-double DFT) into oracle/_ref/libaccfft_ref.so.  This script drives the
reference's public API through oracle/ref_driver.cpp on seeded inputs and
stores inputs and outputs, so the reference's own plan geometry, pass order,
xyz handling, in-place layout, single-axis transposes and wave-number loops
(src/accfft.cpp, src/operators.txx, src/transpose.cpp) are what the oracle
and the CUDA path are checked against.  Runs only where the reference tree is
present:

    python oracle/build_ref.py && python tests/golden/gen_ref_cases.py

Layout of the archive (all float64 / complex128):
  in__<shape>__<name>         seeded inputs of one grid shape
  out__<shape>__<case>        the reference's result for one case
Inputs per shape: u (N(0,1) field), nyq (a field dominated by the Nyquist and
near-Nyquist modes of every axis), c (complex N(0,1) grid), h (complex N(0,1)
half spectrum [n0][n1][n2/2+1], not Hermitian), hy / hx (complex N(0,1) arrays
in the CPU path's y-only [n0][n2][n1/2+1] and x-only [n1][n2][n0/2+1]
layouts), v (3 stacked N(0,1) fields).
Cases: r2c_<field>_<xyz>, r2c_ip (in place), c2r_<xyz>, c2r_ip, c2c<dir>_<xyz>
(dir f / b), ax<a>f_<field> (single-axis r2c, a = 0 x, 1 y, 2 z, CPU layout),
ax<a>b (single-axis c2r of h / hy / hx), <op>_<field> for grad / grad_slow
(3 stacked outputs; grad_p5 with the y component not selected, left zero),
laplace, biharmonic, inv_laplace, inv_biharmonic, and div / div_slow of v.
"""
import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.abspath(os.path.join(HERE, "..", ".."))
OUT = os.path.join(HERE, "ref_cases.npz")

# Grids the CUDA path supports (even N2, lengths with compiled kernels):
# even and odd x / y lengths, length 2, the z half length 9, N0 = 1.
GPU_SHAPES = [(8, 6, 10), (5, 9, 4), (6, 5, 12), (2, 4, 6), (16, 12, 10), (9, 10, 8), (4, 20, 18), (1, 6, 8)]
# Grids only the oracle is checked on: odd N2 (the CUDA r2c needs an even
# N2) and a prime length without kernels.
ORACLE_SHAPES = [(7, 5, 9), (3, 11, 7)]
PARTIAL_XYZ = [1, 2, 3, 4, 5, 6]
OPS = {"grad": 0, "grad_slow": 1, "laplace": 2, "div": 3, "div_slow": 4, "biharmonic": 5, "inv_laplace": 6,
       "inv_biharmonic": 7}


def tag(n):
    return "x".join(map(str, n))


def nyquist_field(n, rng):
    """Dominated by the highest modes of every axis (the Nyquist plane of
    even axes, the two top modes of odd ones), plus a little noise."""
    i, j, k = np.meshgrid(*[np.arange(m) for m in n], indexing="ij")
    f = 0.2 * rng.standard_normal(n)
    for idx, m in ((i, n[0]), (j, n[1]), (k, n[2])):
        f += 2.0 * np.cos(np.pi * idx * (2 * (m // 2)) / max(m, 1))
    f += 1.5 * np.cos(np.pi * (i * (2 * (n[0] // 2)) / n[0] + j * (2 * (n[1] // 2)) / n[1]))
    f += np.cos(np.pi * (i * (2 * (n[0] // 2)) / n[0] + j * (2 * (n[1] // 2)) / n[1] + k * (2 * (n[2] // 2)) / n[2]))
    return f


class Ref:
    def __init__(self, path):
        self.lib = ctypes.CDLL(path)
        self.lib.ref_init(min(8, os.cpu_count() or 1))
        self.dp = ctypes.POINTER(ctypes.c_double)
        self.lib.ref_axis.argtypes = [ctypes.POINTER(ctypes.c_int), ctypes.c_int, ctypes.c_int, self.dp, self.dp,
                                      ctypes.c_longlong]

    def _n(self, n):
        return (ctypes.c_int * 3)(*n)

    def _p(self, a):
        assert a.flags.c_contiguous
        return a.ctypes.data_as(self.dp)

    def _chk(self, rc, what):
        if rc != 0:
            raise RuntimeError(f"reference call {what} failed: {rc}")

    def r2c(self, n, xyz, x):
        h = (n[0], n[1], n[2] // 2 + 1)
        x = np.ascontiguousarray(x, dtype=np.complex128 if not xyz & 4 else np.float64)
        out = np.zeros(h, np.complex128)
        self._chk(self.lib.ref_r2c(self._n(n), xyz, self._p(x), self._p(out)), "r2c")
        return out

    def c2r(self, n, xyz, s):
        s = np.ascontiguousarray(s, np.complex128)
        out = np.zeros(n if xyz & 4 else s.shape, np.float64 if xyz & 4 else np.complex128)
        self._chk(self.lib.ref_c2r(self._n(n), xyz, self._p(s), self._p(out)), "c2r")
        return out

    def r2c_ip(self, n, u):
        out = np.zeros((n[0], n[1], n[2] // 2 + 1), np.complex128)
        self._chk(self.lib.ref_r2c_inplace(self._n(n), self._p(np.ascontiguousarray(u)), self._p(out)), "r2c_ip")
        return out

    def c2r_ip(self, n, s):
        out = np.zeros(n)
        self._chk(self.lib.ref_c2r_inplace(self._n(n), self._p(np.ascontiguousarray(s)), self._p(out)), "c2r_ip")
        return out

    def c2c(self, n, d, xyz, c):
        out = np.zeros(n, np.complex128)
        self._chk(self.lib.ref_c2c(self._n(n), d, xyz, self._p(np.ascontiguousarray(c)), self._p(out)), "c2c")
        return out

    @staticmethod
    def axis_shape(n, a):
        return [(n[1], n[2], n[0] // 2 + 1), (n[0], n[2], n[1] // 2 + 1), (n[0], n[1], n[2] // 2 + 1)][a]

    def axis(self, n, a, d, x):
        x = np.ascontiguousarray(x)
        out = np.zeros(self.axis_shape(n, a), np.complex128) if d < 0 else np.zeros(n)
        cap = out.size * (2 if d < 0 else 1)
        self._chk(self.lib.ref_axis(self._n(n), a, d, self._p(x), self._p(out), cap), f"axis {a} {d}")
        return out

    def op(self, n, kind, x, pxyz=7):
        x = np.ascontiguousarray(x, np.float64)
        outs = 3 if kind in (0, 1) else 1
        out = np.zeros((outs,) + tuple(n)) if outs == 3 else np.zeros(n)
        self._chk(self.lib.ref_op(self._n(n), kind, pxyz, self._p(x), self._p(out)), f"op {kind}")
        return out


def main():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import build_ref

    path = build_ref.build()
    if path is None:
        raise SystemExit("reference tree not found: set ACCFFT_REFERENCE_ROOT")
    ref = Ref(path)
    rng = np.random.default_rng(20261204)
    arc = {}
    for n in GPU_SHAPES + ORACLE_SHAPES:
        t = tag(n)
        gpu = n in GPU_SHAPES
        h = (n[0], n[1], n[2] // 2 + 1)
        inp = {
            "u": rng.standard_normal(n),
            "nyq": nyquist_field(n, rng),
            "c": rng.standard_normal(n) + 1j * rng.standard_normal(n),
            "h": rng.standard_normal(h) + 1j * rng.standard_normal(h),
            "hy": rng.standard_normal(Ref.axis_shape(n, 1)) + 1j * rng.standard_normal(Ref.axis_shape(n, 1)),
            "hx": rng.standard_normal(Ref.axis_shape(n, 0)) + 1j * rng.standard_normal(Ref.axis_shape(n, 0)),
            "v": rng.standard_normal((3,) + tuple(n)),
        }
        for k, v in inp.items():
            arc[f"in__{t}__{k}"] = v
        out = {}
        for f in ("u", "nyq"):
            out[f"r2c_{f}_7"] = ref.r2c(n, 7, inp[f])
            for a in range(3):
                out[f"ax{a}f_{f}"] = ref.axis(n, a, -1, inp[f])
            for name in ("laplace", "biharmonic", "inv_laplace", "inv_biharmonic", "grad", "grad_slow"):
                out[f"{name}_{f}"] = ref.op(n, OPS[name], inp[f])
        out["grad_p5_u"] = ref.op(n, OPS["grad"], inp["u"], pxyz=5)
        out["div_v"] = ref.op(n, OPS["div"], inp["v"])
        out["div_slow_v"] = ref.op(n, OPS["div_slow"], inp["v"])
        out["c2r_7"] = ref.c2r(n, 7, inp["h"])
        out["c2cf_7"] = ref.c2c(n, -1, 7, inp["c"])
        out["c2cb_7"] = ref.c2c(n, 1, 7, inp["c"])
        for a, key in ((0, "hx"), (1, "hy"), (2, "h")):
            out[f"ax{a}b"] = ref.axis(n, a, 1, inp[key])
        if gpu:
            out["r2c_ip"] = ref.r2c_ip(n, inp["u"])
            out["c2r_ip"] = ref.c2r_ip(n, inp["h"])
            for xyz in PARTIAL_XYZ:
                out[f"r2c_{'u' if xyz & 4 else 'h'}_{xyz}"] = ref.r2c(n, xyz, inp["u"] if xyz & 4 else inp["h"])
                out[f"c2r_{xyz}"] = ref.c2r(n, xyz, inp["h"])
                out[f"c2cf_{xyz}"] = ref.c2c(n, -1, xyz, inp["c"])
                out[f"c2cb_{xyz}"] = ref.c2c(n, 1, xyz, inp["c"])
        for k, v in out.items():
            arc[f"out__{t}__{k}"] = v
    np.savez_compressed(OUT, **arc)
    n_out = sum(1 for k in arc if k.startswith("out__"))
    print(f"wrote {OUT}: {n_out} reference results over {len(GPU_SHAPES) + len(ORACLE_SHAPES)} grids, "
          f"{os.path.getsize(OUT) / 1e6:.2f} MB")


if __name__ == "__main__":
    main()
