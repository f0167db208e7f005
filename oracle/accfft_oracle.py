"""Oracle for AccFFT's single-rank 3-D FFT path.  TEST INFRASTRUCTURE ONLY.

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg use
this module, and only as the checker.  The product library (accfft_gb300)
never imports it.

Two independent restatements of the same mathematics live here:

* the C restatement in fft_oracle.c (mixed-radix DFT in double or long
  double, the reference's pass order and layouts), driven by the functions
  below, and
* ``np_*`` functions built on numpy.fft, used to cross-check the C code.

The reference computes with FFTW3 on the CPU (src/accfft.cpp) and cuFFT on the
GPU (src/accfft_gpu.cpp); neither library is part of the reference tree and
neither is installed here, so the oracle restates the DFT those libraries
implement (see fft_oracle.c) and is pinned to the reference's own tests:
round trips (steps/step1-3), analytic operator results (steps/step5) and
analytic spectra (tests/golden/).

Layouts (row-major, z fastest):
  real            [N0][N1][N2]          (in-place plans: rows padded to 2*(N2/2+1))
  r2c spectrum    [N0][N1][N2/2+1] complex
  c2c             [N0][N1][N2] complex
  x-only spectrum [N0/2+1][N1][N2], y-only [N0][N1/2+1][N2], z-only = r2c
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "liboracle.so")
SRCS = [os.path.join(HERE, f) for f in ("fft_oracle.c", "oracle_core.h")]

_lib = None


def build() -> str:
    """Compile fft_oracle.c into oracle/_build/liboracle.so (gcc, no CUDA)."""
    os.makedirs(BUILD, exist_ok=True)
    newest = max(os.path.getmtime(s) for s in SRCS)
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= newest:
        return LIB
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-Wall", "-o", LIB, SRCS[0], "-lpthread", "-lm"]
    subprocess.run(cmd, check=True, capture_output=True)
    return LIB


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB)
        dp = ctypes.POINTER(ctypes.c_double)
        ll = ctypes.c_longlong
        i = ctypes.c_int
        L.orc_fft1d.argtypes = [i, dp, dp, i, i]
        L.orc_c2c_axis.argtypes = [i, i, i, i, dp, i, i, i]
        L.orc_r2c_z.argtypes = [ll, i, dp, ll, dp, ll, i, i]
        L.orc_c2r_z.argtypes = [ll, i, dp, ll, dp, ll, i, i]
        L.orc_r2c_strided.argtypes = [ll, i, ll, dp, dp, i, i]
        L.orc_c2r_strided.argtypes = [ll, i, ll, dp, dp, i, i]
        for f in ("orc_fft1d", "orc_c2c_axis", "orc_r2c_z", "orc_c2r_z", "orc_r2c_strided", "orc_c2r_strided"):
            getattr(L, f).restype = i
        _lib = L
    return _lib


def _threads(nthreads):
    return nthreads if nthreads else (os.cpu_count() or 1)


def _dp(a: np.ndarray):
    assert a.dtype in (np.float64, np.complex128) and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


def _prec(prec: str) -> int:
    return {"d": 0, "ld": 1}[prec]


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"oracle {what} failed ({rc})")


# ----------------------------------------------------------------- 1-D
def fft1d(x, sign=-1, prec="d"):
    x = np.ascontiguousarray(x, dtype=np.complex128)
    out = np.empty_like(x)
    _check(lib().orc_fft1d(x.size, _dp(x), _dp(out), sign, _prec(prec)), "fft1d")
    return out


# ----------------------------------------------------------- passes
def c2c_axis(data: np.ndarray, axis: int, sign: int, prec="d", nthreads=0) -> np.ndarray:
    """Complex transform along `axis` of a complex [n0][n1][w] array (returns a new array)."""
    return _c2c_axis_inplace(np.array(data, dtype=np.complex128, order="C", copy=True), axis, sign, prec, nthreads)


def _c2c_axis_inplace(d: np.ndarray, axis: int, sign: int, prec="d", nthreads=0) -> np.ndarray:
    """c2c_axis on an array the caller owns (C-contiguous complex128), in place."""
    assert d.dtype == np.complex128 and d.flags.c_contiguous and d.ndim == 3
    n0, n1, w = d.shape
    _check(lib().orc_c2c_axis(n0, n1, w, axis, _dp(d), sign, _prec(prec), _threads(nthreads)), "c2c_axis")
    return d


c2c_axis_inplace = _c2c_axis_inplace


def _out(out, shape, dtype):
    """`out` when given (C-contiguous, of the shape and type), else a new array."""
    if out is None:
        return np.empty(shape, dtype)
    assert out.shape == shape and out.dtype == dtype and out.flags.c_contiguous
    return out


def r2c_z(u: np.ndarray, prec="d", nthreads=0, out=None) -> np.ndarray:
    """z pass of r2c: [..][N2] real -> [..][N2/2+1] complex (src/accfft_gpu.cpp:170-206)."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    n2 = u.shape[-1]
    rows = u.size // n2
    out = _out(out, u.shape[:-1] + (n2 // 2 + 1,), np.complex128)
    _check(lib().orc_r2c_z(rows, n2, _dp(u), n2, _dp(out), n2 // 2 + 1, _prec(prec), _threads(nthreads)), "r2c_z")
    return out


def c2r_z(s: np.ndarray, n2: int, prec="d", nthreads=0, out=None) -> np.ndarray:
    """z pass of c2r: [..][N2/2+1] complex -> [..][N2] real, DC/Nyquist imaginary parts ignored."""
    s = np.ascontiguousarray(s, dtype=np.complex128)
    h = s.shape[-1]
    assert h == n2 // 2 + 1
    rows = s.size // h
    out = _out(out, s.shape[:-1] + (n2,), np.float64)
    _check(lib().orc_c2r_z(rows, n2, _dp(s), h, _dp(out), n2, _prec(prec), _threads(nthreads)), "c2r_z")
    return out


def r2c_strided(u: np.ndarray, prec="d", nthreads=0) -> np.ndarray:
    """Real transform along the middle axis of a real [a][L][b] array -> complex [a][L/2+1][b]."""
    u = np.ascontiguousarray(u, dtype=np.float64)
    a, L, b = u.shape
    out = np.empty((a, L // 2 + 1, b), np.complex128)
    _check(lib().orc_r2c_strided(a, L, b, _dp(u), _dp(out), _prec(prec), _threads(nthreads)), "r2c_strided")
    return out


def c2r_strided(s: np.ndarray, L: int, prec="d", nthreads=0) -> np.ndarray:
    s = np.ascontiguousarray(s, dtype=np.complex128)
    a, h, b = s.shape
    assert h == L // 2 + 1
    out = np.empty((a, L, b), np.float64)
    _check(lib().orc_c2r_strided(a, L, b, _dp(s), _dp(out), _prec(prec), _threads(nthreads)), "c2r_strided")
    return out


# --------------------------------------------------------- 3-D transforms
def r2c(u: np.ndarray, xyz: int = 7, prec="d", nthreads=0) -> np.ndarray:
    """Forward real 3-D transform, unnormalised, sign -1.

    Pass order of accfft_execute_gpu (src/accfft_gpu.cpp:470-539): z r2c, y c2c,
    x c2c.  With the z bit cleared the reference runs the y/x passes on the
    input reinterpreted as complex [N0][N1][N2/2+1]; here `u` must then already
    be that complex array.
    """
    if xyz & 4:
        s = r2c_z(u, prec, nthreads)
    else:
        s = np.array(u, dtype=np.complex128, order="C")
    if xyz & 2:
        _c2c_axis_inplace(s, 1, -1, prec, nthreads)
    if xyz & 1:
        _c2c_axis_inplace(s, 0, -1, prec, nthreads)
    return s


def c2r(s: np.ndarray, n2: int, xyz: int = 7, prec="d", nthreads=0) -> np.ndarray:
    """Backward real 3-D transform (src/accfft_gpu.cpp:540-603): x c2c, y c2c, z c2r; unnormalised."""
    s = np.array(s, dtype=np.complex128, order="C")
    if xyz & 1:
        _c2c_axis_inplace(s, 0, +1, prec, nthreads)
    if xyz & 2:
        _c2c_axis_inplace(s, 1, +1, prec, nthreads)
    if xyz & 4:
        return c2r_z(s, n2, prec, nthreads)
    return s


def c2c(d: np.ndarray, direction: int, xyz: int = 7, prec="d", nthreads=0) -> np.ndarray:
    """Complex 3-D transform (src/accfft_gpu.cpp:943-1136), direction -1 or +1, unnormalised."""
    s = np.array(d, dtype=np.complex128, order="C")
    order = (2, 1, 0) if direction == -1 else (0, 1, 2)
    for ax in order:
        if xyz & (1 << ax):
            _c2c_axis_inplace(s, ax, direction, prec, nthreads)
    return s


def r2c_axis(u: np.ndarray, axis: int, prec="d", nthreads=0) -> np.ndarray:
    """Single-axis real transforms (src/accfft_gpu.cpp:1212-1604) with the reference's layouts."""
    n0, n1, n2 = u.shape
    if axis == 2:
        return r2c_z(u, prec, nthreads)
    if axis == 1:
        return r2c_strided(u, prec, nthreads)
    return r2c_strided(u.reshape(1, n0, n1 * n2), prec, nthreads).reshape(n0 // 2 + 1, n1, n2)


def c2r_axis(s: np.ndarray, axis: int, n: tuple, prec="d", nthreads=0) -> np.ndarray:
    n0, n1, n2 = n
    if axis == 2:
        return c2r_z(s, n2, prec, nthreads)
    if axis == 1:
        return c2r_strided(s, n1, prec, nthreads)
    return c2r_strided(s.reshape(1, n0 // 2 + 1, n1 * n2), n0, prec, nthreads).reshape(n0, n1, n2)


# ------------------------------------------------------- wave numbers
def fold(idx: np.ndarray, n: int, nyquist_zero=True) -> np.ndarray:
    """Wave number of index i on an axis of length n, as in grad_mult_wave_number*_cu
    (src/operators_cuda.cu:33-38): i - n above n/2, and 0 at i == n/2 (integer n/2)."""
    w = idx.astype(np.int64).copy()
    w[idx > n // 2] -= n
    if nyquist_zero:
        w[idx == n // 2] = 0
    return w


def _waves(n, h2, nyquist_zero=True):
    n0, n1, n2 = n
    wx = fold(np.arange(n0), n0, nyquist_zero)[:, None, None]
    wy = fold(np.arange(n1), n1, nyquist_zero)[None, :, None]
    wz = fold(np.arange(h2), n2, nyquist_zero)[None, None, :]
    return wx, wy, wz


def symbol(kind: str, n, param: float = 0.0) -> np.ndarray:
    """Multipliers applied to the r2c spectrum by the reference's operators:
    laplace/biharmonic (src/operators_cuda.cu:115-205), inv_laplace
    (src/operators.txx:276-333), inv_biharmonic (src/operators.txx:336-388),
    grad components of the full-3-D path (src/operators_cuda.cu:16-112)."""
    n0, n1, n2 = n
    h2 = n2 // 2 + 1
    scale = 1.0 / (n0 * n1 * n2)
    if kind == "inv_biharmonic":
        wx, wy, wz = _waves(n, h2, nyquist_zero=False)
        w = (-(wx * wx) - wy * wy - wz * wz).astype(np.float64)
        w = w * w
        w[w == 0] = 1
        return scale / w
    wx, wy, wz = _waves(n, h2)
    w2 = -(wx * wx) - wy * wy - wz * wz
    if kind == "laplace":
        return scale * w2.astype(np.float64)
    if kind == "biharmonic":
        return scale * (w2 * w2).astype(np.float64)
    if kind == "inv_laplace":
        w = w2.astype(np.float64)
        out = np.zeros_like(w)
        nz = w != 0
        out[nz] = 1.0 / w[nz]
        return scale * out
    if kind == "heat":
        return scale * np.exp(-(wx * wx + wy * wy + wz * wz).astype(np.float64) * param)
    if kind == "helmholtz":
        d = param + (wx * wx + wy * wy + wz * wz).astype(np.float64)
        out = np.zeros_like(d)
        nz = d != 0
        out[nz] = scale / d[nz]
        return out
    if kind in ("gradx", "grady", "gradz"):
        w = {"gradx": wx, "grady": wy, "gradz": wz}[kind]
        return 1j * scale * np.broadcast_to(w, (n0, n1, h2)).astype(np.float64)
    if kind in ("poisson_fd", "poisson_spec"):
        # steps/step4/kernels.cu:24-110: Poisson filter on the unit cube.
        # method 0 (poisson_fd): finite-difference Laplacian eigenvalues
        #   2 * sum_i (cos(2 pi k_i / N_i) - 1) / dx_i^2, dx_i = 1 / N_i
        # method 1 (poisson_spec): -4 pi^2 |k|^2 with k_i folded above N_i/2
        #   (no Nyquist filter); the zero mode is set to 0 (zero mean)
        ix = np.arange(n0)[:, None, None]
        iy = np.arange(n1)[None, :, None]
        iz = np.arange(h2)[None, None, :]
        if kind == "poisson_fd":
            d = sum(2.0 * (np.cos(2 * np.pi * i / m) - 1.0) * m * m for i, m in ((ix, n0), (iy, n1), (iz, n2)))
        else:
            fx, fy, fz = (np.where(i > m // 2, i - m, i) for i, m in ((ix, n0), (iy, n1), (iz, n2)))
            d = -4.0 * np.pi ** 2 * (fx * fx + fy * fy + fz * fz).astype(np.float64)
        d = np.broadcast_to(d, (n0, n1, h2)).astype(np.float64)
        out = np.zeros_like(d)
        nz = np.broadcast_to((ix != 0) | (iy != 0) | (iz != 0), d.shape)
        out[nz] = scale / d[nz]
        return out
    raise ValueError(kind)


# ----------------------------------------------------------- operators
def spectral_op(u: np.ndarray, kind: str, prec="d", nthreads=0, param: float = 0.0) -> np.ndarray:
    """r2c -> multiply -> c2r (accfft_laplace_gpu_t, src/operators_gpu.txx:281-334,
    and its biharmonic twin :556-609; inv_laplace per src/operators.txx:1270-1322;
    heat / helmholtz are this library's solvers on the same wave numbers)."""
    n = u.shape
    s = r2c(u, 7, prec, nthreads) * symbol(kind, n, param)
    return c2r(s, n[2], 7, prec, nthreads)


def deriv(u: np.ndarray, axis: int, prec="d", nthreads=0) -> np.ndarray:
    """d/dx_axis by a single-axis real transform, multiply by i*w/N_axis
    (Nyquist -> 0), single-axis inverse (accfft_grad_gpu_t, src/operators_gpu.txx:173-278)."""
    n = u.shape
    s = r2c_axis(u, axis, prec, nthreads)
    L = n[axis]
    w = fold(np.arange(L // 2 + 1), L).astype(np.float64)
    shape = [1, 1, 1]
    shape[axis] = L // 2 + 1
    s = s * (1j * w / L).reshape(shape)
    return c2r_axis(s, axis, n, prec, nthreads)


def grad(u, prec="d", nthreads=0):
    return [deriv(u, a, prec, nthreads) for a in (0, 1, 2)]


def grad_slow(u, prec="d", nthreads=0):
    """Full-3-D gradient (accfft_grad_gpu_slow_t, src/operators_gpu.txx:72-170)."""
    s = r2c(u, 7, prec, nthreads)
    return [c2r(s * symbol(k, u.shape), u.shape[2], 7, prec, nthreads) for k in ("gradx", "grady", "gradz")]


def divergence(ax, ay, az, prec="d", nthreads=0):
    """sum_j dA_j/dx_j with x first (accfft_divergence_gpu_t, src/operators_gpu.txx:449-553)."""
    out = deriv(ax, 0, prec, nthreads)
    out = out + deriv(ay, 1, prec, nthreads)
    return out + deriv(az, 2, prec, nthreads)


def divergence_slow(ax, ay, az, prec="d", nthreads=0):
    """The slow divergence (accfft_divergence_gpu_slow_t, src/operators_gpu.txx:337-446;
    CPU src/operators.txx:1019-1119): A_x transformed over {x, z} (xyz = 5),
    A_y over {y, z} (6), A_z over {z} (4); each multiplied by i*fold(k_j)/(N_j*N2)
    with the 3-D multipliers' filter (index N_j/2 -> 0, src/operators.txx:24-110)
    and transformed back over the same axes; the terms summed x, y, z."""
    n = ax.shape
    out = None
    for a, (f, xyz) in enumerate(((ax, 5), (ay, 6), (az, 4))):
        s = r2c(f, xyz, prec, nthreads)
        L = n[a]
        w = fold(np.arange(s.shape[a]), L).astype(np.float64)
        shape = [1, 1, 1]
        shape[a] = s.shape[a]
        scale = 1.0 / (L * n[2]) if a < 2 else 1.0 / n[2]
        t = c2r(s * (1j * w * scale).reshape(shape), n[2], xyz, prec, nthreads)
        out = t if out is None else out + t
    return out


# ---------------------------------------------------- numpy cross-check
def np_r2c(u):
    return np.fft.rfftn(u, axes=(0, 1, 2))


def np_c2r(s, n2):
    s = np.array(s, dtype=np.complex128)
    n = s.shape[0] * s.shape[1] * n2
    return np.fft.irfftn(s, s=(s.shape[0], s.shape[1], n2), axes=(0, 1, 2)) * n


def np_c2c(d, direction):
    if direction == -1:
        return np.fft.fftn(d, axes=(0, 1, 2))
    return np.fft.ifftn(d, axes=(0, 1, 2)) * d.size


# ------------------------------------------------------------- helpers
def pad_rows(u: np.ndarray) -> np.ndarray:
    """Real array in the in-place layout: rows padded to 2*(N2/2+1) (steps/step2/step2_gpu.cpp:40-72)."""
    n0, n1, n2 = u.shape
    out = np.zeros((n0, n1, 2 * (n2 // 2 + 1)), u.dtype)
    out[:, :, :n2] = u
    return out


def rel_l2(a, b) -> float:
    a = np.asarray(a)
    b = np.asarray(b)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))
