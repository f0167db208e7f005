"""The oracle (CPU restatement) against numpy.fft, its long-double twin, the
reference's analytic known answers and the committed golden fixtures."""
import os

import numpy as np
import pytest

from conftest import rng

GOLDEN = os.path.join(os.path.dirname(__file__), "golden")

SHAPES = [(4, 6, 8), (16, 12, 10), (9, 5, 6), (7, 11, 14), (32, 32, 32), (12, 20, 18)]


@pytest.mark.parametrize("n", SHAPES)
def test_r2c_c2r_vs_numpy(oracle, n):
    u = rng(1).standard_normal(n)
    s = oracle.r2c(u)
    assert oracle.rel_l2(s, oracle.np_r2c(u)) < 1e-14
    b = oracle.c2r(s, n[2])
    assert oracle.rel_l2(b, oracle.np_c2r(s, n[2])) < 1e-14
    assert oracle.rel_l2(b / np.prod(n), u) < 1e-14


@pytest.mark.parametrize("n", SHAPES)
def test_c2c_vs_numpy(oracle, n):
    r = rng(2)
    d = r.standard_normal(n) + 1j * r.standard_normal(n)
    for direction in (-1, 1):
        assert oracle.rel_l2(oracle.c2c(d, direction), oracle.np_c2c(d, direction)) < 1e-14


@pytest.mark.parametrize("n", SHAPES[:4])
def test_single_axis_vs_numpy(oracle, n):
    u = rng(3).standard_normal(n)
    for ax in range(3):
        s = oracle.r2c_axis(u, ax)
        assert oracle.rel_l2(s, np.fft.rfft(u, axis=ax)) < 1e-14
        assert oracle.rel_l2(oracle.c2r_axis(s, ax, n) / n[ax], u) < 1e-14


def test_long_double_agrees(oracle):
    u = rng(4).standard_normal((24, 20, 16))
    a = oracle.r2c(u, prec="d")
    b = oracle.r2c(u, prec="ld")
    assert oracle.rel_l2(a, b) < 1e-15


def test_c2r_ignores_dc_and_nyquist_imag(oracle):
    """c2r reads the half spectrum of a Hermitian array: the imaginary parts
    of the kz = 0 and kz = N2/2 entries of each z line do not matter."""
    n = (6, 4, 8)
    s = oracle.r2c(rng(5).standard_normal(n))
    t = s.copy()
    t[:, :, 0] += 3j
    t[:, :, -1] -= 2j
    # after the x and y backward passes those planes stay where they are, so
    # only the z c2r sees them; compare z pass alone
    assert oracle.rel_l2(oracle.c2r_z(t, n[2]), oracle.c2r_z(s, n[2])) < 1e-15


def grid(n):
    x = [2 * np.pi * np.arange(k) / k for k in n]
    return np.meshgrid(*x, indexing="ij")


def test_config1_analytic_modes(oracle):
    """u = sin x + sin y cos 2z on 128^3: the spectrum has exactly four stored
    non-zero modes, -iN/2 at (1,0,0), +iN/2 at (N0-1,0,0), -iN/4 at (0,1,2)
    and +iN/4 at (0,N1-1,2)."""
    n = (128, 128, 128)
    X, Y, Z = grid(n)
    u = np.sin(X) + np.sin(Y) * np.cos(2 * Z)
    s = oracle.r2c(u)
    N = float(np.prod(n))
    expect = np.zeros_like(s)
    expect[1, 0, 0] = -0.5j * N
    expect[-1, 0, 0] = 0.5j * N
    expect[0, 1, 2] = -0.25j * N
    expect[0, -1, 2] = 0.25j * N
    assert np.abs(s - expect).max() / N < 1e-13
    b = oracle.c2r(s, n[2]) / N
    assert np.abs(b - u).max() < 1e-13


def gaussian(n, sigma=4.0):
    X, Y, Z = grid(n)
    return np.exp(-sigma * ((X - np.pi) ** 2 + (Y - np.pi) ** 2 + (Z - np.pi) ** 2))


def test_step1_gaussian_round_trip(oracle):
    """steps/step1/step1_gpu.cpp:94-106: relative L1 error of c2r(r2c(u))/N - u below 1e-10."""
    n = (64, 64, 64)
    u = gaussian(n)
    b = oracle.c2r(oracle.r2c(u), n[2]) / np.prod(n)
    assert np.abs(b - u).sum() / np.abs(u).sum() < 1e-10


SIGMA = 32.0


def step5_field(n):
    """steps/step5/step5_gpu.cpp:20-33: sin x sin y sin z + exp(-32|x-pi|^2)."""
    X, Y, Z = grid(n)
    f = np.exp(-SIGMA * ((X - np.pi) ** 2 + (Y - np.pi) ** 2 + (Z - np.pi) ** 2))
    return np.sin(X) * np.sin(Y) * np.sin(Z) + f, (X, Y, Z, f)


def step5_grad(n):
    """steps/step5/step5_gpu.cpp:34-67"""
    _, (X, Y, Z, f) = step5_field(n)
    return [np.cos(X) * np.sin(Y) * np.sin(Z) - 2 * SIGMA * (X - np.pi) * f,
            np.sin(X) * np.cos(Y) * np.sin(Z) - 2 * SIGMA * (Y - np.pi) * f,
            np.sin(X) * np.sin(Y) * np.cos(Z) - 2 * SIGMA * (Z - np.pi) * f]


def step5_laplace(n):
    """steps/step5/step5_gpu.cpp:69-97"""
    _, (X, Y, Z, f) = step5_field(n)
    r2 = (X - np.pi) ** 2 + (Y - np.pi) ** 2 + (Z - np.pi) ** 2
    return -3 * np.sin(X) * np.sin(Y) * np.sin(Z) + (4 * SIGMA ** 2 * r2 - 6 * SIGMA) * f


def step5_biharmonic(n):
    """steps/step5/step5_gpu.cpp:98-133"""
    _, (X, Y, Z, f) = step5_field(n)
    s2, s3, s4 = SIGMA ** 2, SIGMA ** 3, SIGMA ** 4
    Xp, Yp, Zp = X - np.pi, Y - np.pi, Z - np.pi
    d4 = lambda a: 12 * s2 * f - 48 * s3 * a * a * f + 16 * s4 * a ** 4 * f
    d22 = lambda a, b: 4 * s2 * f - 8 * s3 * b * b * f - 8 * s3 * a * a * f + 16 * s4 * a * a * b * b * f
    return 9 * np.sin(X) * np.sin(Y) * np.sin(Z) + d4(Xp) + 2 * d22(Xp, Yp) + 2 * d22(Xp, Zp) + d4(Yp) + 2 * d22(
        Yp, Zp) + d4(Zp)


def rel_l1(a, b):
    return np.abs(a - b).sum() / np.abs(b).sum()


def test_step5_operators_closed_form(oracle):
    """steps/step5/step5_gpu.cpp:559-699: operators against closed forms (rel. L1)."""
    n = (128, 128, 128)
    u, _ = step5_field(n)
    g = oracle.grad(u)
    for j, ref in enumerate(step5_grad(n)):
        assert rel_l1(g[j], ref) < 1e-10
    assert rel_l1(oracle.spectral_op(u, "laplace"), step5_laplace(n)) < 1e-10
    assert rel_l1(oracle.spectral_op(u, "biharmonic"), step5_biharmonic(n)) < 1e-8
    # divergence of the gradient equals the Laplacian (steps/step5/step5_gpu.cpp:460-467)
    assert rel_l1(oracle.divergence(*g), step5_laplace(n)) < 1e-10
    gs = oracle.grad_slow(u)
    for j in range(3):
        assert oracle.rel_l2(gs[j], g[j]) < 1e-12


def test_inv_laplace_inverts_laplace(oracle):
    """inv_laplace(laplace(u)) = u for zero-mean fields without Nyquist content."""
    n = (32, 24, 16)
    X, Y, Z = grid(n)
    u = np.sin(X) * np.cos(2 * Y) + 0.5 * np.sin(3 * Z + X)
    lap = oracle.spectral_op(u, "laplace")
    assert oracle.rel_l2(oracle.spectral_op(lap, "inv_laplace"), u) < 1e-13


def test_golden_fixtures(oracle):
    """Committed long-double fixtures (tests/golden/gen_golden.py)."""
    path = os.path.join(GOLDEN, "small_cases.npz")
    g = np.load(path)
    for key in g.files:
        if not key.endswith("_in"):
            continue
        name = key[:-3]
        meta = name.split("__")
        op, shape = meta[0], tuple(int(v) for v in meta[1].split("x"))
        x = g[key]
        y = g[name + "_out"]
        if op == "r2c":
            got = oracle.r2c(x)
        elif op == "c2r":
            got = oracle.c2r(x, shape[2])
        elif op == "c2cf":
            got = oracle.c2c(x, -1)
        elif op == "c2cb":
            got = oracle.c2c(x, 1)
        else:
            got = oracle.spectral_op(x, op)
        assert oracle.rel_l2(got, y) < 1e-14, name


def test_step4_poisson_sine_case(oracle):
    """steps/step4/step4_gpu.cpp:100-115 (testcase sine on the unit cube):
    method 1 returns the exact solution -rhs / (12 pi^2); method 0 returns the
    discrete solution rhs / (6 N^2 (cos(2 pi / N) - 1)) of the same mode."""
    N = 32
    x = np.arange(N) / N
    X, Y, Z = np.meshgrid(x, x, x, indexing="ij")
    rhs = np.sin(2 * np.pi * X) * np.sin(2 * np.pi * Y) * np.sin(2 * np.pi * Z)
    exact = -rhs / (3 * 4 * np.pi ** 2)
    assert oracle.rel_l2(oracle.spectral_op(rhs, "poisson_spec"), exact) < 1e-13
    discrete = rhs / (3 * 2 * N * N * (np.cos(2 * np.pi / N) - 1))
    assert oracle.rel_l2(oracle.spectral_op(rhs, "poisson_fd"), discrete) < 1e-13
