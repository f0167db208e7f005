"""C ABI checks that need no GPU: the library loads, exports every symbol the
header declares, answers the local-size queries like the reference, and turns
bad plans into errors instead of crashes."""
import ctypes
import subprocess

import pytest


def test_exports_every_declared_symbol(native):
    L = native.lib()
    names = native.header_symbols()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing


def test_library_is_sm103a_and_exports_cabi(native):
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True, text=True).stdout
    for n in native.header_symbols():
        assert f" T {n}" in out, n


def ref_local_size_r2c(n, rb):
    """accfft_local_size_dft_r2c_t (src/accfft_common.cpp:98-192) at P = 1."""
    nt = (n[2] // 2 + 1) * 2
    amax = max(n[0] * n[1] * nt * rb,
               2 * n[0] * (nt // 2) * n[1] * rb,
               2 * n[1] * (nt // 2) * n[0] * rb,
               n[0] * n[2] * n[1] * rb,
               2 * n[0] * n[2] * (n[1] // 2 + 1) * rb,
               n[0] * n[1] * n[2] * rb,
               2 * (n[0] // 2 + 1) * n[1] * n[2] * rb)
    return amax, (n[0], n[1], n[2]), (n[0], n[1], n[2] // 2 + 1)


@pytest.mark.parametrize("n", [(128, 128, 128), (512, 512, 512), (160, 180, 200), (1024, 1024, 1024), (5, 9, 4)])
@pytest.mark.parametrize("rb", [4, 8])
def test_local_size_r2c(native, n, rb):
    amax, isz, ist, osz, ost = native.local_size_r2c(n, rb)
    ramax, risz, rosz = ref_local_size_r2c(n, rb)
    assert (amax, isz, osz) == (ramax, risz, rosz)
    assert ist == (0, 0, 0) and ost == (0, 0, 0)


def test_local_size_known_values(native):
    # figures quoted for the reference's configurations
    assert native.local_size_r2c((128, 128, 128), 8)[0] == 17_039_360
    assert native.local_size_r2c((512, 512, 512), 8)[0] == 1_077_936_128
    assert native.local_size_r2c((1024, 1024, 1024), 4)[0] == 4_303_355_904   # beyond int: 64-bit here
    assert native.local_size_c2c((512, 512, 512), 8)[0] == 2_147_483_648
    assert native.local_size_c2c((256, 256, 256), 8)[0] == 268_435_456


def test_supported_lengths(native):
    L = native.lib()
    for n in (1, 2, 4, 8, 16, 32, 64, 128, 256, 512, 1024, 48, 90, 96, 100, 160, 180, 192, 200):
        assert L.accfft_c_length_supported(n) == 1, n
    for n in (7, 11, 13, 17, 1000003):
        assert L.accfft_c_length_supported(n) == 0, n
    # lengths without compiled kernels that the generic kernels take: prime
    # factors up to 31, at most 4096
    for n in (7, 11, 13, 14, 18, 27, 31, 36, 62, 121, 2048, 4096):
        assert L.accfft_c_length_generic(n) == 1, n
    for n in (37, 74, 97, 4100, 1000003):
        assert L.accfft_c_length_generic(n) == 0, n


def test_plan_rejects_bad_sizes(native):
    L = native.lib()
    n = (ctypes.c_int * 3)(8, 8, 74)
    assert not L.accfft_c_plan_dft_3d_r2c_gpuf(n, None, None, 2)
    assert "length 74" in native.last_error()
    n = (ctypes.c_int * 3)(8, 37, 8)
    assert not L.accfft_c_plan_dft_3d_c2c_gpu(n, None, None, 2)
    assert "length 37" in native.last_error()
    assert L.accfft_c_last_error_code() == native.EUNSUPPORTED
    # double-float plans need compiled lengths (rejected before any device call)
    n = (ctypes.c_int * 3)(8, 13, 8)
    assert not L.accfft_c_plan_dft_3d_r2c_gpu(n, None, None, native.F64_DF)
    assert L.accfft_c_last_error_code() == native.EUNSUPPORTED
    n = (ctypes.c_int * 3)(0, 8, 8)
    assert not L.accfft_c_plan_dft_3d_r2c_gpu(n, None, None, 2)
    assert L.accfft_c_last_error_code() == native.EINVAL
    # the tensor-core forms are float r2c plans only (rejected before any device call)
    n = (ctypes.c_int * 3)(128, 128, 256)
    assert not L.accfft_c_plan_dft_3d_r2c_gpu(n, None, None, native.TC_TF32)
    assert L.accfft_c_last_error_code() == native.EUNSUPPORTED
    n = (ctypes.c_int * 3)(96, 128, 256)
    assert not L.accfft_c_plan_dft_3d_r2c_gpuf(n, None, None, native.TC_BF16)
    assert "tensor-core" in native.last_error()


def test_python_plan_errors_carry_the_code(native):
    with pytest.raises(native.AccfftError) as e:
        native.PlanR2C((8, 37, 8), "float32")
    assert e.value.code == native.EUNSUPPORTED
    with pytest.raises(native.AccfftError) as e:
        native.PlanC2C((0, 8, 8), "float64")
    assert e.value.code == native.EINVAL


def test_null_plan_is_an_error(native):
    L = native.lib()
    rc = L.accfft_c_execute_r2c_gpu(None, None, None, None, 7)
    assert rc == native.EINVAL
    assert "NULL plan" in native.last_error()
    assert L.accfft_c_laplace(None, None, None, None) == native.EINVAL


def test_pdl_switch_queries_and_restores(native):
    """The launch-overlap switch is process state with query (-1) semantics;
    no GPU is touched."""
    prev = native.set_pdl(None)
    assert prev in (0, 1, 2)
    try:
        assert native.set_pdl(0) == prev
        assert native.set_pdl(None) == 0
        assert native.set_pdl(2) == 0
        assert native.set_pdl(9) == 2       # clamped
        assert native.set_pdl(None) == 2
    finally:
        native.set_pdl(prev)


def test_double_float_flag_needs_a_double_plan(native):
    with pytest.raises(native.AccfftError) as e:
        native.PlanR2C((8, 8, 8), "float32", flags=native.F64_DF)
    assert e.value.code == native.EUNSUPPORTED
    assert "double plans" in str(e.value)


@pytest.mark.parametrize("env,mode", [("0", 0), ("1", 1), ("2", 2), ("7", 1), ("", 1), ("off", 1)])
def test_pdl_mode_from_environment(native, env, mode):
    """ACCFFT_GB300_PDL is read on first use: 0, 1 or 2, anything else the
    default (1)."""
    import os
    import sys

    code = "import accfft_gb300 as ag; print(ag.set_pdl(None))"
    e = dict(os.environ, ACCFFT_GB300_PDL=env)
    out = subprocess.run([sys.executable, "-c", code], env=e, capture_output=True, text=True, check=True,
                         cwd=os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    assert int(out.stdout.strip().splitlines()[-1]) == mode
