"""The C++ API (AccFFT's accfft_gpu.h / accfft_gpuf.h / accfft_operators_gpu.h
signatures) compiled into an AccFFT-style program: it must compile and link
on any machine, and pass its step1/2/3/5-style checks on a GPU."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "api_steps.cpp")
LIBDIR = os.path.join(ROOT, "accfft_gb300", "lib")


def cuda_home():
    for c in ("/usr/local/cuda",):
        if os.path.exists(os.path.join(c, "include", "cuda_runtime_api.h")):
            return c
    pytest.skip("CUDA toolkit headers not found")


def build_program(tmp_path):
    cuda = cuda_home()
    exe = str(tmp_path / "api_steps")
    cmd = ["g++", "-std=c++17", "-O2", "-Wall", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(ROOT, "include", "mpi_shim"), "-I", os.path.join(cuda, "include"), SRC, "-o", exe,
           "-L", LIBDIR, "-laccfft_gpu", "-laccfft_gb300", f"-Wl,-rpath,{LIBDIR}",
           "-L", os.path.join(cuda, "lib64"), "-lcudart", f"-Wl,-rpath,{os.path.join(cuda, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_program_compiles_and_links(native, tmp_path):
    assert os.path.exists(build_program(tmp_path))


@pytest.mark.gpu
def test_program_passes_on_gpu(native, tmp_path):
    exe = build_program(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "NOT CORRECT" not in r.stdout
    assert r.stdout.count("CORRECT") >= 10
    assert "plan has not been made correctly" in r.stdout
