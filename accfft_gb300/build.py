"""Build the accfft_gb300 native libraries in-tree (sm_103a only).

    python -m accfft_gb300.build            # or accfft_gb300.build.build()

Products (git-ignored, under accfft_gb300/lib/):
    libaccfft_gb300.so  kernels + plan layer + C ABI (include/accfft_gb300.h)
    libaccfft_gpu.so    C++ API mirroring AccFFT's accfft_gpu.h / accfft_gpuf.h /
                        accfft_operators_gpu.h, layered on the C ABI

kernels.cu is compiled once per (precision, kernel kind, length group) so the
template instantiations build in parallel; objects are rebuilt only when a
source or header changed.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "lib")
OBJ = os.path.join(LIB, "obj")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr"] + ARCH
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-Wall", "-Wno-unused-function"]
KINDS = 5     # strided, zc2c, zr2c, zc2r, zsym
GROUPS = 2


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _digest(paths, extra) -> str:
    h = hashlib.sha256()
    for p in paths:
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(repr(extra).encode())
    return h.hexdigest()


def _headers():
    out = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC)) if f.endswith((".h", ".cuh"))]
    out += [os.path.join(INCLUDE, f) for f in sorted(os.listdir(INCLUDE)) if f.endswith(".h")]
    return out


def _compile(job):
    src, obj, cmd, key = job
    stamp = obj + ".sha"
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == key:
        return obj, False, ""
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as f:
        f.write(key)
    return obj, True, r.stderr


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile both libraries; returns the path of libaccfft_gb300.so."""
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()
    cuda_inc = os.path.join(_cuda_home(), "include")
    hdrs = _headers()
    work = []
    ksrc = os.path.join(CSRC, "kernels.cu")
    for prec in (0, 1, 2):
        for kind in range(KINDS):
            if prec == 2 and kind == 4:      # double-float: no symbol kernels
                continue
            for grp in range(GROUPS):
                obj = os.path.join(OBJ, f"kernels_p{prec}_k{kind}_g{grp}.o")
                cmd = [nvcc, *NVCC_FLAGS, f"-DAFG_PREC={prec}", f"-DAFG_KIND={kind}", f"-DAFG_GROUP={grp}",
                       "-c", ksrc, "-o", obj]
                work.append((ksrc, obj, cmd, _digest([ksrc] + hdrs, cmd[1:])))
    for name in ("plan.cpp", "dispatch.cpp"):
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJ, name.replace(".cpp", ".o"))
        cmd = ["g++", *CXX_FLAGS, "-I", cuda_inc, "-c", src, "-o", obj]
        work.append((src, obj, cmd, _digest([src] + hdrs, cmd[1:])))
    for name in ("noalloc.cu", "slab.cu", "tc_kernels.cu", "zy_fused.cu", "df_scale.cu", "accum.cu", "variants.cu",
                 "sym_spectrum.cu", "gen.cu"):
        src = os.path.join(CSRC, name)
        obj = os.path.join(OBJ, name.replace(".cu", ".o"))
        cmd = [nvcc, *NVCC_FLAGS, "-c", src, "-o", obj]
        work.append((src, obj, cmd, _digest([src] + hdrs, cmd[1:])))
    # heaviest translation units first
    work.sort(key=lambda w: ("_k0_" not in w[1], "_g1" not in w[1]))
    n = jobs or max(1, os.cpu_count() or 1)
    with ThreadPoolExecutor(max_workers=n) as ex:
        results = list(ex.map(_compile, work))
    rebuilt = any(r[1] for r in results)
    if verbose:
        for obj, did, log in results:
            if did and log.strip():
                print(log)
    core = os.path.join(LIB, "libaccfft_gb300.so")
    objs = [r[0] for r in results]
    if rebuilt or not os.path.exists(core):
        cmd = [nvcc, *ARCH, "-shared", "-o", core, *objs, "-Xlinker", "-z,defs", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    # C++ API layer over the C ABI
    api_src = os.path.join(CSRC, "accfft_gpu_api.cpp")
    api = os.path.join(LIB, "libaccfft_gpu.so")
    if os.path.exists(api_src):
        key = _digest([api_src] + hdrs, ["api"])
        stamp = api + ".sha"
        if rebuilt or not os.path.exists(api) or not os.path.exists(stamp) or open(stamp).read() != key:
            cmd = ["g++", *CXX_FLAGS, "-shared", "-I", INCLUDE, "-I", os.path.join(INCLUDE, "mpi_shim"),
                   "-I", cuda_inc, api_src, "-o", api, "-L", LIB, "-laccfft_gb300", "-Wl,-rpath,$ORIGIN"]
            r = subprocess.run(cmd, capture_output=True, text=True)
            if r.returncode != 0:
                raise RuntimeError(f"API layer build failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
            with open(stamp, "w") as f:
                f.write(key)
    return core


if __name__ == "__main__":
    path = build(verbose="-v" in sys.argv)
    print(path)
