"""Build recipe for oracle/_ref: AccFFT's own CPU host code as the parity reference.

TEST INFRASTRUCTURE ONLY.  Compiles the reference's unmodified sources where
they lie (src/accfft.cpp, src/accfft_common.cpp, src/operators.cpp,
src/transpose.cpp, headers from include/) together with
  - oracle/ref_shim/mpi.h + ref_shim.c: MPI on one rank,
  - oracle/ref_shim/fftw3.h + ref_shim.c: the FFTW3 calls, computed by the
    oracle's long-double DFT,
  - oracle/ref_driver.cpp: extern "C" entry points over the reference's API,
into oracle/_ref/libaccfft_ref.so.  Nothing is copied out of the reference
tree.  The reference's own build system (CMake, real MPI and FFTW) is not
used: neither MPI nor FFTW exists on these machines.

Usage: python oracle/build_ref.py [REFERENCE_ROOT]   (default /root/reference,
or $ACCFFT_REFERENCE_ROOT).  build() returns the library path, or None when
the reference tree is absent (machines that only run the committed fixtures).
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT_DIR = os.path.join(HERE, "_ref")
LIB = os.path.join(OUT_DIR, "libaccfft_ref.so")
REF_SOURCES = ["src/accfft.cpp", "src/accfft_common.cpp", "src/operators.cpp", "src/transpose.cpp"]


def reference_root(arg=None):
    return arg or os.environ.get("ACCFFT_REFERENCE_ROOT") or "/root/reference"


def build(root=None, verbose=False):
    root = reference_root(root)
    if not all(os.path.isfile(os.path.join(root, s)) for s in REF_SOURCES):
        return None
    os.makedirs(OUT_DIR, exist_ok=True)
    shim = os.path.join(HERE, "ref_shim")
    inc = ["-I", shim, "-I", os.path.join(root, "include")]
    # the reference is written for older compilers: keep its warnings quiet
    cxx = ["g++", "-std=c++11", "-O2", "-fPIC", "-fopenmp", "-w"] + inc
    jobs = []
    for s in REF_SOURCES:
        obj = os.path.join(OUT_DIR, os.path.basename(s).replace(".cpp", ".o"))
        jobs.append((cxx + ["-c", os.path.join(root, s), "-o", obj], obj))
    drv = os.path.join(OUT_DIR, "ref_driver.o")
    jobs.append((cxx + ["-c", os.path.join(HERE, "ref_driver.cpp"), "-o", drv], drv))
    sh = os.path.join(OUT_DIR, "ref_shim.o")
    jobs.append((["gcc", "-std=gnu11", "-O2", "-fPIC", "-w", "-I", shim, "-c", os.path.join(shim, "ref_shim.c"),
                  "-o", sh], sh))

    def run(cmd):
        if verbose:
            print(" ".join(cmd))
        subprocess.run(cmd, check=True)

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, [j[0] for j in jobs]))
    run(["g++", "-shared", "-fopenmp", "-Wl,--no-undefined", "-o", LIB] + [j[1] for j in jobs] + ["-lpthread", "-lm"])
    return LIB


if __name__ == "__main__":
    path = build(sys.argv[1] if len(sys.argv) > 1 else None, verbose=True)
    print(path or "reference tree not found: nothing built")
