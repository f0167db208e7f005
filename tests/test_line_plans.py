"""Radix plans (accfft_gb300/csrc/line_plan.h), compiled on the host with
g++: the library's accfft_c_line_plan (what the batch reports print)
returns exactly the header's plans for every supported length and all three
arithmetic types, and double-float plans keep the first radix at 8 or below
wherever such a plan exists (falling back to the double plan elsewhere).
No GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r'''
#include <cstdio>
#include <cstdlib>
#include "line_plan.h"
int main(int argc, char** argv) {
  for (int i = 1; i < argc; ++i) {
    const int L = atoi(argv[i]);
    for (int cls = 0; cls < 3; ++cls) {
      afg::LinePlan pl = afg::plan_select(L, cls, 0);
      printf("%d %d %d %d", L, cls, pl.E, pl.P);
      for (int s = 0; s < pl.ns; ++s) printf(" %d", pl.radix[s]);
      printf("\n");
    }
  }
  return 0;
}
'''


@pytest.fixture(scope="module")
def plans(tmp_path_factory, native):
    if shutil.which("g++") is None:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("plans")
    src, exe = d / "plans.cpp", d / "plans"
    src.write_text(PROGRAM)
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "accfft_gb300", "csrc"), str(src), "-o",
                    str(exe)], check=True)
    lengths = [L for L in range(1, 1025) if native.lib().accfft_c_length_supported(L)]
    out = subprocess.run([str(exe)] + [str(L) for L in lengths], check=True, capture_output=True, text=True).stdout
    res = {}
    for line in out.split("\n"):
        if line.strip():
            v = [int(x) for x in line.split()]
            res[(v[0], v[1])] = {"E": v[2], "P": v[3], "radices": v[4:]}
    return lengths, res


def test_library_reports_the_compiled_plans(plans, native):
    from accfft_gb300.batch import radix_plan

    lengths, res = plans
    assert len(lengths) >= 30
    for L in lengths:
        for cls, prec in ((0, "float32"), (1, "float64"), (2, "double-float")):
            assert native.line_plan(L, prec) == res[(L, cls)], (L, prec)
        assert radix_plan(L, "float32") == res[(L, 0)]
    with pytest.raises(native.AccfftError):
        native.line_plan(37)


def _has_small_plan(L):
    """Some first radix E <= 8 whose greedy factorisation of L / E uses only divisors of E."""
    for E in range(2, min(L, 8) + 1):
        if L % E:
            continue
        rem, ok = L // E, True
        while rem > 1:
            d = next((c for c in range(E, 1, -1) if E % c == 0 and rem % c == 0), 0)
            if d == 0:
                ok = False
                break
            rem //= d
        if ok:
            return True
    return False


def test_double_float_plans_keep_small_radices(plans):
    lengths, res = plans
    for L in lengths:
        if L == 1:
            continue
        df, dbl = res[(L, 2)], res[(L, 1)]
        assert df["E"] * df["P"] == L and all(r <= df["E"] for r in df["radices"])
        if _has_small_plan(L):
            assert df["E"] <= 8, L
        else:
            assert df == dbl, L
    # the 512-point lines of the headline grid: radix 8 in three stages
    assert res[(512, 2)]["radices"] == [8, 8, 8]
