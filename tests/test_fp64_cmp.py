"""The integer-pipe double comparisons the right-hand-side kernels use
(csrc/fp64_cmp.h) against the C comparison operators, on the host: the
header compiles as plain C++ with g++, and every helper must agree with
<, <=, >, >=, == and isnan on signed zeros, subnormals, infinities, NaNs and
random values."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(os.path.dirname(HERE), "pihm-cuda_gb300", "csrc")


@pytest.mark.parametrize("opt", ["-O0", "-O2"])
def test_fp64_cmp_matches_c_comparisons(tmp_path, opt):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("g++ not found")
    exe = str(tmp_path / "fp64_cmp_check")
    subprocess.run([gxx, "-std=c++17", opt, "-I", CSRC, os.path.join(HERE, "fp64_cmp_check.cpp"),
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout
