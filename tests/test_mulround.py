"""CPU: the integer restatement of the plastic traces' skip() rounding, (float)((double)x * f)
(spice2_gb300/csrc/mulround.h), against the host's IEEE double multiply and float conversion:
random pairs over every float exponent, the skip factors of several traces, and constructed
products next to float rounding ties (tests/mulround_check.cpp).  The GPU self-test
(test_gpu_plastic.py) compares the same function with the GPU's double multiply."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_mul_f32_f64_rn_matches_the_double_multiply(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "mulround_check"
    subprocess.run([cxx, "-std=c++17", "-O2", "-fno-fast-math", "-ffp-contract=off",
                    "-I", os.path.join(ROOT, "spice2_gb300", "csrc"), os.path.join(ROOT, "tests", "mulround_check.cpp"),
                    "-o", str(exe)], check=True)
    out = subprocess.run([str(exe), "2000000"], capture_output=True, text=True)
    assert out.returncode == 0, out.stdout + out.stderr
    assert "mismatches 0" in out.stdout, out.stdout
