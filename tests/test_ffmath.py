"""Correctly rounded log / pow of the equation of state (wrf_gb300/csrc/ffmath.h).

calc_p_rho_phi (module_big_step_utilities_em.F:953-1226) needs LOG and
x**cpovcv; the kernels evaluate them in table-driven float-float arithmetic
and round once, with a Ziv rounding test that sends ambiguous cases to FP64.
The host build of the same code is checked here: equal to the FP64 result
rounded to float on every float in [1/4, 4) and on samples elsewhere, and
with a float-float error far below the rounding test's bound."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("g++") is None, reason="g++ not available")
def test_ffmath_correct_rounding(tmp_path):
    exe = str(tmp_path / "ffmath_check")
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17", "-o", exe,
                    os.path.join(HERE, "native", "ffmath_check.cpp"), "-lm"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout
