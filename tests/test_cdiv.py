"""Exact division by the flux denominators 12 and 60 (wrf_gb300/csrc/cdiv.h).

The kernels replace x / 12 and x / 60 of the advection operators
(module_advect_em.F:172-186) by a multiply and two fmas; the result must be
the IEEE-rounded quotient bit for bit, or the plain form would drift from the
reference's rounding.  The check is host code compiled with gcc."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.mark.skipif(shutil.which("gcc") is None, reason="gcc not available")
def test_div_const_matches_ieee(tmp_path):
    exe = str(tmp_path / "cdiv_check")
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-o", exe,
                    os.path.join(HERE, "native", "cdiv_check.c"), "-lm"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0 mismatches" in r.stdout


@pytest.mark.gpu
def test_paired_flux_helpers_match_scalar(gpulib, tmp_path):
    """The two-species packed arithmetic of the scalar transport kernels
    (wrf_gb300/csrc/pair.cuh) gives each lane exactly the scalar helper's
    bits: flux5, flux3, pflux5, pflux3, the upwind flux and the packed
    add / sub / mul, on 2^20 random input pairs (tests/native/pair_check.cu)."""
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    exe = str(tmp_path / "pair_check")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "--fmad=false", "-std=c++17",
                    "--expt-relaxed-constexpr", "-o", exe, os.path.join(HERE, "native", "pair_check.cu")],
                   check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    lines = [ln for ln in r.stdout.splitlines() if "mismatches" in ln]
    assert len(lines) == 8 and all(ln.split()[-1] == "0" for ln in lines), r.stdout
