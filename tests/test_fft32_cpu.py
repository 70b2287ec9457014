"""The register-blocked Stockham line transform of the FP32 FFTs
(crocodile_gb300/csrc/fft32.h, plain C++ compiled for the host) against a
direct DFT in double precision for N = 32 .. 8192 and both signs, and its
per-stage twiddle tables against the exact values (tests/fft32_check.cpp)."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_line_transform_matches_direct_dft(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "fft32_check")
    subprocess.run([gxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "crocodile_gb300", "csrc"),
                    os.path.join(HERE, "fft32_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    worst = float(r.stdout.strip().splitlines()[-1].split()[-1])
    assert worst < 1e-6
