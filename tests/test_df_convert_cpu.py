"""The integer FP64 <-> double-float conversions of the device code
(crocodile_gb300/csrc/df_convert.h, plain C++) compiled for the host and
checked bit for bit against the FP64 forms they replace on 15 million cases
(tests/df_convert_check.cpp)."""

import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_split_and_join_match_fp64(tmp_path):
    gxx = shutil.which("g++")
    if gxx is None:
        pytest.skip("no g++")
    exe = str(tmp_path / "df_convert_check")
    subprocess.run([gxx, "-O2", "-ffp-contract=off", "-std=c++17", "-I",
                    os.path.join(ROOT, "crocodile_gb300", "csrc"),
                    os.path.join(HERE, "df_convert_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "split: 0 of" in r.stdout and "join: 0 of" in r.stdout
