"""Double-float arithmetic of the mixed form's Schur operator
(zeroslam_gb300/csrc/ba_df.cuh) on the host: exact error-free
transformations and the error bounds the operator relies on
(tests/cpp/df_test.cpp, against long double references)."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.mark.skipif(not shutil.which("g++"), reason="needs g++")
def test_double_float_bounds(tmp_path):
    exe = str(tmp_path / "df_test")
    cmd = ["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "zeroslam_gb300", "csrc"),
           os.path.join(ROOT, "tests", "cpp", "df_test.cpp"), "-o", exe]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "OK", r.stdout + r.stderr
