"""The kernels' integer-pipe float<->double conversions (hydro_gb300/csrc/
fpconv.h) give the IEEE results: every float widened exactly, doubles
narrowed with rounding to nearest, ties to even, as the host converts them
(tests/fpconv_check.cpp, compiled with the host compiler)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_conversions_match_host(tmp_path):
    cxx = shutil.which("g++") or shutil.which("c++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "fpconv_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "hydro_gb300", "csrc"),
                    os.path.join(ROOT, "tests", "fpconv_check.cpp"), "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0 and r.stdout.startswith("ok"), r.stdout + r.stderr
