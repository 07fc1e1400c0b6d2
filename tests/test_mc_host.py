"""The motion-compensation helpers of the CUDA kernels (h264r_mc.cuh: the
4x2 luma interpolation, the 2x2 chroma interpolation and the weighting
formula) compiled as host C++ and checked on every fractional position
against scalar restatements of 8.4.2.2.1, 8.4.2.2.2 and 8.4.2.3
(tests/mc/mc_check.cpp)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))


def test_mc_helpers_match_scalar_formulas(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no host C++ compiler")
    exe = str(tmp_path / "mc_check")
    subprocess.run([cxx, "-O2", "-std=c++17", "-D__host__=", "-D__device__=", "-D__forceinline__=inline",
                    "-o", exe, os.path.join(HERE, "mc", "mc_check.cpp")], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip() == "ok"
