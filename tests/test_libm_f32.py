"""The device's acosf / atanf / atan2f (physecs_gb300/csrc/libm_f32.cuh) against the host's
C library, whose results the reference's servo and gear rows use.

The header compiles as plain C++; tests/libm/check_libm.cpp compares it, bit for bit,
with the C library on every float in [-1, 1] (acosf) and on seeded arguments (atanf,
atan2f: random bit patterns, moderate angles, special values)."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_restated_libm_equals_the_c_library(tmp_path):
    if shutil.which("g++") is None:
        pytest.skip("no g++")
    import platform
    exe = str(tmp_path / "check_libm")
    fused = ["-DPSX_LIBM_FUSED"] if platform.machine() in ("aarch64", "arm64") else []   # as the build sets it
    subprocess.run(["g++", "-O2", "-ffp-contract=off", "-std=c++17"] + fused +
                   ["-I", os.path.join(ROOT, "physecs_gb300", "csrc"), os.path.join(HERE, "libm", "check_libm.cpp"),
                    "-o", exe], check=True)
    r = subprocess.run([exe, "4000000"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    assert " 0/" in r.stdout
