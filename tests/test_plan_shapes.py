"""The launch planner's shape choices (csrc/em_plan.h) on a model of a
GB300: tests/plan_shape_check.cpp is compiled against the library's own
headers and run on the CPU (no device calls)."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA_INC = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "include")


def test_planner_shapes(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None or not os.path.exists(os.path.join(CUDA_INC, "cuda_runtime.h")):
        pytest.skip("no C++ compiler or CUDA headers")
    exe = tmp_path / "plan_shape_check"
    subprocess.check_call([cxx, "-std=c++17", "-O1",
                           "-I", os.path.join(ROOT, "include"),
                           "-I", os.path.join(ROOT, "electromag-with-cuda_gb300", "csrc"),
                           "-I", CUDA_INC,
                           os.path.join(ROOT, "tests", "plan_shape_check.cpp"),
                           "-o", str(exe)])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok ") == 12
