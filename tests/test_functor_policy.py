"""The multi-device functor's lifecycle and remap policy (the reference's
AbstractFunctor, GPGPU_Segment/src/Abstract_Functor.cpp:29-160) on fake
devices: tests/functor_policy_check.cpp is compiled against
include/emgb300_functor.hpp and run on the CPU; failures are injected on the
host (devices that fail every functor), never on a GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_remap_policy_on_fake_devices(tmp_path):
    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    exe = tmp_path / "functor_policy_check"
    subprocess.check_call([cxx, "-std=c++17", "-O1", "-pthread",
                           "-I", os.path.join(ROOT, "include"),
                           os.path.join(ROOT, "tests", "functor_policy_check.cpp"),
                           "-o", str(exe)])
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.count("ok ") == 8
