"""Failure paths on the GPU without a fault: a bounded device wait that is
made to expire returns an error status and leaves the device usable; an
injected allocation failure comes back as EM_ERR_NOMEM."""
import ctypes
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import ROOT, lines_from

pytestmark = pytest.mark.gpu


def test_bounded_wait_times_out_and_device_stays_usable(em, gpu):
    ms = ctypes.c_double()
    rc = gpu.em_selftest_wait_timeout(100, ctypes.byref(ms))
    assert rc == em._capi.EM_ERR_TIMEOUT
    assert 90.0 <= ms.value <= 2000.0, ms.value
    # the context still works: a small trace succeeds afterwards
    ch, seeds, _ = em.workloads.make("cpu_256", seed=1)
    x, y, z = lines_from(seeds[:64].astype(np.float32), 8, np.float32)
    rc, _ = em.calc_field(x, y, z, ch, 64, 1.0, True)
    assert rc == 0


def test_injected_allocation_failure_returns_nomem(em, gpu):
    code = r"""
import importlib, sys, numpy as np
sys.path.insert(0, %r)
em = importlib.import_module("electromag-with-cuda_gb300")
ch, seeds, _ = em.workloads.make("cpu_256", seed=1)
s = seeds[:64].astype(np.float32)
x, y, z = em.new_lines(s, 8)
rc, _ = em.calc_field(x, y, z, ch, 64, 1.0, True)
print("RC", rc)
x, y, z = em.new_lines(s, 8)
rc2, _ = em.calc_field(x, y, z, ch, 64, 1.0, True)
print("RC2", rc2)
""" % ROOT
    env = dict(os.environ, EM_INJECT_ALLOC_FAIL="1")
    r = subprocess.run([sys.executable, "-c", code], capture_output=True,
                       text=True, env=env, timeout=300)
    assert "RC 11" in r.stdout, r.stdout + r.stderr
    # the next call allocates normally and succeeds
    assert "RC2 0" in r.stdout, r.stdout + r.stderr
