"""The C ABI library: it loads, exports every declared entry point, and
answers argument errors without a GPU (no compute call is made here)."""
import ctypes
import os
import subprocess

import numpy as np
import pytest

from conftest import ROOT


def test_library_exports_every_declared_symbol(em):
    lib = em.load()
    names = em.declared_symbols()
    assert len(names) >= 10
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing


def test_library_has_no_cpu_fallback_symbols(em):
    """The product library is CUDA-only: nothing from the oracle is linked."""
    out = subprocess.run(["nm", "-D", "--defined-only", em._capi.LIB_PATH],
                         capture_output=True, text=True).stdout
    assert "orc_" not in out and "ref_calc_field" not in out


def test_version_and_strerror(em):
    lib = em.load()
    assert lib.em_version().decode().count(".") == 2
    assert em.strerror(5) == "n is not a multiple of 64"
    assert em.strerror(12) == "device-side wait timed out"


def test_device_count_is_an_int(em):
    assert em.load().em_device_count() >= 0


@pytest.mark.parametrize("n,steps,res,curv,want", [
    (0, 4, 1.0, 1, 1), (64, 4, 0.0, 1, 2), (64, 1, 1.0, 1, 3),
    (32, 4, 1.0, 1, 5), (32, 1, 1.0, 1, 5)])
def test_reference_codes_before_any_device_work(em, n, steps, res, curv, want):
    """Codes 1/2/3/5 come from argument checks made before the device is
    touched (CPU_Implement.cpp:213-230), so they hold without a GPU."""
    x = np.zeros(max(n * steps, 1), np.float32)
    y, z = x.copy(), x.copy()
    ch = np.zeros((4, 4), np.float32)
    rc, _ = em.calc_field(x, y, z, ch, n, res, bool(curv), plain=True)
    assert rc == want


@pytest.mark.parametrize("dtype,kw", [
    (np.float64, dict(arith="mixed")),          # mixed arithmetic is FP32-only
    (np.float32, dict(arith="mixed", null_frac=-1.0)),
])
def test_option_errors_before_any_device_work(em, dtype, kw):
    """Option errors are argument errors (code 4), answered before the
    device is touched."""
    n, steps = 64, 4
    x = np.zeros(n * steps, dtype)
    y, z = x.copy(), x.copy()
    ch = np.zeros((4, 4), dtype)
    rc, _ = em.calc_field(x, y, z, ch, n, 1.0, True, **kw)
    assert rc == 4


@pytest.mark.parametrize("kw", [
    dict(warps_per_cta=-1), dict(warps_per_cta=33), dict(tile_charges=-1),
    dict(tile_charges=1 << 20), dict(threads_per_line=2)])
def test_extended_shape_overrides_checked_before_any_device_work(em, kw):
    """The extended tracer refuses launch-shape overrides it cannot run
    (code 4) before the device is touched; a tile of -1 records used to
    round to a zero tile."""
    seeds = np.zeros((8, 3), np.float32)
    ch = np.array([[0, 0, 0, 1]], np.float32)
    with pytest.raises(em.EmError) as e:
        em.trace_lines(seeds, ch, 4, 1.0, 0.5, **kw)
    assert e.value.code == 4


@pytest.mark.parametrize("tile", [-1, 1 << 20])
def test_batch_tile_override_checked_before_any_device_work(em, tile):
    sets = [(np.array([[0, 0, 0, 1]], np.float32), np.ones((4, 3), np.float32))]
    with pytest.raises(em.EmError) as e:
        em.trace_batch(sets, 4, 1.0, 0.5, tile_charges=tile)
    assert e.value.code == 4


def test_size_limits_before_any_device_work(em):
    """Sizes beyond what an entry point takes return EM_ERR_TOO_LARGE (14)
    from the argument checks, before any buffer is read or the device is
    touched: rows beyond 2^31 - 1 or more than 2^25 - 1 charges for a
    trace; more than 2^29 - 1 charges or points beyond 2^31 - 1 blocks of
    256 for the field at points."""
    lib = em._capi.load()
    a = np.zeros(64, np.float32)
    P = a.ctypes.data
    # rows beyond INT_MAX (n = 64)
    assert lib.em_calc_field_ex_f32(P, P, P, 64, 2 ** 31, P, 1, 1.0, 1,
                                    None, None) == 14
    # charges beyond INT_MAX / 64 (2^25 - 1)
    assert lib.em_calc_field_ex_f32(P, P, P, 64, 4, P, 2 ** 25, 1.0, 1,
                                    None, None) == 14
    # field points beyond the grid limit, charges beyond INT_MAX / 4
    assert lib.em_field_f32(P, P, P, (2 ** 31 - 1) * 256 + 1, P, 1,
                            P, P, P, None) == 14
    assert lib.em_field_f32(P, P, P, 64, P, 2 ** 29, P, P, P, None) == 14


def test_dropin_header_compiles_against_stand_in_types(tmp_path):
    """include/emgb300_dropin.hpp (the CalcField_CPU / CalcField overloads)
    compiles and links against libemgb300.so with containers shaped like
    the reference's (own stand-ins, no reference code)."""
    src = os.path.join(ROOT, "tests", "dropin_check.cpp")
    exe = tmp_path / "dropin_check"
    lib = os.path.join(ROOT, "electromag-with-cuda_gb300")
    r = subprocess.run(["g++", "-std=c++11", "-Wall", "-Werror", src,
                        "-I" + os.path.join(ROOT, "include"), "-L" + lib,
                        "-lemgb300", "-Wl,-rpath," + lib, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    # without a GPU the traced call reports EM_ERR_NO_DEVICE (13); with one
    # it succeeds; the argument-check calls return the reference's codes
    assert r.returncode == 0, r.stdout + r.stderr


REFERENCE = os.environ.get("EM_REFERENCE_DIR", "/root/reference")


@pytest.mark.skipif(not os.path.isfile(os.path.join(
    REFERENCE, "ElectroMag", "src", "CPU Implement.h")),
    reason="reference tree not present")
def test_dropin_against_reference_headers(tmp_path):
    """The reference-side CalcField_CPU forwards compile against its own
    headers, link against libemgb300.so and return its argument codes."""
    src = os.path.join(ROOT, "tests", "dropin_reference_headers.cpp")
    exe = tmp_path / "dropin_ref"
    lib = os.path.join(ROOT, "electromag-with-cuda_gb300")
    r = subprocess.run(["g++", "-std=c++11", src,
                        "-I" + os.path.join(REFERENCE, "include"),
                        "-I" + os.path.join(REFERENCE, "ElectroMag", "src"),
                        "-I" + os.path.join(ROOT, "include"), "-L" + lib,
                        "-lemgb300", "-Wl,-rpath," + lib, "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
