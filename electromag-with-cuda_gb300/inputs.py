"""The reference program's inputs: its presets (ElectroMag.cpp:43-55) and
its charge and line generators ("Electromag utils.h":29-111), through the C
ABI (em_preset, em_init_charges_*, em_init_lines_*).

reference_case() assembles what the reference's main() traces for a preset:
InitializePointChargeArray with srand(1) (ElectroMag.cpp:251), grid seeds
(:266), `len` rows per line, resolution 1, curvature on.
"""
import ctypes

import numpy as np

from . import _capi

PRESET_NAMES = ("normal", "enhanced", "extreme", "insane", "fuckingInsane",
                "cpu", "micro", "bogo")


def preset(name):
    """dict(nx, ny, nz, p_static, p_dynamic, len) of a preset."""
    out = _capi.EmPresetParams()
    rc = _capi.load().em_preset(name.encode(), ctypes.byref(out))
    if rc:
        raise _capi.EmError(rc, f"em_preset({name!r})")
    return {k: int(getattr(out, k)) for k, _ in out._fields_}


def init_charges(p, seed=1, dtype=np.float32):
    """(p, 4) {x, y, z, q} as InitializePointChargeArray draws them after
    srand(seed) (the reference: seed 1)."""
    dt = np.dtype(dtype)
    out = np.zeros((p, 4), dt)
    fn = (_capi.load().em_init_charges_f32 if dt == np.float32
          else _capi.load().em_init_charges_f64)
    rc = fn(out.ctypes.data, p, int(seed) & 0xffffffff)
    if rc:
        raise _capi.EmError(rc, "em_init_charges")
    return out


def init_lines(nx, ny, nz, random=False, seed=1, dtype=np.float32):
    """(3, nx*ny*nz) seeds as InitializeFieldLineArray places them: the grid
    (default) or random positions after srand(seed)."""
    dt = np.dtype(dtype)
    n = nx * ny * nz
    out = np.zeros((3, n), dt)
    fn = (_capi.load().em_init_lines_f32 if dt == np.float32
          else _capi.load().em_init_lines_f64)
    rc = fn(out[0].ctypes.data, out[1].ctypes.data, out[2].ctypes.data, nx, ny,
            nz, int(bool(random)), int(seed) & 0xffffffff)
    if rc:
        raise _capi.EmError(rc, "em_init_lines")
    return out


def reference_case(name="normal", dtype=np.float32, randseed=None):
    """(charges (p, 4), seeds (n, 3), rows) of the reference's run for a
    preset; randseed replaces srand(1) (the reference's --randseed)."""
    pr = preset(name)
    ch = init_charges(pr["p_static"], 1 if randseed is None else randseed,
                      dtype)
    seeds = init_lines(pr["nx"], pr["ny"], pr["nz"], dtype=dtype).T.copy()
    return ch, seeds, pr["len"]
