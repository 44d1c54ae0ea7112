"""Generate tests/golden/reference_inputs.npz from the reference itself.

Runs only where the reference sources exist: it loads
oracle/_ref/libemref_inputs.so (built by oracle/build_ref.sh from the
reference's "Electromag utils.h" generators) and records

  charges_<dt>_p<p>     InitializePointChargeArray(p, random=false), i.e. the
                        srand(1) stream ("Electromag utils.h":91-111)
  grid_<dt>_<w>x<h>x<d> InitializeFieldLineArray grid mode (:29-70)
  rand_<seed>           the first 2000 rand() values after srand(seed)

Large arrays are stored as a SHA-256 of their bytes plus a sample.

    python tests/golden/make_inputs_golden.py
"""
import ctypes
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
LIB = os.path.join(ROOT, "oracle", "_ref", "libemref_inputs.so")
P, S = ctypes.c_void_p, ctypes.c_size_t

CHARGE_SIZES = (50, 1000, 1024, 2048, 5120)   # the presets' charge counts
GRIDS = ((16, 16, 1), (7, 5, 3), (64, 64, 1), (128, 128, 1), (256, 112, 1),
         (1024, 1024, 1))
SEEDS = (1, 0, 12345, 2**31 + 5, 2**32 - 1)
FULL_LIMIT = 4096   # arrays with more elements per component keep a hash


def main():
    if not os.path.exists(LIB):
        sys.exit("oracle/_ref/libemref_inputs.so missing: run bash oracle/build_ref.sh")
    lib = ctypes.CDLL(LIB)
    out, meta = {}, {"generator": "tests/golden/make_inputs_golden.py",
                     "machine": os.uname().machine, "sha256": {}}
    for dt, tag in ((np.float32, "f32"), (np.float64, "f64")):
        fn = getattr(lib, f"ref_init_charges_{tag}")
        fn.argtypes = [P, S]
        for p in CHARGE_SIZES:
            a = np.zeros((p, 4), dt)
            fn(a.ctypes.data, p)
            key = f"charges_{tag}_p{p}"
            meta["sha256"][key] = hashlib.sha256(a.tobytes()).hexdigest()
            out[key] = a if p <= FULL_LIMIT // 4 else a[::97]
        fn = getattr(lib, f"ref_init_grid_{tag}")
        fn.argtypes = [P, P, P, S, S, S]
        for w, h, d in GRIDS:
            n = w * h * d
            g = np.zeros((3, n), dt)
            fn(g[0].ctypes.data, g[1].ctypes.data, g[2].ctypes.data, w, h, d)
            key = f"grid_{tag}_{w}x{h}x{d}"
            meta["sha256"][key] = hashlib.sha256(g.tobytes()).hexdigest()
            out[key] = g if n <= FULL_LIMIT else g[:, ::997]
    lib.ref_libc_rand.argtypes = [ctypes.c_uint, P, S]
    for seed in SEEDS:
        r = np.zeros(2000, np.int32)
        lib.ref_libc_rand(seed, r.ctypes.data, 2000)
        out[f"rand_{seed}"] = r
    meta["full_limit"] = FULL_LIMIT
    path = os.path.join(HERE, "reference_inputs.npz")
    np.savez_compressed(path, meta=np.array(json.dumps(meta)), **out)
    print("wrote", path, f"({len(out)} arrays)")


if __name__ == "__main__":
    main()
