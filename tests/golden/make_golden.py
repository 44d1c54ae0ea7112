"""Generate the golden vectors in tests/golden/ from the reference itself.

Runs only where the reference sources exist (it needs oracle/_ref/, built by
oracle/build_ref.sh from ElectroMag/src/CPU_Implement.cpp).  The fixtures it
writes are committed, so the tests never need the reference at run time.

    python tests/golden/make_golden.py

Every fixture stores its inputs (charges {x,y,z,q}, seeds), the call's
arguments, the reference's return code and its output vertices.  Outputs come
from three builds of the unmodified reference:
  strict   -O3 -msse2 -fopenmp, IEEE arithmetic (x86 SSE specialisations,
           CPU_Implement.cpp:207-351 and :366-498)
  fast     the reference's release flags (CMakeLists.txt:24, -ffast-math)
  generic  __SSE__ undefined: the scalar templates (CPU_Implement.cpp:38-191)
Each build is loaded in its own subprocess: a -ffast-math library can change
the floating-point environment of the process that loads it.
"""
import ctypes
import hashlib
import json
import os
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
REFDIR = os.path.join(ROOT, "oracle", "_ref")


def charges_uniform(rng, p, half, dtype):
    ch = np.empty((p, 4), dtype)
    ch[:, :3] = rng.uniform(-half, half, (p, 3))
    ch[:, 3] = rng.uniform(1.0, 10.0, p) * rng.choice([-1.0, 1.0], p)
    return ch


def fibonacci_seeds(ch, per_charge, radius):
    """Seeds on a sphere of `radius` around every positive charge."""
    ga = np.pi * (3.0 - np.sqrt(5.0))
    i = np.arange(per_charge, dtype=np.float64)
    zz = 1.0 - (2.0 * i + 1.0) / per_charge
    rr = np.sqrt(1.0 - zz * zz)
    d = np.stack([rr * np.cos(ga * i), rr * np.sin(ga * i), zz], 1)
    pos = ch[ch[:, 3] > 0, :3].astype(np.float64)
    return (pos[:, None, :] + radius * d[None]).reshape(-1, 3)


def run_case(lib, dtype, seeds, ch, n, steps, res, curv):
    """Run one reference call in this process; returns (rc, x, y, z)."""
    P, S = ctypes.c_void_p, ctypes.c_size_t
    T = ctypes.c_float if dtype == np.float32 else ctypes.c_double
    fn = lib.ref_calc_field_f32 if dtype == np.float32 else lib.ref_calc_field_f64
    fn.argtypes = [P, P, P, S, S, P, S, T, ctypes.c_int, P]
    arrs = []
    for c in range(3):
        a = np.zeros(max(n * steps, 1), dtype)
        if n:
            a[:n] = seeds[:n, c]
        arrs.append(a)
    chc = np.ascontiguousarray(ch, dtype)
    rc = fn(*(a.ctypes.data_as(P) for a in arrs), n, steps,
            chc.ctypes.data_as(P), ch.shape[0], res, int(curv), None)
    return rc, arrs


def child(build, spec_path, out_path):
    """Subprocess body: load one reference build and run every case."""
    lib = ctypes.CDLL(os.path.join(REFDIR, f"libemref_{build}.so"))
    spec = np.load(spec_path, allow_pickle=False)
    cases = json.loads(str(spec["cases"]))
    out = {}
    for c in cases:
        dtype = np.float32 if c["dtype"] == "f32" else np.float64
        rc, arrs = run_case(lib, dtype, spec[c["name"] + "/seeds"],
                            spec[c["name"] + "/charges"], c["n"], c["steps"],
                            c["res"], c["curv"])
        out[c["name"] + "/rc"] = np.array(rc)
        if rc == 0:
            v = np.stack([a.reshape(c["steps"], c["n"]) for a in arrs])
            out[c["name"] + "/sha256"] = np.array(
                hashlib.sha256(v.tobytes()).hexdigest())
            rows = c.get("rows")
            out[c["name"] + "/vertices"] = v if rows is None else v[:, rows]
    np.savez(out_path, **out)


def main():
    if len(sys.argv) == 4:
        child(*sys.argv[1:])
        return
    if not os.path.exists(os.path.join(REFDIR, "libemref_strict.so")):
        sys.exit("oracle/_ref missing: run bash oracle/build_ref.sh first")
    rng = np.random.default_rng(20101)
    cases, arrays = [], {}

    def add(name, dtype, seeds, ch, n, steps, res, curv, builds, rows=None):
        c = dict(name=name, dtype=dtype, n=n, steps=steps, res=res,
                 curv=curv, builds=builds)
        if rows is not None:
            c["rows"] = rows
        cases.append(c)
        arrays[name + "/seeds"] = np.asarray(seeds, np.float64)
        arrays[name + "/charges"] = np.asarray(ch, np.float64)

    # small cases, full vertex arrays
    for dt in ("f32", "f64"):
        npdt = np.float32 if dt == "f32" else np.float64
        ch = charges_uniform(rng, 29, 50.0, npdt)
        seeds = rng.uniform(-60, 60, (64, 3)).astype(npdt)
        add(f"curv_{dt}", dt, seeds, ch, 64, 48, 1.0, 1,
            ["strict", "fast", "generic"])
        add(f"fixed_{dt}", dt, seeds, ch, 64, 24, 1.0, 0, ["strict"])
    # odd charge count, two line blocks, fractional resolution
    ch = charges_uniform(rng, 37, 50.0, np.float32)
    seeds = rng.uniform(-60, 60, (128, 3)).astype(np.float32)
    add("curv_f32_res05", "f32", seeds, ch, 128, 20, 0.5, 1,
        ["strict", "generic"])
    # a single charge: straight radial lines
    ch = np.array([[1.5, -2.0, 0.25, 3.0]], np.float32)
    seeds = rng.uniform(-5, 5, (64, 3)).astype(np.float32)
    add("curv_f32_p1", "f32", seeds, ch, 64, 16, 1.0, 1, ["strict"])
    # the CPU-runnable configuration: 256 charges in [-50,50]^3, |q| in
    # [1,10] with random sign, 8 Fibonacci seeds per positive charge at radius
    # 1, 2500 steps; n padded to a multiple of 64 with copies of seed 0
    ch = charges_uniform(rng, 256, 50.0, np.float32)
    seeds = fibonacci_seeds(ch.astype(np.float64), 8, 1.0).astype(np.float32)
    n = (len(seeds) + 63) // 64 * 64
    seeds = np.concatenate([seeds, np.repeat(seeds[:1], n - len(seeds), 0)])
    add("cfg_cpu_2500", "f32", seeds, ch, n, 2500, 1.0, 1, ["strict"],
        rows=[0, 1, 2, 5, 10, 50, 100, 250, 500, 1000, 2000, 2499])
    # the reference program's own runs: --bogo (16x16 grid, 50 charges, 500
    # rows) and the default preset (128x128 grid, 1024 charges, 2500 rows),
    # inputs from its generators (InitializePointChargeArray with srand(1),
    # InitializeFieldLineArray grid mode) through oracle/_ref/libemref_inputs.so
    inp = ctypes.CDLL(os.path.join(REFDIR, "libemref_inputs.so"))
    inp.ref_init_charges_f32.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
    inp.ref_init_grid_f32.argtypes = [ctypes.c_void_p] * 3 + [ctypes.c_size_t] * 3
    for name, (w, h, p, rows, sample) in {
            "preset_bogo": (16, 16, 50, 500, [0, 1, 2, 10, 100, 250, 499]),
            "preset_normal": (128, 128, 1024, 2500, [1, 1000, 2499])}.items():
        ch = np.zeros((p, 4), np.float32)
        inp.ref_init_charges_f32(ch.ctypes.data, p)
        g = np.zeros((3, w * h), np.float32)
        inp.ref_init_grid_f32(g[0].ctypes.data, g[1].ctypes.data,
                              g[2].ctypes.data, w, h, 1)
        add(name, "f32", g.T.copy(), ch, w * h, rows, 1.0, 1, ["strict"],
            rows=sample)
    # error codes: n == 0, resolution == 0, total_steps < 2, n % 64 != 0
    ch = charges_uniform(rng, 4, 50.0, np.float32)
    seeds = rng.uniform(-60, 60, (64, 3)).astype(np.float32)
    add("rc_n0", "f32", seeds, ch, 0, 4, 1.0, 1, ["strict"])
    add("rc_res0", "f32", seeds, ch, 64, 4, 0.0, 1, ["strict"])
    add("rc_steps1", "f32", seeds, ch, 64, 1, 1.0, 1, ["strict"])
    add("rc_n32", "f32", seeds, ch, 32, 4, 1.0, 1, ["strict"])
    add("rc_n32_steps1", "f32", seeds, ch, 32, 1, 1.0, 1, ["strict"])
    add("rc_fixed_n32", "f32", seeds, ch, 32, 4, 1.0, 0, ["strict"])

    work = tempfile.mkdtemp(prefix="em_golden_")
    tmp = os.path.join(work, "spec.npz")
    np.savez(tmp, cases=np.array(json.dumps(cases)), **arrays)
    results = {}
    for build in ("strict", "fast", "generic"):
        out = os.path.join(work, f"out_{build}.npz")
        subprocess.check_call([sys.executable, __file__, build, tmp, out])
        with np.load(out) as r:
            for c in cases:
                if build in c["builds"]:
                    for k in r.files:
                        if k.startswith(c["name"] + "/"):
                            results[f"{build}/{k}"] = r[k]
    shutil.rmtree(work)

    meta = dict(cases=cases, generator="tests/golden/make_golden.py",
                reference="ElectroMag/src/CPU_Implement.cpp via oracle/build_ref.sh",
                machine=os.uname().machine)
    np.savez_compressed(os.path.join(HERE, "reference_vectors.npz"),
                        meta=np.array(json.dumps(meta)), **arrays, **results)
    print("wrote", os.path.join(HERE, "reference_vectors.npz"),
          f"({len(cases)} cases)")


if __name__ == "__main__":
    main()
