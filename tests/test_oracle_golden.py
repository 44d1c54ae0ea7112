"""The CPU oracle against the reference's own outputs (tests/golden/).

The fixtures were produced by the unmodified reference (CPU_Implement.cpp)
compiled here (tests/golden/make_golden.py).  The restatement must match its
strict IEEE build bit for bit, its generic-template build bit for bit, and
its fast-math release build to within rounding wherever that build is finite.
"""
import hashlib

import numpy as np
import pytest

from conftest import lines_from

BITEXACT_STRICT = ["curv_f32", "fixed_f32", "curv_f64", "fixed_f64",
                   "curv_f32_res05", "curv_f32_p1"]


def run_oracle(orc, golden, name, variant):
    c, seeds, ch = golden.inputs(name)
    dt = seeds.dtype
    x, y, z = lines_from(seeds[: c["n"]], c["steps"], dt)
    rc = orc.calc_field(x, y, z, ch, c["n"], c["res"], variant)
    return rc, np.stack([a.reshape(c["steps"], c["n"]) for a in (x, y, z)])


def variant_of(orc, c, build):
    if not c["curv"]:
        return orc.FIXED
    return orc.CURV_GENERIC if build == "generic" else orc.CURV_SSE


@pytest.mark.parametrize("name", BITEXACT_STRICT)
def test_strict_bitexact(orc, golden, name):
    c = golden.cases[name]
    rc, v = run_oracle(orc, golden, name, variant_of(orc, c, "strict"))
    assert rc == int(golden.get("strict", name, "rc")) == 0
    ref = golden.get("strict", name, "vertices")
    assert v.dtype == ref.dtype
    assert np.array_equal(v.view(np.uint8), ref.view(np.uint8))


@pytest.mark.parametrize("name", ["curv_f32", "curv_f64", "curv_f32_res05"])
def test_generic_bitexact(orc, golden, name):
    c = golden.cases[name]
    rc, v = run_oracle(orc, golden, name, orc.CURV_GENERIC)
    assert rc == 0
    ref = golden.get("generic", name, "vertices")
    assert np.array_equal(v.view(np.uint8), ref.view(np.uint8))


def test_cpu_config_2500_steps(orc, golden):
    """256 charges, Fibonacci seeds, 2500 steps: sampled rows and the SHA-256
    of the whole vertex array equal the reference's."""
    name = "cfg_cpu_2500"
    c = golden.cases[name]
    rc, v = run_oracle(orc, golden, name, orc.CURV_SSE)
    assert rc == 0
    assert hashlib.sha256(v.tobytes()).hexdigest() == str(
        golden.get("strict", name, "sha256"))
    ref = golden.get("strict", name, "vertices")
    assert np.array_equal(v[:, c["rows"]], ref)


@pytest.mark.parametrize("name", ["curv_f32", "curv_f64"])
def test_fast_math_build_within_rounding(orc, golden, name):
    """The release build (-ffast-math) differs by reassociation; it is NaN
    where |E|^3 overflows, which the strict build handles as k = 0."""
    c = golden.cases[name]
    rc, v = run_oracle(orc, golden, name, orc.CURV_SSE)
    ref = golden.get("fast", name, "vertices")
    fin = np.isfinite(ref).all(axis=0)
    # compare the first 8 steps of lines that stay finite in the fast build
    keep = fin.all(axis=0)
    assert keep.sum() >= c["n"] // 2
    tol = 1e-4 if c["dtype"] == "f32" else 1e-12
    a, b = v[:, :8, keep], ref[:, :8, keep]
    assert np.all(np.abs(a - b) <= tol * np.maximum(1.0, np.abs(b)))


@pytest.mark.parametrize("name", ["rc_n0", "rc_res0", "rc_steps1", "rc_n32",
                                  "rc_n32_steps1", "rc_fixed_n32"])
def test_return_codes(orc, golden, name):
    c, seeds, ch = golden.inputs(name)
    n = c["n"]
    x, y, z = lines_from(seeds[:max(n, 1)], max(c["steps"], 1), seeds.dtype)
    if n:
        x, y, z = x[: n * c["steps"]], y[: n * c["steps"]], z[: n * c["steps"]]
    variant = orc.CURV_SSE if c["curv"] else orc.FIXED
    rc = orc.calc_field(x, y, z, ch, n, c["res"], variant)
    assert rc == int(golden.get("strict", name, "rc"))


def test_oracle_line_subset_matches_full(orc, golden):
    """Tracing a subset of lines gives the same bits as the full run (the
    CPU baseline times subsets)."""
    c, seeds, ch = golden.inputs("curv_f32_res05")
    full = lines_from(seeds, c["steps"], np.float32)
    orc.calc_field(*full, ch, c["n"], c["res"], orc.CURV_SSE)
    part = lines_from(seeds, c["steps"], np.float32)
    orc.calc_field(*part, ch, c["n"], c["res"], orc.CURV_SSE, line0=37,
                   nlines=50)
    for a, b in zip(full, part):
        A = a.reshape(c["steps"], c["n"])[1:, 37:87]
        B = b.reshape(c["steps"], c["n"])[1:, 37:87]
        assert np.array_equal(A, B)


def test_field_f64_single_charge_known_answer(orc):
    """E = k q r / |r|^3 for one charge (include/Electrostatics.h:38-51)."""
    ch = np.array([[1.0, 2.0, 3.0, 2.5]])
    pts = np.array([[4.0, 6.0, 3.0], [1.0, 2.0, 5.0]])
    e = orc.field_f64(pts, ch)
    k = 8.987551787e9
    r = pts - ch[:, :3]
    want = k * 2.5 * r / np.linalg.norm(r, axis=1, keepdims=True) ** 3
    assert np.allclose(e, want, rtol=1e-15, atol=0)


def test_field_f64_null_between_equal_charges(orc):
    ch = np.array([[-1.0, 0, 0, 3.0], [1.0, 0, 0, 3.0]])
    e = orc.field_f64(np.array([[0.0, 0.0, 0.0]]), ch)
    assert np.all(e == 0)


def test_field_f64_dipole_midplane(orc):
    """On the mid-plane of a ±q dipole the field is antiparallel to the
    dipole axis with magnitude k q d / (r^2 + d^2/4)^1.5."""
    d, q = 0.2, 4.0
    ch = np.array([[0, 0, d / 2, q], [0, 0, -d / 2, -q]])
    pts = np.array([[3.0, 0, 0], [0, -2.0, 0]])
    e = orc.field_f64(pts, ch)
    k = 8.987551787e9
    for p, v in zip(pts, e):
        rr = np.linalg.norm(p)
        mag = k * q * d / (rr * rr + d * d / 4) ** 1.5
        assert np.allclose(v, [0, 0, -mag], rtol=1e-13, atol=1e-9 * mag)
