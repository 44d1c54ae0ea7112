"""Parity of the CUDA tracer (through the C ABI) with the reference.

Exact arithmetic must reproduce the reference's strict build bit for bit
(golden vectors from the unmodified reference); fast arithmetic must stay
within the stated tolerances of the oracle (the restatement pinned to those
vectors) on the same inputs.
"""
import hashlib

import numpy as np
import pytest

from conftest import lines_from

pytestmark = pytest.mark.gpu

# Tolerances (fast FP32 arithmetic against the reference's FP32 results):
FIELD_RTOL = 1e-5    # |E_gpu - E_ref| / |E_ref| at identical points
VERTEX_RTOL = 1e-4   # |v_gpu - v_ref| / max(|v_ref|, 1), first 500 steps

FULL_CASES = ["curv_f32", "fixed_f32", "curv_f64", "fixed_f64",
              "curv_f32_res05", "curv_f32_p1"]


def trace(em, golden, name, **kw):
    c, seeds, ch = golden.inputs(name)
    x, y, z = lines_from(seeds[: c["n"]], c["steps"], seeds.dtype)
    rc, perf = em.calc_field(x, y, z, ch, c["n"], c["res"], bool(c["curv"]),
                             **kw)
    v = np.stack([a.reshape(c["steps"], c["n"]) for a in (x, y, z)])
    return rc, perf, v


def bits_equal(a, b):
    return a.dtype == b.dtype and np.array_equal(a.view(np.uint8),
                                                 b.view(np.uint8))


@pytest.mark.parametrize("name", FULL_CASES)
def test_exact_matches_reference_bit_for_bit(em, gpu, golden, name):
    rc, perf, v = trace(em, golden, name, arith="exact")
    assert rc == 0
    assert bits_equal(v, golden.get("strict", name, "vertices"))
    assert perf.progress == 1.0 and perf.time > 0


@pytest.mark.parametrize("name", ["curv_f32", "curv_f64", "curv_f32_res05"])
def test_exact_generic_rule_matches_generic_build(em, gpu, golden, name):
    rc, _, v = trace(em, golden, name, arith="exact", rule="generic")
    assert rc == 0
    assert bits_equal(v, golden.get("generic", name, "vertices"))


@pytest.mark.parametrize("streamed", [False, True])
def test_exact_cpu_config_2500_steps_sha256(em, gpu, golden, streamed):
    """1024 lines x 256 charges x 2500 steps: the whole vertex array hashes
    to the reference's SHA-256, with charges resident or streamed through
    the tile pipeline."""
    kw = dict(force_streamed=True, tile_charges=64) if streamed else {}
    rc, _, v = trace(em, golden, "cfg_cpu_2500", arith="exact", **kw)
    assert rc == 0
    assert hashlib.sha256(v.tobytes()).hexdigest() == str(
        golden.get("strict", "cfg_cpu_2500", "sha256"))


def test_exact_streamed_many_tiles(em, gpu, golden):
    name = "curv_f32_res05"  # p = 37 -> 5 tiles of 8 charges, ring of 4
    rc, _, v = trace(em, golden, name, arith="exact", force_streamed=True,
                     tile_charges=8)
    assert rc == 0
    assert bits_equal(v, golden.get("strict", name, "vertices"))


@pytest.mark.parametrize("name", ["rc_n0", "rc_res0", "rc_steps1", "rc_n32",
                                  "rc_n32_steps1", "rc_fixed_n32"])
def test_plain_entry_return_codes(em, gpu, golden, name):
    c, seeds, ch = golden.inputs(name)
    n, steps = c["n"], c["steps"]
    x, y, z = lines_from(seeds[: max(n, 1)], max(steps, 1), np.float32)
    if n:
        x, y, z = x[: n * steps], y[: n * steps], z[: n * steps]
    rc, _ = em.calc_field(x, y, z, ch, n, c["res"], bool(c["curv"]),
                          plain=True)
    assert rc == int(golden.get("strict", name, "rc"))


def test_any_n_when_restriction_lifted(em, gpu, orc, golden):
    """n = 100 (not a multiple of 64) with require_n64 = 0; each line equals
    the oracle's line traced inside a 128-line array."""
    c, seeds, ch = golden.inputs("curv_f32_res05")
    s100 = seeds[:100]
    x, y, z = lines_from(s100, c["steps"], np.float32)
    rc, _ = em.calc_field(x, y, z, ch, 100, c["res"], True, arith="exact",
                          require_n64=False)
    assert rc == 0
    ox, oy, oz = lines_from(seeds[:128], c["steps"], np.float32)
    assert orc.calc_field(ox, oy, oz, ch, 128, c["res"], orc.CURV_SSE) == 0
    for a, b in zip((x, y, z), (ox, oy, oz)):
        assert np.array_equal(a.reshape(c["steps"], 100),
                              b.reshape(c["steps"], 128)[:, :100])


@pytest.fixture(scope="module")
def cpu_config(em):
    """The CPU-runnable configuration (256 charges in [-50,50]^3, 8 seeds
    per positive charge on a radius-1 Fibonacci sphere), 501 rows."""
    ch, seeds, _ = em.workloads.make("cpu_256", seed=7)
    seeds = em.workloads.pad_lines(seeds.astype(np.float32), 64)
    return ch, seeds, 501


def test_fast_field_within_1e5_of_reference_fp32(em, gpu, orc, cpu_config):
    ch, seeds, steps = cpu_config
    # points: the oracle's own vertices along the lines (realistic spread)
    x, y, z = lines_from(seeds, 40, np.float32)
    orc.calc_field(x, y, z, ch, len(seeds), 1.0, orc.CURV_SSE)
    pts = np.stack([x, y, z], 1)
    e_ref = orc.field_f32(pts, ch, three_arg=True).astype(np.float64)
    e_gpu = em.field(pts.astype(np.float32), ch).astype(np.float64)
    e64 = orc.field_f64(pts.astype(np.float64), ch.astype(np.float64))
    rel = np.linalg.norm(e_gpu - e_ref, axis=1) / np.linalg.norm(e_ref, axis=1)
    assert np.all(rel <= FIELD_RTOL), (rel.max(), np.median(rel))
    # and the fast kernel is no further from FP64 than the reference is
    err_gpu = np.linalg.norm(e_gpu - e64, axis=1) / np.linalg.norm(e64, axis=1)
    err_ref = np.linalg.norm(e_ref - e64, axis=1) / np.linalg.norm(e64, axis=1)
    assert np.median(err_gpu) <= 2 * np.median(err_ref) + 1e-7


def first_approach(v, ch, radius):
    """Per line: first row whose vertex is within `radius` of a negative
    charge (the reference keeps stepping through charges; beyond that point
    a trajectory is chaotic)."""
    neg = ch[ch[:, 3] < 0, :3].astype(np.float64)
    steps, n = v.shape[1], v.shape[2]
    out = np.full(n, steps)
    for s in range(steps):
        d = v[:, s, :].T.astype(np.float64)  # (n, 3)
        dd = ((d[:, None, :] - neg[None]) ** 2).sum(-1).min(1)
        hit = (dd < radius * radius) & (out == steps)
        out[hit] = s
    return out


@pytest.mark.parametrize("pack,kl", [("scalar", 1), ("scalar", 2),
                                     ("pairs", 1), ("pairs", 2)])
def test_fast_vertices_within_1e4_first_500_steps(em, gpu, orc, cpu_config,
                                                  pack, kl):
    ch, seeds, steps = cpu_config
    n = len(seeds)
    ref = lines_from(seeds, steps, np.float32)
    assert orc.calc_field(*ref, ch, n, 1.0, orc.CURV_SSE) == 0
    got = lines_from(seeds, steps, np.float32)
    rc, perf = em.calc_field(*got, ch, n, 1.0, True, pack=pack,
                             lines_per_thread=kl)
    assert rc == 0
    R = np.stack([a.reshape(steps, n) for a in ref]).astype(np.float64)
    G = np.stack([a.reshape(steps, n) for a in got]).astype(np.float64)
    stop = first_approach(R, ch, 0.5)
    err = np.linalg.norm(G - R, axis=0) / np.maximum(
        np.linalg.norm(R, axis=0), 1.0)
    rows = np.arange(steps)[:, None]
    mask = rows < stop[None, :]
    bad_lines = np.any((err > VERTEX_RTOL) & mask, axis=0)
    # lines that graze a charge or a separatrix may diverge; all but 0.1 %
    # must stay within tolerance over their first 500 steps
    assert bad_lines.mean() <= 1e-3, (bad_lines.sum(), err[mask].max())
    assert perf.pairs == n * (steps - 1) * len(ch)


@pytest.mark.parametrize("pack,kl", [("scalar", 1), ("scalar", 2),
                                     ("pairs", 1), ("pairs", 2)])
@pytest.mark.parametrize("tpl", [1, 2, 4, 8])
def test_fast_threads_per_line_variants_agree(em, gpu, golden, tpl, pack, kl):
    name = "curv_f32"
    base = trace(em, golden, name, threads_per_line=1, pack="scalar")[2]
    rc, _, v = trace(em, golden, name, threads_per_line=tpl, pack=pack,
                     lines_per_thread=kl)
    assert rc == 0
    err = np.abs(v.astype(np.float64) - base) / np.maximum(np.abs(base), 1)
    assert err[:, :8].max() <= VERTEX_RTOL


@pytest.mark.parametrize("pack,kl", [("scalar", 1), ("scalar", 2),
                                     ("pairs", 1), ("pairs", 2)])
@pytest.mark.parametrize("tpl", [1, 4])
def test_fast_streamed_equals_resident_bitwise(em, gpu, cpu_config, tpl, pack,
                                               kl):
    ch, seeds, _ = cpu_config
    n, steps = len(seeds), 60
    a = lines_from(seeds, steps, np.float32)
    b = lines_from(seeds, steps, np.float32)
    assert em.calc_field(*a, ch, n, 1.0, True, threads_per_line=tpl,
                         pack=pack, lines_per_thread=kl)[0] == 0
    assert em.calc_field(*b, ch, n, 1.0, True, threads_per_line=tpl,
                         pack=pack, lines_per_thread=kl, force_streamed=True,
                         tile_charges=64)[0] == 0
    for u, w in zip(a, b):
        assert np.array_equal(u, w)


def test_fast_f64_close_to_oracle_f64(em, gpu, orc, golden):
    c, seeds, ch = golden.inputs("curv_f64")
    x, y, z = lines_from(seeds, 12, np.float64)
    assert em.calc_field(x, y, z, ch, c["n"], 1.0, True, plain=False)[0] == 0
    ox, oy, oz = lines_from(seeds, 12, np.float64)
    orc.calc_field(ox, oy, oz, ch, c["n"], 1.0, orc.CURV_SSE)
    for a, b in zip((x, y, z), (ox, oy, oz)):
        assert np.allclose(a, b, rtol=1e-11, atol=1e-11)


def test_device_pointer_entry_matches_host_entry(em, gpu, cpu_config):
    torch = pytest.importorskip("torch")
    ch, seeds, _ = cpu_config
    n, steps = len(seeds), 50
    host = lines_from(seeds, steps, np.float32)
    assert em.calc_field(*host, ch, n, 1.0, True, plain=False)[0] == 0
    dev = [torch.from_numpy(a).cuda() for a in lines_from(seeds, steps,
                                                          np.float32)]
    dch = torch.from_numpy(np.ascontiguousarray(ch)).cuda()
    rc, _ = em.calc_field(*dev, dch, n, 1.0, True)
    torch.cuda.synchronize()
    assert rc == 0
    for h, d in zip(host, dev):
        assert np.array_equal(h, d.cpu().numpy())


def test_field_exact_matches_reference_fp32_bitwise(em, gpu, orc, cpu_config):
    ch, seeds, _ = cpu_config
    pts = seeds[:200].astype(np.float32) + np.float32(0.37)
    e_ref = orc.field_f32(pts, ch, three_arg=True)
    e_gpu = em.field(pts, ch, arith="exact", rule="sse")
    assert np.array_equal(e_ref, e_gpu)
    e_ref2 = orc.field_f32(pts, ch, three_arg=False)
    e_gpu2 = em.field(pts, ch, arith="exact", rule="generic")
    assert np.array_equal(e_ref2, e_gpu2)


def test_field_f64_matches_fp64_oracle(em, gpu, orc, cpu_config):
    """The GPU FP64 field (the reference's double sequence) equals the CPU
    FP64 oracle to rounding; bench.py uses it as the FP64 reference for its
    error statistics."""
    ch, seeds, _ = cpu_config
    rng = np.random.default_rng(9)
    pts = rng.uniform(-60, 60, (4000, 3))
    e_cpu = orc.field_f64(pts, ch.astype(np.float64))
    e_gpu = em.field(pts, ch.astype(np.float64), arith="exact")
    rel = np.linalg.norm(e_gpu - e_cpu, axis=1) / np.linalg.norm(e_cpu, axis=1)
    assert rel.max() <= 1e-13, rel.max()


def test_host_entry_chunked_copy_matches_device_entry(em, gpu):
    """Host arrays above 64 MB are traced in row chunks whose device-to-host
    copies overlap the next chunk: the vertices equal the device-pointer
    entry's (one launch) bit for bit."""
    torch = pytest.importorskip("torch")
    ch, seeds, _ = em.workloads.make("cpu_256", seed=5)
    ch = np.ascontiguousarray(ch, np.float32)
    seeds = np.tile(seeds.astype(np.float32), (8, 1))[:8192]
    n, rows = len(seeds), 1000
    x, y, z = lines_from(seeds, rows, np.float32)
    rc, _ = em.calc_field(x, y, z, ch, n, 1.0, True, require_n64=False,
                          plain=False)
    assert rc == 0
    D = [torch.from_numpy(lines_from(seeds, rows, np.float32)[c]).cuda()
         for c in range(3)]
    rc, _ = em.calc_field(*D, torch.from_numpy(ch).cuda(), n, 1.0, True)
    torch.cuda.synchronize()
    assert rc == 0
    for host, dev in zip((x, y, z), D):
        assert np.array_equal(host, dev.cpu().numpy())


@pytest.mark.parametrize("arith", ["exact", "fast"])
def test_no_charges_traces_a_zero_field(em, gpu, arith):
    """Zero charges: the field is zero and the reference's step is 0/0, so
    every row after the seeds is NaN and the call still returns 0."""
    seeds = np.random.default_rng(2).uniform(-5, 5, (64, 3)).astype(np.float32)
    x, y, z = lines_from(seeds, 6, np.float32)
    rc, _ = em.calc_field(x, y, z, np.zeros((0, 4), np.float32), 64, 1.0,
                          True, arith=arith, plain=False)
    assert rc == 0
    v = np.stack([x, y, z]).reshape(3, 6, 64)
    assert np.array_equal(v[:, 0], seeds.T)
    assert np.all(np.isnan(v[:, 1:]))


def test_indexing_beyond_two_to_the_31(em, gpu):
    """524 288 lines x 5000 rows: 2.6e9 elements per component array (the
    reference's largest presets reach 1e10).  The last lines' rows, stored
    past element 2^31, equal a separate 64-line call with the same shape."""
    torch = pytest.importorskip("torch")
    free, _ = torch.cuda.mem_get_info()
    n, rows = 524288, 5000
    if free < 3 * n * rows * 4 + (4 << 30):
        pytest.skip("not enough device memory")
    rng = np.random.default_rng(8)
    ch = np.zeros((64, 4), np.float32)
    ch[:, :3] = rng.uniform(-50, 50, (64, 3))
    ch[:, 3] = rng.uniform(1, 10, 64) * rng.choice([-1, 1], 64)
    seeds = rng.uniform(-60, 60, (n, 3)).astype(np.float32)
    shape = dict(threads_per_line=4, lines_per_thread=1)
    dch = torch.from_numpy(ch).cuda()
    X = [torch.empty(n * rows, dtype=torch.float32, device="cuda") for _ in range(3)]
    for c in range(3):
        X[c][:n] = torch.from_numpy(np.ascontiguousarray(seeds[:, c])).cuda()
    rc, _ = em.calc_field(*X, dch, n, 1.0, True, **shape)
    assert rc == 0
    tail = np.arange(n - 64, n)
    big = np.stack([X[c].view(rows, n)[:, tail].cpu().numpy() for c in range(3)])
    del X
    torch.cuda.empty_cache()
    Y = [torch.zeros(64 * rows, dtype=torch.float32, device="cuda") for _ in range(3)]
    for c in range(3):
        Y[c][:64] = torch.from_numpy(np.ascontiguousarray(seeds[tail, c])).cuda()
    rc, _ = em.calc_field(*Y, dch, 64, 1.0, True, **shape)
    assert rc == 0
    small = np.stack([Y[c].view(rows, 64).cpu().numpy() for c in range(3)])
    assert np.array_equal(big, small)
