"""Parity of the timed tracer shape on the benchmark charge sets.

bench.py times ref_trace_kernel with 8 lanes per line and 2 lines per lane
(the planner's choice for 32 736 lines x 4096 charges).  These tests run that
shape — forced, since a line subset would make the planner choose another —
on a subset of each benchmark's lines with the FULL charge set:

- uniform 4096-charge set (charges resident in shared memory),
- dipole 16 384-charge set (charges streamed in 1024-record tiles through
  the 4-stage ring),
- uniform 1024-charge set of the adjoint benchmark,

against the oracle's restatement of the reference's SSE float path
(ElectroMag/src/CPU_Implement.cpp:207-351) and its FP64 field.  Lines per
lane and warps per CTA never change a line's bits, so the subset's vertices
are those the full benchmark computes for the same lines.

Tolerances (the parity bar of the fast path against the reference):
- vertices within 1e-4 relative of the reference for the first 500 steps,
  up to a line's first approach within 0.5 of a negative charge (the
  reference keeps stepping through charges, where trajectories turn
  chaotic), on >= 99.9 % of lines — on the uniform sets.  Around the dipoles
  (separation 0.01, lines seeded 1 away) the field cancels by factors of
  100 and more, so two FP32 sums of it in different orders differ by 1e-5
  to 1e-4 at the first vertex already and the trajectories part: there the
  kernel is held to the field bound below, to the reference's own accuracy
  against FP64, and to bit equality in the exact arithmetic;
- the field the kernel used at each vertex within 1e-5 relative of the
  reference's FP32 field at the same point wherever the sum is well
  conditioned (kappa = sum_j |q_j|/r_j^2 / |E| <= 3); where it cancels, two
  FP32 sums of the same terms in different orders, each term rounded a few
  times, differ by up to a few units of FP32 rounding times kappa, and the
  bound is 1e-5 + 32 * 2^-24 * kappa;
- against the FP64 field, the kernel's median error within a factor 8 of
  the reference's own FP32 path (the reference forms each term with IEEE
  square root and divides, about 1.5 rounding units; the fast kernel's
  rsqrt.approx term carries about 3, which the cancellation around the
  dipoles amplifies).
"""
import numpy as np
import pytest

from conftest import lines_from

pytestmark = pytest.mark.gpu

VERTEX_RTOL = 1e-4
FIELD_RTOL = 1e-5
EPS32 = 2.0 ** -24
BENCH_SHAPE = dict(threads_per_line=8, lines_per_thread=2)
ROWS = 501            # 500 steps
N_LINES = 1024


def _subset(em, name):
    ch, seeds, _ = em.workloads.make(name, seed=1234)
    idx = np.linspace(0, len(seeds) - 1, N_LINES).astype(int)
    return np.ascontiguousarray(ch, np.float32), seeds[idx].astype(np.float32)


def _gpu_trace(em, torch, ch, seeds, rows, **kw):
    n = len(seeds)
    X = [torch.from_numpy(a).cuda() for a in lines_from(seeds, rows, np.float32)]
    F = torch.zeros(3 * n * (rows - 1), dtype=torch.float32, device="cuda")
    rc, _ = em.calc_field(*X, torch.from_numpy(ch).cuda(), n, 1.0, True,
                          field_out=F, **kw)
    torch.cuda.synchronize()
    assert rc == 0, em.strerror(rc)
    V = np.stack([a.cpu().numpy().reshape(rows, n) for a in X])
    E = F.cpu().numpy().reshape(3, rows - 1, n)
    return V, E


def _first_approach(V, ch, radius):
    """Per line: first row within `radius` of a negative charge (rows if
    none)."""
    from scipy.spatial import cKDTree
    neg = ch[ch[:, 3] < 0, :3].astype(np.float64)
    steps, n = V.shape[1], V.shape[2]
    d, _ = cKDTree(neg).query(V.reshape(3, -1).T.astype(np.float64))
    hit = (d < radius).reshape(steps, n)
    return np.where(hit.any(0), hit.argmax(0), steps)


def _kappa(pts, ch):
    """sum_j |q_j| / r_j^2 (FP64), the l1 size of the terms."""
    pts = pts.astype(np.float64)
    c = ch.astype(np.float64)
    out = np.zeros(len(pts))
    for i0 in range(0, len(pts), 512):
        d = pts[i0:i0 + 512, None, :] - c[None, :, :3]
        out[i0:i0 + 512] = (np.abs(c[None, :, 3]) / (d * d).sum(-1)).sum(1)
    return out * 8.987551787e9


@pytest.fixture(scope="module")
def torch():
    return pytest.importorskip("torch")


@pytest.mark.parametrize("name", ["gpu_4096", "dipole_16384", "adjoint_1024"])
def test_bench_shape_vertices_and_field(em, gpu, orc, torch, name):
    ch, seeds = _subset(em, name)
    n = len(seeds)
    G, E = _gpu_trace(em, torch, ch, seeds, ROWS, **BENCH_SHAPE)
    ref = lines_from(seeds, ROWS, np.float32)
    assert orc.calc_field(*ref, ch, n, 1.0, orc.CURV_SSE) == 0
    R = np.stack([a.reshape(ROWS, n) for a in ref])

    # vertices: first 500 steps up to the first approach of a negative charge
    stop = _first_approach(R, ch, 0.5)
    err = (np.linalg.norm(G.astype(np.float64) - R, axis=0) /
           np.maximum(np.linalg.norm(R.astype(np.float64), axis=0), 1.0))
    mask = np.arange(ROWS)[:, None] < stop[None, :]
    bad = np.any((err > VERTEX_RTOL) & mask, axis=0)
    if name != "dipole_16384":
        assert bad.mean() <= 1e-3, (name, int(bad.sum()), float(err[mask].max()))

    # field at identical points: every 20th row of the GPU's own vertices
    rows = np.arange(0, ROWS - 1, 20)
    pts = G[:, rows, :].reshape(3, -1).T                     # (m, 3)
    eg = E[:, rows, :].reshape(3, -1).T.astype(np.float64)   # kernel's field
    er = orc.field_f32(pts, ch, three_arg=True).astype(np.float64)
    e64 = orc.field_f64(pts.astype(np.float64), ch.astype(np.float64))
    keep = np.isfinite(eg).all(1) & (np.linalg.norm(e64, axis=1) > 0)
    eg, er, e64, pts = eg[keep], er[keep], e64[keep], pts[keep]
    n64 = np.linalg.norm(e64, axis=1)
    kappa = _kappa(pts, ch) / n64
    rel = np.linalg.norm(eg - er, axis=1) / np.linalg.norm(er, axis=1)
    bound = FIELD_RTOL + 32 * EPS32 * kappa
    well = kappa <= 3.0
    # against FP64: the kernel's error and the reference FP32 path's own
    err_g = np.linalg.norm(eg - e64, axis=1) / n64
    err_r = np.linalg.norm(er - e64, axis=1) / n64
    print(f"{name}: {len(rel)} points; vs reference FP32 max {rel.max():.3g} "
          f"(kappa <= 3 on {well.mean():.4f} of points, max there "
          f"{rel[well].max():.3g}; max rel/bound {(rel / bound).max():.3g}); "
          f"vs FP64 median {np.median(err_g):.3g} max {err_g.max():.3g} "
          f"(reference FP32: median {np.median(err_r):.3g} max "
          f"{err_r.max():.3g}); lines beyond 1e-4: {int(bad.sum())}")
    if well.any():
        assert np.all(rel[well] <= FIELD_RTOL), (name, float(rel[well].max()))
    assert np.all(rel <= bound), (name, float(rel.max()),
                                  float(kappa[np.argmax(rel / bound)]))
    assert np.median(err_g) <= 8 * np.median(err_r) + 1e-8, (
        name, float(np.median(err_g)), float(np.median(err_r)))


@pytest.mark.parametrize("name", ["gpu_4096", "dipole_16384"])
def test_exact_arithmetic_bitwise_on_bench_charge_sets(em, gpu, orc, torch,
                                                       name):
    """The exact arithmetic on the full benchmark charge sets (16 384 dipole
    charges: streamed tiles) equals the reference's strict build, restated
    by the oracle, bit for bit."""
    ch, seeds = _subset(em, name)
    seeds = seeds[:128]
    rows = 40
    ref = lines_from(seeds, rows, np.float32)
    assert orc.calc_field(*ref, ch, len(seeds), 1.0, orc.CURV_SSE) == 0
    got = lines_from(seeds, rows, np.float32)
    rc, _ = em.calc_field(*got, ch, len(seeds), 1.0, True, arith="exact",
                          plain=False)
    assert rc == 0, em.strerror(rc)
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
