"""The mixed arithmetic on the reference-layout tracer (EM_ARITH_MIXED
through em_calc_field_ex_f32): FP32 pairs with the Newton-corrected inv^3,
compensated chunk sums, the line position in FP64 and a double-float
re-evaluation where the sum is ill-conditioned, on the reference's stepping
loop (CPU_Implement.cpp:207-351), against the FP64 oracle of that loop and
the FP64 field at the same points."""
import numpy as np
import pytest

from conftest import lines_from

pytestmark = pytest.mark.gpu

VERTEX_RTOL = 1e-4


@pytest.fixture(scope="module")
def case(em, orc):
    ch, seeds, _ = em.workloads.make("cpu_256", seed=7)
    seeds = em.workloads.pad_lines(seeds.astype(np.float32), 64)
    steps = 60
    n = len(seeds)
    ref = lines_from(seeds.astype(np.float64), steps, np.float64)
    orc.calc_field(*ref, ch.astype(np.float64), n, 1.0, orc.CURV_SSE)
    R = np.stack([a.reshape(steps, n) for a in ref])
    return ch, seeds, steps, R


def run(em, ch, seeds, steps, **kw):
    x, y, z = lines_from(seeds, steps, np.float32)
    rc, perf = em.calc_field(x, y, z, ch, len(seeds), 1.0, True, **kw)
    assert rc == 0
    return np.stack([a.reshape(steps, len(seeds)) for a in (x, y, z)]).astype(np.float64), perf


def rel_err(V, R, rows):
    d = np.linalg.norm(V[:, :rows] - R[:, :rows], axis=0)
    return d / np.maximum(np.linalg.norm(R[:, :rows], axis=0), 1.0)


def test_mixed_tracks_the_fp64_trajectory_closer_than_fp32(em, gpu, case):
    ch, seeds, steps, R = case
    vm, pm = run(em, ch, seeds, steps, arith="mixed")
    vf, _ = run(em, ch, seeds, steps, arith="fast")
    em_ = rel_err(vm, R, 20)
    ef = rel_err(vf, R, 20)
    # lines that graze a charge part in any precision: all but 1 % within
    # the vertex tolerance, and the mixed form closer than FP32 overall
    assert np.mean(em_.max(axis=0) <= VERTEX_RTOL) >= 0.99
    assert np.median(em_) < np.median(ef)
    assert pm.pairs == pytest.approx(len(seeds) * (steps - 1) * len(ch))


@pytest.mark.parametrize("tpl,kl", [(1, 1), (2, 2), (4, 1), (8, 2), (8, 1)])
def test_mixed_shapes_agree(em, gpu, case, tpl, kl):
    ch, seeds, steps, R = case
    v, _ = run(em, ch, seeds, steps, arith="mixed", threads_per_line=tpl,
               lines_per_thread=kl)
    assert np.mean(rel_err(v, R, 20).max(axis=0) <= VERTEX_RTOL) >= 0.99


def test_mixed_streamed_tiles(em, gpu, case):
    ch, seeds, steps, R = case
    v, _ = run(em, ch, seeds, steps, arith="mixed", force_streamed=True,
               tile_charges=64)
    assert np.mean(rel_err(v, R, 20).max(axis=0) <= VERTEX_RTOL) >= 0.99


def test_mixed_with_every_field_reevaluated_is_fp64_class(em, gpu, case):
    """refine_kappa far below 1 re-evaluates every vertex's field in
    double-float: only the FP32 step and the FP32 copy of the position
    remain, so the trajectory stays within 1e-5 of the FP64 one."""
    ch, seeds, steps, R = case
    v, perf = run(em, ch, seeds, steps, arith="mixed", refine_kappa=1e-12)
    assert perf.fp64_refines == len(seeds) * (steps - 1)
    assert np.mean(rel_err(v, R, 20).max(axis=0) <= 1e-5) >= 0.99


@pytest.fixture(scope="module")
def gpu_scale(em):
    """1024 lines of the 4096-charge GPU-scale set, 300 rows."""
    ch, seeds, _ = em.workloads.make("gpu_4096", seed=1234)
    idx = np.linspace(0, len(seeds) - 1, 1024).astype(int)
    return np.ascontiguousarray(ch, np.float32), seeds[idx].astype(np.float32), 300


def field_errors(em, torch, ch, seeds, rows, **kw):
    """Traces on the device with the field output; returns the relative
    error of the field at every vertex against the FP64 field there, the
    perf record, and the condition sqrt(sum |t_j|^2) / |E| per vertex."""
    n = len(seeds)
    X = [torch.from_numpy(a).cuda() for a in lines_from(seeds, rows, np.float32)]
    F = torch.full((3 * n * (rows - 1),), float("nan"), dtype=torch.float32,
                   device="cuda")
    dch = torch.from_numpy(ch).cuda()
    rc, perf = em.calc_field(*X, dch, n, 1.0, True, arith="mixed",
                             field_out=F, **kw)
    torch.cuda.synchronize()
    assert rc == 0, em.strerror(rc)
    V = torch.stack([x.view(rows, n)[:-1] for x in X]).reshape(3, -1)
    E = F.view(3, -1).double()
    ref = em.field(V.double().contiguous(), dch.double().contiguous(),
                   arith="exact")
    err = ((E - ref).norm(dim=0) / ref.norm(dim=0)).cpu().numpy()
    return err, perf


def test_mixed_field_within_1e6_of_fp64_at_every_vertex(em, gpu, gpu_scale):
    """The mixed form's target: the field each step uses within 1e-6
    relative of the FP64 field at the same point, at every vertex (1024
    lines x 299 steps of the GPU-scale set); without the re-evaluations some
    vertices exceed it, so the test of the sum's conditioning is what holds
    the bound."""
    torch = pytest.importorskip("torch")
    ch, seeds, rows = gpu_scale
    err, perf = field_errors(em, torch, ch, seeds, rows)
    assert np.isfinite(err).all()
    assert err.max() <= 1e-6, (err.max(), np.median(err))
    assert perf.fp64_refines < 0.01 * len(seeds) * (rows - 1)
    err_off, perf_off = field_errors(em, torch, ch, seeds, rows,
                                     refine_kappa=1e30)
    assert perf_off.fp64_refines == 0
    assert np.median(err_off) <= 2e-7


def test_mixed_rejects_fp64_arrays(em, gpu, case):
    ch, seeds, steps, _ = case
    x, y, z = lines_from(seeds.astype(np.float64), steps, np.float64)
    rc, _ = em.calc_field(x, y, z, ch.astype(np.float64), len(seeds), 1.0,
                          True, arith="mixed")
    assert rc == 4
