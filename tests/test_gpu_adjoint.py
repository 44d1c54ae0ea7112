"""Gradients through the tracer (em_adjoint_f32) against FP64 references of
the same frozen-step map: its discrete adjoint, the complex-step derivative
and central differences (h = 1e-3), all computed on the CPU."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GRAD_RTOL = 1e-4   # |g_gpu - g_ref| / |g_ref| against the FP64 references
FD_RTOL = 1e-3     # central differences carry O(h^2) truncation error


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def test_adjoint_matches_fp64_discrete_adjoint(em, gpu, adjoint_case):
    ch, seeds, rows, targets, fz = adjoint_case
    out = em.adjoint(seeds, ch, rows, targets)
    assert out["loss"] == pytest.approx(fz.L, rel=1e-4)
    assert rel(out["grad"], fz.grad()) <= GRAD_RTOL


def test_adjoint_matches_complex_step(em, gpu, adjoint_case):
    ch, seeds, rows, targets, fz = adjoint_case
    g = em.adjoint(seeds, ch, rows, targets)["grad"]
    cs = np.array([[fz.complex_step(j, c) for c in range(4)]
                   for j in range(len(ch))])
    assert rel(g, cs) <= GRAD_RTOL


def test_adjoint_matches_central_differences(em, gpu, adjoint_case):
    ch, seeds, rows, targets, fz = adjoint_case
    g = em.adjoint(seeds, ch, rows, targets)["grad"]
    fd = np.array([[fz.central(j, c, 1e-3) for c in range(4)]
                   for j in range(len(ch))])
    assert rel(g, fd) <= FD_RTOL


def test_autograd_function(em, gpu, adjoint_case):
    torch = pytest.importorskip("torch")
    ch, seeds, rows, targets, fz = adjoint_case
    TraceLoss = em.trace_loss_function()
    q = torch.tensor(ch, dtype=torch.float64, requires_grad=True)
    loss = TraceLoss.apply(q, torch.tensor(seeds), rows, torch.tensor(targets))
    (2.0 * loss).backward()
    direct = em.adjoint(seeds, ch, rows, targets)["grad"]
    assert np.allclose(q.grad.numpy(), 2.0 * direct, rtol=1e-12, atol=0)


def test_adjoint_fixed_step_mode(em, gpu, adjoint_case, orc):
    """use_curvature = False: lam_s = 1/res; the loss matches an FP64 trace
    of the fixed-step rule within FP32 rounding."""
    ch, seeds, rows, targets, _ = adjoint_case
    out = em.adjoint(seeds, ch, rows, targets, use_curvature=False)
    x, y, z = em.new_lines(seeds.astype(np.float64), rows, np.float64)
    orc.calc_field(x, y, z, ch, len(seeds), 1.0, orc.FIXED)
    V = np.stack([a.reshape(rows, -1) for a in (x, y, z)])
    L = float(((V - targets.astype(np.float64)) ** 2).sum())
    assert out["loss"] == pytest.approx(L, rel=1e-4)
    assert np.all(np.isfinite(out["grad"]))
