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


@pytest.mark.parametrize("checkpoint", [False, True])
def test_adjoint_matches_fp64_discrete_adjoint(em, gpu, adjoint_case, checkpoint):
    ch, seeds, rows, targets, fz = adjoint_case
    out = em.adjoint(seeds, ch, rows, targets, checkpoint=checkpoint)
    assert out["loss"] == pytest.approx(fz.L, rel=1e-4)
    assert rel(out["grad"], fz.grad()) <= GRAD_RTOL


def _shape_case(orc, p, n=40, rows=150, seed=7):
    """p charges in [-10,10]^3 (70 % positive, so the set's net charge is
    positive and the lines leave the cloud), n lines seeded 35..45 from the
    origin, rows spanning three 64-row segments and a partial 32-row
    block."""
    rng = np.random.default_rng(seed + p)
    ch = np.zeros((p, 4))
    ch[:, :3] = rng.uniform(-10, 10, (p, 3))
    ch[:, 3] = rng.uniform(1, 10, p) * rng.choice([-1, 1], p, p=[0.3, 0.7])
    d = rng.normal(size=(n, 3))
    seeds = d / np.linalg.norm(d, axis=1, keepdims=True) * rng.uniform(35, 45, (n, 1))
    ch = ch.astype(np.float32).astype(np.float64)
    seeds = seeds.astype(np.float32).astype(np.float64)
    fz = orc.Frozen(ch, seeds, rows, np.zeros((3, rows, n)))
    V = np.stack([v.reshape(rows, n) for v in fz.V])
    targets = (V + rng.normal(0, 0.1, V.shape)).astype(np.float32)
    fz = orc.Frozen(ch, seeds, rows, targets.astype(np.float64))
    return ch, seeds, rows, targets, fz


# p -> backward shape: 300 (16 charges per lane), 1000 (32 per lane, one warp
# per line), 1500 and 3000 (two and four warps per line), 5000 (two-pass).
# Over 150 rows the FP32 forward drifts from an FP64 forward wherever a line
# passes near a charge, so the reference here is the FP64 discrete adjoint
# linearised at the GPU's own trajectory: only the backward's arithmetic
# differs.
@pytest.mark.parametrize("p", [300, 1000, 1500, 3000, 5000])
@pytest.mark.parametrize("checkpoint", [False, True])
def test_adjoint_backward_shapes(em, gpu, orc, p, checkpoint):
    ch, seeds, rows, targets, _ = _shape_case(orc, p)
    out = em.adjoint(seeds, ch, rows, targets, checkpoint=checkpoint)
    L, g = orc.adjoint_at(ch, out["vertices"], targets)
    assert out["loss"] == pytest.approx(L, rel=1e-6)
    assert rel(out["grad"], g) <= GRAD_RTOL
    npairs = len(seeds) * (rows - 1) * p
    passes = 3 if p > 4096 else (2 if checkpoint else 1)
    assert out["bwd_pairs"] == pytest.approx(passes * npairs)


def test_adjoint_stored_and_checkpoint_agree(em, gpu, orc):
    """Both modes trace the same vertices and see the same field bits (the
    recompute repeats the forward's order); the gradients differ only where
    the register sums are flushed (every 512 rows, or per 64-row launch)."""
    ch, seeds, rows, targets, _ = _shape_case(orc, 1000)
    a = em.adjoint(seeds, ch, rows, targets, checkpoint=False)
    b = em.adjoint(seeds, ch, rows, targets, checkpoint=True)
    assert np.array_equal(a["vertices"], b["vertices"])
    assert a["loss"] == b["loss"]
    assert rel(a["grad"], b["grad"]) <= 1e-6


@pytest.mark.parametrize("p", [300, 1000, 3000])
def test_checkpoint_recompute_gives_the_forward_field_bits(em, gpu, p):
    """Within one 64-row segment both modes flush their register sums at the
    same point, so the gradients agree bit for bit exactly when the
    recomputed field has the forward's bits.  8192 lines x 59 rows of
    vertices take both the four-vertex and the one-vertex passes of the
    recompute."""
    rng = np.random.default_rng(p)
    n, rows = 8192, 60
    ch = np.zeros((p, 4), np.float32)
    ch[:, :3] = rng.uniform(-10, 10, (p, 3))
    ch[:, 3] = rng.uniform(1, 10, p) * rng.choice([-1, 1], p, p=[0.3, 0.7])
    d = rng.normal(size=(n, 3))
    seeds = (d / np.linalg.norm(d, axis=1, keepdims=True)
             * rng.uniform(35, 45, (n, 1))).astype(np.float32)
    targets = rng.normal(0, 30, (3, rows, n)).astype(np.float32)
    a = em.adjoint(seeds, ch, rows, targets, checkpoint=False)
    b = em.adjoint(seeds, ch, rows, targets, checkpoint=True)
    assert np.array_equal(a["vertices"], b["vertices"])
    assert np.array_equal(a["grad"], b["grad"])


def test_adjoint_repeats_bit_for_bit(em, gpu, adjoint_case):
    """Team partials are summed in a fixed order: two calls agree exactly."""
    ch, seeds, rows, targets, _ = adjoint_case
    a = em.adjoint(seeds, ch, rows, targets)
    b = em.adjoint(seeds, ch, rows, targets)
    assert np.array_equal(a["grad"], b["grad"])


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


@pytest.fixture(scope="module")
def scale_case(em):
    """The adjoint benchmark's charge set (1024 charges uniform in a cube of
    side 100) and length (4000 rows: 62 checkpoint segments and a partial
    one), 256 of its lines; targets a seeded perturbation of the forward.
    The forward runs with its field output in the adjoint's own shape (8
    lanes per line), so F holds the field bits every step used."""
    torch = pytest.importorskip("torch")
    ch, seeds, rows = em.workloads.make("adjoint_1024", seed=1234)
    idx = np.linspace(0, len(seeds) - 1, 256).astype(int)
    n = len(idx)
    V = torch.zeros((3, rows, n), dtype=torch.float32, device="cuda")
    V[:, 0, :] = torch.from_numpy(seeds[idx].T.astype(np.float32)).cuda()
    F = torch.zeros(3 * n * (rows - 1), dtype=torch.float32, device="cuda")
    dch = torch.from_numpy(np.ascontiguousarray(ch, np.float32)).cuda()
    rc, _ = em.calc_field(V[0].reshape(-1), V[1].reshape(-1), V[2].reshape(-1),
                          dch, n, 1.0, True, require_n64=False, field_out=F,
                          threads_per_line=8, lines_per_thread=1)
    assert rc == 0
    gen = torch.Generator(device="cuda")
    gen.manual_seed(5)
    T = V + 0.1 * torch.randn(V.shape, generator=gen, device="cuda")
    W = torch.zeros_like(V)
    W[:, 0, :] = V[:, 0, :]
    return ch, dch, V, W, T, F.view(3, rows - 1, n)


# Over the adjoint benchmark's 4000 rows the backward amplifies per-step
# differences at the level of FP32 rounding about 2000-fold: lines circle
# charges 0.01 to 0.5 away for thousands of steps.  The GPU's frozen map takes
# its directions from the FP32 field (u = E'/|E'| in FP32, within about 6e-8
# of the same direction in FP64), so even the FP64 adjoint of that map differs
# from the GPU's by about 1.2e-4 of the gradient (4.5e-5 at 1000 rows); FP64
# projections in the backward, Newton-corrected 1/|r|, compensated adjoint
# state or gradient flushes every 32 rows all left that figure unchanged.
SCALE_RTOL = 2e-4
SCALE_ENTRY_RTOL = 3e-4


@pytest.mark.parametrize("checkpoint", [False, True])
def test_adjoint_at_benchmark_scale(em, gpu, orc, scale_case, checkpoint):
    """Gradients with respect to all 1024 x 3 positions and 1024 magnitudes
    over 4000 rows, against the FP64 adjoint of the GPU's own frozen map:
    linearised at its trajectory with the step lengths (the reference's FP32
    step sequence), directions and |E| of the field its forward used; the
    Jacobian products in FP64.  Within SCALE_RTOL overall and
    SCALE_ENTRY_RTOL on each of the 32 largest entries (the conditioning
    note above)."""
    import torch
    ch, dch, V, W, T, F = scale_case
    loss, grad, _, _ = em.adjoint_device(W, dch, T, checkpoint=checkpoint)
    torch.cuda.synchronize()
    assert torch.equal(W, V)  # the adjoint's forward is the traced one
    L, g = orc.adjoint_at_field(ch.astype(np.float64), W.double().cpu().numpy(),
                                T.double().cpu().numpy(),
                                F.double().cpu().numpy())
    gg = grad.cpu().numpy()
    assert float(loss.item()) == pytest.approx(L, rel=1e-6)
    assert rel(gg, g) <= SCALE_RTOL
    big = np.argsort(-np.abs(g).ravel())[:32]
    assert np.all(np.abs(gg.ravel()[big] - g.ravel()[big])
                  <= SCALE_ENTRY_RTOL * np.abs(g.ravel()[big]))


def test_adjoint_scale_sensitivity_to_the_forward_field(em, gpu, orc, scale_case):
    """Linearised instead with the FP64 field at the same vertices, the
    reference's step lengths and directions differ from the GPU's by the
    FP32 field's rounding (about 1e-7, up to 1e-5 where terms cancel); over
    4000 rows the backward amplifies those differences to about 1e-3 of the
    gradient (2e-5 at 250 rows, 7e-5 at 1000 and 2000).  The bound records
    that measurement."""
    import torch
    ch, dch, V, W, T, F = scale_case
    _, grad, _, _ = em.adjoint_device(W, dch, T)
    torch.cuda.synchronize()
    _, g64 = orc.adjoint_at(ch.astype(np.float64), W.double().cpu().numpy(),
                            T.double().cpu().numpy())
    assert rel(grad.cpu().numpy(), g64) <= 3e-3
