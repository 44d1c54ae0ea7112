"""The FP64 adjoint references (oracle/em_oracle.c) agree among themselves:
the discrete adjoint with the complex-step derivative to machine precision,
and with central differences (h = 1e-3) to their truncation error."""
import numpy as np
import pytest


def rel(a, b):
    return np.linalg.norm(np.ravel(a) - np.ravel(b)) / np.linalg.norm(np.ravel(b))


def test_discrete_adjoint_equals_complex_step(adjoint_case):
    fz = adjoint_case[-1]
    g = fz.grad()
    cs = np.array([[fz.complex_step(j, c) for c in range(4)]
                   for j in range(len(fz.ch))])
    assert rel(g, cs) <= 1e-12


def test_discrete_adjoint_close_to_central_differences(adjoint_case):
    fz = adjoint_case[-1]
    g = fz.grad()
    fd = np.array([[fz.central(j, c, 1e-3) for c in range(4)]
                   for j in range(len(fz.ch))])
    assert rel(g, fd) <= 1e-3, rel(g, fd)


def test_adjoint_at_trajectory_equals_frozen_adjoint(orc, adjoint_case):
    """Linearised at the FP64 trajectory itself, the at-trajectory adjoint
    recomputes the same step lengths and reproduces the frozen adjoint."""
    ch, seeds, rows, targets, fz = adjoint_case
    V = np.stack([v.reshape(rows, -1) for v in fz.V])
    L, g = orc.adjoint_at(ch, V, targets)
    assert L == pytest.approx(fz.L, rel=1e-14)
    assert np.allclose(g, fz.grad(), rtol=0, atol=1e-12 * np.abs(g).max())


@pytest.fixture(scope="module")
def adjoint_scale_case(em, orc):
    """The adjoint benchmark's charge set (1024 charges uniform in a cube of
    side 100, |q| in U[1,10], random sign), 8 of its lines for the full 4000
    rows, targets a seeded perturbation of the FP64 forward."""
    ch, seeds, rows = em.workloads.make("adjoint_1024", seed=1234)
    idx = np.linspace(0, len(seeds) - 1, 8).astype(int)
    s = seeds[idx].astype(np.float32).astype(np.float64)
    ch = ch.astype(np.float64)
    fz = orc.Frozen(ch, s, rows, np.zeros((3, rows, len(s))))
    V = np.stack([v.reshape(rows, -1) for v in fz.V])
    rng = np.random.default_rng(5)
    fz = orc.Frozen(ch, s, rows, V + rng.normal(0, 0.1, V.shape))
    return fz


def test_adjoint_at_benchmark_length(adjoint_scale_case):
    """At the adjoint benchmark's length (4000 rows, 1024 charges) the FP64
    discrete adjoint still equals the complex-step derivative to rounding
    on sampled entries and on the largest ones.  Central differences with
    h = 1e-3 agree within their truncation error on the sampled entries;
    the largest entries belong to charges that lines circle for thousands
    of steps, where the loss is nonlinear on the scale of h (their central
    differences are off by percents), so the complex step is the reference
    there."""
    fz = adjoint_scale_case
    g = fz.grad()
    rng = np.random.default_rng(11)
    sampled = list(zip(rng.integers(0, len(fz.ch), 4).tolist(),
                       rng.integers(0, 4, 4).tolist()))
    big = np.unravel_index(np.argsort(-np.abs(g).ravel())[:2], g.shape)
    for j, c in sampled + list(zip(big[0].tolist(), big[1].tolist())):
        cs = fz.complex_step(j, c)
        assert abs(g[j, c] - cs) <= 1e-9 * abs(cs) + 1e-12 * np.abs(g).max()
    for j, c in sampled:
        fd = fz.central(j, c, 1e-3)
        assert abs(g[j, c] - fd) <= 1e-3 * abs(fd) + 1e-6 * np.abs(g).max()


def test_adjoint_at_given_fp64_field_equals_adjoint_at(orc, adjoint_case):
    """Given the FP64 field at each vertex, the at-field adjoint is the
    at-trajectory adjoint (the field is what the latter recomputes)."""
    ch, seeds, rows, targets, fz = adjoint_case
    V = np.stack([v.reshape(rows, -1) for v in fz.V])
    n = V.shape[2]
    pts = V[:, :-1, :].reshape(3, -1).T
    F = orc.field_f64(pts, ch).T.reshape(3, rows - 1, n)
    L1, g1 = orc.adjoint_at(ch, V, targets)
    L2, g2 = orc.adjoint_at_field(ch, V, targets, F, lam_fp32=False)
    assert L1 == L2
    assert np.allclose(g2, g1, rtol=0, atol=1e-12 * np.abs(g1).max())
