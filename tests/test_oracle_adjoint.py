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
