"""The FP64 adjoint references (oracle/em_oracle.c) agree among themselves:
the discrete adjoint with the complex-step derivative to machine precision,
and with central differences (h = 1e-3) to their truncation error."""
import numpy as np


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
