"""The FP64 Verlet restatement (oracle/em_nbody_oracle.py) on closed-form
cases: a free particle, Coulomb repulsion of a pair, the magnetic force of a
moving charge, and reflection off the box."""
import numpy as np
import pytest

import em_nbody_oracle as N

BIG = [1e9] * 3


def test_free_particle_moves_ballistically():
    dyn = np.array([[1.0, 2.0, 3.0, 0.0, 0.5, -1.0, 2.0, 3.0]])
    out, acc = N.verlet_step(dyn, np.zeros((1, 3)), np.zeros((0, 4)),
                             [-1e9] * 3, BIG, 0.1)
    assert np.allclose(out[0, :3], [1.05, 1.9, 3.2])
    assert np.all(acc == 0)


def test_pair_coulomb_repulsion():
    """Two charges 2 apart on x, at rest, dt -> 0: a = K q1 q2 / (m d^2)."""
    q1, q2, m = 1e-6, 2e-6, 0.5
    dyn = np.array([[-1.0, 0, 0, q1, 0, 0, 0, m], [1.0, 0, 0, q2, 0, 0, 0, m]])
    _, acc = N.verlet_step(dyn, np.zeros((2, 3)), np.zeros((0, 4)),
                           [-1e9] * 3, BIG, 0.0)
    f = N.ELECTRO_K * q1 * q2 / 4.0
    assert acc[0] == pytest.approx([-f / m, 0, 0])
    assert acc[1] == pytest.approx([f / m, 0, 0])


def test_moving_source_magnetic_force():
    """Source at the origin moving along y; test charge at x = 1 moving
    along z: B = 1e-7 q v x r / r^3 = -1e-7 q v z_hat; F adds q v' x B."""
    qs, vs, qt, vt, m = 3.0, 2.0, 5.0, 4.0, 1.0
    dyn = np.array([[0.0, 0, 0, qs, 0, vs, 0, 1e30],
                    [1.0, 0, 0, qt, 0, 0, vt, m]])
    _, acc = N.verlet_step(dyn, np.zeros((2, 3)), np.zeros((0, 4)),
                           [-1e9] * 3, BIG, 0.0)
    Bz = -N.MAGNETO_K * qs * vs               # v_s x r = (0, vs, 0) x (1, 0, 0)
    Ex = N.ELECTRO_K * qs
    fm = qt * np.cross([0, 0, vt], [0, 0, Bz])   # zero: v parallel to B
    assert acc[1] == pytest.approx(np.array([qt * Ex, 0, 0]) + fm)
    dyn[1, 4:7] = [0, vt, 0]                     # now v' x B along x
    _, acc = N.verlet_step(dyn, np.zeros((2, 3)), np.zeros((0, 4)),
                           [-1e9] * 3, BIG, 0.0)
    assert acc[1] == pytest.approx([qt * Ex + qt * vt * Bz, 0, 0])


def test_box_reflection():
    dyn = np.array([[0.9, -0.95, 0.0, 0.0, 1.0, -1.0, 0.0, 1.0]])
    out, _ = N.verlet_step(dyn, np.zeros((1, 3)), np.zeros((0, 4)),
                           [-1, -1, -1], [1, 1, 1], 0.2)
    assert out[0, :3] == pytest.approx([0.9, -0.85, 0.0])   # mirrored back
    assert out[0, 4:7] == pytest.approx([-1.0, 1.0, 0.0])
