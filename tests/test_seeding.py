"""Seeding (host code in libemgb300.so, no GPU needed)."""
import numpy as np


def test_seed_fibonacci_matches_definition(em):
    ch = em.workloads.uniform_charges(40, 50.0, seed=2)
    got = em.seed_fibonacci(ch, 8, 1.0)
    want = em.workloads.fibonacci_seeds(ch, 8, 1.0)
    assert got.shape == want.shape == (8 * int((ch[:, 3] > 0).sum()), 3)
    assert np.allclose(got, want, rtol=0, atol=1e-5)
    pos = ch[ch[:, 3] > 0, :3].astype(np.float64)
    d = np.linalg.norm(got.reshape(-1, 8, 3) - pos[:, None, :], axis=2)
    assert np.allclose(d, 1.0, atol=1e-5)


def test_seed_fibonacci_directions_spread_evenly(em):
    ch = np.array([[0, 0, 0, 1.0]], np.float32)
    s = em.seed_fibonacci(ch, 64, 1.0).astype(np.float64)
    assert np.linalg.norm(s.mean(0)) < 0.05
