"""The Verlet step of moving charges (em_verlet_step_*) against the FP64
restatement (oracle/em_nbody_oracle.py; the reference's own template cannot
be instantiated, so parity for this step is unpinned)."""
import numpy as np
import pytest

import em_nbody_oracle as N

pytestmark = pytest.mark.gpu


def system(n, p, seed=4, vscale=1e3):
    rng = np.random.default_rng(seed)
    dyn = np.zeros((n, 8))
    dyn[:, :3] = rng.uniform(-10, 10, (n, 3))
    dyn[:, 3] = rng.uniform(-1, 1, n) * 1e-5
    dyn[:, 4:7] = rng.normal(0, vscale, (n, 3))
    dyn[:, 7] = rng.uniform(1e-3, 1e-2, n)
    acc = rng.normal(0, 10, (n, 3))
    ch = np.zeros((p, 4))
    ch[:, :3] = rng.uniform(-12, 12, (p, 3))
    ch[:, 3] = rng.uniform(-1, 1, p) * 1e-6
    return dyn, acc, ch


BOX = ([-11.0] * 3, [11.0] * 3)


def rel(a, b):
    """max |a - b| / max |b| (the absolute difference when b is all zero)."""
    scale = np.abs(b).max()
    return np.abs(a - b).max() / (scale if scale > 0 else 1.0)


@pytest.mark.parametrize("n,p", [(1, 0), (200, 0), (300, 77), (1000, 1500)])
@pytest.mark.parametrize("lanes", [0, 1, 2, 4])
def test_fp64_matches_restatement(em, gpu, n, p, lanes):
    dyn, acc, ch = system(n, p)
    ref_dyn, ref_acc = N.verlet_step(dyn, acc, ch, *BOX, 1e-4)
    d, a = dyn.copy(), acc.copy()
    em.verlet_step(d, a, ch.copy(), *BOX, 1e-4, lanes_per_particle=lanes)
    assert rel(a, ref_acc) <= 1e-12
    assert rel(d[:, :3], ref_dyn[:, :3]) <= 1e-14
    assert rel(d[:, 4:7], ref_dyn[:, 4:7]) <= 1e-12
    assert np.array_equal(d[:, [3, 7]], dyn[:, [3, 7]])


def test_fast_charges_magnetic_term(em, gpu):
    """Speeds near c (v^2/c^2 ~ 0.1): the v x B force is a tenth of the
    electric one, so the magnetic sums are checked too."""
    dyn, acc, ch = system(300, 50, seed=9, vscale=1e8)
    ref_dyn, ref_acc = N.verlet_step(dyn, acc, ch, *BOX, 1e-10)
    d, a = dyn.copy(), acc.copy()
    em.verlet_step(d, a, ch.copy(), *BOX, 1e-10)
    assert rel(a, ref_acc) <= 1e-12
    # the magnetic part alone, from a run without it in the restatement
    saved = N.MAGNETO_K
    try:
        N.MAGNETO_K = 0.0
        _, acc_e = N.verlet_step(dyn, acc, ch, *BOX, 1e-10)
    finally:
        N.MAGNETO_K = saved
    assert rel(a - acc_e, ref_acc - acc_e) <= 1e-9
    assert np.abs(ref_acc - acc_e).max() > 1e-3 * np.abs(ref_acc).max()


def test_fp32_within_tolerance(em, gpu):
    dyn, acc, ch = system(1000, 1500)
    ref_dyn, ref_acc = N.verlet_step(dyn, acc, ch, *BOX, 1e-4)
    d = dyn.astype(np.float32)
    a = acc.astype(np.float32)
    em.verlet_step(d, a, ch.astype(np.float32), *BOX, 1e-4)
    assert rel(a.astype(np.float64), ref_acc) <= 1e-4
    assert rel(d[:, :3].astype(np.float64), ref_dyn[:, :3]) <= 1e-6


def test_steps_equal_repeated_calls_bitwise(em, gpu):
    dyn, acc, ch = system(500, 100)
    d1, a1 = dyn.copy(), acc.copy()
    em.verlet_step(d1, a1, ch.copy(), *BOX, 1e-4, steps=3)
    d2, a2 = dyn.copy(), acc.copy()
    for _ in range(3):
        em.verlet_step(d2, a2, ch.copy(), *BOX, 1e-4)
    assert np.array_equal(d1, d2) and np.array_equal(a1, a2)


def test_device_tensors_match_host(em, gpu):
    torch = pytest.importorskip("torch")
    dyn, acc, ch = system(700, 300)
    dh, ah = dyn.copy(), acc.copy()
    em.verlet_step(dh, ah, ch.copy(), *BOX, 1e-4, steps=2)
    dd = torch.from_numpy(dyn.copy()).cuda()
    ad = torch.from_numpy(acc.copy()).cuda()
    perf = em.verlet_step(dd, ad, torch.from_numpy(ch.copy()).cuda(), *BOX,
                          1e-4, steps=2)
    torch.cuda.synchronize()
    assert np.array_equal(dd.cpu().numpy(), dh)
    assert np.array_equal(ad.cpu().numpy(), ah)
    assert perf.pairs == 2 * 700 * (300 + 699)


def test_empty_system_returns_reference_code(em, gpu):
    import ctypes
    lib = em.load()
    lo = np.zeros(3, np.float32)
    rc = lib.em_verlet_step_f32(None, None, 0, None, 0, lo.ctypes.data,
                                lo.ctypes.data, 0.1, 1, None, None)
    assert rc == 1
