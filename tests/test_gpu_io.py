"""The reference program's own runs and its --autoregress check on the GPU:
the default and --bogo presets traced from the library's generators hash to
the reference's outputs, and the divergence scan with its report matches
the numpy restatement (oracle/em_io_oracle.py)."""
import hashlib

import numpy as np
import pytest

import em_io_oracle as O
from conftest import lines_from

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("preset,name", [("bogo", "preset_bogo"),
                                         ("normal", "preset_normal")])
def test_reference_preset_run_bit_for_bit(em, gpu, golden, preset, name):
    """The reference's main() run for a preset (srand(1) charges, grid
    seeds, curvature, resolution 1): the whole vertex array hashes to the
    reference's own."""
    ch, seeds, rows = em.inputs.reference_case(preset)
    n = len(seeds)
    x, y, z = lines_from(seeds, rows, np.float32)
    rc, _ = em.calc_field(x, y, z, ch, n, 1.0, True, arith="exact")
    assert rc == 0
    v = np.stack([a.reshape(rows, n) for a in (x, y, z)])
    assert hashlib.sha256(v.tobytes()).hexdigest() == str(
        golden.get("strict", name, "sha256"))
    c = golden.cases[name]
    assert np.array_equal(v[:, c["rows"]], golden.get("strict", name, "vertices"))


def crafted(seed=5, n=70, rows=90):
    """Two runs that part at chosen rows: row 0, mid-line, the last row, a
    NaN (never counts), an offset just under the threshold, and none."""
    rng = np.random.default_rng(seed)
    a = rng.normal(0, 50, (3, rows, n)).astype(np.float32)
    b = a.copy()
    plan = {0: 0, 1: 17, 2: rows - 1, 3: 40, 5: 63, 6: 64, 7: 65, 9: 1}
    for line, row in plan.items():
        b[:, row:, line] += np.float32(0.2)
    b[0, 30, 11] = np.nan                     # NaN offset: not > threshold
    b[1, 12:, 12] += np.float32(0.0999)       # just under 0.1
    b[2, 50:, 13] += np.float32(0.1001)       # just over
    return a, b


@pytest.mark.parametrize("device", [False, True])
def test_autoregress_matches_oracle(em, gpu, tmp_path, device):
    a, b = crafted()
    rows, n = a.shape[1], a.shape[2]
    path = tmp_path / "regression.txt"
    if device:
        import torch
        first, count = em.outputs.autoregress(torch.from_numpy(a).cuda(),
                                              torch.from_numpy(b).cuda(),
                                              path=path)
    else:
        first, count = em.outputs.autoregress(a, b, path=path)
    ref_first, ref_text = O.autoregress(n, rows, a.reshape(3, -1), b.reshape(3, -1))
    assert np.array_equal(first, ref_first)
    assert count == int((ref_first >= 0).sum())
    assert path.read_text() == ref_text
    assert first[0] == 0 and first[1] == 17 and first[11] == -1 and first[12] == -1
    assert first[13] == 50


def test_autoregress_exact_against_fast_run(em, gpu):
    """The check used as intended: the same workload (256 charges, 8 seeds
    per positive charge, 501 rows) traced with the reference's arithmetic
    and with the fast arithmetic; the scan agrees with the restatement."""
    ch, seeds, _ = em.workloads.make("cpu_256", seed=7)
    seeds = em.workloads.pad_lines(seeds.astype(np.float32), 64)
    ch = np.ascontiguousarray(ch, np.float32)
    n, rows = len(seeds), 501
    runs = []
    for arith in ("exact", "fast"):
        x, y, z = lines_from(seeds, rows, np.float32)
        rc, _ = em.calc_field(x, y, z, ch, n, 1.0, True, arith=arith,
                              require_n64=False)
        assert rc == 0
        runs.append(np.stack([v.reshape(rows, n) for v in (x, y, z)]))
    first, count = em.outputs.autoregress(runs[0], runs[1])
    ref_first, _ = O.autoregress(n, rows, runs[0].reshape(3, -1),
                                 runs[1].reshape(3, -1))
    assert np.array_equal(first, ref_first)
    assert count == int((ref_first >= 0).sum())


def test_autoregress_identical_runs(em, gpu):
    a, _ = crafted(n=33, rows=200)
    first, count = em.outputs.autoregress(a, a.copy())
    assert count == 0 and np.all(first == -1)
