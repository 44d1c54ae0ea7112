"""The batched tracer's autotuner (autotune.tune_batch) with the timing
replaced by a model: a candidate that wins on the tuning sample but not on
the second, independent sample must not be returned."""
import importlib

import numpy as np


def _sets(n=40):
    rng = np.random.default_rng(1)
    return [(np.zeros((int(rng.integers(8, 64)), 4), np.float32),
             np.zeros((int(rng.integers(4, 16)), 3), np.float32)) for _ in range(n)]


def _run(monkeypatch, timing):
    at = importlib.import_module("electromag-with-cuda_gb300.autotune")
    calls = []

    def fake_time(sub, max_steps, lims, opts, repeats=2):
        calls.append((len(sub), dict(opts)))
        return timing(sub, opts)

    monkeypatch.setattr(at, "_time", fake_time)
    sets = _sets()
    lims = np.full(sum(len(s) for _, s in sets), 100, np.int32)
    return at, at.tune_batch(sets, 100, lims, sample=8, use_cache=False), calls


def test_defaults_when_nothing_wins(monkeypatch):
    at, best, _ = _run(monkeypatch, lambda sub, o: 1.0)
    assert best == {k: v[0] for k, v in at.SPACE.items()}


def test_winner_must_hold_on_a_second_sample(monkeypatch):
    first = {}

    def timing(sub, o):
        key = id(sub[0][0])
        first.setdefault("tuning", key)
        on_tuning_sample = key == first["tuning"]
        return 0.8 if (o["tile_charges"] == 2048 and on_tuning_sample) else 1.0

    at, best, _ = _run(monkeypatch, timing)
    assert best["tile_charges"] == at.SPACE["tile_charges"][0]


def test_winner_that_holds_is_kept(monkeypatch):
    at, best, _ = _run(monkeypatch,
                       lambda sub, o: 0.8 if o["tile_charges"] == 2048 else 1.0)
    assert best["tile_charges"] == 2048
    assert "first_budget" not in best
