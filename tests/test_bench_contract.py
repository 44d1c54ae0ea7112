"""bench.py's reference arm prints the contract's JSON line (CPU only: the
oracle's timing is replaced by a stub, so the test checks the line's form,
not a rate)."""
import argparse
import importlib.util
import json
import os

import pytest

from conftest import ROOT


@pytest.fixture
def bench(monkeypatch):
    spec = importlib.util.spec_from_file_location(
        "bench_under_test", os.path.join(ROOT, "bench.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    calls = []

    def fake_rate(orc, ch, seeds, rows, seconds, nthreads):
        calls.append(seconds)
        return 2.5, dict(lines=64, rows=3, pairs=64 * 2 * len(ch), seconds=0.25)

    monkeypatch.setattr(mod, "cpu_rate", fake_rate)
    mod.calls = calls
    return mod


def args(**kw):
    a = dict(gpus=1, steps=2, warmup=3, impl="reference", workload="gpu_4096",
             rows=None, seed=1234)
    a.update(kw)
    return argparse.Namespace(**a)


def test_reference_arm_line(bench, capsys, monkeypatch):
    monkeypatch.delenv("RANK", raising=False)
    assert bench.run_reference(args()) == 0
    line = json.loads(capsys.readouterr().out.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == bench.UNIT
    assert line["higher_is_better"] is True
    assert line["steps"] == 2 and line["warmup"] == 3 and line["n_gpus"] == 1
    assert line["value"] == 2.5
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == 2.5
    assert line["e2e"] == {"value": 2.5, "unit": bench.UNIT,
                           "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # the same workload keys and values as the GPU arm's line
    ours = bench.workload_config(args(), line["config"]["lines"],
                                 line["config"]["charges"],
                                 line["config"]["rows"], 1, "x")
    assert set(line["config"]) == set(ours)
    for k in ours:
        if k != "arith":
            assert line["config"][k] == ours[k]
    assert line["config"]["lines"] == 32736 and line["config"]["rows"] == 5000
    assert line["data"] == bench.DATA
    # warm-up samples first, then one sample per timed step
    assert len(bench.calls) == 5


def test_reference_arm_other_ranks_exit_quietly(bench, capsys, monkeypatch):
    monkeypatch.setenv("RANK", "1")
    assert bench.run_reference(args(gpus=2)) == 0
    assert capsys.readouterr().out == ""
    assert bench.calls == []
