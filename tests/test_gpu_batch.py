"""Batched tracing (em_trace_batch_f32): many charge sets in persistent
launches.  With lane-group widening off, every line's arithmetic is the
single-set tracer's, so each set must equal its own em_trace_lines call bit
for bit, whatever the work items, phases, tiles or graph capture."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def make_sets(em, nsets, seed, pmin=16, pmax=400, per_pos=4):
    rng = np.random.default_rng(seed)
    sets = []
    for i in range(nsets):
        p = int(np.exp(rng.uniform(np.log(pmin), np.log(pmax))))
        ch = em.workloads.uniform_charges(p, 50.0, seed=seed * 1000 + i)
        seeds = em.workloads.fibonacci_seeds(ch, per_pos).astype(np.float32)
        if len(seeds) == 0:
            ch[0, 3] = abs(ch[0, 3])
            seeds = em.workloads.fibonacci_seeds(ch, per_pos).astype(np.float32)
        sets.append((ch, seeds))
    return sets


BATCH_DEFAULT_TPL = 16   # em_batch_options.threads_per_line = 0


def per_set(em, sets, max_steps, lims, store_rows, tpl=BATCH_DEFAULT_TPL):
    """Each set through em_trace_lines with the batch's lanes per line (the
    same lane order, hence the same bits)."""
    out, k = [], 0
    for ch, seeds in sets:
        m = len(seeds)
        r = em.trace_lines(seeds, ch, max_steps, 1.0, 0.5,
                           steps_per_line=lims[k:k + m] if lims is not None
                           else None, deterministic=True,
                           threads_per_line=tpl)
        out.append(r)
        k += m
    return out


def check_equal(b, ref, sets, store_rows):
    k = 0
    for (ch, seeds), r in zip(sets, ref):
        m = len(seeds)
        assert np.array_equal(b["len"][k:k + m], r["len"])
        assert np.array_equal(b["cls"][k:k + m], r["cls"])
        for i in range(m):
            L = r["len"][i]
            assert np.array_equal(b["last"][k + i], r["vertices"][:, L - 1, i])
            rows = min(L, store_rows)
            assert np.array_equal(b["rows"][:, :rows, k + i],
                                  r["vertices"][:, :rows, i])
        k += m


@pytest.fixture(scope="module")
def batch_case(em):
    sets = make_sets(em, 12, 3)
    n = sum(len(s) for _, s in sets)
    lims = np.random.default_rng(4).integers(2, 300, n).astype(np.int32)
    return sets, lims


@pytest.mark.parametrize("kw", [dict(), dict(first_budget=8, phases=4),
                                dict(use_graph=True),
                                dict(lines_per_item=16, threads_per_line=8),
                                dict(threads_per_line=4, first_budget=4,
                                     phases=6)])
def test_batch_equals_per_set_calls(em, gpu, batch_case, kw):
    sets, lims = batch_case
    b = em.trace_batch(sets, 300, 1.0, 0.5, steps_per_line=lims, store_rows=24,
                       deterministic=True, **kw)
    ref = per_set(em, sets, 300, lims, 24,
                  kw.get("threads_per_line", BATCH_DEFAULT_TPL))
    check_equal(b, ref, sets, 24)
    total = sum(float(np.sum(r["perf"].pairs)) for r in ref)
    assert b["perf"].pairs == total


def test_batch_streamed_set(em, gpu):
    """A set too large for shared memory streams through the tile ring."""
    big = em.workloads.uniform_charges(15000, 100.0, seed=21)
    seeds = em.workloads.fibonacci_seeds(big, 1)[:96].astype(np.float32)
    small = make_sets(em, 3, 22)
    sets = [(big, seeds)] + small
    b = em.trace_batch(sets, 60, 1.0, 0.5, store_rows=8, deterministic=True,
                       first_budget=16)
    ref = per_set(em, sets, 60, None, 8)
    check_equal(b, ref, sets, 8)


def test_batch_widening_agrees(em, gpu, batch_case, orc):
    sets, lims = batch_case
    a = em.trace_batch(sets, 300, 1.0, 0.5, steps_per_line=lims,
                       deterministic=True)
    b = em.trace_batch(sets, 300, 1.0, 0.5, steps_per_line=lims)
    agree = (a["cls"] == b["cls"]).mean()
    assert agree >= 0.999, agree


def test_autotuner_returns_a_working_shape(em, gpu, batch_case):
    """The tuner's answer is a complete option dict from its search space
    (the defaults unless a candidate also wins on a second sample), and a
    batch run with it equals the per-set calls."""
    sets, lims = batch_case
    opts = em.autotune.tune_batch(sets, 300, lims, sample=6, use_cache=False,
                                  rounds=1)
    assert set(opts) == set(em.autotune.SPACE)
    for k, v in opts.items():
        assert v in em.autotune.SPACE[k]
    b = em.trace_batch(sets, 300, 1.0, 0.5, steps_per_line=lims,
                       deterministic=True, **opts)
    ref = per_set(em, sets, 300, lims, 0, tpl=opts["threads_per_line"])
    k = 0
    for (ch, seeds), r in zip(sets, ref):
        m = len(seeds)
        assert np.array_equal(b["len"][k:k + m], r["len"])
        k += m
