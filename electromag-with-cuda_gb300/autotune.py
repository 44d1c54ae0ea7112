"""Autotuner for the batched tracer's launch shape.

Times the batched launch on a sample of the caller's charge sets over the
shape parameters - lanes per line, lines per work item (lines per CTA at a
time), charge-tile size and pipeline stages of the sets streamed through
shared memory - by coordinate descent from the
library's defaults, and caches the winner per GPU and workload signature in
a JSON file (EM_AUTOTUNE_CACHE, default: autotune_cache.json beside this
module).
"""
import json
import os
import time

import numpy as np

from . import tracer

CACHE = os.environ.get("EM_AUTOTUNE_CACHE",
                       os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                    "autotune_cache.json"))

# The first phase's step budget is not searched (it stays the library's
# 64): on sets cut to a sample's line counts a larger budget looked 5-10 %
# faster, on the whole 512-set batch it was 20 % slower (its phases carry
# far more lines than the sample's).
SPACE = {
    "threads_per_line": [16, 8, 4],
    "lines_per_item": [512, 256, 1024],
    "tile_charges": [1024, 2048, 512],
    "stages": [4, 3, 2],
}


def _signature(sets, max_steps):
    p = np.array([len(c) for c, _ in sets])
    n = np.array([len(s) for _, s in sets])
    return (f"sets{len(sets)}_p{int(np.median(p))}_{int(p.max())}"
            f"_n{int(n.sum())}_s{max_steps}")


def _device_key():
    try:
        import torch
        return torch.cuda.get_device_name(0)
    except Exception:  # pragma: no cover - no torch / no device
        return "unknown"


def _load():
    try:
        with open(CACHE) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _time(sets, max_steps, lims, opts, repeats=2):
    best = None
    for _ in range(repeats):
        t0 = time.perf_counter()
        r = tracer.trace_batch(sets, max_steps, 1.0, 0.5,
                               steps_per_line=lims, **opts)
        dt = r["perf"].time or (time.perf_counter() - t0)
        best = dt if best is None else min(best, dt)
    return best


def _sample(sets, steps_per_line, n, seed, lines_cap, cap):
    """`n` sets drawn at random, each cut to its first `lines_cap` lines,
    with their step limits (capped at `cap`)."""
    rng = np.random.default_rng(seed)
    idx = np.sort(rng.choice(len(sets), min(n, len(sets)), replace=False))
    sub = [(sets[i][0], sets[i][1][:lines_cap]) for i in idx]
    lims = None
    if steps_per_line is not None:
        offs = np.concatenate([[0], np.cumsum([len(s) for _, s in sets])])
        lims = np.concatenate([
            np.minimum(steps_per_line[offs[i]:offs[i] + min(lines_cap,
                                                           offs[i + 1] - offs[i])],
                       cap) for i in idx]).astype(np.int32)
    return sub, lims


def tune_batch(sets, max_steps, steps_per_line=None, sample=32, seed=0,
               rounds=2, use_cache=True, lines_cap=1024, steps_cap=None):
    """Returns the best option dict for trace_batch on these sets.

    Trials run on `sample` sets drawn at random, each cut to its first
    `lines_cap` lines: the same mix of set sizes and the same step limits (a
    few long lines carry most of the pairs, and the phase budgets are tuned
    for them, so steps are not capped unless `steps_cap` is given) at a
    fraction of the cost.  A sample of cut sets is noisy and may misjudge the
    whole batch (its phases carry fewer lines), so a step of the descent must
    gain 3 % and the winner must beat the defaults by 5 % on a second,
    independent sample; otherwise the defaults stand."""
    key = _device_key() + "|" + _signature(sets, max_steps)
    cache = _load() if use_cache else {}
    if key in cache:
        return dict(cache[key]["options"])
    cap = max_steps if steps_cap is None else steps_cap
    sub, lims = _sample(sets, steps_per_line, sample, seed, lines_cap, cap)
    max_steps = min(max_steps, cap)
    default = {k: v[0] for k, v in SPACE.items()}
    best = dict(default)
    best_t = _time(sub, max_steps, lims, best)
    trials = [(dict(best), best_t)]
    for _ in range(rounds):
        changed = False
        for k, vals in SPACE.items():
            for v in vals:
                if v == best[k]:
                    continue
                cand = dict(best, **{k: v})
                t = _time(sub, max_steps, lims, cand)
                trials.append((cand, t))
                if t < best_t * 0.97:
                    best, best_t, changed = cand, t, True
        if not changed:
            break
    if best != default:
        vsub, vlims = _sample(sets, steps_per_line, sample, seed + 1, lines_cap, cap)
        if not (_time(vsub, max_steps, vlims, best)
                < 0.95 * _time(vsub, max_steps, vlims, default)):
            best = dict(default)
    if use_cache:
        cache[key] = {"options": best, "seconds": best_t,
                      "trials": len(trials)}
        try:
            with open(CACHE, "w") as f:
                json.dump(cache, f, indent=1)
        except OSError:
            pass
    return dict(best)
