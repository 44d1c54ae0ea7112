"""Seeded synthetic charge sets and seeds for the benchmark workloads.

The reference ships no datasets; these generators stand in with the shapes,
sizes and value distributions of the five benchmark configurations.  All
randomness comes from numpy's PCG64 with the seed recorded by the caller.
"""
import numpy as np

# name -> description used in bench.py's config
CONFIGS = {
    "cpu_256": dict(p=256, half=50.0, lines_per_positive=8, steps=2500),
    "gpu_4096": dict(p=4096, half=100.0, lines_per_positive=16, steps=5000),
    "dipole_16384": dict(dipoles=8192, clusters=32, sigma=5.0, half=100.0,
                         lines=65536, steps=4000),
    "adjoint_1024": dict(p=1024, half=50.0, lines=16384, steps=4000),
}


def uniform_charges(p, half, seed, dtype=np.float32):
    """p charges uniform in [-half, half]^3, |q| in U[1, 10], random sign."""
    rng = np.random.Generator(np.random.PCG64(seed))
    ch = np.empty((p, 4), np.float64)
    ch[:, :3] = rng.uniform(-half, half, (p, 3))
    ch[:, 3] = rng.uniform(1.0, 10.0, p) * rng.choice([-1.0, 1.0], p)
    return ch.astype(dtype)


def dipole_charges(dipoles, clusters, sigma, half, seed, sep=0.01,
                   dtype=np.float32):
    """±q pairs (q in U[1,10], separation sep, random orientation) whose
    centres come from Gaussian clusters (sigma) inside [-half, half]^3."""
    rng = np.random.Generator(np.random.PCG64(seed))
    centres = rng.uniform(-half * 0.9, half * 0.9, (clusters, 3))
    which = rng.integers(0, clusters, dipoles)
    c = np.clip(centres[which] + rng.normal(0, sigma, (dipoles, 3)),
                -half, half)
    d = rng.normal(size=(dipoles, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    q = rng.uniform(1.0, 10.0, dipoles)
    ch = np.empty((2 * dipoles, 4), np.float64)
    ch[0::2, :3] = c + 0.5 * sep * d
    ch[0::2, 3] = q
    ch[1::2, :3] = c - 0.5 * sep * d
    ch[1::2, 3] = -q
    return ch.astype(dtype)


def fibonacci_seeds(charges, per_charge, radius=1.0):
    """per_charge seeds on a sphere of `radius` around every positive charge
    (golden-angle spiral directions), in charge order; float64 (m, 3)."""
    ga = np.pi * (3.0 - np.sqrt(5.0))
    i = np.arange(per_charge, dtype=np.float64)
    zz = 1.0 - (2.0 * i + 1.0) / per_charge
    rr = np.sqrt(1.0 - zz * zz)
    d = np.stack([rr * np.cos(ga * i), rr * np.sin(ga * i), zz], 1)
    pos = np.asarray(charges, np.float64)
    pos = pos[pos[:, 3] > 0, :3]
    return (pos[:, None, :] + radius * d[None]).reshape(-1, 3)


def pad_lines(seeds, multiple):
    """Pads a seed list to a multiple of `multiple` with copies of seed 0
    (the reference's SSE path needs n % 64 == 0)."""
    n = len(seeds)
    m = (n + multiple - 1) // multiple * multiple
    if m == n:
        return seeds
    return np.concatenate([seeds, np.repeat(seeds[:1], m - n, 0)])


def make(name, seed=1234, dtype=np.float32):
    """Returns (charges (p,4), seeds (n,3) float64, steps) for a workload."""
    cfg = CONFIGS[name]
    if name == "dipole_16384":
        ch = dipole_charges(cfg["dipoles"], cfg["clusters"], cfg["sigma"],
                            cfg["half"], seed, dtype=dtype)
        per = max(1, cfg["lines"] // cfg["dipoles"])
        seeds = fibonacci_seeds(ch, per)[: cfg["lines"]]
        return ch, seeds, cfg["steps"]
    ch = uniform_charges(cfg["p"], cfg["half"], seed, dtype=dtype)
    if "lines" in cfg:
        npos = int((ch[:, 3] > 0).sum())
        per = max(1, -(-cfg["lines"] // npos))
        seeds = fibonacci_seeds(ch, per)[: cfg["lines"]]
    else:
        seeds = fibonacci_seeds(ch, cfg["lines_per_positive"])
    return ch, seeds, cfg["steps"]


def make_batch(nsets=512, seed=1234, pmin=64, pmax=32768, half=50.0,
               lines_per_positive=4, steps=(500, 8000)):
    """Independent charge sets for batched tracing: sizes log-uniform in
    [pmin, pmax], charges uniform in [-half, half]^3 with |q| in U[1, 10] and
    random sign, lines_per_positive seeds per positive charge, one step limit
    per set uniform in `steps`.  Returns a list of (charges, seeds, limit)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    sizes = np.exp(rng.uniform(np.log(pmin), np.log(pmax), nsets)).astype(int)
    limits = rng.integers(steps[0], steps[1] + 1, nsets)
    out = []
    for i, (p, lim) in enumerate(zip(sizes, limits)):
        ch = uniform_charges(int(p), half, seed * 7919 + i)
        seeds = fibonacci_seeds(ch, lines_per_positive).astype(np.float32)
        out.append((ch, seeds, int(lim)))
    return out
