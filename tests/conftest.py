import importlib
import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)
ORACLE_DIR = os.path.join(ROOT, "oracle")
if ORACLE_DIR not in sys.path:
    sys.path.insert(0, ORACLE_DIR)

GOLDEN = os.path.join(ROOT, "tests", "golden", "reference_vectors.npz")


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


@pytest.fixture(scope="session")
def em():
    """The package (directory name has hyphens, so import via importlib)."""
    return importlib.import_module("electromag-with-cuda_gb300")


@pytest.fixture(scope="session")
def orc():
    import em_oracle
    em_oracle.load()
    return em_oracle


class Golden:
    def __init__(self, path):
        self.z = np.load(path, allow_pickle=False)
        self.meta = json.loads(str(self.z["meta"]))
        self.cases = {c["name"]: c for c in self.meta["cases"]}

    def inputs(self, name):
        c = self.cases[name]
        dt = np.float32 if c["dtype"] == "f32" else np.float64
        return (c, self.z[name + "/seeds"].astype(dt),
                self.z[name + "/charges"].astype(dt))

    def get(self, build, name, key):
        return self.z[f"{build}/{name}/{key}"]

    def has(self, build, name, key):
        return f"{build}/{name}/{key}" in self.z.files


@pytest.fixture(scope="session")
def golden():
    return Golden(GOLDEN)


@pytest.fixture(scope="session")
def gpu(em):
    """Skips unless a CUDA device is visible; then the library must work."""
    lib = em.load()
    if lib.em_device_count() < 1:
        pytest.skip("no CUDA device")
    return lib


def lines_from(seeds, steps, dtype):
    n = len(seeds)
    out = []
    for c in range(3):
        a = np.zeros(n * steps, dtype)
        a[:n] = seeds[:, c]
        out.append(a)
    return out


@pytest.fixture(scope="session")
def adjoint_case(orc):
    """24 charges in [-10,10]^3, 48 lines seeded 35..45 from the origin
    (well conditioned: no line comes near a charge in 24 rows)."""
    rng = np.random.default_rng(42)
    p, n, rows = 24, 48, 24
    ch = np.zeros((p, 4))
    ch[:, :3] = rng.uniform(-10, 10, (p, 3))
    ch[:, 3] = rng.uniform(1, 10, p) * rng.choice([-1, 1], p)
    d = rng.normal(size=(n, 3))
    seeds = d / np.linalg.norm(d, axis=1, keepdims=True) * rng.uniform(35, 45, (n, 1))
    ch = ch.astype(np.float32).astype(np.float64)
    seeds = seeds.astype(np.float32).astype(np.float64)
    fz = orc.Frozen(ch, seeds, rows, np.zeros((3, rows, n)))
    V = np.stack([v.reshape(rows, n) for v in fz.V])
    targets = (V + rng.normal(0, 0.1, V.shape)).astype(np.float32)
    fz = orc.Frozen(ch, seeds, rows, targets.astype(np.float64))
    return ch, seeds, rows, targets, fz


