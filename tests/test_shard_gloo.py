"""Line sharding across ranks: two gloo ranks on CPU each trace their shard
of lines with the CPU oracle and gather; the result equals one process
tracing every line (lines are independent: no exchange while tracing)."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def test_shard_ranges_cover_exactly(em):
    for n in (0, 1, 7, 64, 1000):
        for w in (1, 2, 3, 8):
            got = []
            for r in range(w):
                b, e = em.shard.shard_range(n, w, r)
                got.extend(range(b, e))
            assert got == list(range(n))
            sizes = [em.shard.shard_range(n, w, r) for r in range(w)]
            assert max(e - b for b, e in sizes) - min(e - b for b, e in sizes) <= 1


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_path):
    import importlib
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    em = importlib.import_module("electromag-with-cuda_gb300")
    import em_oracle as orc
    ch, seeds, _ = em.workloads.make("cpu_256", seed=4)
    n, steps = len(seeds), 30
    b, e = em.shard.shard_range(n, world, rank)
    _, ln, cl = orc.trace_lines_f64(ch.astype(np.float64), seeds[b:e], steps,
                                    1.0, 0.5, nthreads=1)
    L = em.shard.gather_lines(ln, n, world, rank)
    C = em.shard.gather_lines(cl, n, world, rank)
    if rank == 0:
        np.savez(out_path, len=L, cls=C)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_equal_single_process(em, orc, tmp_path):
    out = str(tmp_path / "gathered.npz")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    g = np.load(out)
    ch, seeds, _ = em.workloads.make("cpu_256", seed=4)
    _, ln, cl = orc.trace_lines_f64(ch.astype(np.float64), seeds, 30, 1.0, 0.5)
    assert np.array_equal(g["len"], ln)
    assert np.array_equal(g["cls"], cl)


def _adjoint_worker(rank, world, port, out_path):
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    sys.path.insert(0, os.path.join(root, "tests"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import importlib
    em = importlib.import_module("electromag-with-cuda_gb300")
    import em_oracle as orc
    ch, seeds, rows, targets = _adjoint_inputs()

    def shard_grad(s, t):
        # the FP64 discrete adjoint of this rank's lines (the GPU path calls
        # em.adjoint here)
        fz = orc.Frozen(ch, s, rows, t)
        return fz.L, fz.grad()

    L, g = em.shard.adjoint_sharded(shard_grad, seeds, targets, world, rank)
    np.savez(out_path + f".{rank}.npz", loss=L, grad=g)
    dist.barrier()
    dist.destroy_process_group()


def _adjoint_inputs():
    rng = np.random.default_rng(11)
    p, n, rows = 16, 37, 12
    ch = np.zeros((p, 4))
    ch[:, :3] = rng.uniform(-10, 10, (p, 3))
    ch[:, 3] = rng.uniform(1, 10, p) * rng.choice([-1, 1], p, p=[0.3, 0.7])
    d = rng.normal(size=(n, 3))
    seeds = d / np.linalg.norm(d, axis=1, keepdims=True) * rng.uniform(35, 45, (n, 1))
    targets = rng.normal(0, 40, (3, rows, n))
    return ch, seeds, rows, targets


def test_sharded_adjoint_equals_single_process(em, orc, tmp_path):
    """Two gloo ranks, 18 and 19 lines: one all-reduce of loss and
    gradients gives the one-process adjoint of all 37 lines on both ranks."""
    out = str(tmp_path / "adj")
    mp.spawn(_adjoint_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    ch, seeds, rows, targets = _adjoint_inputs()
    fz = orc.Frozen(ch, seeds, rows, targets)
    ref_g = fz.grad()
    for r in range(2):
        z = np.load(out + f".{r}.npz")
        assert float(z["loss"]) == pytest.approx(fz.L, rel=1e-12)
        assert np.allclose(z["grad"], ref_g, rtol=1e-10, atol=1e-12 * np.abs(ref_g).max())


def _trace_worker(rank, world, port, out_path):
    """bench.py's sharded mode on CPU ranks: shard the lines, trace each
    shard (here with the oracle's restatement of the reference's FP32 path,
    where bench.py calls the GPU tracer), gather along the line axis."""
    import importlib
    import sys
    import torch.distributed as dist
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    sys.path.insert(0, root)
    sys.path.insert(0, os.path.join(root, "oracle"))
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    em = importlib.import_module("electromag-with-cuda_gb300")
    import em_oracle as orc
    ch, seeds, rows = _trace_inputs(em)

    def trace(s):
        X = [np.zeros(len(s) * rows, np.float32) for _ in range(3)]
        for c in range(3):
            X[c][:len(s)] = s[:, c]
        # the generic curvature rule takes any line count (the SSE form
        # wants multiples of 64)
        assert orc.calc_field(*X, ch, len(s), 1.0, orc.CURV_GENERIC, nthreads=1) == 0
        return np.stack([x.reshape(rows, len(s)) for x in X])

    V, (b, e) = em.shard.trace_sharded(trace, seeds, world, rank)
    np.savez(out_path + f".{rank}.npz", V=V, b=b, e=e)
    dist.barrier()
    dist.destroy_process_group()


def _trace_inputs(em):
    ch, seeds, _ = em.workloads.make("cpu_256", seed=9)
    # 1001 lines: the ranks' shards differ in size (500 and 501)
    seeds = np.resize(seeds.astype(np.float32), (1001, 3))
    return np.ascontiguousarray(ch, np.float32), seeds, 40


def test_sharded_trace_gathers_the_single_process_result(em, orc, tmp_path):
    """Two gloo ranks trace 500 and 501 lines of one workload; after the
    gather both hold the vertices of the whole trace, bit for bit those of
    one process tracing every line."""
    out = str(tmp_path / "tr")
    mp.spawn(_trace_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    ch, seeds, rows = _trace_inputs(em)
    n = len(seeds)
    X = [np.zeros(n * rows, np.float32) for _ in range(3)]
    for c in range(3):
        X[c][:n] = seeds[:, c]
    assert orc.calc_field(*X, ch, n, 1.0, orc.CURV_GENERIC) == 0
    ref = np.stack([x.reshape(rows, n) for x in X])
    spans = []
    for r in range(2):
        z = np.load(out + f".{r}.npz")
        assert np.array_equal(z["V"], ref)
        spans.append((int(z["b"]), int(z["e"])))
    assert spans == [(0, 501), (501, 1001)]
