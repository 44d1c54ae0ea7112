#!/usr/bin/env python
"""Throughput of the GB300 field-line tracer, one JSON line on rank 0.

A step is one trace of the GPU-scale workload: 4096 charges uniform in
[-100,100]^3 with |q| in U[1,10] and random sign, 16 lines seeded per
positive charge on a radius-1 Fibonacci sphere, 5000 rows per line, the
reference's curvature stepping rule (CalcField_CPU_T_Curvature, SSE form).
  value  pair interactions/s with inputs resident in HBM (device pointers)
  e2e    the same through the host-pointer C ABI call (em_calc_field_ex_f32):
         seeds and charges copied in, all vertices copied out, every step
--impl reference times the reference algorithm's CPU implementation (the
oracle port of CPU_Implement.cpp, OpenMP over all host cores) on bounded
samples of the same workload.
"""
import argparse
import importlib
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
METRIC = ("Gpair-int/s vs plain FP32 at ≤1e-6 field err vs FP64; "
          "adjoint/fwd time ratio")
UNIT = "Gpair-int/s"
FLOP_PER_PAIR = 20  # the FP32-roofline credit per pair interaction
# DRAM bytes (read + write) per trace launch of the 4096-charge workload at
# 5000 rows, from the ncu launch list in profiles/ref_trace_kernel_gpu4096.md
TRAFFIC_GPU4096 = 1.911e9 + 7.8e6


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", default="gpu_4096")
    ap.add_argument("--rows", type=int, default=None,
                    help="override rows per line (quick runs only)")
    ap.add_argument("--seed", type=int, default=1234)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-e2e", action="store_true")
    # launch-shape overrides (0/auto = the library's choice); for profiling
    ap.add_argument("--tpl", type=int, default=0)
    ap.add_argument("--kl", type=int, default=0)
    ap.add_argument("--warps", type=int, default=0)
    ap.add_argument("--pack", default="auto")
    ap.add_argument("--mode", choices=["replicas", "shard"], default="replicas",
                    help="N > 1: every rank traces the whole workload (weak "
                         "scaling) or its contiguous shard of the lines "
                         "(strong scaling, no exchange while tracing)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the single-GPU blocks of the other workloads "
                         "(always skipped when N > 1)")
    ap.add_argument("--case", choices=["ref-mixed", "ext-fp32", "ext-mixed", "ext-df64",
                                       "ext-tail-dipole", "ext-tail-gpu", "exact", "adjoint",
                                       "adjoint-checkpoint", "adjoint-twopass",
                                       "batch", "verlet"],
                    default=None,
                    help="profiling cases: run one small case and exit")
    return ap.parse_args()


def workload(em, name, seed, rows):
    ch, seeds, steps = em.workloads.make(name, seed=seed)
    if rows:
        steps = rows
    return np.ascontiguousarray(ch, np.float32), seeds.astype(np.float32), steps


class ClockSampler:
    """nvidia-smi samples every 200 ms while the timed region runs."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.t.join(timeout=2)

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [],
                    "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx,
                "reasons": sorted(reasons), "samples": len(sm)}


DATA = "synthetic (seeded PCG64)"


def workload_config(args, n, p, rows, world, arith):
    """The workload both arms report: the same keys and values, with the
    arithmetic each arm computes in."""
    return {"workload": args.workload, "lines": int(n), "charges": int(p),
            "rows": int(rows), "seed": args.seed,
            "rule": "curvature, seed vector (CPU_Implement.cpp:207-351)",
            "arith": arith,
            "parallelism": (f"lines sharded x{world}" if getattr(args, "mode", "") == "shard"
                            else f"replicas x{world}"),
            "l2": "vertex output %.2f GB per step exceeds the 129 MB L2"
                  % (3 * 4 * n * rows / 1e9)}


def cpu_rate(orc, ch, seeds, rows, seconds, nthreads):
    """Oracle port on host cores over a bounded sample: all charges, a
    line subset and a row count sized to take about `seconds`."""
    # the reference's SSE path needs n % 64 == 0 (CPU_Implement.cpp:223);
    # pad with copies of seed 0 as a reference user would
    seeds = np.concatenate([seeds, np.repeat(seeds[:1], (-len(seeds)) % 64, 0)])
    n = len(seeds)
    p = len(ch)
    # calibrate on a small sample
    lines = min(n, 256)
    cal_rows = 4
    x = np.zeros(n * cal_rows, np.float32)
    xs = [x.copy(), x.copy(), x.copy()]
    for c in range(3):
        xs[c][:n] = seeds[:, c]
    t = time.perf_counter()
    orc.calc_field(*xs, ch, n, 1.0, orc.CURV_SSE, 0, lines, nthreads)
    dt = max(time.perf_counter() - t, 1e-4)
    rate = lines * (cal_rows - 1) * p / dt
    want_pairs = rate * seconds
    lines = int(min(n, max(64, want_pairs / (p * max(rows - 1, 1)))))
    lines = max(64, lines // 64 * 64) if n >= 64 else n
    srows = int(min(rows, max(2, want_pairs / (lines * p) + 1)))
    xs = [np.zeros(n * srows, np.float32) for _ in range(3)]
    for c in range(3):
        xs[c][:n] = seeds[:, c]
    t = time.perf_counter()
    rc = orc.calc_field(*xs, ch, n, 1.0, orc.CURV_SSE, 0, lines, nthreads)
    dt = time.perf_counter() - t
    if rc:
        raise RuntimeError(f"oracle returned {rc}")
    pairs = lines * (srows - 1) * p
    return pairs / dt / 1e9, dict(lines=lines, rows=srows, pairs=pairs,
                                  seconds=dt)


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    em = importlib.import_module("electromag-with-cuda_gb300")
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import em_oracle as orc
    ch, seeds, rows = workload(em, args.workload, args.seed, args.rows)
    threads = os.cpu_count() or 1
    per_step = max(2.0, 60.0 / max(1, args.steps + args.warmup))
    for _ in range(args.warmup):
        cpu_rate(orc, ch, seeds, rows, min(per_step, 2.0), threads)
    vals, sample = [], None
    for _ in range(args.steps):
        v, sample = cpu_rate(orc, ch, seeds, rows, per_step, threads)
        vals.append(v)
    value = float(np.median(vals))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": sample["seconds"] * 1e3, "higher_is_better": True,
        "scaling": "strong" if getattr(args, "mode", "") == "shard" else "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": DATA,
        "config": workload_config(
            args, len(seeds), len(ch), rows, args.gpus,
            "the reference's FP32 SSE sequence (sqrt + divide), oracle port "
            "on the host cores"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": threads,
                         "kind": "port",
                         "sample": f"{sample['lines']} lines x {len(ch)} charges"
                                   f" x {sample['rows']} rows per step"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def run_case(args):
    """Small profiling cases (ncu captures): the mixed arithmetic on the
    reference-layout tracer (4096 charges, 200 rows), the extended kernel on the
    4096-charge workload (200 rows, no termination radius; FP32, mixed or
    double-float pairs), the extended tracer with its tail kernel on the
    dipole set (1000 rows, termination radius 0.5) or on the 4096-charge
    workload (5000 rows, termination radius 0.5: lines that escape the
    charges run all rows, on the tail kernel), the reference's arithmetic
    bit for bit on the 256-charge configuration (500 rows), the adjoint
    kernels on the 1024-charge workload (200 rows; stored field, or the
    field recomputed per 64-row segment; adjoint-twopass: 6000 charges, the
    two-pass backward of sets above 4096 charges), the batched tracer on the
    first 24 sets of the 512-set workload with the bench's tuned shape
    (limits capped at 500 rows), or the Verlet step (65 536 moving and 4096
    static charges, FP32, 2 steps)."""
    import torch
    em = importlib.import_module("electromag-with-cuda_gb300")
    dev = torch.device("cuda", 0)
    if args.case == "ref-mixed":
        # the mixed arithmetic on the reference-layout tracer, 4096-charge
        # workload (--rows, default 200): once with the default conditioning
        # test, once with re-evaluations off (the pair pass alone)
        ch, seeds, _ = em.workloads.make("gpu_4096", seed=args.seed)
        rows = args.rows or 200
        n = len(seeds)
        dch = torch.from_numpy(np.ascontiguousarray(ch, np.float32)).to(dev)
        for kappa in (0.0, 1e30):
            X = [torch.zeros(n * rows, dtype=torch.float32, device=dev) for _ in range(3)]
            for c in range(3):
                X[c][:n] = torch.from_numpy(np.ascontiguousarray(seeds[:, c], np.float32)).to(dev)
            rc, perf = em.calc_field(*X, dch, n, 1.0, True, arith="mixed",
                                     require_n64=False, refine_kappa=kappa)
            if rc:
                raise em.EmError(rc, "mixed")
            torch.cuda.synchronize()
            print("mixed kappa", kappa or "default", n * (rows - 1) * len(ch) / perf.time / 1e9,
                  "Gpair/s, re-evaluated vertices", perf.fp64_refines)
        return 0
    if args.case == "batch":
        sets = em.workloads.make_batch(512, args.seed)[:24]
        lims = np.concatenate([np.full(len(s), min(lim, 500), np.int32)
                               for _, s, lim in sets])
        kw = dict(threads_per_line=16, lines_per_item=512, first_budget=64,
                  tile_charges=2048, stages=4)
        for _ in range(2):
            out = em.trace_batch([(c, s) for c, s, _ in sets], 500, 1.0, 0.5,
                                 steps_per_line=lims, **kw)
        torch.cuda.synchronize()
        perf = out["perf"]
        print("batch", perf.pairs / perf.time / 1e9, "Gpair/s")
        return 0
    if args.case == "ext-tail-dipole":
        ch, seeds, _ = em.workloads.make("dipole_16384", seed=args.seed)
        ch = torch.from_numpy(np.ascontiguousarray(ch, np.float32)).to(dev)
        s = torch.from_numpy(seeds.astype(np.float32)).to(dev)
        out = em.trace_lines(s, ch, 1000, 1.0, 0.5)
        torch.cuda.synchronize()
        print("tail", out["perf"].pairs / out["perf"].time / 1e9, "Gpair/s")
        return 0
    if args.case == "exact":
        # the reference's arithmetic bit for bit, on the CPU-runnable
        # configuration (256 charges, 1088 lines; --rows, default 500)
        ch, seeds, _ = em.workloads.make("cpu_256", seed=args.seed)
        rows = args.rows or 500
        n = len(seeds)
        chd = torch.from_numpy(np.ascontiguousarray(ch, np.float32)).to(dev)
        V = torch.zeros((3, rows, n), dtype=torch.float32, device=dev)
        V[:, 0, :] = torch.from_numpy(np.ascontiguousarray(seeds.T, np.float32)).to(dev)
        for _ in range(2):
            W = V.clone()
            rc, perf = em.calc_field(W[0].reshape(-1), W[1].reshape(-1), W[2].reshape(-1),
                                     chd, n, 1.0, True, arith="exact", require_n64=False)
            if rc:
                raise em.EmError(rc, "exact")
        torch.cuda.synchronize()
        print("exact", n * (rows - 1) * len(ch) / perf.time / 1e9, "Gpair/s")
        return 0
    if args.case == "ext-tail-gpu":
        ch, seeds, _ = em.workloads.make("gpu_4096", seed=args.seed)
        ch = torch.from_numpy(np.ascontiguousarray(ch, np.float32)).to(dev)
        s = torch.from_numpy(seeds.astype(np.float32)).to(dev)
        rows = args.rows or 5000
        out = em.trace_lines(s, ch, rows, 1.0, 0.5)
        torch.cuda.synchronize()
        ln = out["len"]
        print("tail", out["perf"].pairs / out["perf"].time / 1e9, "Gpair/s",
              out["perf"].time * 1e3, "ms, lines at the row limit",
              int((ln >= rows).sum()))
        return 0
    if args.case.startswith("ext"):
        ch, seeds, _ = em.workloads.make("gpu_4096", seed=args.seed)
        ch = torch.from_numpy(np.ascontiguousarray(ch, np.float32)).to(dev)
        s = torch.from_numpy(seeds.astype(np.float32)).to(dev)
        prec = args.case.split("-")[1]
        for _ in range(2):
            out = em.trace_lines(s, ch, 200, 1.0, 0.0, precision=prec)
        torch.cuda.synchronize()
        print(prec, out["perf"].pairs / out["perf"].time / 1e9, "Gpair/s")
        return 0
    if args.case == "verlet":
        rng = np.random.Generator(np.random.PCG64(args.seed))
        n, p = 65536, 4096
        dyn = np.zeros((n, 8), np.float32)
        dyn[:, :3] = rng.uniform(-100, 100, (n, 3))
        dyn[:, 3] = rng.uniform(-1, 1, n) * 1e-9
        dyn[:, 4:7] = rng.normal(0, 1e3, (n, 3))
        dyn[:, 7] = rng.uniform(1e-6, 1e-5, n)
        st = np.zeros((p, 4), np.float32)
        st[:, :3] = rng.uniform(-100, 100, (p, 3))
        st[:, 3] = rng.uniform(-1, 1, p) * 1e-8
        d = torch.from_numpy(dyn).to(dev)
        a = torch.zeros((n, 3), dtype=torch.float32, device=dev)
        c = torch.from_numpy(st).to(dev)
        for _ in range(2):
            perf = em.verlet_step(d, a, c, [-100.0] * 3, [100.0] * 3, 1e-6,
                                  steps=2)
        torch.cuda.synchronize()
        print("verlet", perf.pairs / perf.time / 1e9, "Gpair/s")
        return 0
    ch_np, seeds_np, _ = em.workloads.make("adjoint_1024", seed=args.seed)
    if args.case == "adjoint-twopass":
        ch_np = em.workloads.uniform_charges(6000, 50.0, args.seed)
    rows, n = 200, len(seeds_np)
    ch = torch.from_numpy(np.ascontiguousarray(ch_np, np.float32)).to(dev)
    V = torch.zeros((3, rows, n), dtype=torch.float32, device=dev)
    V[:, 0, :] = torch.from_numpy(seeds_np.T.astype(np.float32)).to(dev)
    T = V.clone()
    for _ in range(2):
        W = V.clone()
        _, _, f, b = em.adjoint_device(
            W, ch, T, checkpoint=args.case == "adjoint-checkpoint")
    torch.cuda.synchronize()
    print("fwd ms", f * 1e3, "bwd ms", b * 1e3, "ratio", b / f)
    return 0


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.case:
        return run_case(args)
    import torch
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    em = importlib.import_module("electromag-with-cuda_gb300")
    lib = em.load()
    ch, seeds, rows = workload(em, args.workload, args.seed + 0, args.rows)
    n_all, p = len(seeds), len(ch)
    # strong scaling: this rank's contiguous shard of the lines
    shard = args.mode == "shard" and world > 1
    if shard:
        b, e = em.shard.shard_range(n_all, world, rank)
        seeds = seeds[b:e]
    n = len(seeds)
    pairs = float(n) * (rows - 1) * p           # this rank's work per step
    pairs_all = float(n_all) * (rows - 1) * p * (1 if shard else world)
    dev = torch.device("cuda", local)
    stream = torch.cuda.current_stream(dev)
    X = [torch.zeros(n * rows, dtype=torch.float32, device=dev) for _ in range(3)]
    for c in range(3):
        X[c][:n] = torch.from_numpy(np.ascontiguousarray(seeds[:, c])).to(dev)
    dch = torch.from_numpy(ch).to(dev)

    shape = dict(threads_per_line=args.tpl, lines_per_thread=args.kl,
                 warps_per_cta=args.warps, pack=args.pack)

    def step():
        rc, perf = em.calc_field(*X, dch, n, 1.0, True, require_n64=False,
                                 stream=stream.cuda_stream, **shape)
        if rc:
            raise em.EmError(rc, "em_calc_field_ex_f32")
        return perf

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    for _ in range(args.warmup):
        step()
    peak_tflops = lib_peak(lib)
    barrier()
    launches0 = lib.em_launch_count()
    kern = []
    with ClockSampler(local) as clk:
        t0 = torch.cuda.Event(enable_timing=True)
        t1 = torch.cuda.Event(enable_timing=True)
        barrier()
        t0.record(stream)
        for _ in range(args.steps):
            kern.append(step().time)
        t1.record(stream)
        barrier()
    launches = lib.em_launch_count() - launches0
    ms = t0.elapsed_time(t1)
    if dist:
        t = torch.tensor([ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms = float(t.item())
    value = pairs_all * args.steps / (ms * 1e-3) / 1e9
    kernel_s = float(np.mean(kern))
    achieved = FLOP_PER_PAIR * pairs / kernel_s / 1e12

    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(em, torch, dist, ch, seeds, rows, args, pairs_all)

    extras = {}
    field_err = None
    if not args.no_extras and world == 1:
        # the timed path's own field at sampled vertices of one more
        # (untimed) trace of the same workload and shape
        del X
        torch.cuda.empty_cache()
        _, field_err = traced_field_errors(em, torch, dev, ch, seeds, rows,
                                           20000, args.seed + 1, **shape)
        extras = run_extras(em, torch, dev, args, value)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        sys.path.insert(0, os.path.join(ROOT, "oracle"))
        import em_oracle as orc
        threads = os.cpu_count() or 1
        v, smp = cpu_rate(orc, ch, seeds, rows, args.cpu_seconds, threads)
        cpu = {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"{smp['lines']} of {n} lines x {p} charges x "
                         f"{smp['rows']} rows ({smp['seconds']:.1f} s)"}
    if rank != 0:
        return 0
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms / args.steps, "higher_is_better": True,
        "scaling": "strong" if shard else "weak", "vs_baseline": None, "dtype": "f32",
        "data": DATA,
        "config": workload_config(args, n_all, p, rows, world,
                                  "fast FP32 (rsqrt + FMA)"),
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak_tflops,
                     "unit": "TFLOP/s", "frac": achieved / peak_tflops,
                     "traffic": (TRAFFIC_GPU4096 if args.workload == "gpu_4096"
                                 and not args.rows else None),
                     "algorithmic_bytes": 12.0 * n * (rows - 1),
                     "peak_source": "measured FFMA peak (em_fp32_peak_tflops)",
                     "flop_per_pair": FLOP_PER_PAIR,
                     # the reference's own count (perfPacket): 18 FLOP per
                     # pair and 13 per vertex step
                     "achieved_reference_convention":
                         (18.0 * pairs + 13.0 * n * (rows - 1)) / kernel_s / 1e12,
                     "kernel_ms": kernel_s * 1e3},
        "field_err": field_err,
        "clocks": clk.summary(),
        "gpu_launches": int(launches),
        "e2e": e2e,
        "cpu_baseline": cpu,
    }
    line.update(extras)
    line["metric_parts"] = metric_parts(value, extras, field_err)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()
    return 0


def fastest_within(candidates, bound=1e-6):
    """The fastest (name, rate, max error) candidate whose sampled maximum
    field error is within `bound`, or None."""
    ok = [c for c in candidates if c[1] and c[2] is not None and c[2] <= bound]
    if not ok:
        return None
    name, rate, err = max(ok, key=lambda c: c[1])
    return {"mode": name, "gpair_s": rate, "field_err_max": err}


def metric_parts(value, extras, value_err=None):
    """The metric's parts in one place: the plain FP32 rate (`value`) and
    its field error; the mixed arithmetic on the reference-layout tracer
    (the same loop and workload as `value`) against `value`, with its field
    error; the extended tracer's mixed mode per pair (200 rows, no
    termination) against `value` and against the extended tracer's own FP32
    form; the fastest mode whose maximum sampled field error is within 1e-6
    of FP64 on the GPU-scale and the dipole workloads; the adjoint/forward
    time ratio."""
    parts = {"plain_fp32_gpair_s": value}
    if value_err:
        parts["plain_fp32_field_err_max"] = value_err["vs_fp64"]["max"]
    mref = extras.get("mixed_reference_layout", {})
    if "gpair_s" in mref:
        e = mref["field_err"]["vs_fp64"]
        parts.update({"mixed_reference_layout_gpair_s": mref["gpair_s"],
                      "mixed_reference_layout_vs_plain_fp32": mref["gpair_s"] / value,
                      "mixed_reference_layout_field_err_median": e["median"],
                      "mixed_reference_layout_field_err_max": e["max"],
                      "mixed_reference_layout_frac_le_1e-6": e["frac_le_1e-6"],
                      "mixed_reference_layout_refined_vertex_frac":
                          mref["refined_vertex_frac"]})
    prec = extras.get("precision", {})
    if "mixed_vs_fp32" in prec:
        mixed = prec.get("mixed", {}).get("field_err_vs_fp64") or {}
        rates = prec.get("no_termination_200_rows_gpair_s", {})
        parts.update({"extended_mixed_gpair_s": rates.get("mixed"),
                      "extended_mixed_vs_plain_fp32": (rates["mixed"] / value
                                                       if rates.get("mixed") else None),
                      "extended_mixed_vs_extended_fp32": prec["mixed_vs_fp32"],
                      "extended_mixed_vs_fp64": prec.get("mixed_vs_fp64"),
                      "extended_mixed_field_err_median": mixed.get("median"),
                      "extended_mixed_field_err_max": mixed.get("max"),
                      "extended_mixed_frac_le_1e-6": mixed.get("frac_le_1e-6")})
    fastest = {}
    for wl, blk in (("gpu_4096", prec), ("dipole_16384", extras.get("precision_stress", {}))):
        cands = []
        if wl == "gpu_4096":
            if value_err:
                cands.append(("reference-layout fp32", value, value_err["vs_fp64"]["max"]))
            if "gpair_s" in mref:
                cands.append(("reference-layout mixed", mref["gpair_s"],
                              mref["field_err"]["vs_fp64"]["max"]))
        for mode in ("fp32", "mixed", "mixed_fp64_refine", "mixed_no_refine", "df64", "fp64"):
            m = blk.get(mode) or {}
            err = (m.get("field_err_vs_fp64") or {}).get("max")
            if m.get("gpair_s"):
                cands.append(("extended " + mode + " (termination)", m["gpair_s"], err))
        best = fastest_within(cands)
        if best:
            best["vs_plain_fp32"] = best["gpair_s"] / value
        fastest[wl] = best
    parts["fastest_mode_max_err_le_1e-6"] = fastest
    adj = extras.get("adjoint", {})
    if "stored" in adj:
        parts["adjoint_over_forward"] = adj["stored"]["adjoint_over_forward"]
        parts["adjoint_over_forward_checkpointed"] = (
            adj["checkpoint"]["adjoint_over_forward"])
        parts["adjoint_grad_rel_err_vs_fp64"] = max(
            adj[m].get("grad_rel_err_vs_fp64", float("nan"))
            for m in ("stored", "checkpoint"))
    return parts


def field_errors(em, torch, ch, V, F, ln, samples, seed):
    """Relative field error of a run's stored fields against the FP64 field
    (em_field_f64, the reference's double sequence) at sampled vertices."""
    g = np.random.Generator(np.random.PCG64(seed))
    lnh = ln.cpu().numpy()
    rows_ok = np.maximum(lnh - 1, 0)  # rows with a field that led to a step
    lines = np.nonzero(rows_ok)[0]
    if len(lines) == 0:
        return None
    li = g.choice(lines, samples)
    ri = (g.random(samples) * rows_ok[li]).astype(np.int64)
    li_t = torch.from_numpy(li).to(V.device)
    ri_t = torch.from_numpy(ri).to(V.device)
    pts = V[:, ri_t, li_t].double()                 # (3, m)
    got = F[:, ri_t, li_t].double()
    ref = em.field(pts.contiguous(), ch.double().contiguous(), arith="exact")
    err = (got - ref).norm(dim=0) / ref.norm(dim=0)
    e = err.cpu().numpy()
    return {"median": float(np.median(e)), "p99": float(np.quantile(e, 0.99)),
            "p999": float(np.quantile(e, 0.999)), "max": float(e.max()),
            "frac_le_1e-6": float((e <= 1e-6).mean()), "samples": int(samples)}


def traced(em, torch, ch, seeds, steps, term, precision, want_field,
           refine_kappa=0.0, refine="df64"):
    dt = torch.float64 if precision == "fp64" else torch.float32
    em.trace_lines(seeds.to(dt), ch.to(dt), min(steps, 8), 1.0, term,
                   precision=precision, refine_kappa=refine_kappa,
                   refine=refine)  # warm-up
    torch.cuda.synchronize()
    out = em.trace_lines(seeds.to(dt), ch.to(dt), steps, 1.0, term,
                         precision=precision, want_field=want_field,
                         refine_kappa=refine_kappa, refine=refine)
    torch.cuda.synchronize()
    perf = out["perf"]
    out["gpairs"] = perf.pairs / perf.time / 1e9 if perf.time > 0 else 0.0
    return out


def precision_block(em, torch, dev, name, steps, seed, samples, with_ratio):
    """FP32 / mixed / double-float / FP64 runs of the extended method on one
    workload, with throughput and field error vs FP64; the mixed mode with
    its default conditioning test and double-float re-evaluations, with FP64
    re-evaluations, and with the re-evaluations off."""
    ch_np, seeds_np, _ = em.workloads.make(name, seed=seed)
    ch = torch.from_numpy(np.ascontiguousarray(ch_np, np.float32)).to(dev)
    seeds = torch.from_numpy(seeds_np.astype(np.float32)).to(dev)
    blk = {"workload": name, "lines": int(len(seeds_np)),
           "charges": int(len(ch_np)), "max_rows": steps,
           "term_radius": 0.5}
    for prec, kappa, refine in (("fp32", 0.0, "df64"), ("mixed", 0.0, "df64"),
                                ("mixed_fp64_refine", 0.0, "fp64"),
                                ("mixed_no_refine", 1e30, "df64"),
                                ("df64", 0.0, "df64"), ("fp64", 0.0, "df64")):
        p = "mixed" if prec.startswith("mixed") else prec
        out = traced(em, torch, ch, seeds, steps, 0.5, p, True, kappa, refine)
        ln = out["len"]
        cls = np.bincount(out["cls"].cpu().numpy(), minlength=3)
        errs = field_errors(em, torch, ch, out["vertices"], out["field"], ln,
                            samples, seed + 1)
        blk[prec] = {"gpair_s": out["gpairs"], "ms": out["perf"].time * 1e3,
                     "pairs": out["perf"].pairs,
                     "mean_len": float(ln.double().mean()),
                     "classes": {"steps": int(cls[0]), "charge": int(cls[1]),
                                 "null": int(cls[2])},
                     "fp64_refines": out["perf"].fp64_refines,
                     "field_err_vs_fp64": errs}
        del out
        torch.cuda.empty_cache()
    if with_ratio:
        # per-pair cost without termination: every line runs 200 rows
        r = {}
        for p in ("fp32", "mixed", "df64", "fp64"):
            out = traced(em, torch, ch, seeds, 200, 0.0, p, False)
            r[p] = out["gpairs"]
        blk["no_termination_200_rows_gpair_s"] = r
        blk["mixed_vs_fp32"] = r["mixed"] / r["fp32"]
        blk["mixed_vs_fp64"] = r["mixed"] / r["fp64"]
        blk["df64_vs_fp64"] = r["df64"] / r["fp64"]
    return blk


def adjoint_block(em, torch, dev, seed):
    """Adjoint: 1024 charges (cube side 100), 16384 lines x 4000 rows; the
    loss is sum |v - t|^2 against a seeded perturbed copy of the forward."""
    ch_np, seeds_np, rows = em.workloads.make("adjoint_1024", seed=seed)
    n = len(seeds_np)
    ch = torch.from_numpy(np.ascontiguousarray(ch_np, np.float32)).to(dev)
    V = torch.zeros((3, rows, n), dtype=torch.float32, device=dev)
    V[:, 0, :] = torch.from_numpy(seeds_np.T.astype(np.float32)).to(dev)
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    rc, _ = em.calc_field(V[0].reshape(-1), V[1].reshape(-1), V[2].reshape(-1),
                          ch, n, 1.0, True, require_n64=False)
    if rc:
        raise em.EmError(rc, "forward")
    T = V + 0.1 * torch.randn(V.shape, generator=gen, device=dev)
    W = torch.zeros_like(V)
    W[:, 0, :] = V[:, 0, :]
    pairs = float(n) * (rows - 1) * len(ch_np)
    blk = {"workload": "adjoint_1024", "lines": n, "charges": len(ch_np),
           "rows": rows}
    # stored: the forward keeps its field at every vertex; checkpoint: only
    # the vertices, the field recomputed per 64-row segment
    for mode, ck in (("stored", False), ("checkpoint", True)):
        em.adjoint_device(W, ch, T, checkpoint=ck)  # warm-up
        loss, grad, fwd_s, bwd_s = em.adjoint_device(W, ch, T, checkpoint=ck)
        torch.cuda.synchronize()
        blk[mode] = {"forward_ms": fwd_s * 1e3, "adjoint_ms": bwd_s * 1e3,
                     "adjoint_over_forward": bwd_s / fwd_s,
                     "forward_gpair_s": pairs / fwd_s / 1e9,
                     "loss": float(loss.item()),
                     "grad_norm": float(grad.norm().item())}
    blk["checkpoint_rows"] = 64
    # correctness at this scale: on 256 of the lines (all 4000 rows, all
    # 1024 charges) the gradient of both modes against the FP64 adjoint of
    # the GPU's own frozen map (linearised at its trajectory with the field
    # its forward used, traced again here with the field output in the
    # adjoint's shape), and against the FP64 adjoint with the FP64 field at
    # the same vertices (the sensitivity to the forward field's rounding)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import em_oracle as orc
    sub = torch.from_numpy(np.linspace(0, n - 1, 256).astype(np.int64)).to(dev)
    ns = 256
    Vs = torch.zeros((3, rows, ns), dtype=torch.float32, device=dev)
    Vs[:, 0, :] = V[:, 0, sub]
    Fs = torch.zeros(3 * ns * (rows - 1), dtype=torch.float32, device=dev)
    rc, _ = em.calc_field(Vs[0].reshape(-1), Vs[1].reshape(-1), Vs[2].reshape(-1),
                          ch, ns, 1.0, True, require_n64=False, field_out=Fs,
                          threads_per_line=8, lines_per_thread=1)
    if rc:
        raise em.EmError(rc, "forward with field output")
    Ts = T[:, :, sub].contiguous()
    Ws = torch.zeros_like(Vs)
    Ws[:, 0, :] = Vs[:, 0, :]
    refs = None
    for mode, ck in (("stored", False), ("checkpoint", True)):
        loss, grad, _, _ = em.adjoint_device(Ws, ch, Ts, checkpoint=ck)
        torch.cuda.synchronize()
        if refs is None:
            t0 = time.perf_counter()
            chd = ch_np.astype(np.float64)
            Wh, Th = Ws.double().cpu().numpy(), Ts.double().cpu().numpy()
            refs = (orc.adjoint_at_field(chd, Wh, Th, Fs.view(3, rows - 1, ns)
                                         .double().cpu().numpy()),
                    orc.adjoint_at(chd, Wh, Th))
            blk["grad_check_host_s"] = time.perf_counter() - t0
        (L, g), (_, g64) = refs
        gg = grad.cpu().numpy()
        blk[mode]["grad_rel_err_vs_fp64"] = float(np.linalg.norm(gg - g) /
                                                  np.linalg.norm(g))
        blk[mode]["grad_rel_diff_vs_fp64_field"] = float(
            np.linalg.norm(gg - g64) / np.linalg.norm(g64))
        blk[mode]["loss_rel_err_vs_fp64"] = abs(float(loss.item()) - L) / abs(L)
    blk["grad_check"] = ("256 of the lines, all rows and charges: against the "
                         "FP64 discrete adjoint of the GPU's frozen map (its "
                         "trajectory and forward field); the second figure "
                         "with the FP64 field at the same vertices instead")
    return blk


def batch_block(em, torch, dev, seed):
    """512 independent sets (sizes log-uniform in [64, 32768], cube side 100,
    4 lines per positive charge, step limits per set uniform in [500, 8000],
    termination at negative charges): one graph-captured batched launch
    sequence with autotuned shape, against per-set launches of the single-set
    tracer (same FP32 arithmetic)."""
    sets = em.workloads.make_batch(512, seed)
    max_steps = max(lim for _, _, lim in sets)
    lims = np.concatenate([np.full(len(s), lim, np.int32) for _, s, lim in sets])
    pairs_sets = [(c, s) for c, s, _ in sets]
    t0 = time.perf_counter()
    opts = em.autotune.tune_batch(pairs_sets, max_steps, lims, sample=16,
                                  use_cache=False)
    tune_s = time.perf_counter() - t0
    coff = np.concatenate([[0], np.cumsum([len(c) for c, _, _ in sets])])
    loff = np.concatenate([[0], np.cumsum([len(s) for _, s, _ in sets])])
    d = {"charges": torch.from_numpy(np.concatenate([c for c, _, _ in sets])
                                     .astype(np.float32)).to(dev),
         "seeds": torch.from_numpy(np.concatenate([s for _, s, _ in sets])).to(dev),
         "charge_off": coff, "line_off": loff}
    spl = torch.from_numpy(lims).to(dev)
    em.trace_batch(d, max_steps, 1.0, 0.5, steps_per_line=spl, use_graph=True,
                   **opts)
    torch.cuda.synchronize()
    r = em.trace_batch(d, max_steps, 1.0, 0.5, steps_per_line=spl,
                       use_graph=True, **opts)
    torch.cuda.synchronize()
    bt, bp = r["perf"].time, r["perf"].pairs
    cls = np.bincount(r["cls"].cpu().numpy(), minlength=3)
    # per-set launches of the single-set tracer
    ksum, psum = 0.0, 0.0
    torch.cuda.synchronize()
    w0 = time.perf_counter()
    for (c, s, lim) in sets:
        out = em.trace_lines(torch.from_numpy(s).to(dev),
                             torch.from_numpy(np.ascontiguousarray(c, np.float32))
                             .to(dev), lim, 1.0, 0.5)
        ksum += out["perf"].time
        psum += out["perf"].pairs
        del out
    torch.cuda.synchronize()
    wall = time.perf_counter() - w0
    torch.cuda.empty_cache()
    return {"workload": "batch_512", "sets": len(sets), "lines": int(loff[-1]),
            "charges": int(coff[-1]), "max_rows": max_steps,
            "tuned": opts, "tune_seconds": tune_s,
            "batched_ms": bt * 1e3, "batched_pairs": bp,
            "batched_gpair_s": bp / bt / 1e9,
            "classes": {"steps": int(cls[0]), "charge": int(cls[1]),
                        "null": int(cls[2])},
            "per_set_kernel_ms": ksum * 1e3, "per_set_wall_ms": wall * 1e3,
            "per_set_pairs": psum, "per_set_gpair_s": psum / ksum / 1e9,
            "speedup_vs_per_set_kernels": ksum / bt,
            "speedup_vs_per_set_wall": wall / bt}


def reference_run_block(em, torch, dev, seed):
    """The reference program's own default run (preset "normal": srand(1)
    charges, 128x128 grid seeds, 1024 charges, 2500 rows; ElectroMag.cpp:43,
    251-266): GPU with the reference's arithmetic (bit-exact) and the fast
    arithmetic, the oracle port on host cores over a line sample, the
    --autoregress scan of the two GPU runs and the --save dump of a preset
    run."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import em_oracle as orc
    ch, seeds, rows = em.inputs.reference_case("normal")
    n, p = len(seeds), len(ch)
    pairs = float(n) * (rows - 1) * p
    blk = {"workload": "preset_normal", "lines": n, "charges": p, "rows": rows}
    runs = {}
    chd = torch.from_numpy(ch).to(dev)
    for arith in ("exact", "fast"):
        V = torch.zeros((3, rows, n), dtype=torch.float32, device=dev)
        V[:, 0, :] = torch.from_numpy(seeds.T.copy()).to(dev)
        times = []
        for rep in range(2):
            W = V.clone()
            rc, perf = em.calc_field(W[0].reshape(-1), W[1].reshape(-1),
                                     W[2].reshape(-1), chd, n, 1.0, True,
                                     arith=arith)
            if rc:
                raise em.EmError(rc, f"preset run ({arith})")
            times.append(perf.time)
        runs[arith] = W
        blk[arith] = {"ms": min(times) * 1e3,
                      "gpair_s": pairs / min(times) / 1e9}
    threads = os.cpu_count() or 1
    rate, sample = cpu_rate(orc, ch, seeds, rows, 10.0, threads)
    blk["cpu_port"] = {"gpair_s": rate, "cores": threads,
                       "full_run_s_estimate": pairs / rate / 1e9,
                       "sample": f"{sample['lines']} lines x {p} charges x "
                                 f"{sample['rows']} rows"}
    # --autoregress: exact against fast, then a run against itself (no
    # divergence: every vertex of both runs read once)
    stream = torch.cuda.current_stream(dev)
    for name, b in (("exact_vs_fast", runs["fast"]), ("identical", runs["exact"])):
        em.outputs.autoregress(runs["exact"], b)  # warm-up
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        first, count = em.outputs.autoregress(runs["exact"], b)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        rows_read = np.where(first >= 0, first + 1, rows).sum()
        gbytes = float(rows_read) * 24 / 1e9
        blk["autoregress_" + name] = {
            "ms": ms, "diverged_lines": count,
            "median_first_row": float(np.median(first[first >= 0])) if count else None,
            "algorithmic_gb": gbytes, "gb_s": gbytes / (ms * 1e-3)}
    # --save: the bogo preset's run (256 lines x 500 rows), both tags
    bch, bseeds, brows = em.inputs.reference_case("bogo")
    bn = len(bseeds)
    V = np.zeros((3, brows, bn), np.float32)
    V[:, 0, :] = bseeds.T
    rc, _ = em.calc_field(V[0].reshape(-1), V[1].reshape(-1), V[2].reshape(-1),
                          bch, bn, 1.0, True, arith="exact")
    if rc:
        raise em.EmError(rc, "bogo run")
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, "data.txt")
        t = time.perf_counter()
        em.outputs.save_lines(path, bn, brows, V, V)
        sec = time.perf_counter() - t
        size = os.path.getsize(path)
    blk["save_bogo"] = {"seconds": sec, "mbytes": size / 1e6,
                        "mb_s": size / 1e6 / sec, "threads": threads}
    del runs
    torch.cuda.empty_cache()
    return blk


def nbody_functor_block(em, torch, dev, seed):
    """The Verlet step of moving charges (65 536 particles in the field of
    4096 static charges, 4 steps, FP32 and FP64) and the functor layer's
    cost on one GPU (the 4096-charge workload's first 8192 lines x 1000 rows
    through 4 line ranges on device 0, against one host-pointer call)."""
    rng = np.random.Generator(np.random.PCG64(seed))
    n, p, steps = 65536, 4096, 4
    dyn = np.zeros((n, 8))
    dyn[:, :3] = rng.uniform(-100, 100, (n, 3))
    dyn[:, 3] = rng.uniform(-1, 1, n) * 1e-9
    dyn[:, 4:7] = rng.normal(0, 1e3, (n, 3))
    dyn[:, 7] = rng.uniform(1e-6, 1e-5, n)
    st = np.zeros((p, 4))
    st[:, :3] = rng.uniform(-100, 100, (p, 3))
    st[:, 3] = rng.uniform(-1, 1, p) * 1e-8
    box = ([-100.0] * 3, [100.0] * 3)
    blk = {"workload": f"{n} moving + {p} static charges, {steps} steps"}
    for name, dt in (("fp32", torch.float32), ("fp64", torch.float64)):
        d = torch.from_numpy(dyn).to(dev, dt)
        a = torch.zeros((n, 3), dtype=dt, device=dev)
        c = torch.from_numpy(st).to(dev, dt)
        em.verlet_step(d, a, c, *box, 1e-6, steps=1)  # warm-up
        perf = em.verlet_step(d, a, c, *box, 1e-6, steps=steps)
        torch.cuda.synchronize()
        blk[name] = {"ms": perf.time * 1e3,
                     "gpair_s": perf.pairs / perf.time / 1e9}
    ch, seeds, _ = em.workloads.make("gpu_4096", seed=seed)
    ch = np.ascontiguousarray(ch, np.float32)
    seeds = seeds.astype(np.float32)[:8192]
    nl, rows = len(seeds), 1000

    def fresh():
        x = np.zeros((3, rows * nl), np.float32)
        x[:, :nl] = seeds.T
        return x

    x = fresh()
    em.calc_field(x[0], x[1], x[2], ch, nl, 1.0, True, require_n64=False,
                  plain=False)
    t = time.perf_counter()
    x = fresh()
    rc, _ = em.calc_field(x[0], x[1], x[2], ch, nl, 1.0, True,
                          require_n64=False, plain=False)
    one = time.perf_counter() - t
    y = fresh()
    t = time.perf_counter()
    rc2, _, ran, nfailed = em.calc_field_multi(y[0], y[1], y[2], ch, nl,
                                               [0, 0, 0, 0])
    multi = time.perf_counter() - t
    blk["functor"] = {"one_call_s": one, "four_ranges_s": multi,
                      "ranges_ran_on": ran, "failed": nfailed,
                      "identical": bool(rc == 0 and rc2 == 0
                                        and np.array_equal(x, y))}
    return blk


def traced_field_errors(em, torch, dev, ch, seeds, rows, samples, seed,
                        **kw):
    """One untimed trace of the reference-layout tracer with its field
    output, then the field each step used at `samples` vertices (every row
    and line equally likely) against the FP64 field at the same points
    (em_field_f64, the reference's double sequence) and against the
    reference's FP32 field there (em_field_f32 in the exact arithmetic: the
    reference's own operation sequence, bit for bit)."""
    n = len(seeds)
    X = [torch.zeros(n * rows, dtype=torch.float32, device=dev) for _ in range(3)]
    for c in range(3):
        X[c][:n] = torch.from_numpy(np.ascontiguousarray(seeds[:, c])).to(dev)
    F = torch.zeros(3 * n * (rows - 1), dtype=torch.float32, device=dev)
    dch = torch.from_numpy(np.ascontiguousarray(ch)).to(dev)
    rc, perf = em.calc_field(*X, dch, n, 1.0, True, require_n64=False,
                             field_out=F, **kw)
    if rc:
        raise em.EmError(rc, "em_calc_field_ex_f32 (field output)")
    torch.cuda.synchronize()
    g = np.random.Generator(np.random.PCG64(seed))
    li = torch.from_numpy(g.integers(0, n, samples)).to(dev)
    ri = torch.from_numpy(g.integers(0, rows - 1, samples)).to(dev)
    pts = torch.stack([x.view(rows, n)[ri, li] for x in X])
    got = F.view(3, rows - 1, n)[:, ri, li].double()
    del X, F
    ref64 = em.field(pts.double().contiguous(), dch.double().contiguous(),
                     arith="exact")
    ref32 = em.field(pts.contiguous(), dch, arith="exact", rule="sse").double()
    out = {}
    for key, ref in (("vs_fp64", ref64), ("vs_reference_fp32", ref32)):
        e = ((got - ref).norm(dim=0) / ref.norm(dim=0)).cpu().numpy()
        out[key] = {"median": float(np.median(e)),
                    "p99": float(np.quantile(e, 0.99)),
                    "p999": float(np.quantile(e, 0.999)),
                    "max": float(e.max()),
                    "frac_le_1e-6": float((e <= 1e-6).mean()),
                    "samples": int(samples)}
    torch.cuda.empty_cache()
    return perf, out


def mixed_reference_block(em, torch, dev, args, value):
    """The mixed arithmetic on the reference-layout tracer (EM_ARITH_MIXED):
    the `value` workload and loop (every line all rows, device arrays), so
    its rate divides by `value` directly; its field error at sampled
    vertices, and the share of vertices re-evaluated in double-float."""
    ch, seeds, rows = workload(em, args.workload, args.seed + 0, args.rows)
    n, p = len(seeds), len(ch)
    X = [torch.zeros(n * rows, dtype=torch.float32, device=dev) for _ in range(3)]
    for c in range(3):
        X[c][:n] = torch.from_numpy(np.ascontiguousarray(seeds[:, c])).to(dev)
    dch = torch.from_numpy(ch).to(dev)
    times, refines = [], 0.0
    for i in range(4):
        rc, perf = em.calc_field(*X, dch, n, 1.0, True, require_n64=False,
                                 arith="mixed")
        if rc:
            raise em.EmError(rc, "em_calc_field_ex_f32 (mixed)")
        if i:
            times.append(perf.time)
            refines = perf.fp64_refines
    torch.cuda.synchronize()
    del X
    torch.cuda.empty_cache()
    t = float(np.mean(times))
    pairs = float(n) * (rows - 1) * p
    _, errs = traced_field_errors(em, torch, dev, ch, seeds, rows, 20000,
                                  args.seed + 1, arith="mixed")
    return {"workload": args.workload, "lines": n, "charges": p, "rows": rows,
            "ms": t * 1e3, "gpair_s": pairs / t / 1e9,
            "vs_plain_fp32": pairs / t / 1e9 / value,
            "refined_vertex_frac": refines / (float(n) * (rows - 1)),
            "field_err": errs}


def cpu_config_block(em, torch, dev, seed):
    """The CPU-runnable configuration (256 charges in [-50,50]^3, 8 seeds
    per positive charge, 2500 rows) timed whole: the GPU in the fast and the
    reference's exact arithmetic, and the oracle port of the reference's
    CPU path over all host cores (the whole run, no sampling)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import em_oracle as orc
    ch, seeds, rows = workload(em, "cpu_256", seed, None)
    seeds = em.workloads.pad_lines(seeds, 64)  # the SSE path's n % 64
    n, p = len(seeds), len(ch)
    pairs = float(n) * (rows - 1) * p
    blk = {"workload": "cpu_256", "lines": n, "charges": p, "rows": rows}
    dch = torch.from_numpy(ch).to(dev)
    for arith in ("fast", "exact"):
        best = None
        for _ in range(3):
            V = torch.zeros((3, rows, n), dtype=torch.float32, device=dev)
            V[:, 0, :] = torch.from_numpy(seeds.T.copy()).to(dev)
            rc, perf = em.calc_field(V[0].reshape(-1), V[1].reshape(-1),
                                     V[2].reshape(-1), dch, n, 1.0, True,
                                     arith=arith)
            if rc:
                raise em.EmError(rc, f"cpu_256 ({arith})")
            best = perf.time if best is None else min(best, perf.time)
        blk["gpu_" + arith] = {"ms": best * 1e3, "gpair_s": pairs / best / 1e9}
    threads = os.cpu_count() or 1
    X = [np.zeros(n * rows, np.float32) for _ in range(3)]
    for c in range(3):
        X[c][:n] = seeds[:, c]
    t = time.perf_counter()
    rc = orc.calc_field(*X, ch, n, 1.0, orc.CURV_SSE, nthreads=threads)
    sec = time.perf_counter() - t
    if rc:
        raise RuntimeError(f"oracle port returned {rc}")
    blk["cpu_port"] = {"seconds": sec, "gpair_s": pairs / sec / 1e9,
                       "cores": threads, "sample": "the whole run"}
    blk["gpu_fast_vs_cpu_port"] = blk["gpu_fast"]["gpair_s"] / blk["cpu_port"]["gpair_s"]
    return blk


def run_extras(em, torch, dev, args, value):
    """Single-GPU measurements of the other configurations; a block that
    fails is reported in its place and does not cost the bench line."""
    blocks = [
        ("cpu_config", lambda: cpu_config_block(em, torch, dev, args.seed)),
        ("reference_run", lambda: reference_run_block(em, torch, dev, args.seed)),
        ("batched", lambda: batch_block(em, torch, dev, args.seed)),
        ("precision", lambda: precision_block(em, torch, dev, args.workload,
                                              5000, args.seed, 20000, True)),
        ("mixed_reference_layout", lambda: mixed_reference_block(em, torch, dev, args,
                                                                 value)),
        ("precision_stress", lambda: precision_block(
            em, torch, dev, "dipole_16384", 4000, args.seed, 20000, False)),
        ("adjoint", lambda: adjoint_block(em, torch, dev, args.seed)),
        ("nbody_functor", lambda: nbody_functor_block(em, torch, dev, args.seed)),
    ]
    out = {}
    for name, fn in blocks:
        try:
            out[name] = fn()
        except Exception as exc:  # reported, not fatal
            out[name] = {"error": f"{type(exc).__name__}: {exc}"}
        torch.cuda.empty_cache()
    return out


def lib_peak(lib):
    import ctypes
    t = ctypes.c_double()
    s = ctypes.c_double()
    rc = lib.em_fp32_peak_tflops(ctypes.byref(t), ctypes.byref(s))
    if rc:
        raise RuntimeError(f"em_fp32_peak_tflops failed: {rc}")
    return t.value


def run_e2e(em, torch, dist, ch, seeds, rows, args, pairs_all):
    """Host-pointer C ABI calls on pinned buffers: seeds and charges go in,
    every vertex comes out, each step; pairs_all is the pair count of one
    step over all ranks."""
    n, p = len(seeds), len(ch)
    H = [torch.zeros(n * rows, dtype=torch.float32).pin_memory()
         for _ in range(3)]
    hch = torch.from_numpy(ch).pin_memory()
    Hn = [h.numpy() for h in H]
    for c in range(3):
        Hn[c][:n] = seeds[:, c]
    chn = hch.numpy()

    def step():
        rc, _ = em.calc_field(*Hn, chn, n, 1.0, True, require_n64=False,
                              plain=False)
        if rc:
            raise em.EmError(rc, "em_calc_field_ex_f32 (host)")

    step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t = time.perf_counter()
    for _ in range(args.steps):
        step()
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    sec = time.perf_counter() - t
    if dist:
        tt = torch.tensor([sec], device="cuda")
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        sec = float(tt.item())
    pairs = pairs_all * args.steps
    return {"value": pairs / sec / 1e9, "unit": UNIT,
            "h2d_bytes_per_step": 3 * 4 * n + 16 * p,
            "d2h_bytes_per_step": 3 * 4 * n * (rows - 1) + 4}


if __name__ == "__main__":
    sys.exit(main())
