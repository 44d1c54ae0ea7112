"""Profiling case for ext_trace_kernel: the 4096-charge workload's charges and
seeds (32 736 lines), 200 rows, no termination radius; argv[1] = fp32|mixed."""
import importlib
import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
em = importlib.import_module("electromag-with-cuda_gb300")
ch, seeds, _ = em.workloads.make("gpu_4096", seed=1234)
ch = torch.from_numpy(np.ascontiguousarray(ch, np.float32)).cuda()
s = torch.from_numpy(seeds.astype(np.float32)).cuda()
prec = sys.argv[1] if len(sys.argv) > 1 else "fp32"
for _ in range(2):
    out = em.trace_lines(s, ch, 200, 1.0, 0.0, precision=prec)
torch.cuda.synchronize()
print(prec, out["perf"].pairs / out["perf"].time / 1e9, "Gpair/s")
