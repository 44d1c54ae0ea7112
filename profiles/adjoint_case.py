"""Profiling case for the adjoint kernels: the 1024-charge workload (16 384
lines), 200 rows, targets equal to the seeds' rows (zero-noise)."""
import importlib
import os
import sys

import numpy as np
import torch

sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
em = importlib.import_module("electromag-with-cuda_gb300")
ch_np, seeds_np, _ = em.workloads.make("adjoint_1024", seed=1234)
rows = 200
n = len(seeds_np)
ch = torch.from_numpy(np.ascontiguousarray(ch_np, np.float32)).cuda()
V = torch.zeros((3, rows, n), dtype=torch.float32, device="cuda")
V[:, 0, :] = torch.from_numpy(seeds_np.T.astype(np.float32)).cuda()
T = V.clone()
for _ in range(2):
    W = V.clone()
    loss, grad, f, b = em.adjoint_device(W, ch, T)
torch.cuda.synchronize()
print("fwd ms", f * 1e3, "bwd ms", b * 1e3, "ratio", b / f)
