"""The reference program's outputs around the tracer: the --save text dump
(ElectroMag.cpp:372-397) and the --autoregress comparison of two runs
(:400-453), through the C ABI (em_save_lines_text_f32, em_autoregress_f32).

Line arrays are (3, rows, n) in the reference layout (row-major rows, the
seed row first), numpy float32 arrays or, for autoregress, CUDA tensors.
"""
import ctypes

import numpy as np

from . import _capi


def _host3(a, rows, n):
    a = np.ascontiguousarray(a, np.float32).reshape(3, rows * n)
    return a, [a[c].ctypes.data for c in range(3)]


def save_lines(path, n, rows, cpu=None, gpu=None):
    """Writes the dump: per line and row, " CPUL [line][row] x: .. y: ..
    z: .." from `cpu`, then the "GPUL" line from `gpu` (either may be None)."""
    keep, ptrs = [], []
    for a in (cpu, gpu):
        if a is None:
            ptrs += [None] * 3
        else:
            h, p = _host3(a, rows, n)
            keep.append(h)
            ptrs += p
    rc = _capi.load().em_save_lines_text_f32(str(path).encode(), n, rows, *ptrs)
    if rc:
        raise _capi.EmError(rc, "em_save_lines_text_f32")


def autoregress(cpu, gpu, threshold=0.1, path=None, stream=None):
    """First row where the two runs lie more than `threshold` apart, per line
    (-1: never), scanned on the GPU; writes the reference's regression.txt
    report to `path` if given.  cpu, gpu: (3, rows, n) numpy arrays, or CUDA
    tensors (then no copy is made).  Returns (first (n,) int64, count)."""
    lib = _capi.load()
    o = _capi.EmOptions()
    is_dev = hasattr(cpu, "is_cuda") and cpu.is_cuda
    if is_dev:
        import torch
        for t in (cpu, gpu):
            if t.dtype != torch.float32 or t.dim() != 3 or t.shape[0] != 3:
                raise TypeError("autoregress takes (3, rows, n) float32 arrays")
        if tuple(cpu.shape) != tuple(gpu.shape) or not gpu.is_cuda:
            raise ValueError("both runs must be CUDA tensors of one shape")
        rows, n = cpu.shape[1], cpu.shape[2]
        a, b = cpu.contiguous(), gpu.contiguous()
        ptrs = [a[c].data_ptr() for c in range(3)] + [b[c].data_ptr() for c in range(3)]
        o.device_ptrs = 1
        o.stream = (stream if stream is not None else
                    torch.cuda.current_stream(a.device).cuda_stream)
        keep = (a, b)
    else:
        if np.shape(cpu) != np.shape(gpu) or len(np.shape(cpu)) != 3:
            raise ValueError("autoregress takes two (3, rows, n) arrays of one shape")
        rows, n = np.shape(cpu)[1], np.shape(cpu)[2]
        ha, pa = _host3(cpu, rows, n)
        hb, pb = _host3(gpu, rows, n)
        ptrs = pa + pb
        keep = (ha, hb)
    first = np.zeros(n, np.int64)
    count = ctypes.c_size_t(0)
    rc = lib.em_autoregress_f32(None if path is None else str(path).encode(),
                                n, rows, *ptrs, threshold, first.ctypes.data,
                                ctypes.byref(count), ctypes.byref(o))
    del keep
    if rc:
        raise _capi.EmError(rc, "em_autoregress_f32")
    return first, int(count.value)
