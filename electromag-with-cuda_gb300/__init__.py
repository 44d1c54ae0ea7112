"""GB300-native field-line tracer for ElectroMag (libemgb300.so + bindings).

Import with importlib (the directory name carries hyphens):
    em = importlib.import_module("electromag-with-cuda_gb300")
"""
from . import _capi, autotune, inputs, outputs, shard, tracer, workloads  # noqa: F401
from ._capi import EmError, load, declared_symbols, strerror  # noqa: F401
from .tracer import (adjoint, adjoint_device, calc_field, calc_field_multi,  # noqa: F401
                     field,
                     new_lines, seed_fibonacci,
                     trace_batch, trace_lines, trace_loss_function,
                     verlet_step)

__all__ = ["calc_field", "field", "new_lines", "trace_lines", "seed_fibonacci",
           "adjoint", "adjoint_device", "trace_batch", "trace_loss_function",
           "load", "declared_symbols", "strerror", "EmError", "inputs",
           "outputs", "workloads"]
