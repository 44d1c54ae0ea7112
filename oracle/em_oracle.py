"""TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.

ctypes wrapper of liboracle.so (oracle/em_oracle.c), the CPU restatement of
the reference tracer.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg import this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")

CURV_SSE, CURV_GENERIC, FIXED = 0, 1, 2
# electro_k of include/Electrostatics.h:27 (the oracle's ORC_ELECTRO_K)
ELECTRO_K = 8.987551787e9
TERM_STEPS, TERM_CHARGE, TERM_NULL = 0, 1, 2

P, S, I = ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int
_lib = None


def build():
    subprocess.check_call(["make", "-s", "-C", HERE, "liboracle.so"])


def load():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        lib = ctypes.CDLL(LIB)
        lib.orc_calc_field_f32.argtypes = [P, P, P, S, S, P, S, ctypes.c_float,
                                           I, S, S, I]
        lib.orc_calc_field_f64.argtypes = [P, P, P, S, S, P, S, ctypes.c_double,
                                           I, S, S, I]
        lib.orc_field_f32.argtypes = [P, P, P, S, P, S, I, P, P, P]
        lib.orc_field_f64.argtypes = [P, P, P, S, P, S, P, P, P, P, I]
        lib.orc_trace_lines_f64.argtypes = [P, S, P, P, P, S, S, P,
                                            ctypes.c_double, ctypes.c_double,
                                            P, P, I]
        lib.orc_seed_fibonacci_f64.argtypes = [P, S, S, ctypes.c_double, P, P,
                                               P, S]
        lib.orc_seed_fibonacci_f64.restype = S
        D = ctypes.c_double
        lib.orc_frozen_loss_f64.restype = D
        lib.orc_frozen_loss_f64.argtypes = [P, S, P, P, P, S, S, D, P, P, P,
                                            P, P, P, P, P]
        lib.orc_frozen_loss_cs_f64.restype = D
        lib.orc_frozen_loss_cs_f64.argtypes = [P, S, P, P, P, S, S, D, P, P,
                                               P, P, S, I, D]
        lib.orc_frozen_grad_f64.restype = D
        lib.orc_frozen_grad_f64.argtypes = [P, S, P, P, P, S, S, D, P, P, P,
                                            P, P]
        lib.orc_adjoint_at_f64.restype = D
        lib.orc_adjoint_at_f64.argtypes = [P, S, P, P, P, S, S, D, I, P, P,
                                           P, P]
        lib.orc_adjoint_at_field_f64.restype = D
        lib.orc_adjoint_at_field_f64.argtypes = [P, S, P, P, P, S, S, D, I, P,
                                                 P, P, P, P, P, I, P]
        _lib = lib
    return _lib


def _p(a):
    return a.ctypes.data_as(P) if a is not None else None


def calc_field(x, y, z, charges, n, resolution=1.0, variant=CURV_SSE,
               line0=0, nlines=0, nthreads=0):
    """Runs the restatement in place on the reference layout; returns rc."""
    lib = load()
    f32 = x.dtype == np.float32
    ch = np.ascontiguousarray(charges, x.dtype)
    fn = lib.orc_calc_field_f32 if f32 else lib.orc_calc_field_f64
    steps = x.size // n if n else 0
    return fn(_p(x), _p(y), _p(z), n, steps, _p(ch), ch.size // 4,
              resolution, variant, line0, nlines, nthreads)


def field_f64(points, charges, nthreads=0, with_maxc=False):
    """FP64 field at points (m,3) from charges (p,4); optionally the largest
    single contribution per point."""
    lib = load()
    pts = np.ascontiguousarray(np.asarray(points, np.float64).T)
    ch = np.ascontiguousarray(charges, np.float64)
    m = pts.shape[1]
    e = np.zeros((3, m))
    mc = np.zeros(m) if with_maxc else None
    lib.orc_field_f64(_p(pts[0]), _p(pts[1]), _p(pts[2]), m, _p(ch),
                      ch.size // 4, _p(e[0]), _p(e[1]), _p(e[2]), _p(mc),
                      nthreads)
    return (e.T, mc) if with_maxc else e.T


def field_f32(points, charges, three_arg=True):
    lib = load()
    pts = np.ascontiguousarray(np.asarray(points, np.float32).T)
    ch = np.ascontiguousarray(charges, np.float32)
    m = pts.shape[1]
    e = np.zeros((3, m), np.float32)
    lib.orc_field_f32(_p(pts[0]), _p(pts[1]), _p(pts[2]), m, _p(ch),
                      ch.size // 4, int(three_arg), _p(e[0]), _p(e[1]),
                      _p(e[2]))
    return e.T


def trace_lines_f64(charges, seeds, max_steps, resolution=1.0,
                    term_radius=0.5, max_steps_per_line=None, nthreads=0):
    """Extended method in FP64; returns (vertices (3, max_steps, n), len, cls)."""
    lib = load()
    ch = np.ascontiguousarray(charges, np.float64)
    seeds = np.asarray(seeds, np.float64)
    n = len(seeds)
    v = np.full((3, max_steps, n), np.nan)
    v[:, 0, :] = seeds.T
    ln = np.zeros(n, np.int32)
    cl = np.zeros(n, np.int32)
    msl = None
    if max_steps_per_line is not None:
        msl = np.ascontiguousarray(max_steps_per_line, np.int32)
    rc = lib.orc_trace_lines_f64(_p(ch), ch.size // 4, _p(v[0]), _p(v[1]),
                                 _p(v[2]), n, max_steps, _p(msl), resolution,
                                 term_radius, _p(ln), _p(cl), nthreads)
    if rc:
        raise RuntimeError(f"orc_trace_lines_f64 returned {rc}")
    return v, ln, cl


def adjoint_at(charges, V, targets, resolution=1.0, curvature=True):
    """FP64 discrete adjoint linearised at the trajectory V (3, S, n) (e.g. a
    GPU forward's vertices): returns (L, grad (p, 4))."""
    lib = load()
    ch = np.ascontiguousarray(charges, np.float64)
    V = [np.ascontiguousarray(np.asarray(V[c], np.float64).reshape(-1))
         for c in range(3)]
    T = [np.ascontiguousarray(np.asarray(targets[c], np.float64).reshape(-1))
         for c in range(3)]
    S, n = np.asarray(targets[0]).shape
    g = np.zeros(ch.size)
    L = lib.orc_adjoint_at_f64(_p(ch), len(ch), *map(_p, V), n, S, resolution,
                               int(bool(curvature)), *map(_p, T), _p(g))
    return L, g.reshape(-1, 4)


def adjoint_at_field(charges, V, targets, F, resolution=1.0, curvature=True,
                     lam_fp32=True):
    """adjoint_at with the field each step used given: F (3, S-1, n) with
    the Coulomb constant applied (a forward's own field output); the frozen
    map's directions and |E| come from it and, with lam_fp32, its step
    lengths by the reference's FP32 step sequence (those the FP32 forward
    took; else in FP64); the Jacobian products are FP64 sums.  Returns
    (L, grad (p, 4))."""
    lib = load()
    ch = np.ascontiguousarray(charges, np.float64)
    V = [np.ascontiguousarray(np.asarray(V[c], np.float64).reshape(-1))
         for c in range(3)]
    T = [np.ascontiguousarray(np.asarray(targets[c], np.float64).reshape(-1))
         for c in range(3)]
    S, n = np.asarray(targets[0]).shape
    Fe = [np.ascontiguousarray(np.asarray(F[c], np.float64).reshape(-1) / ELECTRO_K)
          for c in range(3)]
    g = np.zeros(ch.size)
    L = lib.orc_adjoint_at_field_f64(_p(ch), len(ch), *map(_p, V), n, S,
                                     resolution, int(bool(curvature)),
                                     *map(_p, T), *map(_p, Fe),
                                     int(bool(lam_fp32)), _p(g))
    return L, g.reshape(-1, 4)


class Frozen:
    """FP64 frozen-step map of the reference rule (adjoint checks): the
    step lengths come from the unperturbed trajectory of `charges`."""

    def __init__(self, charges, seeds, rows, targets, resolution=1.0):
        self.lib = load()
        self.ch = np.ascontiguousarray(charges, np.float64)
        seeds = np.asarray(seeds, np.float64)
        self.s = [np.ascontiguousarray(seeds[:, c]) for c in range(3)]
        self.n, self.S, self.res = len(seeds), rows, resolution
        self.t = [np.ascontiguousarray(np.asarray(targets[c], np.float64)
                                       .reshape(-1)) for c in range(3)]
        self.lam = np.zeros((rows - 1) * self.n)
        self.V = [np.zeros(rows * self.n) for _ in range(3)]
        self.L = self.lib.orc_frozen_loss_f64(
            _p(self.ch), len(self.ch), *map(_p, self.s), self.n, rows,
            resolution, *map(_p, self.t), None, _p(self.lam),
            *map(_p, self.V))

    def loss(self, charges):
        ch = np.ascontiguousarray(charges, np.float64)
        return self.lib.orc_frozen_loss_f64(
            _p(ch), len(ch), *map(_p, self.s), self.n, self.S, self.res,
            *map(_p, self.t), _p(self.lam), None, None, None, None)

    def grad(self):
        g = np.zeros(self.ch.size)
        self.lib.orc_frozen_grad_f64(_p(self.ch), len(self.ch),
                                     *map(_p, self.s), self.n, self.S,
                                     self.res, *map(_p, self.t),
                                     _p(self.lam), _p(g))
        return g.reshape(-1, 4)

    def complex_step(self, j, c, h=1e-30):
        return self.lib.orc_frozen_loss_cs_f64(
            _p(self.ch), len(self.ch), *map(_p, self.s), self.n, self.S,
            self.res, *map(_p, self.t), _p(self.lam), j, c, h)

    def central(self, j, c, h=1e-3):
        cp = self.ch.copy()
        cm = self.ch.copy()
        cp[j, c] += h
        cm[j, c] -= h
        return (self.loss(cp) - self.loss(cm)) / (2 * h)
