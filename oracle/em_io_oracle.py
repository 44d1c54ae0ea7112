"""TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.

Restatement, in numpy, of the reference program's inputs and outputs around
the tracer, the oracle the tests hold the library's versions to:

  PRESETS          SimulationParams of ElectroMag/src/ElectroMag.cpp:43-55
  init_charges     InitializePointChargeArray, "Electromag utils.h":91-111
  grid_lines       InitializeFieldLineArray grid mode, :29-70
  random_lines     InitializeFieldLineArray random mode, :40-51
  save_text        the --save dump, ElectroMag.cpp:372-397
  autoregress      the --autoregress check, ElectroMag.cpp:400-453

The rand() stream comes from the platform C library through ctypes (the
reference calls the same srand()/rand()).  Only tests/ import this module.
"""
import ctypes
import math

import numpy as np

PRESETS = {
    "normal": (128, 128, 1, 1024, 0, 2500),
    "enhanced": (256, 112, 1, 2048, 0, 5000),
    "extreme": (256, 256, 1, 2048, 0, 5000),
    "insane": (512, 512, 1, 2048, 0, 5000),
    "fuckingInsane": (1024, 1024, 1, 5120, 0, 10000),
    "cpu": (64, 64, 1, 1000, 0, 1000),
    "micro": (16, 16, 1, 1000, 0, 1000),
    "bogo": (16, 16, 1, 50, 0, 500),
}
RAND_MAX = 2147483647

_libc = None


def libc_rand(seed, count):
    """The C library's rand() values after srand(seed)."""
    global _libc
    if _libc is None:
        _libc = ctypes.CDLL(None)
        _libc.srand.argtypes = [ctypes.c_uint]
        _libc.rand.restype = ctypes.c_int
    _libc.srand(seed)
    return np.array([_libc.rand() for _ in range(count)], np.int64)


def init_charges(p, seed=1, dtype=np.float32):
    """(p, 4): x, y, z = (T)(rand() - (T)RAND_MAX/2) / RAND_MAX * 10000,
    q = (T)(rand() - (T)RAND_MAX/10) / RAND_MAX, all in T arithmetic."""
    T = np.dtype(dtype).type
    r = libc_rand(seed, 4 * p).reshape(p, 4).astype(T)
    rm = T(RAND_MAX)
    out = np.empty((p, 4), T)
    out[:, :3] = (r[:, :3] - rm / T(2)) / rm * T(10000)
    out[:, 3] = (r[:, 3] - rm / T(10)) / rm
    return out


def grid_lines(w, h, d, dtype=np.float32):
    """(3, w*h*d) seeds: per axis (T)(-((T)extent)/2 + 1e-5) stepped by ++ in
    T, times (T)10; line k*w*h + j*w + i."""
    T = np.dtype(dtype).type

    def axis(extent):
        v = T(float(-T(extent) / T(2)) + 1e-5)
        out = np.empty(extent, T)
        for i in range(extent):
            out[i] = v
            v = T(v + T(1))
        return T(10) * out

    xs, ys, zs = axis(w), axis(h), axis(d)
    k, j, i = np.meshgrid(np.arange(d), np.arange(h), np.arange(w), indexing="ij")
    return np.stack([xs[i.ravel()], ys[j.ravel()], zs[k.ravel()]])


def random_lines(n, seed, dtype=np.float32):
    """(3, n): (T)(rand() - RAND_MAX/2) / RAND_MAX * 10000 with the integer
    half, x, y, z drawn in turn per line."""
    T = np.dtype(dtype).type
    r = (libc_rand(seed, 3 * n).reshape(n, 3) - RAND_MAX // 2).astype(T)
    return ((r / T(RAND_MAX)) * T(10000)).T.copy()


def _g(v):
    """std::ostream's default float output (printf %g of the widened value,
    which prints a negative NaN as -nan)."""
    v = float(v)
    if math.isnan(v):
        return "-nan" if math.copysign(1.0, v) < 0 else "nan"
    return "%g" % v


def save_text(n, rows, a=None, b=None):
    """The dump text; a, b: (3, rows*n) arrays in the reference layout."""
    out = []
    for line in range(n):
        for row in range(rows):
            i = row * n + line
            for tag, v in (("CPUL", a), ("GPUL", b)):
                if v is not None:
                    out.append(f" {tag} [{line}][{row}] x: {_g(v[0][i])} "
                               f"y: {_g(v[1][i])} z: {_g(v[2][i])}\n")
    return "".join(out)


def _offset(a, b, i):
    """vec3Len(vec3(a[i], b[i])) in float32, left-to-right, no contraction."""
    f = np.float32
    d = [f(a[c][i]) - f(b[c][i]) for c in range(3)]
    return f(np.sqrt(f(f(d[0] * d[0]) + f(d[1] * d[1])) + f(d[2] * d[2])))


def autoregress(n, rows, a, b, threshold=0.1):
    """(first (n,) int64 with -1 for none, report text).  The offsets of all
    rows are formed at once in float32 (one rounding per operation, as the
    reference's per-row loop)."""
    f = np.float32
    A = [np.asarray(a[c], f).reshape(rows, n) for c in range(3)]
    B = [np.asarray(b[c], f).reshape(rows, n) for c in range(3)]
    d = [A[c] - B[c] for c in range(3)]
    with np.errstate(invalid="ignore", over="ignore"):
        off = np.sqrt((d[0] * d[0] + d[1] * d[1]) + d[2] * d[2])
        hit = off > f(threshold)
    first = np.where(hit.any(0), hit.argmax(0), -1).astype(np.int64)
    rep = []
    for line in np.nonzero(first >= 0)[0]:
        step = int(first[line])
        for s in ([step - 1, step] if step > 0 else [step]):
            k = s * n + line
            rep.append(f" CPUL [{line}][{s}] x: {_g(a[0][k])} y: {_g(a[1][k])} "
                       f"z: {_g(a[2][k])}\n")
            rep.append(f" GPUL [{line}][{s}] x: {_g(b[0][k])} y: {_g(b[1][k])} "
                       f"z: {_g(b[2][k])}\n")
            rep.append(f" 3D offset: {_g(_offset(a, b, k))}\n")
        rep.append("\n")
    return first, "".join(rep)
