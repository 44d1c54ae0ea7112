"""Host-side API mirroring the reference's calc-field interface.

calc_field() takes what CalcField_CPU<T> takes (ElectroMag/src/
"CPU Implement.h":25-30): the three component arrays of the field-line
container (n*total_steps elements each, vertex (line, step) at step*n+line,
row 0 = seeds), the charge records {x, y, z, q}, n, the resolution and
useCurvature.  It returns the reference's integer code and a perf record, and
writes rows 1..total_steps-1 in place.  numpy arrays go through the
host-pointer entry points; CUDA torch tensors through the device-pointer ones
on the current torch stream.
"""
import numpy as np

from . import _capi

_ARITH = {"fast": _capi.EM_ARITH_FAST, "exact": _capi.EM_ARITH_EXACT}
_RULE = {"sse": _capi.EM_RULE_SSE, "generic": _capi.EM_RULE_GENERIC}
_PACK = {"auto": _capi.EM_PACK_AUTO, "scalar": _capi.EM_PACK_SCALAR,
         "pairs": _capi.EM_PACK_PAIRS}


def _is_torch(a):
    return type(a).__module__.startswith("torch")


def _ptr(a):
    if _is_torch(a):
        return a.data_ptr()
    return a.ctypes.data


def _check(a, dtype_name):
    if _is_torch(a):
        if not a.is_contiguous():
            raise ValueError("arrays must be contiguous")
        if str(a.dtype).split(".")[-1] != dtype_name:
            raise TypeError(f"expected {dtype_name}, got {a.dtype}")
        return
    if not isinstance(a, np.ndarray) or not a.flags.c_contiguous:
        raise ValueError("arrays must be C-contiguous numpy arrays or tensors")
    if a.dtype.name != dtype_name:
        raise TypeError(f"expected {dtype_name}, got {a.dtype}")


def calc_field(x, y, z, charges, n, resolution=1.0, use_curvature=True, *,
               arith="fast", rule="sse", require_n64=None, stream=None,
               threads_per_line=0, warps_per_cta=0, tile_charges=0,
               force_streamed=False, pack="auto", lines_per_thread=0,
               plain=None):
    """Traces n field lines in place; returns (rc, perf).

    rc is the reference's code (0 ok, 1 n == 0, 2 resolution == 0,
    3 total_steps < 2, 5 n % 64 with require_n64) or a library code >= 4.
    `plain=True` calls em_calc_field_f32/_f64, the exact reference
    signature (host arrays only; the n % 64 restriction applies).
    """
    lib = _capi.load()
    dtype_name = "float32" if str(x.dtype).endswith("float32") else "float64"
    for a in (x, y, z, charges):
        _check(a, dtype_name)
    f32 = dtype_name == "float32"
    size = x.numel() if _is_torch(x) else x.size
    total_steps = size // n if n else 0
    p = (charges.numel() if _is_torch(charges) else charges.size) // 4
    device = _is_torch(x) and x.is_cuda
    perf = _capi.EmPerf()
    if plain is None:
        plain = (not device and arith == "fast" and rule == "sse"
                 and require_n64 in (None, True) and not threads_per_line
                 and not warps_per_cta and not tile_charges
                 and not force_streamed and pack == "auto"
                 and not lines_per_thread)
    if plain:
        if device:
            raise ValueError("the plain entry point takes host arrays")
        fn = lib.em_calc_field_f32 if f32 else lib.em_calc_field_f64
        rc = fn(_ptr(x), _ptr(y), _ptr(z), n, total_steps, _ptr(charges), p,
                resolution, int(bool(use_curvature)), ctypes_byref(perf))
        return rc, perf
    o = _capi.EmOptions()
    o.arith = _ARITH[arith]
    o.rule = _RULE[rule]
    o.require_n64 = int(bool(require_n64))
    o.device_ptrs = int(device)
    if device:
        if stream is None:
            import torch
            stream = torch.cuda.current_stream(x.device).cuda_stream
        o.stream = stream
    o.threads_per_line = threads_per_line
    o.warps_per_cta = warps_per_cta
    o.tile_charges = tile_charges
    o.force_streamed = int(bool(force_streamed))
    o.pack = _PACK[pack]
    o.lines_per_thread = lines_per_thread
    fn = lib.em_calc_field_ex_f32 if f32 else lib.em_calc_field_ex_f64
    rc = fn(_ptr(x), _ptr(y), _ptr(z), n, total_steps, _ptr(charges), p,
            resolution, int(bool(use_curvature)), ctypes_byref(o),
            ctypes_byref(perf))
    return rc, perf


def ctypes_byref(obj):
    import ctypes
    return ctypes.cast(ctypes.pointer(obj), ctypes.c_void_p)


def new_lines(seeds, total_steps, dtype=np.float32):
    """Allocates the reference's SoA line container with `seeds` in row 0."""
    seeds = np.asarray(seeds)
    n = seeds.shape[0]
    out = []
    for c in range(3):
        a = np.zeros(n * total_steps, dtype)
        a[:n] = seeds[:, c]
        out.append(a)
    return out


def field(points, charges, *, arith="fast", rule="sse", stream=None):
    """Field at points (m, 3) from charge records (p, 4); returns (m, 3).

    numpy input: host entry point; CUDA torch tensors: device pointers on the
    current stream (points given as a (3, m) tensor of x, y, z rows)."""
    import ctypes
    lib = _capi.load()
    o = _capi.EmOptions()
    o.arith = _ARITH[arith]
    o.rule = _RULE[rule]
    if _is_torch(points):
        import torch
        pts = points.contiguous()
        dt = pts.dtype
        m = pts.shape[1]
        out = torch.empty_like(pts)
        o.device_ptrs = 1
        o.stream = (stream if stream is not None else
                    torch.cuda.current_stream(pts.device).cuda_stream)
        fn = lib.em_field_f32 if dt == torch.float32 else lib.em_field_f64
        ch = charges.contiguous()
        rc = fn(pts[0].data_ptr(), pts[1].data_ptr(), pts[2].data_ptr(), m,
                ch.data_ptr(), ch.numel() // 4, out[0].data_ptr(),
                out[1].data_ptr(), out[2].data_ptr(), ctypes_byref(o))
        if rc:
            raise _capi.EmError(rc, "em_field")
        return out
    pts = np.asarray(points)
    dt = pts.dtype if pts.dtype in (np.float32, np.float64) else np.float64
    pts = np.ascontiguousarray(pts.T, dt)
    ch = np.ascontiguousarray(charges, dt)
    m = pts.shape[1]
    out = np.zeros((3, m), dt)
    fn = lib.em_field_f32 if dt == np.float32 else lib.em_field_f64
    rc = fn(pts[0].ctypes.data, pts[1].ctypes.data, pts[2].ctypes.data, m,
            ch.ctypes.data, ch.size // 4, out[0].ctypes.data,
            out[1].ctypes.data, out[2].ctypes.data, ctypes_byref(o))
    if rc:
        raise _capi.EmError(rc, "em_field")
    return out.T
