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
import ctypes

import numpy as np

from . import _capi

_ARITH = {"fast": _capi.EM_ARITH_FAST, "exact": _capi.EM_ARITH_EXACT,
          "mixed": _capi.EM_ARITH_MIXED}
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
               plain=None, null_frac=0.0, field_out=None, refine_kappa=0.0):
    """Traces n field lines in place; returns (rc, perf).

    arith: "fast" (FP32/FP64 rsqrt + FMA), "exact" (the reference's IEEE
    sequence) or "mixed" (float32 only: compensated FP32 pairs with a
    Newton-corrected inv^3, the position in FP64, the field re-evaluated in
    double-float where sqrt(sum |t_j|^2) exceeds refine_kappa (default
    2.5; refine_kappa 0 and null_frac > 0: 1/null_frac) times |E|).

    rc is the reference's code (0 ok, 1 n == 0, 2 resolution == 0,
    3 total_steps < 2, 5 n % 64 with require_n64) or a library code >= 4.
    `plain=True` calls em_calc_field_f32/_f64, the exact reference
    signature (host arrays only; the n % 64 restriction applies).
    `field_out` (CUDA tensors only): a tensor of 3 * n * (total_steps - 1)
    values of the arrays' type that receives the field each step used,
    x block, y block, z block, vertex s of line l at s * n + l.
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
        plain = (not device and arith == "fast" and rule == "sse" and not null_frac
                 and require_n64 in (None, True) and not threads_per_line
                 and not warps_per_cta and not tile_charges
                 and not force_streamed and pack == "auto"
                 and not lines_per_thread and field_out is None
                 and not refine_kappa)
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
    o.null_frac = null_frac
    o.refine_kappa = refine_kappa
    if field_out is not None:
        if not (_is_torch(field_out) and field_out.is_cuda and device):
            raise ValueError("field_out needs CUDA tensors throughout")
        _check(field_out, dtype_name)
        if field_out.numel() < 3 * n * (total_steps - 1):
            raise ValueError("field_out holds fewer than 3*n*(total_steps-1) values")
        o.field_out = field_out.data_ptr()
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


_PREC = {"fp32": _capi.EM_PREC_FP32, "mixed": _capi.EM_PREC_MIXED,
         "df64": _capi.EM_PREC_DF64}
_REFINE = {"fp64": _capi.EM_REFINE_FP64, "df64": _capi.EM_REFINE_DF64}


def trace_lines(seeds, charges, max_steps, resolution=1.0, term_radius=0.5, *,
                steps_per_line=None, precision="fp32", want_field=False,
                threads_per_line=0, warps_per_cta=0, tile_charges=0,
                force_streamed=False, null_frac=0.0, deterministic=False,
                refine="df64", refine_kappa=0.0, stream=None):
    """Extended method (seeded lines, termination, step limits).

    seeds (n, 3), charges (p, 4): numpy arrays (host entry point) or CUDA
    torch tensors (device entry point, current stream).  precision: "fp32",
    "mixed" (FP32 pairs, FP64 positions, and the field re-evaluated where
    the sum is ill-conditioned, sqrt(sum |t_j|^2) > refine_kappa |E|
    (default 2.5; refine_kappa 0 and null_frac > 0: 1/null_frac); refine:
    the arithmetic of those re-evaluations, "df64" or "fp64"), "df64"
    (double-float pairs on the FP32 pipes, FP64 field and positions) or
    "fp64".
    Returns a dict with vertices (3, max_steps, n), len (n,), cls (n,),
    field (3, max_steps, n) when want_field, and perf.
    """
    import ctypes
    lib = _capi.load()
    f64 = precision == "fp64"
    o = _capi.EmOptions()
    o.precision = _capi.EM_PREC_FP32 if f64 else _PREC[precision]
    o.threads_per_line = threads_per_line
    o.warps_per_cta = warps_per_cta
    o.tile_charges = tile_charges
    o.force_streamed = int(bool(force_streamed))
    o.null_frac = null_frac
    o.refine_kappa = refine_kappa
    o.deterministic = int(bool(deterministic))
    o.refine = _REFINE[refine]
    perf = _capi.EmPerf()
    fn = lib.em_trace_lines_f64 if f64 else lib.em_trace_lines_f32
    if _is_torch(seeds):
        import torch
        dt = torch.float64 if f64 else torch.float32
        n = seeds.shape[0]
        dev = seeds.device
        V = torch.empty((3, max_steps, n), dtype=dt, device=dev)
        V[:, 0, :] = seeds.T.to(dt)
        ln = torch.zeros(n, dtype=torch.int32, device=dev)
        cl = torch.zeros(n, dtype=torch.int32, device=dev)
        F = (torch.empty((3, max_steps, n), dtype=dt, device=dev)
             if want_field else None)
        ch = charges.to(dt).contiguous()
        spl = (steps_per_line.to(torch.int32).contiguous()
               if steps_per_line is not None else None)
        o.device_ptrs = 1
        o.stream = (stream if stream is not None else
                    torch.cuda.current_stream(dev).cuda_stream)
        rc = fn(V[0].data_ptr(), V[1].data_ptr(), V[2].data_ptr(), n,
                max_steps, spl.data_ptr() if spl is not None else None,
                ch.data_ptr(), ch.numel() // 4, resolution, term_radius,
                ln.data_ptr(), cl.data_ptr(),
                F[0].data_ptr() if F is not None else None,
                F[1].data_ptr() if F is not None else None,
                F[2].data_ptr() if F is not None else None,
                ctypes_byref(o), ctypes_byref(perf))
    else:
        dt = np.float64 if f64 else np.float32
        seeds = np.asarray(seeds)
        n = seeds.shape[0]
        V = np.zeros((3, max_steps, n), dt)
        V[:, 0, :] = seeds.T
        ln = np.zeros(n, np.int32)
        cl = np.zeros(n, np.int32)
        F = np.zeros((3, max_steps, n), dt) if want_field else None
        ch = np.ascontiguousarray(charges, dt)
        spl = (np.ascontiguousarray(steps_per_line, np.int32)
               if steps_per_line is not None else None)
        rc = fn(V[0].ctypes.data, V[1].ctypes.data, V[2].ctypes.data, n,
                max_steps, spl.ctypes.data if spl is not None else None,
                ch.ctypes.data, ch.size // 4, resolution, term_radius,
                ln.ctypes.data, cl.ctypes.data,
                F[0].ctypes.data if F is not None else None,
                F[1].ctypes.data if F is not None else None,
                F[2].ctypes.data if F is not None else None,
                ctypes_byref(o), ctypes_byref(perf))
    if rc:
        raise _capi.EmError(rc, "em_trace_lines")
    out = dict(vertices=V, len=ln, cls=cl, perf=perf)
    if want_field:
        out["field"] = F
    return out


def seed_fibonacci(charges, lines_per_charge, radius=1.0):
    """Seeds around every positive charge (em_seed_fibonacci_f32); (m, 3)."""
    import ctypes
    lib = _capi.load()
    ch = np.ascontiguousarray(charges, np.float32)
    cap = int((ch[:, 3] > 0).sum()) * int(lines_per_charge)
    out = np.zeros((3, max(cap, 1)), np.float32)
    cnt = ctypes.c_size_t()
    rc = lib.em_seed_fibonacci_f32(ch.ctypes.data, len(ch), lines_per_charge,
                                   radius, out[0].ctypes.data,
                                   out[1].ctypes.data, out[2].ctypes.data,
                                   cap, ctypes.addressof(cnt))
    if rc:
        raise _capi.EmError(rc, "em_seed_fibonacci_f32")
    return out[:, : cnt.value].T.copy()


def adjoint(seeds, charges, rows, targets, resolution=1.0, use_curvature=True,
            checkpoint=False):
    """Loss sum |v - t|^2 over the traced vertices and its gradient with
    respect to the charges (em_adjoint_f32, frozen step lengths).

    seeds (n, 3), charges (p, 4), targets (3, rows, n): numpy arrays.
    checkpoint: keep only the vertices and recompute the field per 64-row
    segment instead of storing the forward's field.
    Returns dict(loss, grad (p, 4) float64 [dx, dy, dz, dq], vertices
    (3, rows, n), fwd_time, bwd_time, bwd_pairs)."""
    lib = _capi.load()
    seeds = np.asarray(seeds, np.float32)
    n = seeds.shape[0]
    V = np.zeros((3, rows, n), np.float32)
    V[:, 0, :] = seeds.T
    T = np.ascontiguousarray(targets, np.float32)
    ch = np.ascontiguousarray(charges, np.float32)
    p = ch.shape[0]
    loss = np.zeros(1, np.float64)
    grad = np.zeros((p, 4), np.float64)
    fwd, bwd = _capi.EmPerf(), _capi.EmPerf()
    o = _capi.EmOptions()
    o.adjoint_checkpoint = int(bool(checkpoint))
    rc = lib.em_adjoint_f32(V[0].ctypes.data, V[1].ctypes.data,
                            V[2].ctypes.data, n, rows, ch.ctypes.data, p,
                            resolution, int(bool(use_curvature)),
                            T[0].ctypes.data, T[1].ctypes.data,
                            T[2].ctypes.data, loss.ctypes.data,
                            grad.ctypes.data, ctypes_byref(o),
                            ctypes_byref(fwd), ctypes_byref(bwd))
    if rc:
        raise _capi.EmError(rc, "em_adjoint_f32")
    return dict(loss=float(loss[0]), grad=grad, vertices=V,
                fwd_time=fwd.time, bwd_time=bwd.time, bwd_pairs=bwd.pairs)


def trace_loss_function():
    """torch.autograd.Function: loss = TraceLoss.apply(charges, seeds, rows,
    targets, resolution, use_curvature); charges (p, 4) CPU tensor.  The
    forward runs the tracer and its adjoint together; backward scales the
    stored gradient."""
    import torch

    class TraceLoss(torch.autograd.Function):
        @staticmethod
        def forward(ctx, charges, seeds, rows, targets, resolution=1.0,
                    use_curvature=True):
            out = adjoint(seeds.detach().cpu().numpy(),
                          charges.detach().cpu().numpy(), rows,
                          targets.detach().cpu().numpy(), resolution,
                          use_curvature)
            ctx.save_for_backward(torch.from_numpy(out["grad"]).to(charges))
            return charges.new_tensor(out["loss"])

        @staticmethod
        def backward(ctx, gout):
            (g,) = ctx.saved_tensors
            return gout * g, None, None, None, None, None

    return TraceLoss


def adjoint_device(V, charges, targets, resolution=1.0, use_curvature=True,
                   stream=None, checkpoint=False):
    """em_adjoint_f32 on CUDA torch tensors: V (3, rows, n) float32 with the
    seeds in row 0 (rows written by the forward), charges (p, 4), targets
    (3, rows, n); checkpoint as in adjoint().  Returns (loss, grad (p, 4)
    float64 tensor, fwd_s, bwd_s)."""
    import torch
    lib = _capi.load()
    rows, n = V.shape[1], V.shape[2]
    p = charges.shape[0]
    loss = torch.zeros(1, dtype=torch.float64, device=V.device)
    grad = torch.zeros((p, 4), dtype=torch.float64, device=V.device)
    o = _capi.EmOptions()
    o.device_ptrs = 1
    o.adjoint_checkpoint = int(bool(checkpoint))
    o.stream = (stream if stream is not None else
                torch.cuda.current_stream(V.device).cuda_stream)
    fwd, bwd = _capi.EmPerf(), _capi.EmPerf()
    ch = charges.contiguous()
    T = targets.contiguous()
    rc = lib.em_adjoint_f32(V[0].data_ptr(), V[1].data_ptr(), V[2].data_ptr(),
                            n, rows, ch.data_ptr(), p, resolution,
                            int(bool(use_curvature)), T[0].data_ptr(),
                            T[1].data_ptr(), T[2].data_ptr(), loss.data_ptr(),
                            grad.data_ptr(), ctypes_byref(o),
                            ctypes_byref(fwd), ctypes_byref(bwd))
    if rc:
        raise _capi.EmError(rc, "em_adjoint_f32")
    return loss, grad, fwd.time, bwd.time


def calc_field_multi(x, y, z, charges, n, devices, resolution=1.0,
                     use_curvature=True, *, arith="fast", rule="sse",
                     threads_per_line=0, lines_per_thread=0):
    """The trace split over CUDA devices (em_calc_field_multi_*): one line
    range per entry of `devices` (ordinals may repeat), one host thread per
    range, failed ranges moved to devices that succeeded.  Host arrays in
    the reference layout.  Returns (rc, perf, ran_on list, nfailed)."""
    lib = _capi.load()
    f32 = str(x.dtype).endswith("float32")
    for a in (x, y, z, charges):
        _check(a, "float32" if f32 else "float64")
    steps = x.size // n if n else 0
    p = charges.size // 4
    o = _capi.EmOptions()
    o.arith = _ARITH[arith]
    o.rule = _RULE[rule]
    o.threads_per_line = threads_per_line
    o.lines_per_thread = lines_per_thread
    devs = np.ascontiguousarray(devices, np.int32)
    ran = np.full(len(devs), -1, np.int32)
    nfailed = ctypes.c_size_t(0)
    perf = _capi.EmPerf()
    fn = lib.em_calc_field_multi_f32 if f32 else lib.em_calc_field_multi_f64
    rc = fn(devs.ctypes.data, len(devs), _ptr(x), _ptr(y), _ptr(z), n, steps,
            _ptr(charges), p, resolution, int(bool(use_curvature)),
            ctypes_byref(o), ctypes_byref(perf), ctypes_byref(nfailed),
            ran.ctypes.data)
    return rc, perf, ran.tolist(), int(nfailed.value)


def verlet_step(dyn, accel, charges, box_min, box_max, dt, steps=1,
                stream=None, lanes_per_particle=0):
    """Velocity-Verlet steps of moving charges (em_verlet_step_*), in place.
    dyn (n, 8) {x, y, z, q, vx, vy, vz, m}, accel (n, 3), charges (p, 4):
    numpy arrays, or CUDA tensors (then on the current torch stream).
    lanes_per_particle: 1, 2 or 4 (0: the library's choice).
    Returns the perf record."""
    lib = _capi.load()
    dev = _is_torch(dyn) and dyn.is_cuda
    f32 = str(dyn.dtype).endswith("float32")
    for a in (dyn, accel, charges):
        _check(a, "float32" if f32 else "float64")
    n = dyn.shape[0]
    p = charges.shape[0]
    npt = np.float32 if f32 else np.float64
    lo = np.ascontiguousarray(box_min, npt)
    hi = np.ascontiguousarray(box_max, npt)
    o = _capi.EmOptions()
    o.threads_per_line = lanes_per_particle
    if dev:
        import torch
        o.device_ptrs = 1
        o.stream = (stream if stream is not None else
                    torch.cuda.current_stream(dyn.device).cuda_stream)
    perf = _capi.EmPerf()
    fn = lib.em_verlet_step_f32 if f32 else lib.em_verlet_step_f64
    rc = fn(_ptr(dyn), _ptr(accel), n, _ptr(charges), p, lo.ctypes.data,
            hi.ctypes.data, dt, steps, ctypes_byref(o), ctypes_byref(perf))
    if rc:
        raise _capi.EmError(rc, "em_verlet_step")
    return perf


def trace_batch(sets, max_steps, resolution=1.0, term_radius=0.5, *,
                steps_per_line=None, store_rows=0, threads_per_line=0,
                lines_per_item=0, first_budget=0, phases=0, tile_charges=0,
                stages=0, use_graph=False, deterministic=False, stream=None):
    """Batched extended method (em_trace_batch_f32).

    sets: list of (charges (p, 4), seeds (m, 3)) numpy arrays, or a dict of
    concatenated CUDA tensors {charges, seeds, charge_off, line_off} (the
    offsets as host int64 numpy arrays).  steps_per_line: concatenated
    per-line limits or None.  Returns dict(len, cls, last (N, 3),
    rows (3, store_rows, N) or None, perf, charge_off, line_off)."""
    lib = _capi.load()
    o = _capi.EmBatchOptions()
    o.threads_per_line = threads_per_line
    o.lines_per_item = lines_per_item
    o.first_budget = first_budget
    o.phases = phases
    o.tile_charges = tile_charges
    o.stages = stages
    o.use_graph = int(bool(use_graph))
    o.deterministic = int(bool(deterministic))
    perf = _capi.EmPerf()
    if isinstance(sets, dict):
        import torch
        ch = sets["charges"].contiguous()
        sd = sets["seeds"].contiguous()
        coff = np.ascontiguousarray(sets["charge_off"], np.int64)
        loff = np.ascontiguousarray(sets["line_off"], np.int64)
        N = int(loff[-1])
        dev = ch.device
        S = sd.T.contiguous()
        last = torch.empty((3, N), dtype=torch.float32, device=dev)
        ln = torch.empty(N, dtype=torch.int32, device=dev)
        cl = torch.empty(N, dtype=torch.int32, device=dev)
        R = (torch.empty((3, store_rows, N), dtype=torch.float32, device=dev)
             if store_rows else None)
        spl = (steps_per_line.to(torch.int32).contiguous()
               if steps_per_line is not None else None)
        o.device_ptrs = 1
        o.stream = (stream if stream is not None else
                    torch.cuda.current_stream(dev).cuda_stream)
        ptr = lambda a: a.data_ptr()  # noqa: E731
    else:
        coff = np.zeros(len(sets) + 1, np.int64)
        loff = np.zeros(len(sets) + 1, np.int64)
        for i, (c, s) in enumerate(sets):
            coff[i + 1] = coff[i] + len(c)
            loff[i + 1] = loff[i] + len(s)
        ch = np.ascontiguousarray(np.concatenate([np.asarray(c, np.float32)
                                                  for c, _ in sets]))
        sd = np.concatenate([np.asarray(s, np.float32) for _, s in sets])
        S = np.ascontiguousarray(sd.T)
        N = int(loff[-1])
        last = np.zeros((3, N), np.float32)
        ln = np.zeros(N, np.int32)
        cl = np.zeros(N, np.int32)
        R = np.zeros((3, store_rows, N), np.float32) if store_rows else None
        spl = (np.ascontiguousarray(steps_per_line, np.int32)
               if steps_per_line is not None else None)
        ptr = lambda a: a.ctypes.data  # noqa: E731
    rc = lib.em_trace_batch_f32(
        len(coff) - 1, ptr(ch), coff.ctypes.data, ptr(S[0]), ptr(S[1]),
        ptr(S[2]), loff.ctypes.data, ptr(spl) if spl is not None else None,
        max_steps, resolution, term_radius, store_rows,
        ptr(R[0]) if R is not None else None,
        ptr(R[1]) if R is not None else None,
        ptr(R[2]) if R is not None else None,
        ptr(last[0]), ptr(last[1]), ptr(last[2]), ptr(ln), ptr(cl),
        ctypes_byref(o), ctypes_byref(perf))
    if rc:
        raise _capi.EmError(rc, "em_trace_batch_f32")
    return dict(len=ln, cls=cl, last=last.T, rows=R, perf=perf,
                charge_off=coff, line_off=loff)
