"""ctypes binding of libemgb300.so (the C ABI declared in include/emgb300.h).

Loading fails loudly when the library has not been built: there is no CPU
fallback anywhere in this package.
"""
import ctypes
import os
import re

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libemgb300.so")
HEADER_DIR = os.path.join(os.path.dirname(_HERE), "include")

P = ctypes.c_void_p
S = ctypes.c_size_t
I = ctypes.c_int
F = ctypes.c_float
D = ctypes.c_double

EM_OK = 0
EM_ERR_N_ZERO = 1
EM_ERR_RESOLUTION = 2
EM_ERR_STEPS = 3
EM_ERR_ARG = 4
EM_ERR_N_ALIGN = 5
EM_ERR_CUDA = 10
EM_ERR_NOMEM = 11
EM_ERR_TIMEOUT = 12
EM_ERR_NO_DEVICE = 13
EM_ERR_TOO_LARGE = 14

EM_NOALLOC_MAX_CHARGES = 16384
EM_ARITH_FAST = 0
EM_ARITH_EXACT = 1
EM_ARITH_MIXED = 2
EM_PACK_AUTO = 0
EM_PACK_SCALAR = 1
EM_PACK_PAIRS = 2
EM_PREC_FP32 = 0
EM_PREC_MIXED = 1
EM_PREC_DF64 = 2
EM_REFINE_DF64 = 0
EM_REFINE_FP64 = 1
EM_TERM_STEPS = 0
EM_TERM_CHARGE = 1
EM_TERM_NULL = 2
EM_RULE_SSE = 0
EM_RULE_GENERIC = 1


class EmPerf(ctypes.Structure):
    """em_perf: perfPacket's fields ("Data Structures.h":221-236) + counters."""
    _fields_ = [("performance", D), ("time", D), ("progress", D),
                ("pairs", D), ("wall_time", D), ("fp64_refines", D)]


class EmBatchOptions(ctypes.Structure):
    _fields_ = [("threads_per_line", I), ("lines_per_item", I),
                ("first_budget", I), ("phases", I), ("tile_charges", I),
                ("stages", I), ("use_graph", I), ("deterministic", I),
                ("device_ptrs", I), ("stream", P)]


class EmOptions(ctypes.Structure):
    _fields_ = [("arith", I), ("rule", I), ("require_n64", I),
                ("device_ptrs", I), ("stream", P), ("threads_per_line", I),
                ("warps_per_cta", I), ("tile_charges", I),
                ("force_streamed", I), ("pack", I),
                ("lines_per_thread", I), ("precision", I),
                ("null_frac", D), ("deterministic", I),
                ("adjoint_checkpoint", I), ("refine", I),
                ("field_out", P), ("refine_kappa", D)]


_SIGNATURES = {
    "em_calc_field_f32": (I, [P, P, P, S, S, P, S, F, I, P]),
    "em_calc_field_f64": (I, [P, P, P, S, S, P, S, D, I, P]),
    "em_calc_field_ex_f32": (I, [P, P, P, S, S, P, S, F, I, P, P]),
    "em_calc_field_ex_f64": (I, [P, P, P, S, S, P, S, D, I, P, P]),
    "em_calc_field_noalloc_f32": (I, [P, P, P, S, S, P, S, F, I, P]),
    "em_trace_lines_f32": (I, [P, P, P, S, S, P, P, S, F, F, P, P, P, P, P,
                               P, P]),
    "em_trace_lines_f64": (I, [P, P, P, S, S, P, P, S, D, D, P, P, P, P, P,
                               P, P]),
    "em_seed_fibonacci_f32": (I, [P, S, S, F, P, P, P, S, P]),
    "em_trace_batch_f32": (I, [S, P, P, P, P, P, P, P, I, F, F, I, P, P, P,
                               P, P, P, P, P, P, P]),
    "em_adjoint_f32": (I, [P, P, P, S, S, P, S, F, I, P, P, P, P, P, P, P,
                           P]),
    "em_field_f32": (I, [P, P, P, S, P, S, P, P, P, P]),
    "em_field_f64": (I, [P, P, P, S, P, S, P, P, P, P]),
    "em_fp32_peak_tflops": (I, [P, P]),
    "em_selftest_rounded_ops": (I, [ctypes.c_ulonglong, P]),
    "em_selftest_wait_timeout": (I, [I, P]),
    "em_launch_count": (ctypes.c_ulonglong, []),
    "em_device_count": (I, []),
    "em_release": (I, []),
    "em_strerror": (ctypes.c_char_p, [I]),
    "em_version": (ctypes.c_char_p, []),
    "em_calc_field_part_f32": (I, [I, P, P, P, S, S, S, S, P, S, F, I, P, P]),
    "em_calc_field_part_f64": (I, [I, P, P, P, S, S, S, S, P, S, D, I, P, P]),
    "em_calc_field_multi_f32": (I, [P, S, P, P, P, S, S, P, S, F, I, P, P, P,
                                    P]),
    "em_calc_field_multi_f64": (I, [P, S, P, P, P, S, S, P, S, D, I, P, P, P,
                                    P]),
    "em_release_device": (I, [I]),
    "em_verlet_step_f32": (I, [P, P, S, P, S, P, P, F, S, P, P]),
    "em_verlet_step_f64": (I, [P, P, S, P, S, P, P, D, S, P, P]),
    "em_preset": (I, [ctypes.c_char_p, P]),
    "em_init_charges_f32": (I, [P, S, ctypes.c_uint]),
    "em_init_charges_f64": (I, [P, S, ctypes.c_uint]),
    "em_init_lines_f32": (I, [P, P, P, S, S, S, I, ctypes.c_uint]),
    "em_init_lines_f64": (I, [P, P, P, S, S, S, I, ctypes.c_uint]),
    "em_save_lines_text_f32": (I, [ctypes.c_char_p, S, S, P, P, P, P, P, P]),
    "em_autoregress_f32": (I, [ctypes.c_char_p, S, S, P, P, P, P, P, P, F, P,
                               P, P]),
}


class EmPresetParams(ctypes.Structure):
    _fields_ = [("nx", S), ("ny", S), ("nz", S), ("p_static", S),
                ("p_dynamic", S), ("len", S)]


def declared_symbols():
    """Every entry point declared with EM_API in include/*.h."""
    names = []
    for fn in sorted(os.listdir(HEADER_DIR)):
        if fn.endswith(".h"):
            with open(os.path.join(HEADER_DIR, fn)) as f:
                names += re.findall(r"EM_API\s+[^;(]*?\b(em_\w+)\s*\(", f.read())
    return names


_lib = None


def load():
    """Returns the loaded library; raises if it is missing or incomplete."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(
            f"{LIB_PATH} is not built; run "
            "python -c 'import __graft_entry__ as g; g.build()' first")
    lib = ctypes.CDLL(LIB_PATH)
    for name, (res, args) in _SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def strerror(code):
    return load().em_strerror(int(code)).decode()


class EmError(RuntimeError):
    def __init__(self, code, what=""):
        self.code = int(code)
        super().__init__(f"{what}: error {self.code} ({strerror(self.code)})")
