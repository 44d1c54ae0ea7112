"""perfPacket.progress during a host-pointer call.

The reference adds each finished block's share to `perfData.progress`
(ElectroMag/src/CPU_Implement.cpp:340-342) while a monitor thread polls it
("Electromag utils.h":133-156).  em_calc_field_f32 raises `progress` as each
row chunk's trace completes, so a polling thread sees values strictly between
0 and 1 before the call returns with 1.0.
"""
import ctypes
import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_progress_rises_during_host_call(em, gpu):
    lib = gpu
    ch, seeds, _ = em.workloads.make("gpu_4096", seed=5)
    n, rows = 8192, 2000  # 197 MB of host arrays: traced in row chunks
    seeds = seeds[:n].astype(np.float32)
    X = em.new_lines(seeds, rows, np.float32)
    perf = em._capi.EmPerf()
    perf.progress = -1.0
    seen = []
    done = threading.Event()

    def monitor():
        while not done.is_set():
            seen.append(perf.progress)

    th = threading.Thread(target=monitor)
    th.start()
    try:
        rc = lib.em_calc_field_f32(
            X[0].ctypes.data, X[1].ctypes.data, X[2].ctypes.data, n, rows,
            ch.ctypes.data, len(ch), ctypes.c_float(1.0), 1,
            ctypes.cast(ctypes.pointer(perf), ctypes.c_void_p))
    finally:
        done.set()
        th.join()
    assert rc == 0, em.strerror(rc)
    assert perf.progress == 1.0
    between = sorted({v for v in seen if 0.0 < v < 1.0})
    assert len(between) >= 2, between
    # never decreases once the call has started
    started = [v for v in seen if v >= 0.0]
    assert all(b >= a for a, b in zip(started, started[1:]))
    assert np.isfinite(X[0][-n:]).all()
