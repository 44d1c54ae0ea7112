"""The trace split over devices by the functor layer (em_calc_field_multi_*,
include/emgb300_functor.hpp) and its per-range entry (em_calc_field_part_*).
This pool gives one GPU, so ranges share device 0 (listed several times);
a device ordinal that does not exist is the injected failure (the call
returns EM_ERR_NO_DEVICE on the host; no GPU is faulted), and its range must
move to a device that succeeded."""
import numpy as np
import pytest

from conftest import lines_from

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def case(em):
    ch, seeds, _ = em.workloads.make("cpu_256", seed=11)
    return np.ascontiguousarray(ch, np.float32), seeds.astype(np.float32)[:1000], 301


def single(em, ch, seeds, rows, dtype=np.float32, **kw):
    x, y, z = lines_from(seeds.astype(dtype), rows, dtype)
    rc, _ = em.calc_field(x, y, z, ch.astype(dtype), len(seeds), 1.0, True,
                          require_n64=False, plain=False, **kw)
    assert rc == 0
    return np.stack([x, y, z])


def multi(em, ch, seeds, rows, devices, dtype=np.float32, **kw):
    x, y, z = lines_from(seeds.astype(dtype), rows, dtype)
    rc, perf, ran, nfailed = em.calc_field_multi(
        x, y, z, ch.astype(dtype), len(seeds), devices, 1.0, True, **kw)
    return rc, perf, ran, nfailed, np.stack([x, y, z])


@pytest.mark.parametrize("dtype", [np.float32, np.float64])
def test_ranges_equal_one_call_bitwise(em, gpu, case, dtype):
    ch, seeds, rows = case
    ref = single(em, ch, seeds, rows, dtype, arith="exact")
    rc, perf, ran, nfailed, v = multi(em, ch, seeds, rows, [0, 0, 0], dtype,
                                      arith="exact")
    assert rc == 0 and nfailed == 0 and ran == [0, 0, 0]
    assert np.array_equal(v.view(np.uint8), ref.view(np.uint8))
    assert perf.pairs == pytest.approx(len(seeds) * (rows - 1) * len(ch))


def test_fast_ranges_equal_one_call_with_fixed_shape(em, gpu, case):
    ch, seeds, rows = case
    kw = dict(threads_per_line=8, lines_per_thread=1)
    ref = single(em, ch, seeds, rows, **kw)
    rc, _, ran, nfailed, v = multi(em, ch, seeds, rows, [0] * 5, **kw)
    assert rc == 0 and nfailed == 0
    assert np.array_equal(v, ref)


def test_failed_device_range_is_remapped(em, gpu, case):
    """Range 1 starts on an ordinal that does not exist; it completes on a
    device that succeeded and the result is the one-call result."""
    ch, seeds, rows = case
    bad = em.load().em_device_count()
    ref = single(em, ch, seeds, rows, arith="exact")
    rc, _, ran, nfailed, v = multi(em, ch, seeds, rows, [0, bad, 0],
                                   arith="exact")
    assert rc == 0 and nfailed == 0
    assert ran == [0, 0, 0]
    assert np.array_equal(v.view(np.uint8), ref.view(np.uint8))


def test_no_working_device_reports_every_range(em, gpu, case):
    ch, seeds, rows = case
    bad = em.load().em_device_count()
    rc, _, ran, nfailed, v = multi(em, ch, seeds, rows, [bad, bad + 1])
    assert rc == 13 and nfailed == 2 and ran == [-1, -1]
    assert np.all(v[:, len(seeds):] == 0)   # nothing written past the seeds


def test_part_entry_writes_only_its_range(em, gpu, case):
    ch, seeds, rows = case
    n = len(seeds)
    ref = single(em, ch, seeds, rows, arith="exact")
    x, y, z = lines_from(seeds, rows, np.float32)
    o = em._capi.EmOptions()
    o.arith = em._capi.EM_ARITH_EXACT
    lo, cnt = 333, 250
    rc = em.load().em_calc_field_part_f32(
        0, x.ctypes.data, y.ctypes.data, z.ctypes.data, n, rows, lo, cnt,
        ch.ctypes.data, len(ch), 1.0, 1, em.tracer.ctypes_byref(o), None)
    assert rc == 0
    v = np.stack([x, y, z]).reshape(3, rows, n)
    r = ref.reshape(3, rows, n)
    assert np.array_equal(v[:, :, lo:lo + cnt], r[:, :, lo:lo + cnt])
    outside = np.ones(n, bool)
    outside[lo:lo + cnt] = False
    assert np.all(v[:, 1:, outside] == 0)
