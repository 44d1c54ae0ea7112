"""em_calc_field_noalloc_f32: tracing for callers that cannot let the library
allocate device memory (their own pool holds the GPU, or an allocation's
implicit synchronisation would stall their streams).

The entry point keeps its scratch in one static device array per GPU, so it
must give what the allocating device-pointer entry point gives, call after
call, even though every call reuses the same array.  Collected last (file
name) so that a stop at the first failure has run every other test.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _lines(torch, seeds, rows):
    n = len(seeds)
    out = []
    for c in range(3):
        a = torch.zeros(n * rows, dtype=torch.float32, device="cuda")
        a[:n] = torch.from_numpy(np.ascontiguousarray(seeds[:, c]))
        out.append(a)
    return out


def _allocating(em, torch, seeds, ch, rows):
    """The existing device-pointer entry point (em_calc_field_ex_f32)."""
    X = _lines(torch, seeds, rows)
    dch = torch.from_numpy(np.ascontiguousarray(ch)).cuda()
    rc, _ = em.calc_field(*X, dch, len(seeds), 1.0, True, require_n64=False)
    torch.cuda.synchronize()
    assert rc == 0, em.strerror(rc)
    return np.stack([a.cpu().numpy() for a in X])


def _noalloc(lib, torch, seeds, ch, rows):
    X = _lines(torch, seeds, rows)
    dch = torch.from_numpy(np.ascontiguousarray(ch)).cuda()
    stream = torch.cuda.current_stream().cuda_stream
    rc = lib.em_calc_field_noalloc_f32(
        X[0].data_ptr(), X[1].data_ptr(), X[2].data_ptr(), len(seeds), rows,
        dch.data_ptr(), len(ch), ctypes.c_float(1.0), 1,
        ctypes.c_void_p(stream))
    torch.cuda.synchronize()
    return rc, np.stack([a.cpu().numpy() for a in X])


def test_noalloc_matches_allocating_entry_two_calls(em, gpu):
    """Both entry points plan the same launch (default options) and run the
    same kernel on the same staged records, so the vertices agree bit for
    bit; the shared array must be fully rewritten by each call (different
    counts and padding, back to back)."""
    torch = pytest.importorskip("torch")
    lib = gpu
    rows = 64
    ch_a, seeds_a, _ = em.workloads.make("cpu_256", seed=11)
    ch_b = em.workloads.uniform_charges(300, 50.0, seed=12)
    seeds_b = em.workloads.fibonacci_seeds(ch_b, 4)[:700].astype(np.float32)
    seeds_a = seeds_a.astype(np.float32)
    for ch, seeds in ((ch_a, seeds_a), (ch_b, seeds_b), (ch_a, seeds_a)):
        want = _allocating(em, torch, seeds, ch, rows)
        rc, got = _noalloc(lib, torch, seeds, ch, rows)
        assert rc == 0, em.strerror(rc)
        assert np.array_equal(got, want)


def test_noalloc_streamed_at_the_limit(em, gpu):
    """EM_NOALLOC_MAX_CHARGES charges do not fit shared memory: the kernel
    streams them in tiles from the static array, whose staged copy then uses
    its full padded size.  Two calls in a row, each equal to the allocating
    entry point bit for bit."""
    torch = pytest.importorskip("torch")
    lib = gpu
    limit = em._capi.EM_NOALLOC_MAX_CHARGES
    ch = em.workloads.uniform_charges(limit, 100.0, seed=21)
    seeds = em.workloads.fibonacci_seeds(ch, 1)[:384].astype(np.float32)
    rows = 24
    want = _allocating(em, torch, seeds, ch, rows)
    for _ in range(2):
        rc, got = _noalloc(lib, torch, seeds, ch, rows)
        assert rc == 0, em.strerror(rc)
        assert np.array_equal(got, want)


def test_noalloc_rejects_too_many_charges(em, gpu):
    torch = pytest.importorskip("torch")
    lib = gpu
    limit = em._capi.EM_NOALLOC_MAX_CHARGES
    ch = em.workloads.uniform_charges(limit + 1, 50.0, seed=5)
    seeds = np.zeros((64, 3), np.float32)
    rc, _ = _noalloc(lib, torch, seeds, ch, 4)
    assert rc == em._capi.EM_ERR_TOO_LARGE
