"""The entry point that allocates nothing (gbsort_sort_device_noalloc).

Some callers cannot call cudaMalloc -- a framework's caching allocator owns
the device memory, or an allocation on their path would stall it -- so this
entry point takes its scratch space from a fixed array inside the library.
Its output must equal the allocating entry point's, call after call: the
array keeps the previous call's data, so the second call checks that
nothing stale leaks into the result.  Collected last on purpose.
"""
import ctypes

import numpy
import pytest

pytestmark = pytest.mark.gpu

MAX_BYTES = 8 << 20


@pytest.fixture(scope="module")
def env():
    import __graft_entry__ as g
    g.build()
    import torch
    import mpsort
    L = mpsort._lib.lib()
    if L.gbsort_device_count() < 1:
        pytest.fail("no CUDA device visible to libgbsort")
    return L, mpsort, torch


def _records(n, seed, dups):
    rng = numpy.random.default_rng(seed)
    a = numpy.zeros(n, dtype=[('key', 'i8'), ('val', 'i8')])
    a['key'] = rng.integers(-50, 50, n) if dups else rng.integers(-2**63, 2**63 - 1, n, dtype=numpy.int64)
    a['val'] = numpy.arange(n)
    return a


def _sort_both(env, a):
    L, mpsort, torch = env
    dt = a.dtype
    desc = mpsort._lib.key_desc(dt, 'key')
    din = torch.from_numpy(a.view(numpy.uint8).copy()).cuda()
    ref = torch.empty_like(din)
    got = torch.full_like(din, 0x5a)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.gbsort_sort_device(din.data_ptr(), ref.data_ptr(), len(a), dt.itemsize, ctypes.byref(desc), 1, stream)
    assert rc == 0
    torch.cuda.synchronize()
    rc = L.gbsort_sort_device_noalloc(din.data_ptr(), got.data_ptr(), len(a), dt.itemsize, ctypes.byref(desc),
                                      stream)
    assert rc == 0
    torch.cuda.synchronize()
    return ref.cpu().numpy(), got.cpu().numpy()


def test_noalloc_matches_allocating_entry_point_twice(env):
    # two calls in a row, different data and sizes, the second smaller
    for n, seed, dups in ((MAX_BYTES // 16, 1, False), (300_001, 2, True)):
        ref, got = _sort_both(env, _records(n, seed, dups))
        assert got.tobytes() == ref.tobytes(), (n, seed)


def test_noalloc_rejects_oversize(env):
    L, mpsort, torch = env
    dt = numpy.dtype([('key', 'i8'), ('val', 'i8')])
    desc = mpsort._lib.key_desc(dt, 'key')
    n = MAX_BYTES // 16 + 1
    buf = torch.empty(16, dtype=torch.uint8, device='cuda')  # never touched
    rc = L.gbsort_sort_device_noalloc(buf.data_ptr(), buf.data_ptr(), n, 16, ctypes.byref(desc), None)
    assert rc == 1  # GBSORT_ERR_BAD_ARG
