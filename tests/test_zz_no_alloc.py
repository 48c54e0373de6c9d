"""The entry point that allocates nothing (gbsort_sort_device_noalloc).

Some callers of this library cannot call cudaMalloc: code running inside a
framework whose caching allocator owns the device memory budget, code on a
latency-critical path where an allocation would synchronise the device, or
code that must not run out of memory half-way through.  This entry point
takes its scratch space from one fixed array inside the library instead.

Its output must be the oracle's stable order, and equal to the allocating
entry point's, call after call: the array keeps the previous call's data,
so every comparison runs right after another call.  Once the first call on
the device has set the array up, a call must leave the device's free
memory unchanged.  Collected last on purpose (file name), so a run that
stops at the first failure has run every other test before this one.
"""
import ctypes

import numpy
import pytest

import oracle as O

pytestmark = pytest.mark.gpu

MAX_BYTES = 8 << 20
BAD_ARG = 1


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


def _records(dtype, key, n, seed, dist):
    rng = numpy.random.default_rng(seed)
    a = numpy.zeros(n, dtype=dtype)
    info = numpy.iinfo(a[key].dtype)
    if dist == "dups":
        a[key] = rng.integers(0, 100, n).astype(a[key].dtype)
    else:
        a[key] = rng.integers(info.min, info.max, n, dtype=a[key].dtype, endpoint=True)
    other = [f for f in a.dtype.names if f != key][0]
    if a[other].ndim == 1:
        a[other] = numpy.arange(n).astype(a[other].dtype)
    return a


def _noalloc(env, a, key):
    """Sort a with the no-allocation entry point; returns the output."""
    L, mpsort, torch = env
    desc = mpsort._lib.key_desc(a.dtype, key)
    din = torch.from_numpy(a.view(numpy.uint8).copy()).cuda()
    got = torch.full_like(din, 0x5a)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.gbsort_sort_device_noalloc(din.data_ptr(), got.data_ptr(), len(a), a.dtype.itemsize,
                                      ctypes.byref(desc), stream)
    assert rc == 0, mpsort._lib.lib().gbsort_last_error()
    torch.cuda.synchronize()
    return got.cpu().numpy().view(a.dtype)


def _allocating(env, a, key):
    L, mpsort, torch = env
    desc = mpsort._lib.key_desc(a.dtype, key)
    din = torch.from_numpy(a.view(numpy.uint8).copy()).cuda()
    ref = torch.empty_like(din)
    stream = torch.cuda.current_stream().cuda_stream
    rc = L.gbsort_sort_device(din.data_ptr(), ref.data_ptr(), len(a), a.dtype.itemsize, ctypes.byref(desc), 1,
                              stream)
    assert rc == 0
    torch.cuda.synchronize()
    return ref.cpu().numpy().view(a.dtype)


def test_noalloc_matches_oracle_and_allocating_entry_point_twice(env):
    # two calls in a row, different data and sizes, the second smaller
    dt = [('key', 'i8'), ('val', 'i8')]
    for n, seed, dist in ((MAX_BYTES // 16, 1, "uniform"), (300_001, 2, "dups")):
        a = _records(dt, 'key', n, seed, dist)
        got = _noalloc(env, a, 'key')
        assert got.tobytes() == O.numpy_sorted(a, 'key').tobytes(), (n, seed)
        assert got.tobytes() == _allocating(env, a, 'key').tobytes(), (n, seed)


LAYOUTS = [  # record sizes with their own alignment paths, at the byte limit
    ([('key', 'i4'), ('payload', 'u4')], 'key'),       # 8 B: 2^20 records, 512 buckets
    ([('key', 'u8'), ('value', 'f4')], 'key'),         # 12 B
    ([('key', 'u4'), ('pad', 'u4'), ('v', 'u8')], 'key'),  # 16 B, unsigned 4-byte key
    ([('k', 'u8'), ('pad', ('u8', 7))], 'k'),          # 64 B
]


@pytest.mark.parametrize("layout", range(len(LAYOUTS)))
def test_noalloc_layouts_at_the_limit(env, layout):
    dtype, key = LAYOUTS[layout]
    n = MAX_BYTES // numpy.dtype(dtype).itemsize
    for dist in ("uniform", "dups"):
        a = _records(dtype, key, n, 10 + layout, dist)
        assert _noalloc(env, a, key).tobytes() == O.numpy_sorted(a, key).tobytes(), (layout, dist)


@pytest.mark.parametrize("n", [1, 2, 4096, 4097])
def test_noalloc_small_and_single_bucket(env, n):
    # 4096 records or fewer take one bucket (no splitters at all)
    a = _records([('key', 'u8'), ('val', 'i8')], 'key', n, n, "uniform")
    assert _noalloc(env, a, 'key').tobytes() == O.numpy_sorted(a, 'key').tobytes()


def test_noalloc_call_leaves_free_memory_unchanged(env):
    L, mpsort, torch = env
    a = _records([('key', 'u8'), ('val', 'i8')], 'key', MAX_BYTES // 16, 7, "uniform")
    desc = mpsort._lib.key_desc(a.dtype, 'key')
    din = torch.from_numpy(a.view(numpy.uint8).copy()).cuda()
    out = torch.empty_like(din)
    stream = torch.cuda.current_stream().cuda_stream
    args = (din.data_ptr(), out.data_ptr(), len(a), 16, ctypes.byref(desc), stream)
    assert L.gbsort_sort_device_noalloc(*args) == 0  # set-up on this device (if not done yet)
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info()[0]
    for _ in range(2):
        assert L.gbsort_sort_device_noalloc(*args) == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info()[0] == free0
    assert out.cpu().numpy().view(a.dtype).tobytes() == O.numpy_sorted(a, 'key').tobytes()


def test_noalloc_rejects_oversize(env):
    L, mpsort, torch = env
    dt = numpy.dtype([('key', 'i8'), ('val', 'i8')])
    desc = mpsort._lib.key_desc(dt, 'key')
    n = MAX_BYTES // 16 + 1
    buf = torch.empty(16, dtype=torch.uint8, device='cuda')  # never touched
    rc = L.gbsort_sort_device_noalloc(buf.data_ptr(), buf.data_ptr(), n, 16, ctypes.byref(desc), None)
    assert rc == BAD_ARG
