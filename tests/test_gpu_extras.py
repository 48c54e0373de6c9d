"""GPU tests of the self-check, the device gather, the one-process MPI entry
points and sorts of 2^32 records or more."""
import ctypes

import numpy
import pytest

import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mp():
    import __graft_entry__ as g
    g.build()
    import mpsort
    if mpsort._lib.lib().gbsort_device_count() < 1:
        pytest.fail("no CUDA device visible to libgbsort")
    return mpsort


def _records(n, seed, dtype=(('key', 'u8'), ('val', 'i8'))):
    rng = numpy.random.default_rng(seed)
    a = numpy.zeros(n, dtype=list(dtype))
    a['key'] = rng.integers(0, 1 << 20, n).astype(a['key'].dtype)
    a['val'] = numpy.arange(n).astype(a['val'].dtype)
    return a


def test_multiset_hash_and_self_checked_sort(mp):
    import torch
    from mpsort import device as dev
    a = _records(300_001, 1)
    d = torch.from_numpy(a.view(numpy.uint8).copy()).cuda()
    out = torch.empty_like(d)
    h = torch.zeros(3, dtype=torch.int64, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    dev.multiset_hash(d.data_ptr(), len(a), a.dtype, h.data_ptr(), sp)
    for method in ("plain", "learned", "lsd"):
        dev.sort(d.data_ptr(), out.data_ptr(), len(a), a.dtype, 'key', method, sp, verify=True)
        assert out.cpu().numpy().view(a.dtype).tobytes() == O.numpy_sorted(a, 'key').tobytes()
    dev.multiset_hash(out.data_ptr(), len(a), a.dtype, h.data_ptr() + 8, sp)
    torch.cuda.synchronize()
    assert h[0].item() == h[1].item()  # a permutation hashes equally
    # one byte of one record changed between the two hashes: the hashes differ
    out[16 * 1234 + 9] ^= 1
    dev.multiset_hash(out.data_ptr(), len(a), a.dtype, h.data_ptr() + 16, sp)
    torch.cuda.synchronize()
    assert h[2].item() != h[0].item()
    # two records swapped: still the same multiset
    o = out.view(-1, 16)
    o[[5, 7]] = o[[7, 5]].clone()
    o[16 * 1234 // 16].view(torch.uint8)[9] ^= 1
    dev.multiset_hash(out.data_ptr(), len(a), a.dtype, h.data_ptr() + 16, sp)
    torch.cuda.synchronize()
    assert h[2].item() == h[0].item()


def test_host_sort_verify_flag(mp):
    a = _records(100_000, 2, (('key', 'i4'), ('val', 'u4')))
    out = numpy.empty_like(a)
    mp.sort(a, 'key', out=out, verify=True)
    assert out.tobytes() == O.numpy_sorted(a, 'key').tobytes()


@pytest.mark.parametrize("dtype", [(('key', 'u8'), ('val', 'i8')), (('k', 'i4'), ('a', 'u1'), ('b', 'u1')),
                                   (('x', 'f4', (3,)), ('key', 'i8'))])
def test_device_take_and_permute(mp, dtype):
    import torch
    from mpsort import device as dev
    rng = numpy.random.default_rng(3)
    n = 70_001
    src = numpy.zeros(n, dtype=list(dtype))
    src.view(numpy.uint8)[...] = rng.integers(0, 256, n * src.dtype.itemsize).astype(numpy.uint8)
    idx = rng.integers(0, n, 90_000)
    d_src = torch.from_numpy(src.view(numpy.uint8).copy()).cuda()
    d_idx = torch.from_numpy(idx).cuda()
    d_out = torch.empty(len(idx) * src.dtype.itemsize, dtype=torch.uint8, device="cuda")
    dev.take(d_src.data_ptr(), n, d_idx.data_ptr(), len(idx), src.dtype, d_out.data_ptr())
    assert d_out.cpu().numpy().view(src.dtype).tobytes() == src[idx].tobytes()
    perm = rng.permutation(n)
    assert mp.permute(src, perm, None).tobytes() == src[perm].tobytes()
    assert mp.take(src, idx, None).tobytes() == src[idx].tobytes()
    bad = idx.copy()
    bad[777] = n
    with pytest.raises(mp.GBSortError):
        mp.take(src, bad, None)
    with pytest.raises(ValueError):
        mp.permute(src, perm[:-1], None)


def test_mpi_entry_points_one_process(mp):
    L = mp._lib.lib()
    a = _records(50_003, 4)
    d = mp._lib.key_desc(a.dtype, 'key')
    radix = ctypes.cast(L.mpsort_radix_desc, ctypes.c_void_p)
    base = a.copy()
    out = numpy.zeros_like(a)
    L.mpsort_mpi_newarray_impl(base.ctypes.data, len(a), out.ctypes.data, len(a), 16, radix, 8,
                               ctypes.byref(d), 0, 1, b"test")
    assert L.mpsort_last_status() == 0
    exp = O.numpy_sorted(a, 'key')
    assert out.tobytes() == exp.tobytes() and base.tobytes() == exp.tobytes()
    inplace = a.copy()
    L.mpsort_mpi_impl(inplace.ctypes.data, len(a), 16, radix, 8, ctypes.byref(d), 0, 2, b"test")
    assert L.mpsort_last_status() == 0 and inplace.tobytes() == exp.tobytes()
    L.mpsort_mpi_newarray_impl(a.copy().ctypes.data, len(a), out.ctypes.data, len(a) - 1, 16, radix, 8,
                               ctypes.byref(d), 0, 3, b"test")
    assert L.mpsort_last_status() == mp._lib.ERR_BAD_ARG


def test_sort_of_more_than_2_to_the_32_records(mp):
    """2^32 + 4099 records of 12 bytes (u4 key, u8 input index): the first
    stable partition into key ranges, then the 32-bit pipeline per range.
    Checked on the device: keys ascend, equal keys keep ascending input
    index, and the multiset hash of the output equals the input's."""
    import torch
    from mpsort import device as dev
    L = mp._lib.lib()
    L.gbsort_release()
    torch.cuda.empty_cache()
    free = torch.cuda.mem_get_info()[0]
    n = (1 << 32) + 4099
    need = n * 12 * 3 + 2 * (n // 3 + (1 << 24)) * 12 + (4 << 30)
    if free < need:
        pytest.skip("needs %.0f GB of free device memory, %.0f GB free" % (need / 1e9, free / 1e9))
    dt = numpy.dtype([('key', 'u4'), ('val', 'u8')], align=False)
    rec = torch.empty((n, 3), dtype=torch.int32, device="cuda")
    g = torch.Generator(device="cuda")
    g.manual_seed(11)
    step = 1 << 28
    for s in range(0, n, step):
        e = min(n, s + step)
        rec[s:e, 0] = torch.randint(-2**31, 2**31 - 1, (e - s,), dtype=torch.int64, device="cuda", generator=g).to(torch.int32)
        rec[s:e, 0] >>= 20  # 4096 distinct keys: long runs of equal keys
        ix = torch.arange(s, e, dtype=torch.int64, device="cuda")
        rec[s:e, 1] = (ix & 0xFFFFFFFF).to(torch.int32)
        rec[s:e, 2] = (ix >> 32).to(torch.int32)
        del ix
    out = torch.empty_like(rec)
    h = torch.zeros(2, dtype=torch.int64, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    dev.multiset_hash(rec.data_ptr(), n, dt, h.data_ptr(), sp)
    dev.sort(rec.data_ptr(), out.data_ptr(), n, dt, 'key', 'auto', sp)
    dev.multiset_hash(out.data_ptr(), n, dt, h.data_ptr() + 8, sp)
    torch.cuda.synchronize()
    assert h[0].item() == h[1].item()
    del rec
    ok_sorted = ok_stable = True
    for s in range(0, n, step):
        e = min(n, s + step + 1)
        k = out[s:e, 0].to(torch.int64) & 0xFFFFFFFF  # u4 keys
        v = (out[s:e, 2].to(torch.int64) << 32) | (out[s:e, 1].to(torch.int64) & 0xFFFFFFFF)
        ok_sorted &= bool((k[1:] >= k[:-1]).all().item())
        ok_stable &= bool(((k[1:] != k[:-1]) | (v[1:] > v[:-1])).all().item())
    assert ok_sorted and ok_stable
    del out
    L.gbsort_release()
    torch.cuda.empty_cache()
