"""GPU parity at the benchmark configurations' own sizes and distributions.

  * configuration 1 at its full size (1e6 x 12 B, PCG64 seed 0) and the
    sorted-with-1%-swapped and Zipf(1.2) workloads of configuration 2 at
    2e7 records: the output's SHA-256 must equal that of the unmodified
    reference mpsort_omp's output on the same input
    (tests/golden/digests.json, written by tests/golden/make_golden.py from
    the reference build);
  * configuration 2b / 2c at 5e7 records and configuration 4 at 2e7: equal
    to the oracle's stable sort, record for record;
  * configurations 3 (all 4096 segments) and 5 (both snapshots) at full
    size: size-independent properties on the device, plus a per-segment
    comparison with the oracle for a spread of segments.
"""
import hashlib
import json
import os

import numpy
import pytest

import oracle as O
import workloads as W

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
with open(os.path.join(HERE, "golden", "digests.json")) as _f:
    DIGESTS = json.load(_f)


@pytest.fixture(scope="module")
def mp():
    import __graft_entry__ as g
    g.build()
    import mpsort
    if mpsort._lib.lib().gbsort_device_count() < 1:
        pytest.fail("no CUDA device visible to libgbsort")
    return mpsort


def sha(a):
    return hashlib.sha256(numpy.ascontiguousarray(a).tobytes()).hexdigest()


def _digest_input(name):
    d = DIGESTS[name]
    arr = W.records_1(None) if name == "cfg1_full" else W.records_2_host(d["n"], name[3:5])
    assert sha(arr) == d["sha256_in"], "the seeded generator no longer reproduces %s" % name
    return arr, d


@pytest.mark.parametrize("method", ["auto", "plain", "learned", "lsd"])
def test_config1_full_size_equals_reference(mp, method):
    arr, d = _digest_input("cfg1_full")
    out = numpy.empty_like(arr)
    mp.sort(arr, 'key', out=out, method=method)
    assert sha(out) == d["sha256_out"], method


@pytest.mark.parametrize("method", ["auto", "plain", "learned"])
@pytest.mark.parametrize("name", ["cfg2b_2e7", "cfg2c_2e7"])
def test_config2_workloads_equal_reference(mp, name, method):
    arr, d = _digest_input(name)
    out = numpy.empty_like(arr)
    mp.sort(arr, 'key', out=out, method=method)
    assert sha(out) == d["sha256_out"], (name, method)


@pytest.fixture(scope="module")
def torch_dev():
    import torch
    return torch


def _device_sort(mp, torch, arr, orderby, method):
    from mpsort import device as dev
    din = torch.from_numpy(arr.view(numpy.uint8)).cuda()
    dout = torch.empty_like(din)
    dev.sort(din.data_ptr(), dout.data_ptr(), len(arr), arr.dtype, orderby, method,
             torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    return dout.cpu().numpy().view(arr.dtype), mp.last_stats()


@pytest.mark.parametrize("dist", ["2b", "2c"])
def test_config2_5e7_equals_stable_sort(mp, torch_dev, dist):
    arr = W.records_2_host(5 * 10**7, dist, seed=7)
    exp = O.numpy_sorted(arr, 'key')
    for method in ("plain", "learned"):
        got, st = _device_sort(mp, torch_dev, arr, 'key', method)
        assert got.tobytes() == exp.tobytes(), (dist, method)
        assert st["method"] in ("plain", "learned")
        if dist == "2c":
            assert st["heavy_keys"] > 0  # the Zipf head owns single-key buckets


def test_config4_particles_2e7_equals_stable_sort(mp, torch_dev):
    torch = torch_dev
    n = 2 * 10**7
    buf, dt = W.particles_4(torch, n)
    arr = buf.cpu().numpy().view(dt)
    exp = O.numpy_sorted(arr, 'key')
    for method in ("plain", "learned"):
        got, st = _device_sort(mp, torch, arr, 'key', method)
        assert got.tobytes() == exp.tobytes(), method
        assert st["splits"] > 0


def test_config3_all_segments(mp, torch_dev):
    """All 4096 log-normal segments (about 6.1e8 records of 8 B) in one
    call: every segment sorted stably in place of its range."""
    torch = torch_dev
    from mpsort import device as dev
    buf, dt, offs = W.segments_3(torch)
    n = int(offs[-1])
    out = torch.empty_like(buf)
    dev.sort_segments(buf.data_ptr(), out.data_ptr(), offs, dt, 'key', 'auto',
                      torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    start = torch.zeros(n, dtype=torch.bool, device="cuda")
    start[torch.from_numpy(offs[:-1].astype(numpy.int64)).cuda().clamp_(max=n - 1)] = True
    par = W.device_parity(torch, buf.view(torch.int32).view(-1, 2), out.view(torch.int32).view(-1, 2), n,
                          key_col=0, ident_col=1, segment_start=start, signed=True)
    assert all(par.values()), par
    # a spread of segments against the oracle: the largest, the smallest, and some between
    sizes = numpy.diff(offs.astype(numpy.int64))
    order = numpy.argsort(sizes, kind='stable')
    pick = set(order[:8]) | set(order[-3:]) | set(order[::256])
    for i in sorted(pick):
        a, b = int(offs[i]), int(offs[i + 1])
        if b == a:
            continue
        seg_in = buf[a * 8:b * 8].cpu().numpy().view(dt)
        seg_out = out[a * 8:b * 8].cpu().numpy().view(dt)
        assert seg_out.tobytes() == O.numpy_sorted(seg_in, 'key').tobytes(), (i, b - a)


def test_config5_full_join(mp, torch_dev):
    """Both 2.56e8-record snapshots sorted by id as one two-segment batch,
    then joined on the device: the expected number of pairs, each pair of
    equal ids, and every common id found."""
    torch = torch_dev
    from mpsort import device as dev
    buf, dt, na, nb, common = W.snapshots_5(torch)
    out = torch.empty_like(buf)
    offs = numpy.array([0, na, na + nb], dtype=numpy.uint64)
    pa = torch.empty(min(na, nb), dtype=torch.int64, device="cuda")
    pb = torch.empty_like(pa)
    npairs = torch.zeros(1, dtype=torch.int64, device="cuda")
    sp = torch.cuda.current_stream().cuda_stream
    dev.sort_segments(buf.data_ptr(), out.data_ptr(), offs, dt, 'id', 'auto', sp)
    dev.merge_join(out.data_ptr(), na, out.data_ptr() + na * 16, nb, dt, 'id', pa.data_ptr(), pb.data_ptr(),
                   npairs.data_ptr(), sp)
    torch.cuda.synchronize()
    k = int(npairs.item())
    assert k == common
    ids = out.view(torch.int64).view(-1, 2)[:, 0]
    ida, idb = ids[:na], ids[na:]
    assert bool((ida[1:] > ida[:-1]).all().item()) and bool((idb[1:] > idb[:-1]).all().item())
    assert bool((ida[pa[:k]] == idb[pb[:k]]).all().item())
    assert bool((pa[1:k] > pa[:k - 1]).all().item())
    # every record of each snapshot is still there: the sorted ids equal the
    # input ids sorted by torch
    inp = buf.view(torch.int64).view(-1, 2)[:, 0]
    assert torch.equal(torch.sort(inp[:na])[0], ida) and torch.equal(torch.sort(inp[na:])[0], idb)
