"""GPU parity: the CUDA sort against the oracle and the reference's vectors.

Every comparison is bit-exact on whole records: the reference's output is
the stable order by radix (stdlib/msort.c keeps ties in input order), so
the expected result is unique.
"""
import ctypes
import os

import numpy
import pytest

import oracle as O
from conftest import golden_cases

pytestmark = pytest.mark.gpu
REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

METHODS = ["plain", "learned", "lsd"]


@pytest.fixture(scope="module")
def mp():
    import __graft_entry__ as g
    g.build()
    import mpsort
    if mpsort._lib.lib().gbsort_device_count() < 1:
        pytest.fail("no CUDA device visible to libgbsort")
    return mpsort


def check(mp, arr, orderby, method):
    out = numpy.empty_like(arr)
    mp.sort(arr, orderby, out=out, method=method)
    exp = O.numpy_sorted(arr, orderby)
    assert out.tobytes() == exp.tobytes(), (arr.dtype, len(arr), method)
    return out


# ------------------------------------------------------------- golden --
@pytest.mark.parametrize("method", ["auto"] + METHODS)
def test_golden_vectors(mp, golden, method):
    for name, arr, out, orderby in golden_cases(golden):
        res = numpy.empty_like(arr)
        try:
            mp.sort(arr, orderby, out=res, method=method)
        except mp.GBSortError as e:
            assert e.status == 6 and method in ("plain", "learned"), (name, e)  # unsupported layout
            continue
        assert res.tobytes() == out.tobytes(), (name, method)


def test_golden_callbacks_through_dropin_symbols(mp, golden):
    """radix_sort / mpsort_omp with the reference tests' own radix() callbacks."""
    L = mp._lib.lib()
    olib = O.oracle_lib()
    for fn, sym in ((L.radix_sort, "radix_sort"), (L.mpsort_omp, "mpsort_omp")):
        ints = golden["cb_int__in"].copy()
        fn(ints.ctypes.data, len(ints), 4, ctypes.cast(olib.ref_radix_int, ctypes.c_void_p), 4, None)
        assert L.mpsort_last_status() == 0, sym
        assert ints.tobytes() == golden["cb_int__out"].tobytes(), sym
        recs = golden["cb_issue7__in"].copy()
        fn(recs.ctypes.data, len(recs), 40, ctypes.cast(olib.ref_radix_issue7, ctypes.c_void_p), 16, None)
        assert recs.tobytes() == golden["cb_issue7__out"].tobytes(), sym


def test_dropin_with_key_descriptor(mp, golden):
    L = mp._lib.lib()
    arr = golden["cfg1_4096__in"].copy()
    d = mp._lib.key_desc(arr.dtype, 'key')
    L.mpsort_omp(arr.ctypes.data, len(arr), arr.dtype.itemsize,
                 ctypes.cast(L.mpsort_radix_desc, ctypes.c_void_p), 8, ctypes.byref(d))
    assert L.mpsort_last_status() == 0
    assert arr.tobytes() == golden["cfg1_4096__out"].tobytes()


def test_reference_build_live(mp):
    """Against the unmodified reference mpsort_omp where it was built."""
    if O.ref_lib() is None:
        pytest.skip("reference build absent")
    rng = numpy.random.default_rng(0)
    a = numpy.empty(300_000, dtype=[('key', 'u8'), ('value', 'f4')])
    a['key'] = rng.integers(0, 2**64, len(a), dtype=numpy.uint64, endpoint=False)
    a['value'] = numpy.arange(len(a), dtype=numpy.float32)
    exp = O.ref_sort(a, 'key', 'omp')
    for m in METHODS:
        out = numpy.empty_like(a)
        mp.sort(a, 'key', out=out, method=m)
        assert out.tobytes() == exp.tobytes(), m


# --------------------------------------------------- edges and layouts --
SIZES = [1, 2, 3, 31, 32, 33, 511, 4095, 4096, 4097, 8193, 65537, 300_001]


def make(dtype, key, n, dist, rng):
    a = numpy.zeros(n, dtype=dtype)
    kd = a[key].dtype
    info = numpy.iinfo(kd)
    if dist == "uniform":
        k = rng.integers(info.min, info.max, n, dtype=kd, endpoint=True)
    elif dist == "dups":
        k = rng.integers(-3, 4, n).astype(kd) if info.min < 0 else rng.integers(0, 7, n).astype(kd)
    elif dist == "equal":
        k = numpy.full(n, 5, dtype=kd)
    elif dist == "sorted":
        k = numpy.arange(n).astype(kd)
    elif dist == "reversed":
        k = numpy.arange(n)[::-1].astype(kd)
    elif dist == "zipf":
        vals = rng.integers(info.min, info.max, 1000, dtype=kd, endpoint=True)
        k = vals[numpy.minimum(rng.zipf(1.2, n) - 1, 999)]
    elif dist == "extremes":
        k = rng.choice(numpy.array([info.min, info.max, 0, 1, info.max - 1], dtype=kd), n)
    a[key] = k
    for f in a.dtype.names:
        if f != key and a[f].dtype.kind in "iu" and a[f].ndim == 1:
            a[f] = (numpy.arange(n, dtype=numpy.uint64) % numpy.uint64(1 << 31)).astype(a[f].dtype)
    return a


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("n", SIZES)
def test_sizes_u8_16B(mp, n, method):
    rng = numpy.random.default_rng(n)
    for dist in ("uniform", "dups", "sorted", "reversed"):
        check(mp, make([('key', 'u8'), ('val', 'i8')], 'key', n, dist, rng), 'key', method)


LAYOUTS = [
    ([('key', 'i4'), ('payload', 'u4')], 'key'),                    # 8 B, signed 32-bit
    ([('key', 'u8'), ('value', 'f4')], 'key'),                      # 12 B packed
    ([('id', 'i8'), ('mass', 'f4'), ('halo', 'i4')], 'id'),         # 16 B, signed 64-bit
    ([('a', 'u4'), ('key', 'u4'), ('b', 'u8'), ('c', 'u8')], 'key'),  # 24 B, key at offset 4
    ([('pos', ('f4', 3)), ('vel', ('f4', 3)), ('id', 'u8'), ('key', 'u8')], 'key'),  # 40 B
    ([('k', 'i8'), ('pad', ('u8', 7))], 'k'),                       # 64 B
    ([('key', 'u8'), ('x', 'u4'), ('y', 'u4'), ('z', 'u4'), ('w', 'u4')], 'key'),  # 24 B
]


@pytest.mark.parametrize("method", METHODS)
@pytest.mark.parametrize("layout", range(len(LAYOUTS)))
def test_layouts_and_distributions(mp, layout, method):
    dtype, key = LAYOUTS[layout]
    rng = numpy.random.default_rng(layout)
    for n in (5000, 200_003):
        for dist in ("uniform", "dups", "equal", "zipf", "extremes", "sorted"):
            check(mp, make(dtype, key, n, dist, rng), key, method)


@pytest.mark.parametrize("n", [17, 5000, 70_001])
def test_generic_path_layouts(mp, n):
    """Records the histogram sort does not take: odd sizes, unaligned keys,
    multi-word keys.  AUTO routes them to the LSD path."""
    rng = numpy.random.default_rng(n)
    cases = [
        (numpy.dtype([('c', 'u1'), ('key', 'i4')]), 'key'),         # 5 B, key at offset 1
        (numpy.dtype([('key', 'u8'), ('c', 'u1')]), 'key'),         # 9 B
        (numpy.dtype([('v', ('u8', 3)), ('w', 'u4')]), 'v'),        # 3-word key
        (numpy.dtype([('v', ('i4', 2)), ('w', 'u1')]), 'v'),        # 2 x i4, 9 B
        (numpy.dtype([('v', ('i8', 4))]), 'v'),                     # 4-word key
    ]
    for dt, key in cases:
        a = numpy.zeros(n, dt)
        f = a[key]
        info = numpy.iinfo(f.dtype)
        a[key] = rng.integers(max(info.min, -20), min(info.max, 20), f.shape)
        check(mp, a, key, "auto")


def test_lsd_record_passes(mp, tmp_path):
    """The LSD passes that carry records of 8-32 bytes (GBSORT_LSD_RECORDS=1,
    read at load time, so in a child process) give the same bytes as the
    default key + index passes and gather, which this process runs.  The
    child also sorts one case in place on the device in one pass (only one
    digit varies, found by the constant-digit check at >= 2^22 records)."""
    import subprocess
    import sys
    rng = numpy.random.default_rng(21)
    cases = {
        "r16": make([('key', 'u8'), ('v', 'i8')], 'key', 300_001, "dups", rng),
        "r12": make([('key', 'i8'), ('v', 'u4')], 'key', 70_001, "uniform", rng),
        "r24": numpy.zeros(50_000, numpy.dtype([('k', ('u8', 2)), ('v', 'u8')])),
        "r32": numpy.zeros(40_000, numpy.dtype([('k', ('i8', 4))])),
    }
    cases["r24"]['k'] = rng.integers(0, 50, cases["r24"]['k'].shape, dtype=numpy.uint64)
    cases["r24"]['v'] = numpy.arange(50_000)
    cases["r32"]['k'] = rng.integers(-5, 5, cases["r32"]['k'].shape)
    keys = {"r16": 'key', "r12": 'key', "r24": 'k', "r32": 'k'}
    for name, a in cases.items():
        numpy.save(tmp_path / (name + "_in.npy"), a)
        out = check(mp, a, keys[name], "lsd")
        assert mp.last_stats()["lsd_passes"] == 8 * (a.dtype[keys[name]].itemsize // 8)
        numpy.save(tmp_path / (name + "_default.npy"), out)
    # one pass, in place on the device: keys below 256 in 8-byte records
    dt8 = numpy.dtype([('key', 'u8')])
    big = numpy.zeros((1 << 22) + 5, dt8)
    big['key'] = numpy.arange(len(big), dtype=numpy.uint64)[::-1] % 251
    numpy.save(tmp_path / "big_in.npy", big)
    numpy.save(tmp_path / "big_exp.npy", O.numpy_sorted(big, 'key'))
    script = (
        "import sys, numpy, torch\n"
        "sys.path[:0] = %r\n"
        "import mpsort\n"
        "from mpsort import device\n"
        "t = %r\n"
        "for name, key in %r.items():\n"
        "    a = numpy.load(t + '/' + name + '_in.npy')\n"
        "    out = numpy.empty_like(a)\n"
        "    mpsort.sort(a, key, out=out, method='lsd')\n"
        "    numpy.save(t + '/' + name + '_records.npy', out)\n"
        "big = numpy.load(t + '/big_in.npy')\n"
        "d = torch.from_numpy(big.view(numpy.uint8).copy()).cuda()\n"
        "device.sort(d.data_ptr(), d.data_ptr(), len(big), big.dtype, 'key', 'lsd')\n"
        "torch.cuda.synchronize()\n"
        "assert mpsort.last_stats()['lsd_passes'] == 1\n"
        "assert d.cpu().numpy().tobytes() == numpy.load(t + '/big_exp.npy').tobytes()\n"
        % ([os.path.join(REPO, "mp-sort_gb300"), os.path.join(REPO, "oracle")], str(tmp_path), keys))
    env = dict(os.environ, GBSORT_LSD_RECORDS="1")
    subprocess.run([sys.executable, "-c", script], env=env, check=True, timeout=600)
    for name in cases:
        assert numpy.load(tmp_path / (name + "_records.npy")).tobytes() == \
            numpy.load(tmp_path / (name + "_default.npy")).tobytes(), name


def test_in_place_and_aliasing(mp):
    rng = numpy.random.default_rng(9)
    for m in METHODS:
        a = make([('key', 'i8'), ('v', 'i8')], 'key', 100_000, "dups", rng)
        exp = O.numpy_sorted(a, 'key')
        mp.sort(a, 'key', method=m)
        assert a.tobytes() == exp.tobytes(), m


# ------------------------------------------- ports of test_mpsort.py --
def test_sort_i4_i8_u8_u4(mp):
    s = numpy.int32(numpy.random.random(size=1000) * 1000 - 400)
    r = s.copy()
    mp.sort(r, orderby=None, out=None)
    assert (r == numpy.sort(s)).all()
    s = numpy.int64(numpy.random.random(size=1000) * 1000 - 400)
    r = s.copy()
    mp.sort(r)
    assert (r == numpy.sort(s)).all()
    s = numpy.uint64(numpy.random.uniform(size=1000, low=-1000000, high=1000000) * 1000 - 400)
    r = s.copy()
    mp.sort(r)
    assert (r == numpy.sort(s)).all()
    s = numpy.uint32(numpy.random.random(size=1000) * 1000 - 400)
    r = s.copy()
    mp.sort(r)
    assert (r == numpy.sort(s)).all()


@pytest.mark.parametrize("tuning", [[], ['DISABLE_SPARSE_ALLTOALLV'], ['REQUIRE_SPARSE_ALLTOALLV'],
                                    ['REQUIRE_GATHER_SORT'], ['DISABLE_GATHER_SORT']])
def test_sort_tunings(mp, tuning):
    s = numpy.int32(numpy.random.random(size=1000) * 1000)
    r = s.copy()
    mp.sort(r, orderby=None, out=None, tuning=tuning)
    assert (r == numpy.sort(s)).all()


def test_sort_inplace_outplace_flatiter(mp):
    s = numpy.int32(numpy.random.random(size=1000) * 1000)
    local = s.copy()
    mp.sort(local, local, out=None)
    assert (local == numpy.sort(s)).all()
    local = s.copy()
    res = numpy.zeros(local.size, dtype=local.dtype)
    mp.sort(local, local, out=res)
    assert (res == numpy.sort(s)).all()
    local = s.copy()
    res = numpy.zeros(local.size, dtype=local.dtype)
    mp.sort(local.flat, local.flat, out=res.flat)
    assert (res == numpy.sort(s)).all()


def test_sort_struct_and_vectors(mp):
    s = numpy.empty(10, dtype=[('value', 'i8'), ('key', 'i8')])
    numpy.random.seed(1234)
    s['value'] = numpy.int32(numpy.random.random(size=10) * 1000 - 400)
    s['key'] = s['value']
    backup = s.copy()
    res = numpy.zeros_like(s)
    mp.sort(s, 'key', out=res)
    backup.sort(order='key')
    assert (backup['value'] == res['value']).all()

    s = numpy.empty(10, dtype=[('value', 'i8'), ('key', 'i8'), ('vkey', ('i8', 2))])
    s['value'] = numpy.int32(numpy.random.random(size=len(s)) * 1000)
    s['key'][:][...] = s['value']
    s['vkey'][:, 0][...] = s['value']
    s['vkey'][:, 1][...] = s['value']
    res = numpy.zeros_like(s)
    mp.sort(s, 'vkey', out=res)
    s.sort(order='key')
    assert (s['value'] == res['value']).all()

    s = numpy.empty(10, dtype=[('value', 'i8')])
    s['value'] = numpy.int32(numpy.random.random(size=len(s)) * 1000)
    k = numpy.empty(len(s), ('i8', 2))
    k[:, 0][...] = s['value']
    k[:, 1][...] = s['value']
    res = numpy.zeros_like(s)
    mp.sort(s, k, out=res)
    s.sort(order='value')
    assert (s['value'] == res['value']).all()


def test_permute_take(mp):
    s = numpy.arange(10)
    i = numpy.arange(9, -1, -1)
    assert (mp.permute(s, i, None) == s[i]).all()
    res = numpy.empty(10, s.dtype)
    mp.permute(s, i, None, out=res)
    assert (res == s[i]).all()
    assert (mp.take(s, i, None) == s[i]).all()
    res = numpy.empty(10, s.dtype)
    mp.take(s, i, None, out=res)
    assert (res == s[i]).all()
    rng = numpy.random.default_rng(4)
    src = rng.integers(0, 1 << 40, 50_000)
    idx = rng.integers(0, 50_000, 50_000)      # not a permutation, repeats
    assert (mp.take(src, idx, None) == src[idx]).all()
    perm = rng.permutation(50_000)
    assert (mp.permute(src, perm, None) == src[perm]).all()


def test_few_items_exhaustive(mp):
    from itertools import product
    for sizes in product(*([[0, 1, 2]] * 4)):
        A = [numpy.arange(sizes[i], dtype='u8') for i in range(4)]
        s = numpy.empty(sum(sizes), dtype=[('vkey', ('u8', 3)), ('vector', ('u4', 3))])
        s['vkey'] = numpy.concatenate(A)[:, None]
        s['vector'] = 1
        S = s.copy()
        S.sort()
        r = numpy.empty(len(s), dtype=s.dtype)
        mp.sort(s, 'vkey', out=r)
        assert (r['vkey'] == S['vkey']).all()


# ------------------------------------------ splitters and the model --
def test_device_bisection_matches_oracle(mp):
    from mpsort import device
    lib = O.oracle_lib()
    rng = numpy.random.default_rng(2)
    for s, nsplit, dist in ((10_000, 63, "u"), (50_000, 1023, "dup"), (4096, 4095, "u"), (777, 8, "dup")):
        if dist == "u":
            x = numpy.sort(rng.integers(0, 2**64, s, dtype=numpy.uint64, endpoint=False))
        else:
            x = numpy.sort(rng.integers(0, 50, s).astype(numpy.uint64) * numpy.uint64(1 << 40))
        S, clt, cle, rounds = device.debug_bisect(x, nsplit)
        P = numpy.zeros(nsplit, numpy.uint64)
        CLT = numpy.zeros(nsplit + 2, numpy.int64)
        CLE = numpy.zeros(nsplit + 2, numpy.int64)
        it = lib.oracle_bisect_splitters(x.ctypes.data, s, 8, nsplit, P.ctypes.data, CLT.ctypes.data,
                                         CLE.ctypes.data)
        assert (S == P).all()
        assert (clt == CLT[1:nsplit + 1]).all() and (cle == CLE[1:nsplit + 1]).all()
        assert rounds == it
        C = numpy.array([s * (i + 1) // (nsplit + 1) for i in range(nsplit)])
        assert ((clt < C) & (C <= cle)).all()


def test_cdf_forward_backward_matches_numpy(mp):
    """Gradient check of the hand-written forward/backward kernels."""
    from mpsort import device
    import cdf_oracle
    rng = numpy.random.default_rng(7)
    for lbits, gen in ((6, lambda: rng.integers(0, 2**64, 20000, dtype=numpy.uint64, endpoint=False)),
                       (8, lambda: rng.integers(10**6, 10**6 + 5000, 20000).astype(numpy.uint64)),
                       (4, lambda: (rng.normal(0, 1e9, 20000) + 2**62).astype(numpy.uint64))):
        x = numpy.sort(gen())
        y = numpy.sort(rng.random((1 << lbits) + 1)).astype(numpy.float32)
        y[0], y[-1] = 0, 1
        loss, pred, grad = device.cdf_forward_backward(x, x[0], x[-1], lbits, y)
        l2, p2, g2 = cdf_oracle.forward_backward(x, int(x[0]), int(x[-1]), lbits, y)
        assert abs(loss - l2) <= 1e-4 * max(1e-6, l2) + 1e-7
        numpy.testing.assert_allclose(pred, p2, rtol=1e-5, atol=1e-6)
        numpy.testing.assert_allclose(grad, g2, rtol=2e-3, atol=1e-7)
        # the gradient the training steps use: T y - b from the statistics pass
        gt = device.cdf_train_gradient(x, x[0], x[-1], lbits, y)
        numpy.testing.assert_allclose(gt, g2, rtol=2e-3, atol=2e-6)
        # finite-difference check of the numpy gradient itself
        j = len(y) // 2
        h = 1e-3
        yp = y.astype(numpy.float64).copy(); yp[j] += h
        ym = y.astype(numpy.float64).copy(); ym[j] -= h
        fd = (cdf_oracle.forward_backward(x, int(x[0]), int(x[-1]), lbits, yp)[0] -
              cdf_oracle.forward_backward(x, int(x[0]), int(x[-1]), lbits, ym)[0]) / (2 * h)
        assert abs(fd - g2[j]) <= 1e-3 * max(abs(fd), 1e-4) + 1e-6


@pytest.mark.parametrize("dist", ["uniform", "zipf", "clustered", "narrow"])
def test_learned_lookup_equals_search(mp, dist):
    from mpsort import device
    rng = numpy.random.default_rng(11)
    n = 400_000
    if dist == "uniform":
        keys = rng.integers(0, 2**64, n, dtype=numpy.uint64, endpoint=False)
    elif dist == "zipf":
        vals = rng.integers(0, 2**64, 10000, dtype=numpy.uint64, endpoint=False)
        keys = vals[numpy.minimum(rng.zipf(1.2, n) - 1, 9999)]
    elif dist == "clustered":
        c = rng.integers(0, 2**60, 50, dtype=numpy.uint64)
        keys = c[rng.integers(0, 50, n)] + rng.integers(0, 1 << 20, n).astype(numpy.uint64)
    else:
        keys = rng.integers(1000, 3000, n).astype(numpy.uint64)
    sample = keys[:: 8]
    for nb in (16, 1024, 8192):
        probe = numpy.concatenate([keys[:100_000], numpy.array([0, 2**64 - 1, 1], dtype=numpy.uint64)])
        bs, bl, S, widest = device.debug_buckets(sample, nb, probe)
        assert (bs == bl).all(), (dist, nb)
        assert (numpy.diff(S.astype(object)) >= 0).all()


@pytest.mark.parametrize("dist", ["lognormal", "mixture", "uniform"])
def test_trained_model_gain(mp, dist):
    """What the trained model gains over the full splitter search: the same
    bucket for every key while reading a fraction of the splitters (none at
    all where the splitters come from the model itself), and gradient steps
    that lower the fit's loss below the initial empirical-CDF knots."""
    from mpsort import device
    rng = numpy.random.default_rng(21)
    n = 1_000_000
    if dist == "lognormal":
        keys = (rng.lognormal(0.0, 2.0, n) * 1e9).astype(numpy.uint64)
    elif dist == "mixture":
        c = rng.uniform(0, 2**50, 300)
        sd = numpy.exp(rng.uniform(numpy.log(2**30), numpy.log(2**40), 300))
        i = rng.integers(0, 300, n)
        keys = numpy.abs(rng.normal(c[i], sd[i])).astype(numpy.uint64)
    else:
        keys = rng.integers(0, 2**64, n, dtype=numpy.uint64, endpoint=False)
    sample = keys[rng.integers(0, n, 262_144)]
    probe = keys[:200_000]
    res = {}
    for epochs in (0, 8):
        bs, bl, loss, rl, rp, widest = device.debug_model(sample, 2048, probe, epochs)
        assert (bs == bl).all(), (dist, epochs)
        res[epochs] = (loss, rl / len(probe), rp / len(probe), widest)
    (l0, r0, p0, w0), (l8, r8, p8, w8) = res[0], res[8]
    print(dist, "loss %.3g -> %.3g, splitter reads per key: full search %.2f, learned %.2f (untrained %.2f)"
          % (l0, l8, p8, r8, r0))
    assert p8 >= 10.0                      # 2047 splitters: ~11 reads per full search
    assert r8 <= 0.4 * p8                  # the model reads a fraction of them
    assert l8 < l0                         # the gradient steps improve on the initial fit


# --------------------------------------------- batched and join paths --
@pytest.mark.parametrize("big", [False, True])
def test_segments(mp, big):
    import torch
    from mpsort import device
    rng = numpy.random.default_rng(5)
    sizes = numpy.concatenate([[0, 1, 2, 4096, 4097, 70_000], rng.integers(0, 3000, 200)])
    if big:  # segments above 2^22 records take the whole-grid sort one by one
        sizes = numpy.concatenate([[5_000_000], sizes[:100], [(1 << 22) + 1, 1 << 22], sizes[100:]])
    offs = numpy.concatenate([[0], numpy.cumsum(sizes)]).astype(numpy.uint64)
    n = int(offs[-1])
    dt = numpy.dtype([('key', 'i4'), ('payload', 'u4')])
    a = numpy.zeros(n, dt)
    a['key'] = rng.integers(-2**31, 2**31 - 1, n)
    a['key'][::10] = -2**31 + rng.integers(0, 5, len(a['key'][::10]))
    a['payload'] = numpy.arange(n)
    din = torch.from_numpy(a.view(numpy.uint8).copy()).cuda()
    dout = torch.empty_like(din)
    device.sort_segments(din.data_ptr(), dout.data_ptr(), offs, dt, 'key')
    torch.cuda.synchronize()
    got = dout.cpu().numpy().view(dt)
    for i in range(len(sizes)):
        lo, hi = int(offs[i]), int(offs[i + 1])
        assert got[lo:hi].tobytes() == O.numpy_sorted(a[lo:hi], 'key').tobytes(), i


def test_segments_plan_and_tuning(mp, tmp_path):
    """A segmented plan (one graph launch per replay) against the oracle per
    segment, through the tuned entry the segment autotuner stores: replays
    on two output buffers (the second re-captures), the tuning entry's
    threshold and level-2 choice honoured, and the tuning file round trip."""
    import torch
    import mpsort
    from mpsort import device
    rng = numpy.random.default_rng(15)
    sizes = numpy.concatenate([[0, 1, 4096, 4097, 70_000, 1_500_000], rng.integers(0, 30_000, 300),
                               [2_100_000, 5000]])
    offs = numpy.concatenate([[0], numpy.cumsum(sizes)]).astype(numpy.uint64)
    n = int(offs[-1])
    dt = numpy.dtype([('key', 'u8'), ('payload', 'u8')])
    a = numpy.zeros(n, dt)
    a['key'] = rng.integers(0, 2**64 - 1, n, dtype=numpy.uint64)
    a['key'][::7] = rng.integers(0, 9, len(a['key'][::7]))
    a['payload'] = numpy.arange(n)
    din = torch.from_numpy(a.view(numpy.uint8).copy()).cuda()
    outs = [torch.empty_like(din), torch.empty_like(din)]
    device.tuning_clear()
    try:
        best = device.autotune_segments(offs, dt, 'key', din.data_ptr())
        assert best["level2"] in ("rounds", "engine") and best["big_above"] >= 1 << 20 and best["ms"] > 0
        assert device.tuning_get_segments(n, dt, 'key') == best
        # a hand-set entry: segments above 10^6 records sorted on their own, level 2 as rounds
        path = tmp_path / "tune.txt"
        device.tuning_save(path)
        text = path.read_text().splitlines()
        seg = [l for l in text if not l.startswith('#') and int(l.split()[2]) >= 128]
        assert len(seg) == 1 and int(seg[0].split()[8]) == best["big_above"]
        f = seg[0].split()
        f[7], f[8] = "1", "1000000"
        path.write_text("\n".join(text + [" ".join(f)]) + "\n")
        device.tuning_clear()
        device.tuning_load(path)
        assert device.tuning_get_segments(n, dt, 'key')["big_above"] == 1_000_000
        plan = device.Plan(0, dt, 'key', segments=offs)
        for rep in range(3):
            out = outs[rep % 2]
            out.zero_()
            plan.sort(din.data_ptr(), out.data_ptr())
            plan.wait()
            st = mpsort.last_stats()
            assert st["engine"] == 0 and st["sample"] == 2      # two segments above 10^6, level 2 as rounds
            assert st["launches"] >= 4
            got = out.cpu().numpy().view(dt)
            for i in range(len(sizes)):
                lo, hi = int(offs[i]), int(offs[i + 1])
                assert got[lo:hi].tobytes() == O.numpy_sorted(a[lo:hi], 'key').tobytes(), (rep, i)
        plan.close()
        # the engine and the default threshold through the synchronous call
        device.tuning_clear()
        outs[0].zero_()
        device.sort_segments(din.data_ptr(), outs[0].data_ptr(), offs, dt, 'key')
        torch.cuda.synchronize()
        st = mpsort.last_stats()
        assert st["engine"] == 1 and st["sample"] == 0
        got = outs[0].cpu().numpy().view(dt)
        for i in range(len(sizes)):
            lo, hi = int(offs[i]), int(offs[i + 1])
            assert got[lo:hi].tobytes() == O.numpy_sorted(a[lo:hi], 'key').tobytes(), i
    finally:
        device.tuning_clear()


def test_merge_join(mp):
    import torch
    from mpsort import device
    rng = numpy.random.default_rng(6)
    dt = numpy.dtype([('id', 'i8'), ('mass', 'f4'), ('halo', 'i4')])
    ids = rng.choice(numpy.arange(-10**7, 10**7), 300_000, replace=False)
    a = numpy.zeros(200_000, dt)
    a['id'] = ids[:200_000]
    b = numpy.zeros(200_000, dt)
    b['id'] = numpy.concatenate([ids[4000:196_000], ids[200_000:208_000]])
    a = O.numpy_sorted(a, 'id')
    b = O.numpy_sorted(b, 'id')
    da = torch.from_numpy(a.view(numpy.uint8).copy()).cuda()
    db = torch.from_numpy(b.view(numpy.uint8).copy()).cuda()
    pa = torch.empty(200_000, dtype=torch.int64, device='cuda')
    pb = torch.empty_like(pa)
    npairs = torch.zeros(1, dtype=torch.int64, device='cuda')
    device.merge_join(da.data_ptr(), len(a), db.data_ptr(), len(b), dt, 'id', pa.data_ptr(), pb.data_ptr(),
                      npairs.data_ptr())
    torch.cuda.synchronize()
    k = int(npairs.item())
    common, ia, ib = numpy.intersect1d(a['id'], b['id'], assume_unique=True, return_indices=True)
    assert k == len(common)
    assert (pa[:k].cpu().numpy() == ia).all() and (pb[:k].cpu().numpy() == ib).all()


def test_stats_report_method(mp):
    rng = numpy.random.default_rng(8)
    a = make([('key', 'u8'), ('val', 'i8')], 'key', 1_000_000, "uniform", rng)
    for m in METHODS:
        check(mp, a, 'key', m)
        st = mp.last_stats()
        assert st["method"] == m
        if m != "lsd":
            assert st["nbuckets"] > 1 and st["window_misses"] == 0


@pytest.mark.parametrize("nvals", [1000, 100_000])
def test_learned_heavy_keys_balanced(mp, nvals):
    """Zipf keys put several heavy keys between neighbouring model splitters;
    the learned path must still sort stably and keep every bucket that holds
    more than one key near the mean size (else it falls back to the sample
    quantiles and says so)."""
    rng = numpy.random.default_rng(nvals)
    n = 4_000_000
    dt = numpy.dtype([('key', 'u8'), ('val', 'i8')])
    a = numpy.zeros(n, dt)
    vals = rng.integers(0, 2**64, nvals, dtype=numpy.uint64, endpoint=False)
    a['key'] = vals[numpy.minimum(rng.zipf(1.2, n) - 1, nvals - 1)]
    a['val'] = numpy.arange(n)
    check(mp, a, 'key', "learned")
    st = mp.last_stats()
    assert st["splitter_fallback"] in (0, 1)
    keys, counts = numpy.unique(a['key'], return_counts=True)
    # a bucket is either one key, or at most ~2.5x the mean plus one heavy key
    limit = 3 * n // st["nbuckets"] + 64
    assert st["max_bucket"] <= max(limit, int(counts.max()))


@pytest.mark.parametrize("method", ["plain", "learned"])
def test_split_refines_crowded_bins(mp, method):
    """Particles in Gaussian clusters with Morton keys (40-byte records):
    level-1 buckets hold dense cores beside sparse background, so split bins
    crowd; those bins are cut finer within the same split and the records
    still come out in the stable order.  32 level-1 buckets (a tuning
    entry) make buckets of 250,000 records, large enough to be refined."""
    import torch
    import workloads as W
    from mpsort import device
    n = 8_000_000
    buf, dt = W.particles_4(torch, n)
    a = buf.cpu().numpy().view(dt)
    device.tuning_set(n, dt, 'key', method, max_buckets=32)
    try:
        check(mp, a, 'key', "auto")
        st = mp.last_stats()
    finally:
        device.tuning_clear()
    assert st["method"] == method and st["nbuckets"] == 32, st
    assert st["splits"] > 0 and st["refined_splits"] > 0, st


@pytest.mark.parametrize("method", ["plain", "learned"])
@pytest.mark.parametrize("nheavy", [100, 600])
def test_heavy_key_table(mp, method, nheavy):
    """Keys that own single-key buckets worth several splitters are looked
    up by hash before the bucket search: hundreds of them (hash collisions
    included) over a uniform background sort exactly as the stable sort, and
    the statistics report the table in use."""
    rng = numpy.random.default_rng(nheavy)
    n = 4_000_000
    dt = numpy.dtype([('key', 'u8'), ('val', 'i8')])
    a = numpy.zeros(n, dt)
    heavy = rng.integers(0, 2**64, nheavy, dtype=numpy.uint64, endpoint=False)
    a['key'] = rng.integers(0, 2**64, n, dtype=numpy.uint64, endpoint=False)
    pick = rng.random(n) < 0.9
    a['key'][pick] = heavy[rng.integers(0, nheavy, int(pick.sum()))]
    a['val'] = numpy.arange(n)
    check(mp, a, 'key', method)
    st = mp.last_stats()
    assert st["heavy_keys"] >= (50 if nheavy == 100 else 1), st
    assert st["window_misses"] == 0


# ------------------------------------------------------------ graph plans --
@pytest.mark.parametrize("method", ["auto"] + METHODS)
def test_plan_graph_replay(mp, method):
    """A plan replays the captured pipeline on new contents of the same
    buffers, re-captures for new buffers, and matches the stable sort."""
    import torch
    from mpsort import device
    rng = numpy.random.default_rng(31)
    dt = numpy.dtype([('key', 'u8'), ('val', 'i8')])
    n = 300_001
    plan = device.Plan(n, dt, 'key', method)
    din = torch.empty(n * dt.itemsize, dtype=torch.uint8, device='cuda')
    dout = torch.empty_like(din)
    for rep, dist in enumerate(("uniform", "dups", "zipf", "sorted")):
        a = make(dt, 'key', n, dist, rng)
        din.copy_(torch.from_numpy(a.view(numpy.uint8)))
        plan.sort(din.data_ptr(), dout.data_ptr())
        plan.wait()
        got = dout.cpu().numpy().view(dt)
        assert got.tobytes() == O.numpy_sorted(a, 'key').tobytes(), (method, dist)
        st = mp.last_stats()
        assert st["launches"] > 0
    # new output buffer: re-captured
    dout2 = torch.empty_like(din)
    plan.sort(din.data_ptr(), dout2.data_ptr())
    plan.wait()
    assert torch.equal(dout2, dout)
    plan.close()


def test_plan_on_torch_stream(mp):
    import torch
    from mpsort import device
    rng = numpy.random.default_rng(32)
    dt = numpy.dtype([('key', 'i4'), ('payload', 'u4')])
    n = 70_000
    a = make(dt, 'key', n, "uniform", rng)
    din = torch.from_numpy(a.view(numpy.uint8).copy()).cuda()
    dout = torch.empty_like(din)
    s = torch.cuda.Stream()
    plan = device.Plan(n, dt, 'key', "learned")
    for _ in range(3):
        plan.sort(din.data_ptr(), dout.data_ptr(), s.cuda_stream)
    plan.wait()
    assert dout.cpu().numpy().view(dt).tobytes() == O.numpy_sorted(a, 'key').tobytes()


# -------------------------------------------------------------- autotuner --
@pytest.mark.parametrize("given", [False, True])
def test_autotune_feeds_auto(mp, given):
    """The autotuner times its candidates, stores the winner, and sorts with
    method='auto' then run that configuration (same stable result)."""
    import torch
    from mpsort import device
    rng = numpy.random.default_rng(41)
    dt = numpy.dtype([('key', 'u8'), ('val', 'i8')])
    n = 2_000_000
    a = make(dt, 'key', n, "uniform", rng)
    din = torch.from_numpy(a.view(numpy.uint8).copy()).cuda()
    before = din.clone()
    device.tuning_clear()
    best = device.autotune(n, dt, 'key', din.data_ptr() if given else 0)
    assert torch.equal(din, before)                    # the caller's records are read only
    assert best["method"] in ("plain", "learned", "lsd") and best["ms"] > 0
    assert device.tuning_get(n, dt, 'key')["method"] == best["method"]
    check(mp, a, 'key', "auto")
    st = mp.last_stats()
    assert st["method"] == best["method"]
    if best["method"] != "lsd":
        assert st["nbuckets"] <= best["max_buckets"]
    device.tuning_clear()


# ------------------------------------------------- pipelined host sorts --
@pytest.mark.parametrize("regions", [True, False])
@pytest.mark.parametrize("method", ["auto", "plain", "learned"])
@pytest.mark.parametrize("dist", ["uniform", "zipf", "equal", "sorted"])
def test_host_sort_pipelined_pinned(mp, method, dist, regions, monkeypatch):
    """Pinned host arrays of 2^22 records or more take the pipelined host
    sort (pieces scattered into reserved bucket regions as they land, waves
    down while sorting; or, without regions, the exact level 1 the sort
    falls back to when a region overflows); the result is the same stable
    order, out of place and in place."""
    import torch
    if not regions:
        monkeypatch.setenv("GBSORT_NO_REGIONS", "1")
    rng = numpy.random.default_rng(51)
    dt = numpy.dtype([('key', 'u8'), ('val', 'i8')])
    n = 5_000_000
    a = make(dt, 'key', n, dist, rng)
    pin_in = torch.empty(n * dt.itemsize, dtype=torch.uint8, pin_memory=True)
    pin_out = torch.empty_like(pin_in, pin_memory=True)
    hin = pin_in.numpy().view(dt)
    hout = pin_out.numpy().view(dt)
    hin[:] = a
    mp.sort(hin, 'key', out=hout, method=method)
    st = mp.last_stats()
    exp = O.numpy_sorted(a, 'key')
    assert hout.tobytes() == exp.tobytes()
    assert hin.tobytes() == a.tobytes()
    if st["method"] != "lsd":
        # regions reserved from the sample hold every bucket, skewed keys too
        assert st["pipelined"] == 1 and (st["region_overflow"] == 0 or not regions), st
    mp.sort(hin, 'key', method=method)  # in place
    assert hin.tobytes() == exp.tobytes()


@pytest.mark.parametrize("regions", [True, False])
def test_host_sort_pipelined_4096_buckets(mp, regions, monkeypatch):
    """A tuning entry of 4096 level-1 buckets for a pipelined host sort: its
    (bucket x chunk) count matrix (4096 buckets x 16 pieces x 304 chunks,
    19.9M cells) is past one block's scan of the segment sums, so the count
    scan takes its second level.  Same stable order as the oracle's."""
    import torch
    from mpsort import device
    if not regions:
        monkeypatch.setenv("GBSORT_NO_REGIONS", "1")
    rng = numpy.random.default_rng(53)
    dt = numpy.dtype([('key', 'u8'), ('val', 'i8')])
    n = 10_000_000
    a = make(dt, 'key', n, "uniform", rng)
    pin_in = torch.empty(n * dt.itemsize, dtype=torch.uint8, pin_memory=True)
    pin_out = torch.empty_like(pin_in, pin_memory=True)
    hin = pin_in.numpy().view(dt)
    hout = pin_out.numpy().view(dt)
    hin[:] = a
    device.tuning_clear()
    device.tuning_set(n, dt, 'key', "learned", max_buckets=4096)
    try:
        mp.sort(hin, 'key', out=hout, method="auto")
        st = mp.last_stats()
    finally:
        device.tuning_clear()
    assert st["nbuckets"] == 4096 and st["pipelined"] == 1, st
    assert hout.tobytes() == O.numpy_sorted(a, 'key').tobytes()


@pytest.mark.parametrize("kind,method", [("uniform", "learned"), ("uniform", "plain"), ("intervals", "plain")])
def test_uniform_bucket_splits(mp, kind, method):
    """Level-1 buckets of 8-16 byte records whose keys spread evenly are cut
    into equal key ranges and scattered into regions of their scratch area
    without a histogram pass (uniform_splits); keys that bunch inside their
    buckets (here short intervals 2^51 apart, four or five to a bucket)
    overflow a group's region, and the bucket is split by its histogram
    instead (uniform_fallbacks), until the failures stop further attempts.
    Every key appears twice, so the stable order is checked too."""
    rng = numpy.random.default_rng(61)
    dt = numpy.dtype([('key', 'u8'), ('val', 'i8')])
    n = 8_000_000
    a = numpy.empty(n, dtype=dt)
    if kind == "uniform":
        a['key'] = rng.integers(0, 2**64, n, dtype=numpy.uint64, endpoint=False)
    else:
        k = rng.integers(0, 2**13, n, dtype=numpy.uint64)
        a['key'] = (k << numpy.uint64(51)) + rng.integers(0, 2**40, n, dtype=numpy.uint64)
    a['key'][1::2] = a['key'][0::2]
    a['val'] = numpy.arange(n)
    out = numpy.empty_like(a)
    mp.sort(a, 'key', out=out, method=method)
    st = mp.last_stats()
    assert out.tobytes() == O.numpy_sorted(a, 'key').tobytes()
    if kind == "uniform":
        assert st["uniform_splits"] > 1000 and st["uniform_fallbacks"] == 0, st
    else:
        assert st["uniform_fallbacks"] > 0, st


@pytest.mark.parametrize("layout", [
    [('key', 'u8')],                                  # 8 bytes
    [('key', 'i8'), ('v', 'u4')],                     # 12 bytes, signed key
    [('v', 'u4'), ('key', 'u4'), ('w', 'u8')],        # 16 bytes, 4-byte key at offset 4
])
def test_uniform_splits_record_sizes_in_place(mp, layout):
    """Uniform bucket splits and the split areas for the other record sizes
    of the staged path (8 and 12 bytes) and a 4-byte key, sorted in place
    (the output is the input buffer, which level 1 has consumed before any
    split writes it)."""
    import torch
    from mpsort import device
    rng = numpy.random.default_rng(71)
    dt = numpy.dtype(layout)
    n = 6_000_003
    a = numpy.zeros(n, dtype=dt)
    info = numpy.iinfo(dt['key'].base)
    a['key'] = rng.integers(info.min, info.max, n, dtype=dt['key'].base, endpoint=True)
    a['key'][7::3] = a['key'][0:(n - 7 + 2) // 3]  # equal keys
    for f in dt.names:
        if f != 'key':
            a[f] = numpy.arange(n).astype(dt[f].base)
    d = torch.from_numpy(a.view(numpy.uint8).copy()).cuda()
    device.sort(d.data_ptr(), d.data_ptr(), n, dt, 'key', 'learned', torch.cuda.current_stream().cuda_stream)
    torch.cuda.synchronize()
    st = mp.last_stats()
    got = d.cpu().numpy().view(dt)
    assert got.tobytes() == O.numpy_sorted(a, 'key').tobytes()
    if dt['key'].itemsize == 8:
        assert st["uniform_splits"] > 0, st


@pytest.mark.parametrize("layout", [
    [('key', '<u8'), ('val', '<i8')],
    [('key', '<i8'), ('val', '<u4')],
    [('key', '<u4'), ('val', '<u4')],
])
def test_local_runs_of_equal_keys(mp, layout):
    """20,000 distinct keys of about 150 copies each (plus a uniform rest):
    the local sorts of the staged path (8, 12 and 16-byte records) meet
    runs of equal keys longer than an insertion bin, whose packed words
    differ only in their input indices; such a bin is put in order by a
    bitmap of its indices instead of a counting pass.  Same stable order as
    the oracle's, and the statistics count the crowded bins."""
    rng = numpy.random.default_rng(73)
    dt = numpy.dtype(layout)
    n = 3_000_001
    a = numpy.zeros(n, dtype=dt)
    info = numpy.iinfo(dt['key'].base)
    vals = rng.integers(info.min, info.max, 20_000, dtype=dt['key'].base, endpoint=True)
    a['key'] = rng.integers(info.min, info.max, n, dtype=dt['key'].base, endpoint=True)
    pick = rng.random(n) < 0.97
    a['key'][pick] = vals[rng.integers(0, len(vals), int(pick.sum()))]
    a['val'] = numpy.arange(n).astype(dt['val'].base)
    for method in ("plain", "learned"):
        check(mp, a, 'key', method)
        st = mp.last_stats()
        assert st["bigbin_passes"] > 0, st


@pytest.mark.parametrize("method", ["plain", "learned"])
def test_deep_split_rounds(mp, method):
    """A run of 5000 consecutive keys with one outlier at every power of two
    above it, in a uniform background: each split round narrows the run's
    key range only down to the next outlier, so the run stays one crowded
    group for several rounds.  With 16-byte records the third and later
    rounds go from scratch A to the output and back (the level-1 areas of
    scratch B hold their groups until the local sorts), and local sorts read
    their input from the output itself (deep_splits counts those rounds'
    splits).  Same stable order as the oracle's."""
    rng = numpy.random.default_rng(67)
    dt = numpy.dtype([('key', 'u8'), ('val', 'i8')])
    n = 20_000_000
    a = numpy.empty(n, dtype=dt)
    a['key'] = rng.integers(0, 2**64, n, dtype=numpy.uint64, endpoint=False)
    x = numpy.uint64(2**63 + 12345)
    run = x + numpy.arange(5000, dtype=numpy.uint64)
    outliers = x + (numpy.uint64(1) << numpy.arange(13, 59, dtype=numpy.uint64))
    special = numpy.concatenate([run, run[:1000], outliers])  # (with equal keys)
    pos = rng.choice(n, size=len(special), replace=False)
    a['key'][pos] = special
    a['val'] = numpy.arange(n)
    out = numpy.empty_like(a)
    mp.sort(a, 'key', out=out, method=method)
    st = mp.last_stats()
    assert out.tobytes() == O.numpy_sorted(a, 'key').tobytes()
    assert st["deep_splits"] > 0, st


# ----------------------------------------------- bounded look-back wait --
def test_lookback_wait_runs_out_and_reports(mp):
    """One LSD pass in which a tile never publishes its counts: the next
    tile's look-back wait gives up after a few polls, the call returns
    GBSORT_ERR_INTERNAL with the timeout message, and the device stays
    usable (the same pass without the withheld tile, then a sort, succeed)."""
    L = mp._lib.lib()
    n = 8 * 4096
    rc = L.gbsort_debug_lookback(n, 1, 64)
    assert rc == mp._lib.ERR_INTERNAL
    assert b"gave up" in L.gbsort_last_error()
    assert L.gbsort_debug_lookback(n, 0xFFFFFFFF, 64) == 0
    rng = numpy.random.default_rng(3)
    check(mp, make([('key', 'u8'), ('val', 'i8')], 'key', 100_000, "uniform", rng), 'key', "lsd")


# ------------------------------------------------- level 2: engine vs rounds --
@pytest.mark.parametrize("level2", ["rounds", "engine"])
@pytest.mark.parametrize("layout", [([('key', 'u8'), ('val', 'i8')], 'key'),
                                    ([('key', 'i4'), ('payload', 'u4')], 'key'),
                                    ([('key', 'u8'), ('value', 'f4')], 'key')])
def test_level2_engine_and_rounds(mp, level2, layout):
    """Level 2 as the persistent engine (one launch over a device task queue)
    and as split rounds give the oracle's order on uniform, Zipf and
    duplicate-heavy keys, for both splitter methods (selected through the
    tuning table, as the autotuner would)."""
    from mpsort import device
    dtype, key = layout
    n = 3_000_017
    rng = numpy.random.default_rng(11)
    device.tuning_clear()
    try:
        for dist in ("uniform", "zipf", "dups"):
            a = make(dtype, key, n, dist, rng)
            exp = O.numpy_sorted(a, key)
            for method in ("plain", "learned"):
                device.tuning_set(n, a.dtype, key, method, level2=level2)
                out = numpy.empty_like(a)
                mp.sort(a, key, out=out)
                assert out.tobytes() == exp.tobytes(), (dist, method)
                assert mp.last_stats()["engine"] == (1 if level2 == "engine" else 0)
    finally:
        device.tuning_clear()
