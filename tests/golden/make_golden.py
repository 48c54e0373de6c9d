"""Generate the golden input/output vectors under tests/golden/.

Run in a container where the MP-sort reference tree and its built library
(``oracle/_ref/libref_omp.so``, from ``make -C oracle``) are available:

    python tests/golden/make_golden.py --reference <reference tree>

Every expected output here is produced by the UNMODIFIED reference
``mpsort_omp`` and ``radix_sort`` (compiled from the reference sources),
and cross-checked against ``radix_sort`` and numpy's stable lexsort before
it is written.  The ``issue7`` input is the reference's only frozen test
fixture (``Issue7B64`` in mpsort/tests/test_mpsort.py), decoded here with an
unpickler that can build nothing but numpy scalars and dtypes.
"""
import argparse
import base64
import io
import os
import pickle
import re
import sys

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(REPO, "oracle"))
import oracle as O  # noqa: E402


class _NumpyScalarsOnly(pickle.Unpickler):
    """Allows exactly the two globals the fixture uses."""

    def find_class(self, module, name):
        if (module, name) == ("numpy", "dtype"):
            return numpy.dtype
        if (module, name) in (("numpy.core.multiarray", "scalar"),
                              ("numpy._core.multiarray", "scalar")):
            def scalar(dtype, data=None):
                return numpy.frombuffer(data, dtype=dtype)[0]
            return scalar
        raise pickle.UnpicklingError("refusing global %s.%s" % (module, name))


def issue7_arrays(refdir):
    src = open(os.path.join(refdir, "mpsort", "tests", "test_mpsort.py")).read()
    m = re.search(r'Issue7B64\s*=\s*b?"""(.*?)"""', src, re.S)
    raw = base64.decodebytes(m.group(1).encode())
    lists = _NumpyScalarsOnly(io.BytesIO(raw)).load()
    return [numpy.array(a, dtype='u4').reshape(-1, 10) for a in lists]


def expect(arr, orderby):
    """Reference outputs of mpsort_omp and radix_sort, checked to agree."""
    omp = O.ref_sort(arr, orderby, "omp")
    rad = O.ref_sort(arr, orderby, "radix")
    npy = O.numpy_sorted(arr, orderby)
    assert omp.tobytes() == rad.tobytes() == npy.tobytes(), "reference paths disagree"
    return omp


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--reference", required=True, help="the MP-sort source tree")
    ap.add_argument("--digests-only", action="store_true",
                    help="rewrite digests.json only (golden.npz unchanged)")
    args = ap.parse_args()
    if O.ref_lib() is None:
        sys.exit("oracle/_ref/libref_omp.so is missing: run make -C oracle first")
    O.set_ref_threads(4)
    cases = {}

    # the reference's frozen fixture: 40-byte records, 16-byte two-word radix
    A = issue7_arrays(args.reference)
    parts = []
    for a in A:
        s = numpy.zeros(len(a), dtype=[('radix', ('u8', 2)), ('ext', ('u8', 3))])
        s['radix'][:, 0] = a[:, 5].astype('u8') + (a[:, 4].astype('u8') << numpy.uint64(32))
        s['radix'][:, 1] = a[:, 0]
        parts.append(s)
    s = numpy.concatenate(parts)
    cases["issue7"] = (s, "radix")

    # the only seeded reference test: test_sort_struct (seed 1234, 10 records)
    numpy.random.seed(1234)
    t = numpy.empty(10, dtype=[('value', 'i8'), ('key', 'i8')])
    t['value'] = numpy.int32(numpy.random.random(size=10) * 1000 - 400)
    t['key'] = t['value']
    cases["struct_seed1234"] = (t, "key")

    # test_few_items: sizes {0,1,2}^4 gathered into one array, 3-word key
    for sizes in [(0, 1, 2, 2), (2, 2, 2, 2), (1, 0, 0, 1)]:
        chunks = []
        for n in sizes:
            c = numpy.empty(n, dtype=[('vkey', ('u8', 3)), ('vector', ('u4', 3))])
            c['vkey'] = numpy.arange(n, dtype='u8')[:, None]
            c['vector'] = 1
            chunks.append(c)
        cases["few_items_%d%d%d%d" % sizes] = (numpy.concatenate(chunks), "vkey")

    rng = numpy.random.Generator(numpy.random.PCG64(0))
    # configuration-1 layout (packed 12-byte records, u8 key), 4096 records
    n = 4096
    c1 = numpy.empty(n, dtype=[('key', 'u8'), ('value', 'f4')])
    c1['key'] = rng.integers(0, 2**64, n, dtype=numpy.uint64, endpoint=False)
    c1['value'] = numpy.arange(n, dtype=numpy.float32)
    cases["cfg1_4096"] = (c1, "key")

    # heavy duplicates with a payload that records the input position
    n = 20011
    d = numpy.empty(n, dtype=[('key', 'i4'), ('payload', 'u4')])
    d['key'] = rng.integers(-50, 50, n)
    d['payload'] = numpy.arange(n)
    cases["dup_i4_20011"] = (d, "key")

    # signed 64-bit keys spanning the sign boundary, 16-byte records
    n = 5003
    e = numpy.empty(n, dtype=[('key', 'i8'), ('val', 'i8')])
    e['key'] = rng.integers(-2**62, 2**62, n)
    e['key'][::7] = -1
    e['key'][::11] = 0
    e['val'] = numpy.arange(n)
    cases["i8_5003"] = (e, "key")

    # u4 keys at a non-zero offset in a 40-byte record
    n = 3001
    f = numpy.zeros(n, dtype=[('pos', ('f4', 3)), ('vel', ('f4', 3)), ('id', 'u8'),
                              ('key', 'u4'), ('pad', 'u4')])
    f['key'] = rng.integers(0, 2**32, n, dtype=numpy.uint64).astype('u4')
    f['key'][::5] = 7
    f['id'] = numpy.arange(n)
    cases["u4_off32_3001"] = (f, "key")

    out = {}
    for name, (arr, orderby) in cases.items():
        out[name + "__in"] = arr
        out[name + "__out"] = expect(arr, orderby)
        out[name + "__orderby"] = numpy.array(orderby)

    # callback-keyed buffers: main.c's int radix (rsize 4, unsigned compare)
    ints = rng.integers(-10000, 10000, 10007).astype('i4')
    out["cb_int__in"] = ints
    omp = O.ref_sort_callback(ints, 4, "ref_radix_int", 4, "omp")
    rad = O.ref_sort_callback(ints, 4, "ref_radix_int", 4, "radix")
    assert omp.tobytes() == rad.tobytes()
    assert omp.tobytes() == ints[numpy.argsort(ints.view('u4'), kind='stable')].tobytes()
    out["cb_int__out"] = omp

    # test-issue7.c's composite callback radix on 40-byte records
    recs = numpy.zeros((2003, 10), dtype='u4')
    recs[:, 0] = rng.integers(0, 4, 2003)
    recs[:, 4] = rng.integers(0, 3, 2003)
    recs[:, 5] = rng.integers(0, 2**32, 2003, dtype=numpy.uint64).astype('u4')
    recs[:, 9] = numpy.arange(2003)
    out["cb_issue7__in"] = recs
    omp = O.ref_sort_callback(recs, 40, "ref_radix_issue7", 16, "omp")
    rad = O.ref_sort_callback(recs, 40, "ref_radix_issue7", 16, "radix")
    assert omp.tobytes() == rad.tobytes()
    lo = recs[:, 4].astype('u8') | (recs[:, 5].astype('u8') << numpy.uint64(32))
    order = numpy.lexsort((lo, recs[:, 0].astype('u8')))
    assert omp.tobytes() == recs[order].tobytes()
    out["cb_issue7__out"] = omp

    path = os.path.join(HERE, "golden.npz")
    if not args.digests_only:
        numpy.savez_compressed(path, **out)
        print("wrote", path, os.path.getsize(path), "bytes,", len(cases) + 2, "cases")
    write_digests()


# Benchmark workloads too large to commit as vectors: the SHA-256 of the
# unmodified reference's output (mpsort_omp, checked against radix_sort and
# numpy's stable sort) on inputs that workloads.py regenerates bit for bit
# from a seed, without a GPU.
DIGEST_CASES = {
    "cfg1_full": lambda W: (W.records_1(None), "key"),               # 1e6 x 12 B, PCG64 seed 0
    "cfg2b_2e7": lambda W: (W.records_2_host(2 * 10**7, "2b"), "key"),  # sorted, 1 % swapped
    "cfg2c_2e7": lambda W: (W.records_2_host(2 * 10**7, "2c"), "key"),  # Zipf(1.2) over 1e6 values
}


def write_digests():
    import hashlib
    import json
    sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
    import workloads as W
    dig = {}
    for name, make in DIGEST_CASES.items():
        arr, orderby = make(W)
        ref = expect(arr, orderby)
        dig[name] = {"n": len(arr), "dtype": str(arr.dtype.descr), "orderby": orderby,
                     "sha256_in": hashlib.sha256(arr.tobytes()).hexdigest(),
                     "sha256_out": hashlib.sha256(ref.tobytes()).hexdigest()}
        print(name, dig[name]["sha256_out"])
    path = os.path.join(HERE, "digests.json")
    with open(path, "w") as f:
        json.dump(dig, f, indent=1)
        f.write("\n")
    print("wrote", path)


if __name__ == "__main__":
    main()
