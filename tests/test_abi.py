"""The C ABI and the host-side logic, without a GPU."""
import ctypes
import os
import re
import subprocess

import numpy
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
INCLUDE = os.path.join(REPO, "include")


def _declared_symbols():
    names = set()
    for h in ("gbsort.h", "mpsort.h"):
        src = open(os.path.join(INCLUDE, h)).read()
        names |= set(re.findall(r"GBSORT_API\s+[\w\s\*]+?\b(\w+)\s*\(", src))
    return names


@pytest.fixture(scope="module")
def lib():
    import __graft_entry__ as g
    g.build()
    import mpsort
    return mpsort._lib.lib()


def test_library_exports_every_declared_symbol(lib):
    declared = _declared_symbols()
    assert {"radix_sort", "mpsort_omp", "gbsort_sort_device", "gbsort_sort_host"} <= declared
    so = os.path.join(REPO, "mp-sort_gb300", "lib", "libgbsort.so")
    out = subprocess.run(["nm", "-D", "--defined-only", so], capture_output=True, text=True).stdout
    exported = {line.split()[-1] for line in out.splitlines() if " T " in line}
    assert declared <= exported, declared - exported
    for name in declared:
        assert hasattr(lib, name)


def test_headers_compile_as_c_and_cpp(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "gbsort.h"\n#include "mpsort.h"\nint main(void){gbsort_key_desc d; (void)d; return 0;}\n')
    for cc, lang in (("gcc", "c"), ("g++", "c++")):
        r = subprocess.run([cc, "-x", lang, "-I", INCLUDE, "-fsyntax-only", str(src)], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_key_descriptor_layout_matches_header(lib):
    import mpsort._lib as L
    assert ctypes.sizeof(L.KeyDesc) == 8 + 16 * 4
    assert ctypes.sizeof(L.Stats) == 4 * 30
    assert ctypes.sizeof(L.Tuning) == 4 * 8


def test_struct_fields_match_header_offsets(tmp_path):
    """Every ctypes field of the Python binding sits at the offset the C
    compiler gives the header's field of the same name."""
    import mpsort._lib as L
    pairs = [(L.Stats, "gbsort_stats"), (L.Tuning, "gbsort_tuning"), (L.KeyDesc, "gbsort_key_desc"),
             (L.KeyWord, "gbsort_key_word")]
    lines = ['#include <stdio.h>', '#include <stddef.h>', '#include "gbsort.h"', 'int main(void) {']
    expect = []
    for cls, cname in pairs:
        lines.append('printf("%%zu\\n", sizeof(%s));' % cname)
        expect.append(ctypes.sizeof(cls))
        for f, _ in cls._fields_:
            lines.append('printf("%%zu\\n", offsetof(%s, %s));' % (cname, f))
            expect.append(getattr(cls, f).offset)
    lines += ['return 0;', '}']
    src, exe = tmp_path / "off.c", tmp_path / "off"
    src.write_text("\n".join(lines) + "\n")
    r = subprocess.run(["gcc", "-I", INCLUDE, str(src), "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got = [int(x) for x in subprocess.run([str(exe)], capture_output=True, text=True).stdout.split()]
    assert got == expect


def test_key_desc_follows_binding_rules():
    import mpsort._lib as L
    dt = numpy.dtype([('a', 'u1'), ('k', 'i4'), ('v', ('u8', 2))], align=False)
    d = L.key_desc(dt, 'k')
    assert (d.nwords, d.word[0].offset, d.word[0].width, d.word[0].is_signed) == (1, 1, 4, 1)
    d = L.key_desc(dt, 'v')
    assert d.nwords == 2 and d.word[1].offset == 13 and d.word[1].width == 8
    with pytest.raises(TypeError):
        L.key_desc(numpy.dtype([('f', 'f8')]), 'f')
    with pytest.raises(ValueError):
        L.key_desc(numpy.dtype([('m', ('u8', (2, 2)))]), 'm')


def test_radix_desc_callback_matches_oracle(lib):
    """mpsort_radix_desc writes the same radix bytes as the binding's callbacks."""
    import mpsort._lib as L
    import oracle as O
    rng = numpy.random.default_rng(3)
    dt = numpy.dtype([('i', 'i4'), ('u', 'u4'), ('I', 'i8'), ('U', 'u8'), ('v', ('i4', 3))])
    a = numpy.zeros(64, dt)
    for f in ('i', 'u', 'I', 'U'):
        a[f] = rng.integers(numpy.iinfo(a[f].dtype).min, numpy.iinfo(a[f].dtype).max, 64, dtype=a[f].dtype)
    a['v'] = rng.integers(-5, 5, (64, 3))
    for f in ('i', 'u', 'I', 'U', 'v'):
        d = L.key_desc(dt, f)
        kw = O.key_words(a, f)
        for r in range(64):
            buf = (ctypes.c_uint8 * (8 * d.nwords))()
            lib.mpsort_radix_desc(a[r:r + 1].ctypes.data, buf, ctypes.byref(d))
            assert bytes(buf) == kw[r].tobytes()


def test_no_device_is_an_error_not_a_crash(lib):
    """Without a GPU every entry point returns a status; nothing aborts."""
    import mpsort
    if lib.gbsort_device_count() > 0:
        pytest.skip("a GPU is visible")
    a = numpy.arange(10, dtype='i8')
    with pytest.raises(mpsort.GBSortError) as e:
        mpsort.sort(a)
    assert e.value.status == 4  # GBSORT_ERR_NO_DEVICE
    buf = numpy.arange(5, dtype='i4')
    lib.radix_sort(buf.ctypes.data, 5, 4, ctypes.cast(lib.mpsort_radix_desc, ctypes.c_void_p), 8, None)
    assert lib.mpsort_last_status() != 0


def test_binding_argument_errors(lib):
    import mpsort
    a = numpy.zeros(10, dtype=[('k', 'i8'), ('v', 'f8')])
    with pytest.raises(ValueError):
        mpsort.sort(a[::2], 'k')                      # not C-contiguous
    with pytest.raises(ValueError):
        mpsort.sort(a, 'k', out=numpy.zeros(9, a.dtype))   # size changed
    with pytest.raises(ValueError):
        mpsort.sort(a, 'k', out=numpy.zeros(10, dtype='i4'))   # item size
    with pytest.raises(TypeError):
        mpsort.sort(a, 'v')                           # float key
    with pytest.raises((ValueError, KeyError)):
        mpsort.sort(a, 'nope')

    class TwoRanks:
        size = 2
        rank = 0
    with pytest.raises(NotImplementedError):
        mpsort.sort(a, 'k', comm=TwoRanks())


def test_empty_sort_needs_no_device(lib):
    import mpsort
    s = numpy.empty(0, dtype=[('vkey', ('u8', 3)), ('vector', ('u4', 3))])
    mpsort.sort(s, 'vkey', out=s, tuning=['REQUIRE_GATHER_SORT'])
    assert mpsort.histogram([], [1], None).tolist() == [0, 0]


def test_tuning_flags_are_stored(lib):
    import mpsort
    a = numpy.empty(0, dtype='i8')
    mpsort.sort(a, tuning=['DISABLE_GATHER_SORT', 'REQUIRE_SPARSE_ALLTOALLV'])
    assert lib.mpsort_mpi_has_options((1 << 3) | (1 << 6))
    assert not lib.mpsort_mpi_has_options(1 << 4)


def test_tuning_table_roundtrip_without_gpu(lib, tmp_path):
    """The autotuner's table: set, look up by nearest size class, save,
    clear, load -- host logic only, no device call."""
    from mpsort import device
    dt = numpy.dtype([('key', 'u8'), ('val', 'i8')])
    device.tuning_clear()
    assert device.tuning_get(10**6, dt, 'key') is None
    device.tuning_set(10**6, dt, 'key', 'plain', max_buckets=1024, sample_per_bucket=64)
    got = device.tuning_get(10**6, dt, 'key')
    assert got["method"] == "plain" and got["max_buckets"] == 1024 and got["sample_per_bucket"] == 64
    assert device.tuning_get(3 * 10**6, dt, 'key')["method"] == "plain"   # nearest size class
    assert device.tuning_get(10**9, dt, 'key') is None                     # too far away
    dt4 = numpy.dtype([('key', 'i4'), ('payload', 'u4')])
    assert device.tuning_get(10**6, dt4, 'key') is None                    # other layout
    device.tuning_set(10**8, dt4, 'key', 'lsd')
    path = tmp_path / "tune.txt"
    device.tuning_save(path)
    device.tuning_clear()
    assert device.tuning_get(10**6, dt, 'key') is None
    device.tuning_load(path)
    assert device.tuning_get(10**6, dt, 'key')["max_buckets"] == 1024
    assert device.tuning_get(10**8, dt4, 'key')["method"] == "lsd"
    bad = tmp_path / "bad.txt"
    bad.write_text("16 8 20 2 3000 128 1.0\n")                             # cap not a power of two
    with pytest.raises(Exception):
        device.tuning_load(bad)
    with pytest.raises(Exception):
        device.tuning_set(10**6, dt, 'key', 'plain', max_buckets=8192)
    device.tuning_clear()
