"""CPU checker for the GB300 histogram sort.  TEST INFRASTRUCTURE ONLY.

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline
leg import this module, and only to check or time the reference behaviour;
the shipped library never calls it.

Three checkers, all with the reference's semantics (a stable sort of whole
records by the order-preserving radix of ``mpsort/binding.pyx:81-121``):

* ``liboracle.so`` -- this project's C restatement (``oracle.c``) of
  ``radix_sort`` / ``mpsort_omp`` and the splitter machinery;
* ``_ref/libref_omp.so`` -- the unmodified reference ``radixsort.c`` +
  ``mpsort-omp.c`` built by ``oracle/Makefile`` (present where the reference
  tree was available at build time);
* ``numpy_order`` -- ``numpy.lexsort`` on the mapped key words, which is a
  stable sort and therefore equals the reference.
"""
import ctypes
import os
import subprocess
import sys
import time
from contextlib import contextmanager

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)

MAX_KEY_WORDS = 4


class KeyWord(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_uint32), ("width", ctypes.c_uint32),
                ("is_signed", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class KeyDesc(ctypes.Structure):
    _fields_ = [("nwords", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("word", KeyWord * MAX_KEY_WORDS)]


class RefRadixData(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_int64), ("kind", ctypes.c_int32),
                ("nmemb", ctypes.c_int32)]


RADIX_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)

_KINDS = {numpy.dtype('u8'): (0, 8, 0), numpy.dtype('i8'): (1, 8, 1),
          numpy.dtype('u4'): (2, 4, 0), numpy.dtype('i4'): (3, 4, 1)}


def key_field(dtype, orderby):
    """(base dtype, byte offset, element count) of the key field, following
    ``radix_data_init`` (binding.pyx:50-79)."""
    dtype = numpy.dtype(dtype)
    if orderby is not None:
        fdt, off = dtype.fields[orderby][:2]
    else:
        fdt, off = dtype, 0
    if len(fdt.shape) == 0:
        nmemb = 1
    elif len(fdt.shape) == 1:
        nmemb = fdt.shape[0]
    else:
        raise ValueError("key field is not 0-d or 1-d")
    if fdt.base not in _KINDS:
        raise TypeError("key field is not u8, i8, u4 or i4")
    return fdt.base, off, nmemb


def key_desc(dtype, orderby):
    base, off, nmemb = key_field(dtype, orderby)
    if nmemb > MAX_KEY_WORDS:
        raise ValueError("key has more than %d words" % MAX_KEY_WORDS)
    _, width, signed = _KINDS[base]
    d = KeyDesc()
    d.nwords = nmemb
    for i in range(nmemb):
        d.word[i].offset = off + i * width
        d.word[i].width = width
        d.word[i].is_signed = signed
    return d


def ref_radix_data(dtype, orderby):
    base, off, nmemb = key_field(dtype, orderby)
    kind = _KINDS[base][0]
    return RefRadixData(off, kind, nmemb)


def key_words(arr, orderby):
    """(n, nwords) uint64 order-preserving key words of each record."""
    base, off, nmemb = key_field(arr.dtype, orderby)
    raw = numpy.ascontiguousarray(arr).view(numpy.uint8).reshape(len(arr), arr.dtype.itemsize)
    width = base.itemsize
    cols = []
    for i in range(nmemb):
        b = numpy.ascontiguousarray(raw[:, off + i * width: off + (i + 1) * width])
        v = b.view(base).reshape(len(arr))
        if base == numpy.dtype('u8'):
            w = v.astype(numpy.uint64)
        elif base == numpy.dtype('u4'):
            w = v.astype(numpy.uint64)
        else:
            w = v.astype(numpy.int64).view(numpy.uint64) ^ numpy.uint64(1 << 63)
        cols.append(w)
    return numpy.stack(cols, axis=1) if cols else numpy.zeros((len(arr), 0), numpy.uint64)


def numpy_order(arr, orderby):
    """Stable order of the records; last key word most significant."""
    kw = key_words(arr, orderby)
    if len(arr) == 0:
        return numpy.zeros(0, numpy.int64)
    return numpy.lexsort(kw.T[::1]).astype(numpy.int64) if kw.shape[1] > 1 else \
        numpy.argsort(kw[:, 0], kind='stable').astype(numpy.int64)


def numpy_sorted(arr, orderby):
    return arr[numpy_order(arr, orderby)]


# --------------------------------------------------------------- libraries

_LIBS = {}


def _build(target_dir=HERE):
    subprocess.run(["make", "-s", "-C", target_dir], check=True,
                   stdout=subprocess.DEVNULL)


def oracle_lib():
    """ctypes handle on liboracle.so (built on first use)."""
    if "oracle" not in _LIBS:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            _build()
        lib = ctypes.CDLL(path)
        lib.oracle_radix_sort.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                          ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        lib.oracle_radix_sort.restype = ctypes.c_int
        lib.oracle_argsort.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                       ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                       ctypes.c_void_p]
        lib.oracle_argsort.restype = ctypes.c_int
        lib.oracle_mpsort_tasks.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                            ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p,
                                            ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        lib.oracle_mpsort_tasks.restype = ctypes.c_int
        lib.oracle_compar.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_size_t]
        lib.oracle_compar.restype = ctypes.c_int
        lib.oracle_bisect.argtypes = [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                      ctypes.c_size_t]
        lib.oracle_bisect.restype = None
        lib.oracle_histogram.argtypes = [ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p,
                                         ctypes.c_size_t, ctypes.c_size_t, ctypes.c_void_p,
                                         ctypes.c_void_p]
        lib.oracle_histogram.restype = None
        lib.oracle_solve_layout.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                            ctypes.c_void_p, ctypes.c_void_p]
        lib.oracle_solve_layout.restype = ctypes.c_int
        lib.oracle_bisect_splitters.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                                                ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p]
        lib.oracle_bisect_splitters.restype = ctypes.c_int
        _LIBS["oracle"] = lib
    return _LIBS["oracle"]


def ref_lib():
    """ctypes handle on the unmodified reference build, or None if it was
    not built (the reference tree was absent when ``make`` ran)."""
    if "ref" not in _LIBS:
        path = os.path.join(HERE, "_ref", "libref_omp.so")
        if not os.path.exists(path):
            _LIBS["ref"] = None
            return None
        lib = ctypes.CDLL(path)
        for name in ("radix_sort", "mpsort_omp"):
            f = getattr(lib, name)
            f.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t,
                          ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
            f.restype = None
        _LIBS["ref"] = lib
    return _LIBS["ref"]


@contextmanager
def _quiet_stdout():
    """mpsort_omp prints per-stage timings to stdout (mpsort-omp.c:269-392);
    send file descriptor 1 to /dev/null while it runs."""
    sys.stdout.flush()
    libc = ctypes.CDLL(None)
    saved = os.dup(1)
    devnull = os.open(os.devnull, os.O_WRONLY)
    try:
        os.dup2(devnull, 1)
        yield
    finally:
        libc.fflush(None)
        os.dup2(saved, 1)
        os.close(saved)
        os.close(devnull)


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def oracle_sort(arr, orderby):
    """Sorted copy by this project's C restatement of radix_sort."""
    out = numpy.ascontiguousarray(arr).copy()
    if len(out) == 0:
        return out
    lib = oracle_lib()
    d = key_desc(arr.dtype, orderby)
    fn = ctypes.cast(lib.oracle_radix_desc, ctypes.c_void_p)
    rc = lib.oracle_radix_sort(_ptr(out), len(out), out.dtype.itemsize, fn, 8 * d.nwords,
                               ctypes.byref(d))
    if rc:
        raise MemoryError("oracle_radix_sort failed")
    return out


def oracle_mpsort(arr, orderby, ntasks):
    """Sorted copy by the C restatement of mpsort_omp with `ntasks` tasks."""
    out = numpy.ascontiguousarray(arr).copy()
    if len(out) == 0:
        return out
    lib = oracle_lib()
    d = key_desc(arr.dtype, orderby)
    fn = ctypes.cast(lib.oracle_radix_desc, ctypes.c_void_p)
    rc = lib.oracle_mpsort_tasks(_ptr(out), len(out), out.dtype.itemsize, fn, 8 * d.nwords,
                                 ctypes.byref(d), int(ntasks), None, None)
    if rc:
        raise RuntimeError("oracle_mpsort_tasks failed")
    return out


def set_ref_threads(threads):
    """Thread count of the reference's OpenMP region (omp_set_num_threads)."""
    try:
        ctypes.CDLL("libgomp.so.1").omp_set_num_threads(int(threads))
    except OSError:
        os.environ["OMP_NUM_THREADS"] = str(threads)


def ref_sort(arr, orderby, method="omp", threads=None):
    """Sorted copy by the UNMODIFIED reference (``mpsort_omp`` or
    ``radix_sort``), or None if the reference build is absent."""
    lib = ref_lib()
    if lib is None:
        return None
    out = numpy.ascontiguousarray(arr).copy()
    if len(out) == 0:
        return out
    rd = ref_radix_data(arr.dtype, orderby)
    fn = ctypes.cast(lib.ref_radix_field, ctypes.c_void_p)
    f = lib.mpsort_omp if method == "omp" else lib.radix_sort
    if threads is not None:
        set_ref_threads(threads)
    with _quiet_stdout():
        f(_ptr(out), len(out), out.dtype.itemsize, fn, 8 * rd.nmemb, ctypes.byref(rd))
    return out


def ref_sort_callback(buf, elsize, callback_name, rsize, method="omp"):
    """Sort a raw byte buffer in place with one of ref_keys.c's fixed
    callbacks (``ref_radix_int`` / ``ref_radix_issue7``)."""
    lib = ref_lib()
    if lib is None:
        return None
    out = numpy.ascontiguousarray(buf).copy()
    n = out.nbytes // elsize
    if n == 0:
        return out
    fn = ctypes.cast(getattr(lib, callback_name), ctypes.c_void_p)
    f = lib.mpsort_omp if method == "omp" else lib.radix_sort
    with _quiet_stdout():
        f(_ptr(out), n, elsize, fn, rsize, None)
    return out


def time_ref_sort(arr, orderby, method="omp", repeat=3):
    """Median wall time (s) of the reference sort on copies of `arr`."""
    lib = ref_lib()
    if lib is None:
        return None
    rd = ref_radix_data(arr.dtype, orderby)
    fn = ctypes.cast(lib.ref_radix_field, ctypes.c_void_p)
    f = lib.mpsort_omp if method == "omp" else lib.radix_sort
    times = []
    for _ in range(repeat):
        out = numpy.ascontiguousarray(arr).copy()
        with _quiet_stdout():
            t0 = time.perf_counter()
            f(_ptr(out), len(out), out.dtype.itemsize, fn, 8 * rd.nmemb, ctypes.byref(rd))
            t1 = time.perf_counter()
        times.append(t1 - t0)
    times.sort()
    return times[len(times) // 2]
