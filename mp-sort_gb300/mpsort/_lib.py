"""ctypes binding of libgbsort.so (the C ABI declared in include/gbsort.h).

The library is the product: if it is missing this module raises on import,
there is no CPU fallback.
"""
import ctypes
import os

import numpy

HERE = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.dirname(HERE)
LIB_PATH = os.path.join(PKG, "lib", "libgbsort.so")

MAX_KEY_WORDS = 4

OK, ERR_BAD_ARG, ERR_OOM, ERR_CUDA, ERR_NO_DEVICE, ERR_INTERNAL, ERR_UNSUPPORTED = range(7)
METHODS = {"auto": 0, "plain": 1, "learned": 2, "lsd": 3}
VERIFY = 0x100  # GBSORT_VERIFY: self-checked sort (multiset hash of input and output)
METHOD_NAMES = {v: k for k, v in METHODS.items()}


class KeyWord(ctypes.Structure):
    _fields_ = [("offset", ctypes.c_uint32), ("width", ctypes.c_uint32),
                ("is_signed", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class KeyDesc(ctypes.Structure):
    _fields_ = [("nwords", ctypes.c_uint32), ("reserved", ctypes.c_uint32),
                ("word", KeyWord * MAX_KEY_WORDS)]


class Stats(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int32), ("nbuckets", ctypes.c_uint32),
                ("sample", ctypes.c_uint32), ("splitter_rounds", ctypes.c_uint32),
                ("local_sorts", ctypes.c_uint32), ("splits", ctypes.c_uint32),
                ("copies", ctypes.c_uint32), ("resplits", ctypes.c_uint32),
                ("bigbin_passes", ctypes.c_uint32), ("window_misses", ctypes.c_uint32),
                ("max_bucket", ctypes.c_uint32), ("lsd_passes", ctypes.c_uint32),
                ("widest_window", ctypes.c_uint32), ("model_loss", ctypes.c_float),
                ("stage_ms", ctypes.c_float * 6), ("launches", ctypes.c_uint32),
                ("splitter_fallback", ctypes.c_uint32), ("heavy_keys", ctypes.c_uint32),
                ("refined_splits", ctypes.c_uint32), ("pipelined", ctypes.c_uint32),
                ("region_overflow", ctypes.c_uint32), ("engine", ctypes.c_uint32),
                ("uniform_splits", ctypes.c_uint32), ("uniform_fallbacks", ctypes.c_uint32),
                ("deep_splits", ctypes.c_uint32)]

    STAGES = ("splitters", "count", "scan", "scatter", "split", "local")

    def as_dict(self):
        d = {f: getattr(self, f) for f, _ in self._fields_ if f not in ("reserved", "stage_ms")}
        d["stage_ms"] = {k: round(float(v), 4) for k, v in zip(self.STAGES, self.stage_ms)}
        d["method"] = METHOD_NAMES.get(self.method, self.method)
        return d


class GBSortError(RuntimeError):
    def __init__(self, status, message):
        super().__init__("gbsort status %d (%s): %s" % (status, status_string(status), message))
        self.status = status


RADIX_FN = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p)

_P = ctypes.c_void_p
_SZ = ctypes.c_size_t
_U32 = ctypes.c_uint32
_U64 = ctypes.c_uint64
_I = ctypes.c_int

LEVEL2 = {"default": 0, "rounds": 1, "engine": 2}
LEVEL2_NAMES = {v: k for k, v in LEVEL2.items()}


class Tuning(ctypes.Structure):
    _fields_ = [("method", ctypes.c_int32), ("max_buckets", ctypes.c_uint32),
                ("sample_per_bucket", ctypes.c_uint32), ("ms", ctypes.c_float),
                ("level2", ctypes.c_uint32), ("reserved", ctypes.c_uint32 * 3)]

    def as_dict(self):
        return {"method": METHOD_NAMES.get(self.method, self.method), "max_buckets": self.max_buckets,
                "sample_per_bucket": self.sample_per_bucket, "ms": self.ms,
                "level2": LEVEL2_NAMES.get(self.level2, self.level2), "big_above": self.reserved[0]}


# name: (restype, argtypes)
SIGNATURES = {
    "gbsort_sort_device": (_I, [_P, _P, _SZ, _SZ, _P, _I, _P]),
    "gbsort_sort_device_noalloc": (_I, [_P, _P, _SZ, _SZ, _P, _P]),
    "gbsort_sort_host": (_I, [_P, _P, _SZ, _SZ, _P, _I]),
    "gbsort_sort_radix_host": (_I, [_P, _SZ, _SZ, _P, _SZ, _P]),
    "gbsort_sort_segments_device": (_I, [_P, _P, _P, _SZ, _SZ, _P, _I, _P]),
    "gbsort_merge_join_device": (_I, [_P, _SZ, _P, _SZ, _SZ, _P, _P, _P, _P, _P]),
    "gbsort_cdf_forward_backward": (_I, [_P, _U32, _U64, _U64, _I, _P, _P, _P, _P]),
    "gbsort_cdf_train_gradient": (_I, [_P, _U32, _U64, _U64, _I, _P, _P]),
    "gbsort_debug_buckets": (_I, [_P, _U32, _I, _P, _U32, _P, _P, _P, _P]),
    "gbsort_debug_model": (_I, [_P, _U32, _I, _I, _P, _U32, _P, _P, _P, _P, _P]),
    "gbsort_debug_bisect": (_I, [_P, _U32, _I, _P, _P, _P, _P]),
    "gbsort_debug_lookback": (_I, [_U32, _U32, _U32]),
    "gbsort_multiset_hash_device": (_I, [_P, _SZ, _SZ, _P, _P]),
    "gbsort_take_device": (_I, [_P, _SZ, _SZ, _P, _SZ, _P, _P]),
    "mpsort_mpi_newarray_impl": (None, [_P, _SZ, _P, _SZ, _SZ, _P, _SZ, _P, ctypes.c_ssize_t, _I, ctypes.c_char_p]),
    "mpsort_mpi_impl": (None, [_P, _SZ, _SZ, _P, _SZ, _P, ctypes.c_ssize_t, _I, ctypes.c_char_p]),
    "mpsort_mpi_report_last_run": (None, []),
    "gbsort_plan_create": (_I, [_P, _SZ, _SZ, _P, _I]),
    "gbsort_plan_create_segments": (_I, [_P, _P, _SZ, _SZ, _P, _I]),
    "gbsort_plan_sort": (_I, [_P, _P, _P, _P]),
    "gbsort_plan_wait": (_I, [_P]),
    "gbsort_plan_destroy": (_I, [_P]),
    "gbsort_autotune": (_I, [_SZ, _SZ, _P, _P, _P]),
    "gbsort_tuning_set": (_I, [_SZ, _SZ, _P, _P]),
    "gbsort_tuning_get": (_I, [_SZ, _SZ, _P, _P]),
    "gbsort_autotune_segments": (_I, [_P, _SZ, _SZ, _P, _P, _P]),
    "gbsort_tuning_get_segments": (_I, [_SZ, _SZ, _P, _P]),
    "gbsort_tuning_clear": (_I, []),
    "gbsort_tuning_save": (_I, [ctypes.c_char_p]),
    "gbsort_tuning_load": (_I, [ctypes.c_char_p]),
    "gbsort_last_stats": (_I, [_P]),
    "gbsort_status_string": (ctypes.c_char_p, [_I]),
    "gbsort_last_error": (ctypes.c_char_p, []),
    "gbsort_device_count": (_I, []),
    "gbsort_release": (_I, []),
    "gbsort_version": (ctypes.c_char_p, []),
    "radix_sort": (None, [_P, _SZ, _SZ, _P, _SZ, _P]),
    "mpsort_omp": (None, [_P, _SZ, _SZ, _P, _SZ, _P]),
    "mpsort_radix_desc": (None, [_P, _P, _P]),
    "mpsort_last_status": (_I, []),
    "mpsort_mpi_set_options": (None, [_I]),
    "mpsort_mpi_has_options": (_I, [_I]),
    "mpsort_mpi_unset_options": (None, [_I]),
}

_lib = None


def lib():
    """The loaded libgbsort (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libgbsort.so is not built (%s); run "
                              "`python mp-sort_gb300/build.py` or __graft_entry__.build()" % LIB_PATH)
        L = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            f = getattr(L, name)
            f.restype = res
            f.argtypes = args
        _lib = L
    return _lib


def status_string(status):
    try:
        return lib().gbsort_status_string(status).decode()
    except Exception:
        return "status %d" % status


def check(status):
    if status != OK:
        raise GBSortError(status, lib().gbsort_last_error().decode(errors="replace"))


def last_stats():
    s = Stats()
    check(lib().gbsort_last_stats(ctypes.byref(s)))
    return s.as_dict()


_KINDS = {numpy.dtype('u8'): (8, 0), numpy.dtype('i8'): (8, 1),
          numpy.dtype('u4'): (4, 0), numpy.dtype('i4'): (4, 1)}


def key_desc(dtype, orderby):
    """gbsort_key_desc of field `orderby` of `dtype`, following the binding's
    radix_data_init (mpsort/binding.pyx:50-79): u8/i8/u4/i4 fields, scalar or
    1-d, a 1-d field's last element most significant."""
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
        raise ValueError("data[%s] is not 1d nor 2d" % (orderby,))
    if fdt.base not in _KINDS:
        raise TypeError("data[%s] is not u8 or i8" % (orderby,))
    if nmemb > MAX_KEY_WORDS:
        raise ValueError("keys of more than %d elements are not supported" % MAX_KEY_WORDS)
    width, signed = _KINDS[fdt.base]
    d = KeyDesc()
    d.nwords = nmemb
    for i in range(nmemb):
        d.word[i].offset = off + i * width
        d.word[i].width = width
        d.word[i].is_signed = signed
    return d
