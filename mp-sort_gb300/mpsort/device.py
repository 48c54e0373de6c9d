"""Device-memory entry points for records already in GPU memory.

Pointers are plain integers (e.g. ``torch.Tensor.data_ptr()``) and streams
are ``cudaStream_t`` values as integers (e.g. ``torch.cuda.Stream.cuda_stream``);
0 selects the library's own stream, which orders after work issued earlier on
the legacy default stream (torch's default stream).  Every call returns once the work is
enqueued on that stream.
"""
import ctypes

import numpy

from . import _lib


def _desc(dtype, orderby):
    return _lib.key_desc(dtype, orderby)


def sort(d_in, d_out, n, dtype, orderby, method="auto", stream=0, verify=False):
    """Sort n records of `dtype` from d_in into d_out by field `orderby`.
    verify=True hashes the records before and after (and waits); a result
    that is not a permutation of the input raises GBSortError."""
    dtype = numpy.dtype(dtype)
    desc = _desc(dtype, orderby)
    m = _lib.METHODS[method] | (_lib.VERIFY if verify else 0)
    _lib.check(_lib.lib().gbsort_sort_device(d_in, d_out, n, dtype.itemsize, ctypes.byref(desc), m, stream or None))


def take(d_source, nsource, d_index, nindex, dtype, d_out, stream=0):
    """out[i] = source[index[i]] for device records of `dtype` and int64
    device indices (waits; an index outside the source raises GBSortError)."""
    dtype = numpy.dtype(dtype)
    _lib.check(_lib.lib().gbsort_take_device(d_source, nsource, dtype.itemsize, d_index, nindex, d_out,
                                             stream or None))


def multiset_hash(d_records, n, dtype, d_hash, stream=0):
    """Order-independent 64-bit hash of n device records into the uint64 at
    d_hash (device memory); equal multisets of records hash equally."""
    dtype = numpy.dtype(dtype)
    _lib.check(_lib.lib().gbsort_multiset_hash_device(d_records, n, dtype.itemsize, d_hash, stream or None))


class Plan:
    """The sort of n records of `dtype` by `orderby` captured as one CUDA
    graph: ``plan.sort(d_in, d_out, stream)`` enqueues it (one graph launch,
    no host synchronisation), ``plan.wait()`` waits and raises on a device
    error.  The graph is re-captured when the buffers change.  With
    `segments` (nseg + 1 offsets) the plan is the segmented sort of that
    batch (``sort_segments``) and `n` is ignored."""

    def __init__(self, n, dtype, orderby, method="auto", segments=None):
        dtype = numpy.dtype(dtype)
        self._desc = _desc(dtype, orderby)
        self._h = ctypes.c_void_p()
        if segments is None:
            _lib.check(_lib.lib().gbsort_plan_create(ctypes.byref(self._h), n, dtype.itemsize,
                                                     ctypes.byref(self._desc), _lib.METHODS[method]))
        else:
            offs = numpy.ascontiguousarray(segments, dtype=numpy.uint64)
            _lib.check(_lib.lib().gbsort_plan_create_segments(ctypes.byref(self._h), offs.ctypes.data,
                                                              len(offs) - 1, dtype.itemsize,
                                                              ctypes.byref(self._desc), _lib.METHODS[method]))

    def sort(self, d_in, d_out, stream=0):
        _lib.check(_lib.lib().gbsort_plan_sort(self._h, d_in, d_out, stream or None))

    def wait(self):
        _lib.check(_lib.lib().gbsort_plan_wait(self._h))

    def close(self):
        if self._h:
            _lib.lib().gbsort_plan_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def autotune(n, dtype, orderby, d_records=0):
    """Time the candidate configurations on n records of `dtype` (the device
    records at d_records, read only, or pseudo-random ones) and store the
    fastest in the tuning table used by method='auto'.  Returns it as a dict."""
    dtype = numpy.dtype(dtype)
    desc = _desc(dtype, orderby)
    t = _lib.Tuning()
    _lib.check(_lib.lib().gbsort_autotune(n, dtype.itemsize, ctypes.byref(desc), d_records or None,
                                          ctypes.byref(t)))
    return t.as_dict()


def autotune_segments(offsets, dtype, orderby, d_records=0):
    """Time segmented sorts of this batch (level 2 as rounds / engine, three
    thresholds for sorting a segment on its own) and store the fastest in the
    segment tuning table.  Returns it as a dict."""
    dtype = numpy.dtype(dtype)
    desc = _desc(dtype, orderby)
    offs = numpy.ascontiguousarray(offsets, dtype=numpy.uint64)
    t = _lib.Tuning()
    _lib.check(_lib.lib().gbsort_autotune_segments(offs.ctypes.data, len(offs) - 1, dtype.itemsize,
                                                   ctypes.byref(desc), d_records or None, ctypes.byref(t)))
    return t.as_dict()


def tuning_get_segments(n, dtype, orderby):
    """The segment tuning entry for batches of n records, or None."""
    dtype = numpy.dtype(dtype)
    desc = _desc(dtype, orderby)
    t = _lib.Tuning()
    rc = _lib.lib().gbsort_tuning_get_segments(n, dtype.itemsize, ctypes.byref(desc), ctypes.byref(t))
    if rc == 6:
        return None
    _lib.check(rc)
    return t.as_dict()


def tuning_set(n, dtype, orderby, method, max_buckets=0, sample_per_bucket=0, level2="default"):
    dtype = numpy.dtype(dtype)
    desc = _desc(dtype, orderby)
    t = _lib.Tuning(_lib.METHODS[method], max_buckets, sample_per_bucket, 0.0, _lib.LEVEL2[level2])
    _lib.check(_lib.lib().gbsort_tuning_set(n, dtype.itemsize, ctypes.byref(desc), ctypes.byref(t)))


def tuning_get(n, dtype, orderby):
    """The table entry used for this shape, or None."""
    dtype = numpy.dtype(dtype)
    desc = _desc(dtype, orderby)
    t = _lib.Tuning()
    rc = _lib.lib().gbsort_tuning_get(n, dtype.itemsize, ctypes.byref(desc), ctypes.byref(t))
    if rc == 6:  # GBSORT_ERR_UNSUPPORTED: no entry
        return None
    _lib.check(rc)
    return t.as_dict()


def tuning_clear():
    _lib.check(_lib.lib().gbsort_tuning_clear())


def tuning_save(path):
    _lib.check(_lib.lib().gbsort_tuning_save(str(path).encode()))


def tuning_load(path):
    _lib.check(_lib.lib().gbsort_tuning_load(str(path).encode()))


def sort_segments(d_in, d_out, offsets, dtype, orderby, method="auto", stream=0):
    """Sort every segment [offsets[i], offsets[i+1]) of d_in independently."""
    dtype = numpy.dtype(dtype)
    desc = _desc(dtype, orderby)
    offs = numpy.ascontiguousarray(offsets, dtype=numpy.uint64)
    _lib.check(_lib.lib().gbsort_sort_segments_device(d_in, d_out, offs.ctypes.data, len(offs) - 1,
                                                      dtype.itemsize, ctypes.byref(desc),
                                                      _lib.METHODS[method], stream or None))


def merge_join(d_a, na, d_b, nb, dtype, orderby, d_pairs_a, d_pairs_b, d_npairs, stream=0):
    """Index pairs of equal keys of two key-sorted arrays (unique keys per side)."""
    dtype = numpy.dtype(dtype)
    desc = _desc(dtype, orderby)
    _lib.check(_lib.lib().gbsort_merge_join_device(d_a, na, d_b, nb, dtype.itemsize, ctypes.byref(desc),
                                                   d_pairs_a, d_pairs_b, d_npairs, stream or None))


def sort_host(a, orderby, out=None, method="auto"):
    """Host-array sort through the device pipeline (numpy in, numpy out)."""
    a = numpy.ascontiguousarray(a)
    if out is None:
        out = numpy.empty_like(a)
    desc = _desc(a.dtype, orderby)
    if len(a):
        _lib.check(_lib.lib().gbsort_sort_host(a.ctypes.data, out.ctypes.data, len(a), a.dtype.itemsize,
                                               ctypes.byref(desc), _lib.METHODS[method]))
    return out


def cdf_forward_backward(x, kmin, kmax, lbits, y):
    """Loss, predictions and knot gradient of the learned CDF on sorted keys x."""
    x = numpy.ascontiguousarray(x, dtype=numpy.uint64)
    y = numpy.ascontiguousarray(y, dtype=numpy.float32)
    loss = numpy.zeros(1, numpy.float32)
    pred = numpy.zeros(len(x), numpy.float32)
    grad = numpy.zeros(len(y), numpy.float32)
    _lib.check(_lib.lib().gbsort_cdf_forward_backward(x.ctypes.data, len(x), int(kmin), int(kmax), int(lbits),
                                                      y.ctypes.data, loss.ctypes.data, pred.ctypes.data,
                                                      grad.ctypes.data))
    return float(loss[0]), pred, grad


def cdf_train_gradient(x, kmin, kmax, lbits, y):
    """The training's gradient T y - b (statistics pass) at knots y."""
    x = numpy.ascontiguousarray(x, dtype=numpy.uint64)
    y = numpy.ascontiguousarray(y, dtype=numpy.float32)
    grad = numpy.zeros(len(y), numpy.float32)
    _lib.check(_lib.lib().gbsort_cdf_train_gradient(x.ctypes.data, len(x), int(kmin), int(kmax), lbits,
                                                    y.ctypes.data, grad.ctypes.data))
    return grad


def debug_buckets(sample, nbuckets, keys):
    """(full-search buckets, learned buckets, splitters, widest window)."""
    sample = numpy.ascontiguousarray(sample, dtype=numpy.uint64)
    keys = numpy.ascontiguousarray(keys, dtype=numpy.uint64)
    bs = numpy.zeros(len(keys), numpy.uint32)
    bl = numpy.zeros(len(keys), numpy.uint32)
    S = numpy.zeros(nbuckets - 1, numpy.uint64)
    w = ctypes.c_uint32(0)
    _lib.check(_lib.lib().gbsort_debug_buckets(sample.ctypes.data, len(sample), nbuckets, keys.ctypes.data,
                                               len(keys), bs.ctypes.data, bl.ctypes.data, S.ctypes.data,
                                               ctypes.byref(w)))
    return bs, bl, S, w.value


def debug_model(sample, nbuckets, keys, epochs):
    """Model trained for `epochs` steps: (full-search buckets, learned
    buckets, final loss, splitters read by the learned lookups, splitters read
    by the full searches, widest window)."""
    sample = numpy.ascontiguousarray(sample, dtype=numpy.uint64)
    keys = numpy.ascontiguousarray(keys, dtype=numpy.uint64)
    bs = numpy.zeros(len(keys), numpy.uint32)
    bl = numpy.zeros(len(keys), numpy.uint32)
    loss = ctypes.c_float(0)
    reads = numpy.zeros(2, numpy.uint64)
    w = ctypes.c_uint32(0)
    _lib.check(_lib.lib().gbsort_debug_model(sample.ctypes.data, len(sample), nbuckets, epochs, keys.ctypes.data,
                                             len(keys), bs.ctypes.data, bl.ctypes.data, ctypes.byref(loss),
                                             reads.ctypes.data, ctypes.byref(w)))
    return bs, bl, loss.value, int(reads[0]), int(reads[1]), w.value


def debug_bisect(sorted_keys, nsplit):
    """(splitters, CLT, CLE, rounds) of the device bisection splitter search."""
    x = numpy.ascontiguousarray(sorted_keys, dtype=numpy.uint64)
    S = numpy.zeros(nsplit, numpy.uint64)
    clt = numpy.zeros(nsplit, numpy.int64)
    cle = numpy.zeros(nsplit, numpy.int64)
    r = ctypes.c_uint32(0)
    _lib.check(_lib.lib().gbsort_debug_bisect(x.ctypes.data, len(x), nsplit, S.ctypes.data, clt.ctypes.data,
                                              cle.ctypes.data, ctypes.byref(r)))
    return S, clt, cle, r.value
