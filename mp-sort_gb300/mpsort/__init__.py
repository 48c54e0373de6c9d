"""mpsort -- MP-sort's Python interface, served by the GB300 histogram sort.

Functions, arguments and errors follow the reference module
(mpsort/__init__.py): ``sort``, ``permute``, ``take``, ``histogram``,
``globalrange`` and ``globalindices``.

  * With ``comm=None`` (or any communicator of one rank) the data lives in
    this process and every call runs on the current CUDA device through
    libgbsort.so: the sort is the device histogram sort, take / permute a
    device gather.
  * With a communicator of several ranks -- a torch.distributed process
    group, or any object with the small interface of
    ``mpsort.distributed.ProcessGroupComm`` -- each rank holds a chunk of the
    global array and the calls are the reference's distributed algorithms
    (mpsort.distributed): local sorts on each rank's GPU, splitters by
    bisection with a sum over ranks of the counts per round, one exchange
    of records.

There is no CPU path: without the built library the import of the ctypes
binding raises, and without a device the calls raise GBSortError.
"""
import ctypes

import numpy

from . import _lib
from ._lib import GBSortError, last_stats  # noqa: F401

__version__ = "0.3.0"

_TUNING_FLAGS = {  # the reference's option bits (mpsort.h:17-20)
    'DISABLE_SPARSE_ALLTOALLV': 1 << 1,
    'DISABLE_GATHER_SORT': 1 << 3,
    'REQUIRE_GATHER_SORT': 1 << 4,
    'REQUIRE_SPARSE_ALLTOALLV': 1 << 6,
}


def _ranks(comm):
    """(rank, size) of a communicator; None is one rank."""
    if comm is None:
        return 0, 1
    from . import distributed
    c = distributed.as_comm(comm)
    return c.rank, c.size


def _multi(comm):
    return comm is not None and _ranks(comm)[1] > 1


def _apply_tuning(tuning):
    L = _lib.lib()
    L.mpsort_mpi_unset_options(-1)
    for name in tuning:
        if name in _TUNING_FLAGS:
            L.mpsort_mpi_set_options(_TUNING_FLAGS[name])


def _sort_records(data, orderby, out, comm, tuning, method, verify):
    """Sort of a structured array by one of its fields (the binding's sort,
    mpsort/binding.pyx:123-209): the same argument checks and errors."""
    data[orderby]  # an unknown field raises here, as in the reference
    if not data.flags['C_CONTIGUOUS']:
        raise ValueError("data must be C_CONTIGUOUS")
    if out is None:
        out = data
    if not out.flags['C_CONTIGUOUS']:
        raise ValueError("out must be C_CONTIGUOUS")
    if data.dtype.itemsize != out.dtype.itemsize:
        raise ValueError("item size mismatch")
    _apply_tuning(tuning)
    if _multi(comm):
        from . import distributed
        return distributed.sort_records(data, orderby, out, comm, method=method)
    if len(data) != len(out):
        raise ValueError("total size of array changed %d != %d" % (len(data), len(out)))
    desc = _lib.key_desc(data.dtype, orderby)
    if len(data):
        m = _lib.METHODS[method] | (_lib.VERIFY if verify else 0)
        _lib.check(_lib.lib().gbsort_sort_host(data.ctypes.data, out.ctypes.data, len(data),
                                               data.dtype.itemsize, ctypes.byref(desc), m))
    return out


def _as_array(x):
    """The array behind x (a flat iterator stands for its base array)."""
    return x.base if isinstance(x, numpy.flatiter) else x


def sort(source, orderby=None, out=None, comm=None, tuning=[], method="auto", verify=False):
    """Sort `source` by `orderby` into `out`, stably.

    source   1-d array (or its .flat), a chunk of the global array when comm
             has several ranks.
    orderby  None: the values of source themselves; a field name of a
             structured source; or an array of keys, one per record.  Keys are
             integers (u8, i8, u4, i4) or 1-d vectors of them, compared with
             the last element most significant.
    out      where the sorted records go (None: in place); its global length
             must equal the source's, its item size the source's.
    comm     None / one rank, or a multi-rank communicator (see the module).
    tuning   the reference's flags: 'DISABLE_SPARSE_ALLTOALLV',
             'DISABLE_GATHER_SORT', 'REQUIRE_GATHER_SORT',
             'REQUIRE_SPARSE_ALLTOALLV' (stored; they steer MPI exchanges).
    method   'auto', 'plain', 'learned' or 'lsd': the device algorithm; every
             method gives the same order.
    verify   True: also check that the result is a permutation of the input
             (an order-independent hash of the records before and after).

    Returns out.
    """
    if isinstance(orderby, (str, bytes)):
        return _sort_records(source, orderby, out, comm, tuning, method, verify)
    src = _as_array(source)
    dst = src if out is None else _as_array(out)
    vdt = (src.dtype, src.shape[1:])
    if orderby is None:  # the values are their own keys: one-field records
        rec = numpy.empty(len(src), dtype=[('v', vdt)])
        rec['v'][...] = src
        res = rec if out is None else numpy.empty(len(dst), dtype=rec.dtype)
        _sort_records(rec, 'v', res, comm, tuning, method, verify)
        dst[...] = res['v']
        return out if out is not None else source
    keys = _as_array(orderby)
    rec = numpy.empty(len(src), dtype=[('v', vdt), ('k', (keys.dtype, keys.shape[1:]))])
    rec['v'][...] = src
    rec['k'][...] = keys
    res = numpy.empty(len(dst), dtype=rec.dtype)
    _sort_records(rec, 'k', res, comm, tuning, method, verify)
    dst[...] = res['v']
    return out if out is not None else source


def globalrange(array, comm):
    """[start, end) of this rank's chunk in the global array."""
    rank, size = _ranks(comm)
    if size == 1:
        return (0, len(array))
    from . import distributed
    lens = distributed.as_comm(comm).allgather_int(len(array))
    start = int(sum(lens[:rank]))
    return (start, start + int(lens[rank]))


def globalindices(array, comm):
    """Global indices of this rank's chunk: int64 when the global array has
    more than 2^30 records, else int32 (as the reference chooses)."""
    rank, size = _ranks(comm)
    start, end = globalrange(array, comm)
    total = end if size == 1 else int(sum(_distributed_lens(array, comm)))
    return numpy.arange(start, end, dtype='i8' if total > (1 << 30) else 'i4')


def _distributed_lens(array, comm):
    from . import distributed
    return distributed.as_comm(comm).allgather_int(len(array))


def guess_dtype(array):
    """(dtype, shape of one item) of an array or of a flat iterator's base."""
    a = _as_array(array)
    return (a.dtype, () if isinstance(array, numpy.flatiter) else a.shape[1:])


def take(source, argindex, comm, out=None):
    """out[i] = global_source[argindex[i]]: the records of the global array at
    the global indices argindex, partitioned as argindex (indices may repeat
    and need not cover the array)."""
    argindex = numpy.asarray(argindex)
    if out is None:
        out = numpy.empty(len(argindex), guess_dtype(source))
    if _multi(comm):
        from . import distributed
        return distributed.take(source, argindex, comm, out)
    return _take_device(source, argindex, out)


def permute(source, argindex, comm, out=None):
    """source[argindex] where argindex is a permutation of the global
    indices, partitioned as argindex."""
    rank, size = _ranks(comm)
    if size == 1:
        n_src, n_idx = len(source), len(argindex)
    else:
        from . import distributed
        c = distributed.as_comm(comm)
        n_src, n_idx = sum(c.allgather_int(len(source))), sum(c.allgather_int(len(argindex)))
    if n_src != n_idx:
        raise ValueError("Global size of source and argindex is different")
    return take(source, argindex, comm, out)


def histogram(array, bins, comm, right=False):
    """Global count of array values in each bin of the edges `bins` (len(bins)
    + 1 counts, numpy.digitize's convention, summed over ranks)."""
    bins = numpy.asarray(bins)
    a = numpy.asarray(array)
    where = numpy.searchsorted(bins, a, side='left' if right else 'right') if len(a) else numpy.zeros(0, int)
    counts = numpy.bincount(where, minlength=len(bins) + 1).astype('i8')
    if _multi(comm):
        from . import distributed
        counts = distributed.as_comm(comm).allreduce_sum(counts)
    return counts


def _take_device(source, argindex, out):
    """One process: the source and the indices go to the device, the gather
    runs there (gbsort_take_device), the records come back into out."""
    import torch  # device buffers only; the gather is libgbsort's kernel
    src = numpy.ascontiguousarray(_as_array(source))
    idx = numpy.ascontiguousarray(argindex, dtype=numpy.int64)
    item = src.dtype.itemsize * int(numpy.prod(src.shape[1:], dtype=numpy.int64))
    dst = _as_array(out)
    if len(idx) == 0:
        return out
    d_src = torch.from_numpy(src.reshape(-1).view(numpy.uint8)).cuda()
    d_idx = torch.from_numpy(idx).cuda()
    d_out = torch.empty(len(idx) * item, dtype=torch.uint8, device='cuda')
    _lib.check(_lib.lib().gbsort_take_device(d_src.data_ptr() if len(src) else None, len(src), item,
                                             d_idx.data_ptr(), len(idx), d_out.data_ptr(), None))
    dst.reshape(-1).view(numpy.uint8)[...] = d_out.cpu().numpy()
    return out
