"""mpsort -- the MP-sort Python API (mpsort/__init__.py) on the GB300 sort.

Same names, arguments and errors as the reference module for one process:
``sort``, ``permute``, ``take``, ``histogram``, ``globalrange``,
``globalindices``.  The sort runs on the current CUDA device through
libgbsort.so; the reference ran it over MPI ranks.  ``comm`` may be None or
any communicator of size 1 (e.g. mpi4py's COMM_SELF); larger communicators
raise NotImplementedError, since the multi-rank exchange is not part of this
single-GPU library.
"""
import ctypes

import numpy

from . import _lib
from ._lib import GBSortError, last_stats  # noqa: F401

__version__ = "0.2.0"

_TUNING_FLAGS = {
    'DISABLE_SPARSE_ALLTOALLV': 1 << 1,
    'DISABLE_GATHER_SORT': 1 << 3,
    'REQUIRE_GATHER_SORT': 1 << 4,
    'REQUIRE_SPARSE_ALLTOALLV': 1 << 6,
}


class _SelfComm(object):
    """Stand-in for a one-rank communicator (rank 0 of 1)."""
    rank = 0
    size = 1

    def allreduce(self, x, op=None):
        return x

    def allgather(self, x):
        return [x]

    def bcast(self, x, root=0):
        return x

    def barrier(self):
        pass


def _comm(comm):
    if comm is None:
        return _SelfComm()
    size = getattr(comm, "size", None)
    if size is None and hasattr(comm, "Get_size"):
        size = comm.Get_size()
    if size != 1:
        raise NotImplementedError("mpsort on GB300 sorts within one process; "
                                  "communicators with %s ranks are not supported" % size)
    return comm


def _sort(data, orderby=None, out=None, comm=None, tuning=[], method="auto"):
    """The binding's sort (mpsort/binding.pyx:123-209) for one rank."""
    key = data[orderby]  # noqa: F841 -- raises as the reference does for a bad field

    if not data.flags['C_CONTIGUOUS']:
        raise ValueError("data must be C_CONTIGUOUS")
    if out is None:
        out = data
    if not out.flags['C_CONTIGUOUS']:
        raise ValueError("out must be C_CONTIGUOUS")
    comm = _comm(comm)
    Ntot = comm.allreduce(len(data))
    Ntotout = comm.allreduce(len(out))
    if Ntot != Ntotout:
        raise ValueError("total size of array changed %d != %d" % (Ntot, Ntotout))
    if data.dtype.itemsize != out.dtype.itemsize:
        raise ValueError("item size mismatch")

    desc = _lib.key_desc(data.dtype, orderby)
    L = _lib.lib()
    L.mpsort_mpi_unset_options(-1)
    for name, flag in _TUNING_FLAGS.items():
        if name in tuning:
            L.mpsort_mpi_set_options(flag)
    if len(data) == 0:
        return out
    _lib.check(L.gbsort_sort_host(data.ctypes.data, out.ctypes.data, len(data),
                                  data.dtype.itemsize, ctypes.byref(desc),
                                  _lib.METHODS[method]))
    return out


def sort(source, orderby=None, out=None, comm=None, tuning=[], method="auto"):
    """
        Sort source array with orderby as the key.
        Store result to out.

        Parameters
        ----------
        source : array, 1d

        orderby : array, 1d, or string.
            Only integer types are supported.
            If orderby is string, it refers to the field in source.

        out : array, 1d
            the total length must be the same as source.
            the itemsize must be the same as source
            if None, the sort is in-place.

        tuning: list of strings
            'DISABLE_SPARSE_ALLTOALLV', 'DISABLE_GATHER_SORT',
            'REQUIRE_GATHER_SORT', 'REQUIRE_SPARSE_ALLTOALLV'
            (accepted; they steer the MPI exchange, which one GPU does not have)

        method : 'auto', 'plain', 'learned' or 'lsd' (GPU algorithm; the
            result is the same stable order for every method)

        Returns
        -------
            out
    """
    key = orderby
    if isinstance(key, (str, bytes)):
        return _sort(source, key, out, comm=comm, tuning=tuning, method=method)

    if key is None:
        D, I = 'DD'
        data1 = numpy.empty(len(source), dtype=[('D', guess_dtype(source))])
        data1['D'][...] = source
    else:
        D, I = 'DI'
        data1 = numpy.empty(len(source), dtype=[('D', guess_dtype(source)),
                                                ('I', guess_dtype(key))])
        data1['D'][...] = source
        data1['I'][...] = key

    if out is None:
        out = source
        _sort(data1, orderby=I, comm=comm, tuning=tuning, method=method)
        out[...] = data1[D][...]
    else:
        data2 = numpy.empty(len(out), dtype=data1.dtype)
        _sort(data1, orderby=I, out=data2, comm=comm, tuning=tuning, method=method)
        out[...] = data2[D][...]
    return out


def globalrange(array, comm):
    """The start and end of local chunk in the global array."""
    comm = _comm(comm)
    s = comm.allgather(len(array))
    start = sum(s[:comm.rank])
    end = start + s[comm.rank]
    return (start, end)


def globalindices(array, comm):
    """Construct a list of indices in the global array."""
    comm = _comm(comm)
    start, end = globalrange(array, comm)
    globalsize = comm.bcast(end, root=comm.size - 1)
    dtype = 'i8' if globalsize > 1024 * 1024 * 1024 else 'i4'
    return numpy.arange(start, end, dtype=dtype)


def guess_dtype(array):
    if isinstance(array, numpy.flatiter):
        array = array.base
        return array.dtype, ()
    return array.dtype, array.shape[1:]


def permute(source, argindex, comm, out=None):
    """source[argindex], partitioned as argindex (two sorts, as in the
    reference, mpsort/__init__.py:116-149)."""
    comm = _comm(comm)
    source_size = comm.allreduce(len(source))
    argindex_size = comm.allreduce(len(argindex))
    if source_size != argindex_size:
        raise ValueError("Global size of source and argindex is different")
    if out is None:
        out = numpy.empty(len(argindex), guess_dtype(source))
    originind = globalindices(argindex, comm)
    originind2 = numpy.empty(len(source), dtype=originind.dtype)
    sort(originind, orderby=argindex, out=originind2, comm=comm)
    sort(source, orderby=originind2, out=out, comm=comm)
    return out


def histogram(array, bins, comm, right=False):
    """Histogram of array over bin edges (mpsort/__init__.py:151-172)."""
    comm = _comm(comm)
    if len(array) == 0:
        originrank = []
    else:
        originrank = numpy.digitize(array, bins, right)
    recv = numpy.bincount(originrank, minlength=len(bins) + 1)
    return comm.allreduce(recv)


def take(source, argindex, comm, out=None):
    """source[argindex] partitioned as argindex; argindex need not be a
    permutation nor unique (mpsort/__init__.py:174-204)."""
    comm = _comm(comm)
    start, end = globalrange(source, comm)
    bins = comm.allgather(end)
    h = histogram(argindex, bins, comm)
    nactive = h[comm.rank]
    if out is None:
        out = numpy.empty(len(argindex), guess_dtype(source))
    originind = globalindices(argindex, comm)
    myargindex = numpy.empty(nactive, dtype=guess_dtype(argindex))
    myoriginind = numpy.empty(nactive, dtype=originind.dtype)
    sort(originind, orderby=argindex, out=myoriginind, comm=comm)
    sort(argindex, orderby=argindex, out=myargindex, comm=comm)
    myresult = source[myargindex - start]
    sort(myresult, orderby=myoriginind, out=out, comm=comm)
    return out
