"""Multi-rank form of mpsort: the reference's distributed histogram sort.

The reference sorts an array spread over MPI ranks (mpsort-mpi.c:161-604):

  1. every rank sorts its chunk (radix_sort, mpsort-mpi.c:367);
  2. the global least and greatest keys and the target cumulative counts
     C[i] of the output partition (_find_Pmax_Pmin_C, mpsort-mpi.c:606-661);
  3. P - 1 splitters by bisection on key values, one round at a time: every
     rank counts its keys below (CLT) and not above (CLE) each candidate,
     the counts are summed over ranks, and a splitter is accepted once
     CLT < C <= CLE (piter_*, internal-parallel.h:128-248; the loop at
     mpsort-mpi.c:385-437);
  4. the send counts: each receiver takes every key below its splitter and
     fills the rest of its quota from the senders in rank order among the
     keys equal to the splitter (_solve_for_layout_mpi, mpsort-mpi.c:663-727),
     which keeps equal keys in global input order;
  5. one exchange of records (MPIU_Alltoallv, mp-mpiu.c:69-156), then a
     stable sort of what each rank received (ordered by sender).

Here the local sorts of steps 1 and 5 run on each rank's GPU through
libgbsort, and the collectives are torch.distributed's (gloo for host
arrays, nccl when the group's backend is nccl).  The result is the same as
the reference's: the global stable order by key, cut into the ranks' output
lengths.  Keys are one integer field (u8, i8, u4, i4); vector keys sort on
one rank only.

take / permute of several ranks exchange requests and records directly: each
rank sends every index it wants to the rank holding that record and gets
the records back in two all-to-all exchanges (the reference reaches the same
result through two or three distributed sorts, mpsort/__init__.py:116-204).
"""
import numpy

_SIGN = numpy.uint64(1 << 63)


class ProcessGroupComm(object):
    """The collectives the multi-rank calls use, over a torch.distributed
    process group (None: the default group).  Host arrays in, host arrays
    out; with the nccl backend the buffers pass through the current device."""

    def __init__(self, group=None):
        import torch.distributed as dist
        self._dist = dist
        self._group = group
        self.rank = dist.get_rank(group)
        self.size = dist.get_world_size(group)
        self._device = "cuda" if dist.get_backend(group) == "nccl" else "cpu"

    def _tensor(self, a):
        import torch
        return torch.from_numpy(numpy.ascontiguousarray(a)).to(self._device)

    def allreduce_sum(self, a):
        t = self._tensor(numpy.asarray(a, dtype=numpy.int64))
        self._dist.all_reduce(t, group=self._group)
        return t.cpu().numpy()

    def allgather_array(self, a):
        """Arrays of one length per rank, stacked by rank."""
        import torch
        t = self._tensor(numpy.asarray(a, dtype=numpy.int64).reshape(-1))
        out = torch.empty(self.size * t.numel(), dtype=t.dtype, device=t.device)
        self._dist.all_gather_into_tensor(out, t, group=self._group)
        return out.cpu().numpy().reshape(self.size, -1)

    def allgather_int(self, x):
        return [int(v) for v in self.allgather_array([x])[:, 0]]

    def alltoall_int(self, a):
        """a[j] goes to rank j; returns what every rank sent this one."""
        import torch
        t = self._tensor(numpy.asarray(a, dtype=numpy.int64))
        out = torch.empty_like(t)
        self._dist.all_to_all_single(out, t, group=self._group)
        return out.cpu().numpy()

    def alltoallv_bytes(self, send, counts):
        """send[ranges of counts[j] bytes, in rank order] to rank j; returns the
        bytes received, ordered by sender."""
        import torch
        counts = numpy.asarray(counts, dtype=numpy.int64)
        recv_counts = self.alltoall_int(counts)
        t = self._tensor(numpy.ascontiguousarray(send).view(numpy.uint8).reshape(-1))
        out = torch.empty(int(recv_counts.sum()), dtype=torch.uint8, device=t.device)
        self._dist.all_to_all_single(out, t, [int(x) for x in recv_counts], [int(x) for x in counts],
                                     group=self._group)
        return out.cpu().numpy()


class _OneRank(object):
    rank = 0
    size = 1


def as_comm(comm):
    """A communicator the module can use: a ProcessGroupComm (or any object
    with its methods) as is, a torch.distributed ProcessGroup wrapped, and
    one-rank communicators of other kinds (e.g. mpi4py's COMM_SELF) as a
    one-rank stand-in."""
    if comm is None:
        return _OneRank()
    if hasattr(comm, "alltoallv_bytes"):
        return comm
    try:
        import torch.distributed as dist
        if isinstance(comm, dist.ProcessGroup):
            return ProcessGroupComm(comm)
    except ImportError:
        pass
    size = getattr(comm, "size", None)
    if size is None and hasattr(comm, "Get_size"):
        size = comm.Get_size()
    if size == 1:
        return _OneRank()
    raise NotImplementedError("communicators of %s ranks other than torch.distributed process groups "
                              "are not supported" % size)


def radix_u64(arr, orderby):
    """The order-preserving uint64 of a one-integer key field
    (mpsort/binding.pyx:81-121: u8 as is, u4 zero-extended, i8 / i4
    sign-extended and offset by 2^63)."""
    k = arr[orderby]
    if k.ndim != 1:
        raise NotImplementedError("vector keys sort on one rank only")
    kind = k.dtype
    if kind == numpy.dtype('u8'):
        return k.astype(numpy.uint64, copy=False)
    if kind == numpy.dtype('u4'):
        return k.astype(numpy.uint64)
    if kind in (numpy.dtype('i8'), numpy.dtype('i4')):
        return k.astype(numpy.int64).view(numpy.uint64) ^ _SIGN
    raise TypeError("data[%s] is not u8 or i8" % (orderby,))


def _gpu_sort(arr, orderby, method="auto"):
    from . import _sort_records
    _sort_records(arr, orderby, arr, None, [], method, False)


def bisect_splitters(keys, C, comm):
    """The P - 1 splitters of the output partition C (cumulative counts,
    P + 1 entries) by bisection over key values, one round of counts summed
    over ranks at a time; returns (splitters, my CLT, my CLE, rounds)."""
    P = comm.size
    n = len(keys)
    # global least and greatest key among ranks holding data
    ends = comm.allgather_array([n, int(keys[0].view(numpy.int64)) if n else 0,
                                 int(keys[-1].view(numpy.int64)) if n else 0])
    have = ends[:, 0] > 0
    lo_all = ends[have, 1].view(numpy.uint64) if have.any() else numpy.zeros(1, numpy.uint64)
    hi_all = ends[have, 2].view(numpy.uint64) if have.any() else numpy.zeros(1, numpy.uint64)
    pmin, pmax = lo_all.min(), hi_all.max()
    ns = P - 1
    left = numpy.full(ns, pmin, dtype=numpy.uint64)
    right = numpy.full(ns, pmax, dtype=numpy.uint64)
    stable = numpy.zeros(ns, dtype=bool)
    narrow = numpy.zeros(ns, dtype=bool)
    trial = numpy.zeros(ns, dtype=numpy.uint64)
    C = numpy.asarray(C, dtype=numpy.int64)

    def counts(S):
        lt = numpy.concatenate([[0], numpy.searchsorted(keys, S, side='left'), [n]]).astype(numpy.int64)
        le = numpy.concatenate([[0], numpy.searchsorted(keys, S, side='right'), [n]]).astype(numpy.int64)
        return lt, le

    rounds = 0
    while ns and not stable.all():
        rounds += 1
        todo = ~stable
        last = todo & narrow            # the range is down to [left, right]: try right itself
        trial[last] = right[last]
        stable[last] = True
        mid = todo & ~narrow
        trial[mid] = left[mid] + ((right[mid] - left[mid]) >> numpy.uint64(1))
        narrow[mid & (trial <= left)] = True
        my_lt, my_le = counts(trial)
        lt = comm.allreduce_sum(my_lt)
        le = comm.allreduce_sum(my_le)
        ok = (lt[1:P] < C[1:P]) & (C[1:P] <= le[1:P])
        stable |= ok
        too_big = ~ok & (lt[1:P] >= C[1:P])
        right[too_big] = trial[too_big]
        too_small = ~ok & ~too_big
        left[too_small] = trial[too_small]
    my_lt, my_le = counts(trial)
    return trial, my_lt, my_le, rounds


def solve_layout(C, t_lt, t_le, rank):
    """Cumulative counts this rank takes from each sender: everything below
    its splitter (t_lt[j] from sender j), the rest of its quota C[rank + 1]
    from the keys equal to the splitter, senders in rank order."""
    take = numpy.array(t_lt, dtype=numpy.int64)
    deficit = int(C[rank + 1]) - int(take.sum())
    for j in range(len(take)):
        if deficit <= 0:
            break
        extra = min(int(t_le[j]) - int(take[j]), deficit)
        if extra < 0:
            raise RuntimeError("inconsistent splitter counts")
        take[j] += extra
        deficit -= extra
    if deficit != 0:
        raise RuntimeError("the splitters do not bracket the output partition")
    return take


def sort_records(data, orderby, out, comm, method="auto", local_sort=None):
    """Global stable sort of the records spread over the ranks of comm, by
    field `orderby`, into each rank's `out` (lengths may differ from the
    input's; the totals must agree).  local_sort(array, orderby) sorts one
    rank's records in place, stably; the default is this rank's GPU."""
    c = as_comm(comm)
    P, r = c.size, c.rank
    sort_local = local_sort or (lambda a, f: _gpu_sort(a, f, method))
    n, nout = len(data), len(out)
    sizes = c.allgather_int(n)
    outsizes = c.allgather_int(nout)
    if sum(sizes) != sum(outsizes):
        raise ValueError("total size of array changed %d != %d" % (sum(sizes), sum(outsizes)))
    if n:
        sort_local(data, orderby)  # data ends locally sorted, as the reference's does
    keys = radix_u64(data, orderby)
    C = numpy.concatenate([[0], numpy.cumsum(outsizes)]).astype(numpy.int64)
    S, my_lt, my_le, rounds = bisect_splitters(keys, C, c)
    # what every sender holds below / up to this rank's splitter
    t_lt = c.alltoall_int(my_lt[1:P + 1])
    t_le = c.alltoall_int(my_le[1:P + 1])
    take = solve_layout(C, t_lt, t_le, r)
    # my records' cumulative boundaries per receiver
    bounds = numpy.concatenate([[0], c.alltoall_int(take)]).astype(numpy.int64)
    if bounds[-1] != n:
        raise RuntimeError("send layout covers %d of %d records" % (bounds[-1], n))
    item = data.dtype.itemsize
    recv = c.alltoallv_bytes(data.view(numpy.uint8).reshape(-1), numpy.diff(bounds) * item)
    if len(recv) != nout * item:
        raise RuntimeError("received %d records, expected %d" % (len(recv) // item, nout))
    out.view(numpy.uint8).reshape(-1)[...] = recv
    if nout:
        sort_local(out, orderby)  # runs from lower ranks first: stable over the whole array
    sort_records.last_rounds = rounds
    return out


def take(source, argindex, comm, out, local_take=None):
    """out[i] = global_source[argindex[i]] over the ranks of comm: requests go
    to the ranks holding the records, the records come back.
    local_take(array, local_indices) gathers from this rank's chunk (default:
    the device gather)."""
    c = as_comm(comm)
    P = c.size
    lens = numpy.array(c.allgather_int(len(source)), dtype=numpy.int64)
    ends = numpy.cumsum(lens)
    start = int(ends[c.rank] - lens[c.rank])
    idx = numpy.asarray(argindex, dtype=numpy.int64).reshape(-1)
    if len(idx) and (idx.min() < 0 or idx.max() >= ends[-1]):
        raise IndexError("index out of range for a global array of %d records" % ends[-1])
    owner = numpy.searchsorted(ends, idx, side='right')
    order = numpy.argsort(owner, kind='stable')
    want = numpy.bincount(owner, minlength=P).astype(numpy.int64)
    asked = c.alltoallv_bytes(idx[order].view(numpy.uint8), want * 8).view(numpy.int64)
    if local_take is None:
        from . import _take_device
        mine = numpy.empty(len(asked), dtype=source.dtype)
        _take_device(source, asked - start, mine)
    else:
        mine = local_take(source, asked - start)
    item = source.dtype.itemsize
    asked_by = c.alltoall_int(want)  # how many records each rank asked of this one, in the order asked
    got = c.alltoallv_bytes(numpy.ascontiguousarray(mine).view(numpy.uint8), asked_by * item)
    res = numpy.empty(len(idx), dtype=source.dtype)
    res[order] = got.view(source.dtype)
    out[...] = res
    return out
