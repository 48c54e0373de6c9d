"""The multi-rank sort and take (mpsort.distributed) on CPU ranks (gloo).

The host logic of the reference's distributed histogram sort -- splitter
bisection with counts summed over ranks, the layout solve, the record
exchange -- runs on 2 and 3 gloo ranks; each rank's local sorts use the
oracle's stable sort here (on a GPU machine they run on the rank's GPU).  The
result must equal the oracle's stable sort of the whole array, cut into the
ranks' output lengths, record for record.
"""
import os
import socket
import sys

import numpy
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _chunks(P, seed, kind):
    """Each rank's input chunk and output length (uneven on purpose)."""
    rng = numpy.random.default_rng(seed)
    lens = rng.integers(0, 3000, P)
    lens[seed % P] = 0  # an empty rank
    total = int(lens.sum())
    cut = numpy.sort(rng.integers(0, total + 1, P - 1))
    outlens = numpy.diff(numpy.concatenate([[0], cut, [total]]))
    dt = [('key', 'i8'), ('val', 'i8')] if kind == "i8" else [('key', 'u4'), ('val', 'u4')]
    parts = []
    base = 0
    for p in range(P):
        a = numpy.zeros(lens[p], dtype=dt)
        if kind == "i8":
            a['key'] = rng.integers(-40, 40, lens[p]) * (1 << 40)  # heavy duplicates, signed
        else:
            a['key'] = rng.integers(0, 2**32, lens[p], dtype=numpy.uint64).astype('u4')
        a['val'] = numpy.arange(base, base + lens[p])
        base += lens[p]
        parts.append(a)
    return parts, outlens


def _worker(rank, world, port, seed, kind, results):
    sys.path.insert(0, os.path.join(REPO, "mp-sort_gb300"))
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import torch.distributed as dist
    import oracle as O
    from mpsort import distributed as D
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank, world_size=world)
    comm = D.ProcessGroupComm()
    parts, outlens = _chunks(world, seed, kind)
    mine = parts[rank].copy()
    out = numpy.zeros(outlens[rank], dtype=mine.dtype)

    def local_sort(a, f):
        a[...] = O.numpy_sorted(a, f)

    D.sort_records(mine, 'key', out, comm, local_sort=local_sort)
    results[("sort", rank)] = out.tobytes()
    results[("input_sorted", rank)] = mine.tobytes()
    # take: each rank asks for records anywhere in the global array (repeats allowed)
    rng = numpy.random.default_rng(seed + rank)
    total = sum(len(p) for p in parts)
    want = rng.integers(0, total, 500) if total else numpy.zeros(0, numpy.int64)
    got = numpy.zeros(len(want), dtype=mine.dtype)
    D.take(parts[rank], want, comm, got, local_take=lambda a, i: a[i])
    results[("take", rank)] = (want.tobytes(), got.tobytes())
    dist.destroy_process_group()


@pytest.mark.parametrize("world,seed,kind", [(2, 1, "i8"), (3, 2, "i8"), (3, 5, "u4"), (2, 4, "u4")])
def test_distributed_sort_and_take_match_oracle(world, seed, kind):
    import torch.multiprocessing as mp
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    import oracle as O
    manager = mp.Manager()
    results = manager.dict()
    mp.spawn(_worker, args=(world, _port(), seed, kind, results), nprocs=world, join=True)
    parts, outlens = _chunks(world, seed, kind)
    whole = numpy.concatenate(parts)
    expect = O.numpy_sorted(whole, 'key')
    starts = numpy.concatenate([[0], numpy.cumsum(outlens)])
    for r in range(world):
        got = numpy.frombuffer(results[("sort", r)], dtype=whole.dtype)
        assert got.tobytes() == expect[starts[r]:starts[r + 1]].tobytes(), r
        # as in the reference, each rank's input ends locally sorted
        assert results[("input_sorted", r)] == O.numpy_sorted(parts[r], 'key').tobytes()
        want, tk = results[("take", r)]
        want = numpy.frombuffer(want, dtype=numpy.int64)
        assert numpy.frombuffer(tk, dtype=whole.dtype).tobytes() == whole[want].tobytes(), r


def test_layout_solver_fills_from_lower_ranks():
    sys.path.insert(0, os.path.join(REPO, "mp-sort_gb300"))
    from mpsort import distributed as D
    # three senders; ranks 0 and 1 together receive 10 records: 3 lie below
    # rank 1's splitter, the other 7 come from keys equal to it, senders in
    # rank order (2 from sender 0, 3 from sender 1, 2 from sender 2)
    C = numpy.array([0, 4, 10, 15])
    take = D.solve_layout(C, t_lt=[1, 1, 1], t_le=[3, 4, 5], rank=1)
    assert list(take) == [3, 4, 3]
    with pytest.raises(RuntimeError):  # the equal keys cannot make up the quota
        D.solve_layout(C, t_lt=[1, 1, 1], t_le=[1, 2, 2], rank=1)
