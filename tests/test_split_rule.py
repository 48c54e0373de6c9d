"""The bucket split's grouping rule, restated in NumPy, against the property
the split rounds rely on to end: every group that is split again covers a
strictly narrower key range than its bucket (CPU only).

Rule (split_task in mp-sort_gb300/csrc/hsort.cu): with exclusive-scanned bin
counts h and m records, bin b goes to group floor((h[b] + h[b+1]) / (2 t)),
t = min(max(1792, ceil(m / 512)), m / 2), capped at 511; bins past the last
used bin belong to no group.  Refined bins are the same rule over finer
bins, so the check runs on both kinds of histograms.
"""
import numpy


def groups(counts):
    counts = numpy.asarray(counts, dtype=numpy.int64)
    m = int(counts.sum())
    h = numpy.concatenate([[0], numpy.cumsum(counts)])
    t = min(max(2048 - 2048 // 8, -(-m // 512)), m // 2)
    mid2 = h[:-1] + h[1:]
    return numpy.minimum(mid2 // (2 * t), 511), m, t


def check(counts):
    g, m, t = groups(counts)
    nb = len(counts)
    assert (numpy.diff(g) >= 0).all()  # groups are runs of consecutive bins
    for gid in numpy.unique(g):
        bins = numpy.nonzero(g == gid)[0]
        size = int(numpy.asarray(counts)[bins].sum())
        if size > 2048:  # split again: its range must be narrower than the bucket's
            assert not (bins[0] == 0 and bins[-1] == nb - 1), (gid, size, m, t)


def test_grouping_narrows_on_random_histograms():
    rng = numpy.random.default_rng(5)
    for _ in range(300):
        nb = int(rng.integers(2, 4097))
        m = int(rng.integers(4096, 2_000_000))
        kind = rng.integers(0, 4)
        if kind == 0:    # uniform
            counts = rng.multinomial(m, numpy.full(nb, 1.0 / nb))
        elif kind == 1:  # one crowded bin
            p = numpy.full(nb, 0.2 / nb)
            p[rng.integers(0, nb)] += 0.8
            counts = rng.multinomial(m, p / p.sum())
        elif kind == 2:  # the first and the last bin only
            counts = numpy.zeros(nb, numpy.int64)
            counts[0] = m // 2
            counts[-1] = m - m // 2
        else:            # clusters
            p = rng.random(nb) ** 8
            counts = rng.multinomial(m, p / p.sum())
        check(counts)


def test_everything_in_one_bin_is_alone():
    for nb in (2, 3, 100, 4096):
        for b in (0, nb // 2, nb - 1):
            counts = numpy.zeros(nb, numpy.int64)
            counts[b] = 1_000_000
            g, _, _ = groups(counts)
            assert (g == g[b]).sum() == 1 or nb == 1, (nb, b)
