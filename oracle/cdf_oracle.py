"""NumPy restatement of the learned CDF model's forward and backward passes.
TEST INFRASTRUCTURE ONLY: the checker for the device kernels in
mp-sort_gb300/csrc/cdf.cu (gradient check).

Model: leaves L = 2**lbits uniform in (key - kmin) >> lshift, with
lshift = max(0, bitlen(kmax - kmin) - lbits); leaf j interpolates linearly
between knots y[j] and y[j+1]; targets r_i = i / s over the sorted keys;
loss = mean (F(x_i) - r_i)^2.
"""
import numpy


def shape(kmin, kmax, lbits):
    bits = int(kmax - kmin).bit_length() if kmax > kmin else 0
    return int(kmin), max(0, bits - lbits), lbits


def features(x, kmin, lshift, lbits):
    x = numpy.asarray(x, dtype=numpy.uint64)
    nleaf = 1 << lbits
    below = x < numpy.uint64(kmin)
    d = (x - numpy.uint64(kmin)).astype(numpy.uint64)
    d[below] = 0
    leaf = (d >> numpy.uint64(lshift)).astype(numpy.uint64)
    if lshift:
        frac = (d & numpy.uint64((1 << lshift) - 1)).astype(numpy.float64) / float(1 << lshift)
    else:
        frac = numpy.zeros(len(x))
    over = leaf >= nleaf
    leaf = numpy.minimum(leaf, nleaf - 1).astype(numpy.int64)
    frac[over] = 1.0
    frac[below] = 0.0
    return leaf, frac.astype(numpy.float32)


def forward_backward(x, kmin, kmax, lbits, y):
    """(loss, predictions, gradient) in float64 arithmetic."""
    kmin_, lshift, lbits = shape(kmin, kmax, lbits)
    y = numpy.asarray(y, dtype=numpy.float64)
    s = len(x)
    leaf, frac = features(x, kmin_, lshift, lbits)
    frac = frac.astype(numpy.float64)
    pred = y[leaf] + frac * (y[leaf + 1] - y[leaf])
    r = numpy.arange(s, dtype=numpy.float64) / s
    e = pred - r
    loss = float(numpy.mean(e * e))
    g = 2.0 * e / s
    grad = numpy.zeros(len(y))
    numpy.add.at(grad, leaf, g * (1.0 - frac))
    numpy.add.at(grad, leaf + 1, g * frac)
    return loss, pred, grad
