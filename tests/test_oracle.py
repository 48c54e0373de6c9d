"""The oracle pinned against the reference's golden vectors (CPU only)."""
import ctypes

import numpy
import pytest

import oracle as O
from conftest import golden_cases


def test_oracle_matches_golden(golden):
    for name, arr, out, orderby in golden_cases(golden):
        assert O.oracle_sort(arr, orderby).tobytes() == out.tobytes(), name
        assert O.numpy_sorted(arr, orderby).tobytes() == out.tobytes(), name


@pytest.mark.parametrize("tasks", [1, 2, 3, 4, 7])
def test_oracle_mpsort_matches_golden(golden, tasks):
    for name, arr, out, orderby in golden_cases(golden):
        assert O.oracle_mpsort(arr, orderby, tasks).tobytes() == out.tobytes(), (name, tasks)


def test_oracle_callback_int_unsigned_compare(golden):
    ints = golden["cb_int__in"]
    order = numpy.argsort(ints.view('u4'), kind='stable')
    assert ints[order].tobytes() == golden["cb_int__out"].tobytes()


def test_reference_build_agrees_live(golden):
    if O.ref_lib() is None:
        pytest.skip("reference build absent")
    for name, arr, out, orderby in golden_cases(golden):
        assert O.ref_sort(arr, orderby, "omp").tobytes() == out.tobytes(), name


def test_bisect_and_compare_semantics():
    lib = O.oracle_lib()
    rng = numpy.random.default_rng(5)
    for rsize in (2, 4, 8, 16, 24, 3, 5):
        for _ in range(200):
            a = rng.integers(0, 256, rsize).astype(numpy.uint8)
            b = rng.integers(0, 256, rsize).astype(numpy.uint8)
            ia = int.from_bytes(a.tobytes(), 'little')
            ib = int.from_bytes(b.tobytes(), 'little')
            c = lib.oracle_compar(a.ctypes.data, b.ctypes.data, rsize)
            assert c == (ia > ib) - (ia < ib)
            lo, hi = (a, b) if ia <= ib else (b, a)
            r = numpy.zeros(rsize, numpy.uint8)
            lib.oracle_bisect(r.ctypes.data, lo.ctypes.data, hi.ctypes.data, rsize)
            ilo, ihi = min(ia, ib), max(ia, ib)
            assert int.from_bytes(r.tobytes(), 'little') == ilo + ((ihi - ilo) >> 1)


def test_layout_solver_brackets():
    """_solve_for_layout invariants on a random bracket set."""
    lib = O.oracle_lib()
    rng = numpy.random.default_rng(11)
    T = 5
    keys = numpy.sort(rng.integers(0, 6, 57)).astype('u8')
    chunks = numpy.array_split(numpy.sort(rng.permutation(keys)), T)
    chunks = [numpy.sort(c) for c in numpy.array_split(rng.permutation(keys), T)]
    n = len(keys)
    C = numpy.array([n * i // T for i in range(T + 1)], dtype=numpy.int64)
    P = numpy.sort(keys)[C[1:T] - 1 + 0].astype('u8')  # splitter = value at target rank
    GL_CLT = numpy.zeros((T + 1, T + 1), numpy.int64)
    GL_CLE = numpy.zeros((T + 1, T + 1), numpy.int64)
    for t, c in enumerate(chunks):
        GL_CLT[t, 0] = 0
        GL_CLE[t, 0] = 0
        for i, p in enumerate(P):
            GL_CLT[t, i + 1] = numpy.searchsorted(c, p, 'left')
            GL_CLE[t, i + 1] = numpy.searchsorted(c, p, 'right')
        GL_CLT[t, T] = GL_CLE[t, T] = len(c)
    GL_C = numpy.zeros_like(GL_CLT)
    assert lib.oracle_solve_layout(T, C.ctypes.data, GL_CLT.ctypes.data,
                                   GL_CLE.ctypes.data, GL_C.ctypes.data) == 0
    recv = (GL_C[:T, 1:] - GL_C[:T, :-1]).sum(axis=0)
    assert (recv == numpy.diff(C)).all()
    assert (GL_C[:T] >= GL_CLT[:T]).all() and (GL_C[:T] <= GL_CLE[:T]).all()


def test_cdf_oracle_gradient_matches_finite_differences():
    """The NumPy model oracle (the checker of the device's forward and
    backward kernels): its analytic gradient equals central differences of
    its loss at every knot, for uniform, narrow and clustered keys."""
    import cdf_oracle
    rng = numpy.random.default_rng(17)
    cases = ((5, rng.integers(0, 2**64, 3000, dtype=numpy.uint64, endpoint=False)),
             (4, rng.integers(10**6, 10**6 + 700, 3000).astype(numpy.uint64)),
             (6, (rng.normal(0, 1e9, 3000) + 2**62).astype(numpy.uint64)))
    for lbits, keys in cases:
        x = numpy.sort(keys)
        y = numpy.sort(rng.random((1 << lbits) + 1))
        y[0], y[-1] = 0.0, 1.0
        kmin, kmax = int(x[0]), int(x[-1])
        loss, pred, grad = cdf_oracle.forward_backward(x, kmin, kmax, lbits, y)
        assert pred.shape == x.shape and grad.shape == y.shape
        h = 1e-6
        for j in range(len(y)):
            yp, ym = y.copy(), y.copy()
            yp[j] += h
            ym[j] -= h
            fd = (cdf_oracle.forward_backward(x, kmin, kmax, lbits, yp)[0] -
                  cdf_oracle.forward_backward(x, kmin, kmax, lbits, ym)[0]) / (2 * h)
            assert abs(fd - grad[j]) <= 1e-5 * max(abs(fd), 1e-3), (lbits, j, fd, grad[j])
