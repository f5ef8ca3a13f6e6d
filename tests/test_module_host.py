"""The drop-in module's host types, no GPU needed: diaQMatrix, vector and the numpy conversions
(include/pythonWrappers.cpp:41-109, :146-228 of the reference), checked against numpy's own view
of the same dense matrices -- the round trips of python_tests/test_api_vs_numpy.py that need no
device."""
import numpy as np
import pytest


@pytest.fixture(scope="module")
def d():
    from diaq_gb300 import build

    build.build()
    from diaq_gb300 import diaq_gpu

    return diaq_gpu


def _banded(rng, rows, cols, offsets):
    D = np.zeros((rows, cols), complex)
    for o in offsets:
        r0, c0 = (0, o) if o >= 0 else (-o, 0)
        n = min(rows - r0, cols - c0)
        if n > 0:
            D[np.arange(r0, r0 + n), np.arange(c0, c0 + n)] = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    return D


def _nonzero_diagonals(D):
    rows, cols = D.shape
    return [o for o in range(-(rows - 1), cols) if np.any(np.diagonal(D, o) != 0)]


SHAPES = [(1, 1, [0]), (8, 8, [0, -1, 3, 7, -7]), (5, 9, [-4, 0, 2, 8]), (9, 5, [-8, -3, 0, 4]),
          (16, 16, [-15, 15]), (6, 6, []), (3, 11, [10]), (12, 2, [-11, 1])]


@pytest.mark.parametrize("rows,cols,offsets", SHAPES)
def test_from_numpy_to_numpy_round_trip(d, rows, cols, offsets):
    rng = np.random.default_rng(rows * 100 + cols)
    D = _banded(rng, rows, cols, offsets)
    A = d.from_numpy(D)
    assert list(A.matrix_shape) == [rows, cols]
    assert list(A.dIndices) == _nonzero_diagonals(D)   # ascending, exactly the nonzero diagonals
    assert A.num_diags() == len(A.dIndices)
    assert A.totalLength == sum(np.diagonal(D, o).size for o in A.dIndices)
    assert np.array_equal(d.to_numpy(A), D)
    # the flat overload with an explicit shape builds the same matrix
    F = d.from_numpy(D.ravel(), [rows, cols])
    assert list(F.dIndices) == list(A.dIndices) and np.array_equal(d.to_numpy(F), D)


def test_packed_layout_and_items(d):
    rng = np.random.default_rng(3)
    D = _banded(rng, 7, 10, [-6, -2, 0, 5, 9])
    A = d.from_numpy(D)
    off, re, im = A.diagonal_data()
    assert list(off) == [-6, -2, 0, 5, 9]
    starts = list(A.diagOffsets)
    for k, o in enumerate(off):   # diagonals back to back in slot order, real and imaginary apart
        seg = np.diagonal(D, o)
        assert starts[k] == sum(np.diagonal(D, p).size for p in off[:k])
        assert np.array_equal(re[starts[k]:starts[k] + seg.size], seg.real)
        assert np.array_equal(im[starts[k]:starts[k] + seg.size], seg.imag)
    for i in range(7):
        for j in range(10):
            assert A.getItem([i, j]) == D[i, j]


def test_set_at_diag_prune_and_copy(d):
    A = d.diaQMatrix([5, 5], [-2, 0, 1, 3])
    assert A.totalLength == 3 + 5 + 4 + 2
    A.set_at_diag(1, 2, 0.5, -2.0)
    A.set_at_diag(-2, 0, 3.0, 0.0)
    B = A.copy()
    B.set_at_diag(0, 4, 9.0, 9.0)   # a deep copy: A is unchanged
    assert A.getItem([4, 4]) == 0 and B.getItem([4, 4]) == 9 + 9j
    A.pruneMatrix()
    assert list(A.dIndices) == [-2, 1]
    want = np.zeros((5, 5), complex)
    want[2, 3] = 0.5 - 2j
    want[2, 0] = 3.0
    assert np.array_equal(d.to_numpy(A), want)
    assert A.sparsity() == pytest.approx(1 - 2 / 25)
    with pytest.raises(RuntimeError, match="not present"):
        A.set_at_diag(0, 0, 1.0, 0.0)
    with pytest.raises(RuntimeError):
        A.set_at_diag(1, 4, 1.0, 0.0)   # diagonal +1 of a 5x5 matrix has 4 entries


def test_symmetric_constructor_order(d):
    """diaQMatrix(size, numDiags) lays its diagonals out as 0, -1, +1, -2, +2, ...
    (src/diaQMatrix.hpp:24-39)."""
    assert list(d.diaQMatrix(8, 5).dIndices) == [0, -1, 1, -2, 2]
    assert list(d.diaQMatrix(4, 1).dIndices) == [0]


def test_vector_round_trip(d):
    rng = np.random.default_rng(5)
    x = rng.standard_normal(37) + 1j * rng.standard_normal(37)
    v = d.from_numpy_vector(x)
    assert v.numRows == 37
    assert np.array_equal(d.to_numpy_vector(v), x)
    w = v.copy()
    assert np.array_equal(d.to_numpy_vector(w), x)
    assert d.vector(4).numRows == 4


def test_from_diagonals_and_errors(d):
    A = d.from_diagonals(4, 4, [1, -1], np.arange(6.0), np.zeros(6))
    D = d.to_numpy(A)
    assert D[0, 1] == 0 and D[2, 3] == 2 and D[1, 0] == 3 and D[3, 2] == 5
    with pytest.raises(RuntimeError, match="must hold 6 values"):
        d.from_diagonals(4, 4, [1, -1], np.arange(5.0), np.zeros(5))
    with pytest.raises(RuntimeError, match="outside the matrix"):
        d.diaQMatrix([4, 4], [4])
    with pytest.raises(RuntimeError, match="shape does not match"):
        d.from_numpy(np.zeros(6, complex), [4, 2])
    with pytest.raises(RuntimeError, match="2-D"):
        d.from_numpy(np.zeros((2, 2, 2), complex))
