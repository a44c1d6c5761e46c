"""Matrix construction semantics of the reference's SymmetricCSRMatrix
(CAESolvers/SymmetricCSRMatrix.cs) and the synthetic generators."""
import numpy as np
import pytest

import oracle
from magla_gb300 import (ArgumentException, IndexOutOfRangeException, InvalidOperationException, LinearSystem,
                         MatrixEntry, SymmetricCSRMatrix, SymmetricCSRMatrixBuilder)
from magla_gb300 import generators as G


def test_normalisation_duplicates_and_drop():
    m = SymmetricCSRMatrix(3, [MatrixEntry(1, 0, 2.0), MatrixEntry(0, 1, 3.0), (2, 2, 1.0), (0, 2, 1e-16),
                               (1, 2, 0.5), (2, 1, -0.5), (0, 0, 4.0)])
    # (0,1) and (1,0) merge to 5; (1,2)+(2,1) cancel to 0 and are dropped; 1e-16 is dropped
    assert m.NonZeroCount == 3
    assert m[0, 1] == 5.0 and m[1, 0] == 5.0
    assert m.IsZero(1, 2) and m.IsZero(0, 2)
    assert m.RowPointers.tolist() == [0, 2, 2, 3]
    assert m.ColumnIndices.tolist() == [0, 1, 2]
    assert m.GetDiagonal(1) == 0.0 and m.GetDiagonal(0) == 4.0


def test_diagonal_first_in_row():
    m = G.grid_matrix(3, 3, 3, 2)
    for r in range(m.Size):
        k0 = m.RowPointers[r]
        assert m.ColumnIndices[k0] == r
        assert np.all(np.diff(m.ColumnIndices[k0:m.RowPointers[r + 1]]) > 0)


def test_multiply_matches_dense_and_reference_order():
    m = G.elasticity(3, 2, 2)[0]
    x = np.random.default_rng(1).uniform(-1, 1, m.Size)
    y = m.Multiply(x)
    assert np.allclose(y, m.to_dense() @ x, rtol=1e-13, atol=1e-13)
    assert np.allclose(y, oracle.multiply(m, x), rtol=1e-13, atol=1e-13)


def test_accumulate_and_indexer():
    m = G.grid_matrix(2, 2, 2, 1)
    v = m[0, 1]
    m.AccumulateAt(1, 0, 2.0)
    assert m[0, 1] == v + 2.0
    with pytest.raises(InvalidOperationException):
        m.AccumulateAt(0, 7, 1.0)
    with pytest.raises(IndexOutOfRangeException):
        m.AccumulateAt(0, 8, 1.0)
    m[2, 0] = 9.0
    assert m[0, 2] == 9.0
    m.ClearValues()
    assert np.all(m.Values == 0.0)


def test_line_cross_keeps_structure():
    m = G.grid_matrix(3, 3, 1, 1)
    nnz = m.NonZeroCount
    b = np.ones(m.Size)
    m.LineCross(b, 2.0, 4)
    assert m.NonZeroCount == nnz
    assert m[4, 4] == 1.0
    assert b[4] == 2.0
    for j in range(m.Size):
        if j != 4:
            assert m[4, j] == 0.0


def test_builder_and_linear_system():
    b = SymmetricCSRMatrixBuilder(2)
    b.AddToElement(0, 0, 1.0)
    b.AddToElement(0, 1, 0.5)
    b.AddToElement(1, 0, 0.5)
    b.AddToElement(1, 1, 2.0)
    m = b.Build()
    assert m[0, 1] == 1.0
    with pytest.raises(IndexOutOfRangeException):
        b.AddToElement(2, 0, 1.0)
    with pytest.raises(ArgumentException):
        LinearSystem(m, np.zeros(3))


def test_elasticity_clamped_face_is_identity_rows():
    m, load = G.elasticity(2, 2, 2)
    d = m.to_dense()
    for node in range(9):  # z = 0 face of a 3x3x3 node grid
        for c in range(3):
            i = 3 * node + c
            assert d[i, i] == 1.0
            assert np.count_nonzero(d[i]) == 1
            assert load[i] == 0.0
    assert np.allclose(d, d.T)
    assert np.all(np.linalg.eigvalsh(d) > 0)


def test_laplacian_sizes():
    m = G.laplacian3d(20, 20, 20)
    assert m.Size == 8000 and m.NonZeroCount == 8000 + 3 * 19 * 20 * 20
    m2 = G.laplacian2d(16, 9, np.full(256, 0.05))
    assert m2.Size == 256 and m2.GetDiagonal(0) == 8.05
