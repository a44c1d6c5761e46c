"""Symmetric upper-triangle CSR matrix and the linear-system container.

Python mirror of the reference's container types:

* ``SymmetricCSRMatrix``        CAESolvers/SymmetricCSRMatrix.cs:19-425
* ``SymmetricCSRMatrixBuilder`` CAESolvers/SymmetricCSRMatrixBuilder.cs:11-51
* ``MatrixEntry``               CAESolvers/CSRMatrixBuilder.cs:50-75
* ``LinearSystem``              CAESolvers/LinearSystem.cs:6-23

Construction (normalisation to (min, max), ordered summation of duplicates,
the 1e-15 drop) runs in the native host library so that the structure fed to
the symbolic phase is exactly what the reference would build.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Iterable

import numpy as np

from . import _native
from .errors import (ArgumentException, ArgumentNullException, ArgumentOutOfRangeException,
                     IndexOutOfRangeException, InvalidOperationException, raise_for_status)


@dataclass(frozen=True)
class MatrixEntry:
    Row: int
    Col: int
    Value: float


class SymmetricCSRMatrix:
    """Immutable-structure symmetric matrix stored as its upper triangle (row <= col).

    Columns are strictly ascending inside a row, so the diagonal, when it is
    structurally present, is the first entry of its row.
    """

    def __init__(self, size: int, elements: Iterable = ()):
        if size < 0:
            raise ArgumentOutOfRangeException("size")
        rows, cols, vals = [], [], []
        for e in elements:
            if isinstance(e, MatrixEntry):
                rows.append(e.Row), cols.append(e.Col), vals.append(e.Value)
            else:
                r, c, v = e
                rows.append(r), cols.append(c), vals.append(v)
        self._from_triplets(size, np.asarray(rows, np.int32), np.asarray(cols, np.int32), np.asarray(vals, np.float64))

    # -- construction -------------------------------------------------------
    def _from_triplets(self, size, rows, cols, vals):
        lib = _native.host()
        h = C.c_void_p()
        rows = np.ascontiguousarray(rows, np.int32)
        cols = np.ascontiguousarray(cols, np.int32)
        vals = np.ascontiguousarray(vals, np.float64)
        if len(rows) and (rows.min() < 0 or cols.min() < 0 or rows.max() >= size or cols.max() >= size):
            raise IndexOutOfRangeException("Indices are out of range.")
        st = lib.uchol_csr_from_triplets(size, len(rows), _native.ptr(rows), _native.ptr(cols),
                                         _native.ptr(vals, C.c_double), C.byref(h))
        raise_for_status(st, lib.uchol_host_last_error())
        self._adopt(h)

    def _adopt(self, h):
        lib = _native.host()
        try:
            n, nnz = C.c_int(), C.c_int()
            raise_for_status(lib.uchol_csr_shape(h, C.byref(n), C.byref(nnz)), lib.uchol_host_last_error())
            self._size = n.value
            self._row_ptr = np.zeros(n.value + 1, np.int32)
            self._col = np.zeros(nnz.value, np.int32)
            self._val = np.zeros(nnz.value, np.float64)
            self._diag = np.zeros(n.value, np.int32)
            raise_for_status(lib.uchol_csr_copy(h, _native.ptr(self._row_ptr), _native.ptr(self._col),
                                                _native.ptr(self._val, C.c_double), _native.ptr(self._diag)),
                             lib.uchol_host_last_error())
        finally:
            lib.uchol_csr_destroy(h)

    @classmethod
    def from_triplets(cls, size, rows, cols, values) -> "SymmetricCSRMatrix":
        m = cls.__new__(cls)
        m._from_triplets(size, rows, cols, values)
        return m

    @classmethod
    def _from_handle(cls, h) -> "SymmetricCSRMatrix":
        m = cls.__new__(cls)
        m._adopt(h)
        return m

    # -- structure ------------------------------------------------------------
    @property
    def Size(self) -> int:
        return self._size

    RowCount = Size
    ColumnCount = Size

    @property
    def NonZeroCount(self) -> int:
        return int(self._col.shape[0])

    @property
    def RowPointers(self) -> np.ndarray:
        return self._row_ptr

    @property
    def ColumnIndices(self) -> np.ndarray:
        return self._col

    @property
    def Values(self) -> np.ndarray:
        """Values of the stored half; the array reflects AccumulateAt / indexer writes."""
        return self._val

    @property
    def DiagonalIndices(self) -> np.ndarray:
        return self._diag

    def _check(self, row, col):
        if row < 0 or row >= self._size or col < 0 or col >= self._size:
            raise IndexOutOfRangeException(f"Indices are out of range: ({row}, {col}).")

    def _find(self, row, col) -> int:
        if row > col:
            row, col = col, row
        if row == col:
            return int(self._diag[row])
        lo, hi = self._row_ptr[row], self._row_ptr[row + 1]
        k = lo + int(np.searchsorted(self._col[lo:hi], col))
        return k if k < hi and self._col[k] == col else -1

    def __getitem__(self, rc):
        row, col = rc
        self._check(row, col)
        k = self._find(row, col)
        return float(self._val[k]) if k >= 0 else 0.0

    def __setitem__(self, rc, value):
        row, col = rc
        self._check(row, col)
        k = self._find(row, col)
        if k < 0:
            raise InvalidOperationException(f"Position ({min(row, col)}, {max(row, col)}) is absent from the sparse structure.")
        self._val[k] = value

    def IsZero(self, row, col) -> bool:
        self._check(row, col)
        return self._find(row, col) < 0

    def AccumulateAt(self, row: int, col: int, value: float) -> None:
        """Adds to an existing structural position (SymmetricCSRMatrix.cs:98-110)."""
        self._check(row, col)
        k = self._find(row, col)
        if k < 0:
            raise InvalidOperationException(
                f"Position ({min(row, col)}, {max(row, col)}) is absent from the sparse structure. "
                "Add this position to SymmetricSparseMatrixCSRBuilder before assembly.")
        self._val[k] += value

    def ClearValues(self) -> None:
        self._val[:] = 0.0

    def GetDiagonal(self, row: int) -> float:
        if row < 0 or row >= self._size:
            raise IndexOutOfRangeException(f"Row index {row} is out of range.")
        k = self._diag[row]
        return float(self._val[k]) if k >= 0 else 0.0

    def LineCross(self, right_hand_side, prescribed_value: float, index: int) -> None:
        """Dirichlet condition keeping the structure (SymmetricCSRMatrix.cs:125-167)."""
        if right_hand_side is None:
            raise ArgumentNullException("rightHandSide")
        if len(right_hand_side) != self._size:
            raise ArgumentException(
                f"The right-hand side length {len(right_hand_side)} does not match the matrix size {self._size}.",
                "rightHandSide")
        if index < 0 or index >= self._size:
            raise ArgumentOutOfRangeException("index")
        di = self._diag[index]
        if di < 0:
            raise InvalidOperationException(f"Diagonal position ({index}, {index}) is absent from the sparse structure.")
        rows = np.repeat(np.arange(self._size, dtype=np.int64), np.diff(self._row_ptr))
        hit = ((rows == index) | (self._col == index)) & (rows != self._col)
        for k in np.nonzero(hit)[0]:
            other = self._col[k] if rows[k] == index else rows[k]
            right_hand_side[other] -= self._val[k] * prescribed_value
            self._val[k] = 0.0
        self._val[di] = 1.0
        right_hand_side[index] = prescribed_value

    def Multiply(self, vector) -> np.ndarray:
        """Symmetric product from the stored half, FP64 (SymmetricCSRMatrix.cs:259-283)."""
        x = np.asarray(vector, dtype=np.float64)
        if x.shape[0] != self._size:
            raise ArgumentException(f"Vector length {x.shape[0]} does not match the matrix size {self._size}.")
        rows = np.repeat(np.arange(self._size), np.diff(self._row_ptr))
        off = rows != self._col
        y = np.zeros((self._size,) + x.shape[1:], np.float64)
        if x.ndim == 1:
            np.add.at(y, rows, self._val * x[self._col])
            np.add.at(y, self._col[off], self._val[off] * x[rows[off]])
        else:
            np.add.at(y, rows, self._val[:, None] * x[self._col])
            np.add.at(y, self._col[off], self._val[off, None] * x[rows[off]])
        return y

    def GetRow(self, row: int) -> dict:
        if row < 0 or row >= self._size:
            raise IndexOutOfRangeException(f"Row index {row} is out of range.")
        out = {int(self._col[k]): float(self._val[k]) for k in range(self._row_ptr[row], self._row_ptr[row + 1])}
        for c in range(row):
            k = self._find(c, row)
            if k >= 0:
                out[c] = float(self._val[k])
        return dict(sorted(out.items()))

    def to_dense(self) -> np.ndarray:
        a = np.zeros((self._size, self._size))
        rows = np.repeat(np.arange(self._size), np.diff(self._row_ptr))
        a[rows, self._col] = self._val
        a[self._col, rows] = self._val
        return a


class SymmetricCSRMatrixBuilder:
    """Accumulates (row, col) += value with (min, max) normalisation; Build() creates the matrix."""

    def __init__(self, size: int):
        self._size = size
        self._r, self._c, self._v = [], [], []

    def AddToElement(self, row: int, col: int, value: float) -> None:
        if row < 0 or row >= self._size or col < 0 or col >= self._size:
            raise IndexOutOfRangeException(f"Indices are out of range: ({row}, {col}).")
        self._r.append(row)
        self._c.append(col)
        self._v.append(value)

    def Build(self) -> SymmetricCSRMatrix:
        return SymmetricCSRMatrix.from_triplets(self._size, np.asarray(self._r, np.int32),
                                                np.asarray(self._c, np.int32), np.asarray(self._v, np.float64))


class LinearSystem:
    """A matrix and its right-hand side (CAESolvers/LinearSystem.cs:8-17)."""

    def __init__(self, matrix, right_hand_side):
        if matrix is None:
            raise ArgumentNullException("matrix")
        if right_hand_side is None:
            raise ArgumentNullException("rightHandSide")
        rhs = np.asarray(right_hand_side, dtype=np.float64)
        if matrix.RowCount != rhs.shape[0]:
            raise ArgumentException("The right-hand side length does not match the matrix row count.", "rightHandSide")
        self.Matrix = matrix
        self.RightHandSide = rhs
