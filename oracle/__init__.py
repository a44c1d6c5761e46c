"""ORACLE — test infrastructure only (tests, smoke check, CPU baseline).

Python wrapper of ``oracle_numeric.cpp``, the CPU restatement of the
reference's numeric phase (CAESolvers/UCHOL/UtduNumericFactorization.cs),
and of ``oracle_values.cpp``, the restatement of the values-refresh
operations of CAESolvers/SymmetricCSRMatrix.cs (AccumulateAt, LineCross)
and of the Jacobi-preconditioned CG of
CAESolvers/CGGP/ConjugateGradientGaussPreSolver.cs.
It consumes the symbolic arrays of a ``UtduSymbolicFactorization`` exactly
as the reference's numeric phase consumes its symbolic object.  The product
(``magla_gb300``) never imports this package.

Pinned against the reference's own known answers in
``tests/test_oracle_pins.py`` (diagonal systems, zero right-hand side, the
4x4 interface system, the 8x8 workbook system with its exact solution and
LDL^T factors, the regularisation and negative-pivot cases).
"""
from __future__ import annotations

import ctypes as C
import os
import threading

import numpy as np

from . import build as _build

_LIB = None
_LOCK = threading.Lock()
_ip = C.POINTER(C.c_int)
_dp = C.POINTER(C.c_double)


def lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            path = _build.build()
            L = C.CDLL(str(path))
            L.oracle_factorize.restype = C.c_int
            L.oracle_factorize.argtypes = [C.c_int, C.c_int] + [_ip] * 12 + [
                C.c_int, _dp, C.c_int, C.c_double, C.c_double, C.c_int, C.c_longlong, C.c_int,
                C.POINTER(C.c_void_p), _ip, _ip, _dp, _dp, _ip]
            L.oracle_diagonal.argtypes = [C.c_void_p, _dp]
            L.oracle_block.argtypes = [C.c_void_p, C.c_int, _dp]
            L.oracle_solve.argtypes = [C.c_void_p, _ip, _dp, _dp]
            L.oracle_destroy.argtypes = [C.c_void_p]
            L.oracle_destroy.restype = None
            L.oracle_last_error.restype = C.c_char_p
            L.oracle_residual_norm.restype = C.c_double
            L.oracle_residual_norm.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp]
            L.oracle_multiply.argtypes = [C.c_int, _ip, _ip, _dp, _dp, _dp]
            L.oracle_multiply.restype = None
            L.oracle_accumulate.restype = C.c_int
            L.oracle_accumulate.argtypes = [C.c_int, _ip, _ip, _ip, _dp, C.c_int, _ip, _ip, _dp, _ip]
            L.oracle_line_cross.restype = C.c_int
            L.oracle_line_cross.argtypes = [C.c_int, _ip, _ip, _ip, _dp, _dp, C.c_double, C.c_int]
            L.oracle_jacobi_pcg.restype = C.c_int
            L.oracle_jacobi_pcg.argtypes = [C.c_int, _ip, _ip, _ip, _dp, _dp, _dp, C.c_double, C.c_int, C.c_int,
                                            C.c_double, _dp, _ip]
            _LIB = L
        return _LIB


def _i(a):
    a = np.ascontiguousarray(a, np.int32)
    return a, a.ctypes.data_as(_ip)


def _d(a):
    a = np.ascontiguousarray(a, np.float64)
    return a, a.ctypes.data_as(_dp)


class OracleError(RuntimeError):
    def __init__(self, status, message, column=-1):
        super().__init__(message)
        self.status = status
        self.column = column


class OracleFactor:
    """CPU multifrontal U^T D U of the reference (see module docstring)."""

    def __init__(self, symbolic, values, allow_regularization=True, pivot_tolerance=1e-13,
                 diagonal_regularization=1e-10, panel_width=32, parallel_threshold=1 << 20, workers=None):
        L = lib()
        a = symbolic.arrays
        self.n = symbolic.Size
        self.count = symbolic.SupernodeCount
        self.permutation = a["PERMUTATION"].copy()
        self.front_ptr = a["FRONT_PTR"].copy()
        self.first_column = a["FIRST_COLUMN"].copy()
        keep = []
        args = []
        for name in ("DIAG_VALUE_INDEX", "PATTERN_PTR", "PATTERN_ROWS", "LOWER_START", "LOWER_VALUE_PTR",
                     "LOWER_VALUE_INDEX", "FIRST_COLUMN", "SN_PARENT", "CHILD_PTR", "CHILDREN", "FRONT_PTR",
                     "FRONT_ROWS"):
            arr, p = _i(a[name])
            keep.append(arr)
            args.append(p)
        vals, vp = _d(values)
        h = C.c_void_p()
        reg, neg, failed = C.c_int(), C.c_int(), C.c_int()
        small, large = C.c_double(), C.c_double()
        workers = workers or (os.cpu_count() or 1)
        st = L.oracle_factorize(self.n, self.count, *args, max(1, symbolic.MaxFrontSize), vp,
                                1 if allow_regularization else 0, pivot_tolerance, diagonal_regularization,
                                panel_width, parallel_threshold, workers, C.byref(h), C.byref(reg), C.byref(neg),
                                C.byref(small), C.byref(large), C.byref(failed))
        if st != 0:
            raise OracleError(st, L.oracle_last_error().decode(), failed.value)
        self._h = h
        self.RegularizedPivotCount = reg.value
        self.NegativePivotCount = neg.value
        self.SmallestPivotMagnitude = small.value
        self.LargestPivotMagnitude = large.value

    @property
    def IsPositiveDefinite(self):
        return self.RegularizedPivotCount == 0 and self.NegativePivotCount == 0

    @property
    def Diagonal(self):
        d = np.zeros(self.n)
        lib().oracle_diagonal(self._h, d.ctypes.data_as(_dp))
        return d

    def block(self, s):
        m = int(self.front_ptr[s + 1] - self.front_ptr[s])
        w = int(self.first_column[s + 1] - self.first_column[s])
        out = np.zeros(m * w - w * (w - 1) // 2)
        lib().oracle_block(self._h, s, out.ctypes.data_as(_dp))
        return out

    def Solve(self, b):
        b = np.asarray(b, np.float64)
        if b.ndim == 2:
            return np.stack([self.Solve(b[:, j]) for j in range(b.shape[1])], axis=1)
        perm, pp = _i(self.permutation)
        bb, bp = _d(b)
        x = np.zeros(self.n)
        lib().oracle_solve(self._h, pp, bp, x.ctypes.data_as(_dp))
        return x

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _LIB is not None:
            _LIB.oracle_destroy(h)
            self._h = None


def residual_norm(matrix, b, x) -> float:
    """||b - A x||_2 with the reference's product order (SymmetricCSRMatrix.Multiply)."""
    rp, rpp = _i(matrix.RowPointers)
    cp, cpp = _i(matrix.ColumnIndices)
    v, vp = _d(matrix.Values)
    bb, bp = _d(b)
    xx, xp = _d(x)
    return float(lib().oracle_residual_norm(matrix.Size, rpp, cpp, vp, bp, xp))


def multiply(matrix, x) -> np.ndarray:
    rp, rpp = _i(matrix.RowPointers)
    cp, cpp = _i(matrix.ColumnIndices)
    v, vp = _d(matrix.Values)
    xx, xp = _d(x)
    y = np.zeros(matrix.Size)
    lib().oracle_multiply(matrix.Size, rpp, cpp, vp, xp, y.ctypes.data_as(_dp))
    return y


class _Csr:
    """The structure and a private copy of the values of a SymmetricCSRMatrix."""

    def __init__(self, matrix):
        self.n = matrix.Size
        self.rp, self.rpp = _i(matrix.RowPointers)
        self.cp, self.cpp = _i(matrix.ColumnIndices)
        self.dg, self.dgp = _i(matrix.DiagonalIndices)
        self.val = np.array(matrix.Values, np.float64)
        self.vp = self.val.ctypes.data_as(_dp)


def accumulate(matrix, rows, cols, items):
    """Values after AccumulateAt(rows[i], cols[i], items[i]) in order; raises
    OracleError(1) for an index out of range, OracleError(2) for an absent
    position (``column`` = the item)."""
    m = _Csr(matrix)
    r, rp = _i(rows)
    c, cp = _i(cols)
    v, vp = _d(items)
    bad = C.c_int()
    st = lib().oracle_accumulate(m.n, m.rpp, m.cpp, m.dgp, m.vp, len(r), rp, cp, vp, C.byref(bad))
    if st:
        raise OracleError(st, "index out of range" if st == 1 else "position absent from the structure", bad.value)
    return m.val


def line_cross(matrix, rhs, prescribed, indices):
    """(values, rhs) after LineCross(rhs, prescribed[t], indices[t]) for t in order;
    rhs may have several columns (one LineCross sequence per column, the values
    taken from the first)."""
    rhs = np.array(rhs, np.float64)
    cols = rhs.reshape(rhs.shape[0], -1)
    pres = np.asarray(prescribed, np.float64).reshape(len(indices), -1)
    out_val = None
    for j in range(cols.shape[1]):
        m = _Csr(matrix)
        b = np.ascontiguousarray(cols[:, j])
        for t, k in enumerate(indices):
            st = lib().oracle_line_cross(m.n, m.rpp, m.cpp, m.dgp, m.vp, b.ctypes.data_as(_dp),
                                         float(pres[t, j]), int(k))
            if st:
                raise OracleError(st, "index out of range" if st == 1 else "diagonal absent", t)
        cols[:, j] = b
        if out_val is None:
            out_val = m.val
    if out_val is None:
        out_val = np.array(matrix.Values, np.float64)
    return out_val, cols.reshape(rhs.shape)


def jacobi_pcg(matrix, b, x0=None, tolerance=1e-8, max_iterations=0, use_preconditioner=True,
               pivot_tolerance=1e-300):
    """(x, iterations, converged, residual norm, relative residual) of the
    reference's Jacobi-PCG; raises OracleError(3) for a bad diagonal entry
    (``column`` = its row) and OracleError(4) for p^T A p <= 0."""
    m = _Csr(matrix)
    bb, bp = _d(b)
    x = np.zeros(m.n) if x0 is None else np.array(x0, np.float64)
    out = np.zeros(4)
    bad = C.c_int()
    st = lib().oracle_jacobi_pcg(m.n, m.rpp, m.cpp, m.dgp, m.vp, bp, x.ctypes.data_as(_dp), tolerance,
                                 max_iterations, 1 if use_preconditioner else 0, pivot_tolerance,
                                 out.ctypes.data_as(_dp), C.byref(bad))
    if st:
        raise OracleError(st, "zero or invalid diagonal" if st == 3 else "p^T A p <= 0", bad.value)
    return x, int(out[0]), bool(out[1]), float(out[2]), float(out[3])


def dense_ldlt(a: np.ndarray):
    """Unpivoted dense L D L^T (small known-answer checks)."""
    n = a.shape[0]
    L = np.eye(n)
    d = np.zeros(n)
    w = a.astype(np.float64).copy()
    for k in range(n):
        d[k] = w[k, k]
        L[k + 1:, k] = w[k + 1:, k] / d[k]
        w[k + 1:, k + 1:] -= np.outer(L[k + 1:, k], L[k + 1:, k]) * d[k]
    return L, d
