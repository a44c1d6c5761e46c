"""Device-resident values of a SymmetricCSRMatrix, refreshed on the GPU, and
the Jacobi-preconditioned CG on the GPU's FP64 product.

Mirror of the reference's container operations and iterative solver, run by
libuchol_gpu.so (``uchol_dmatrix_*``, ``uchol_jacobi_pcg`` in
include/uchol_gpu.h):

* ``DeviceSymmetricCSRMatrix.ClearValues``   CAESolvers/SymmetricCSRMatrix.cs:113-116
* ``DeviceSymmetricCSRMatrix.AccumulateAt``  CAESolvers/SymmetricCSRMatrix.cs:98-110
  (item lists: ``AccumulatePlan``)
* ``DeviceSymmetricCSRMatrix.LineCross``     CAESolvers/SymmetricCSRMatrix.cs:125-167
  (index lists: ``LineCrossPlan``)
* ``DeviceSymmetricCSRMatrix.Multiply``      CAESolvers/SymmetricCSRMatrix.cs:259-324
* ``ConjugateGradientGaussPreSolver``        CAESolvers/CGGP/ConjugateGradientGaussPreSolver.cs:40-197
* ``JacobiPreconditioner``                   CAESolvers/CGGP/JacobiPreconditioner.cs:7-58
* ``IterativeSolverResult``                  CAESolvers/CGGP/IterativeSolverResult.cs:8-40

The values never need to leave the device between a refresh and a
refactorisation: ``UtduNumericFactorization.RefactorizeFrom(dmatrix)`` reads
them in place.  Plans resolve the listed positions once on the host (raising
the reference's exceptions there); applying a plan gives the values the
reference's sequential calls give, bit for bit.
"""
from __future__ import annotations

import ctypes as C
import sys

import numpy as np

from . import _native
from .errors import (ArgumentException, ArgumentNullException, ArgumentOutOfRangeException, IndexOutOfRangeException,
                     InvalidOperationException, raise_for_status)
from .matrix import LinearSystem, SymmetricCSRMatrix


def _lib():
    return _native.gpu()


def _check(status):
    lib = _lib()
    raise_for_status(status, lib.uchol_last_error())


def _vp(a):
    return C.c_void_p(a.ctypes.data) if a is not None else None


class DeviceSymmetricCSRMatrix:
    """A SymmetricCSRMatrix whose values live on the device (structure fixed at creation)."""

    def __init__(self, matrix: SymmetricCSRMatrix, stream: int | None = None):
        if matrix is None:
            raise ArgumentNullException("matrix")
        lib = _lib()
        self._n = matrix.Size
        self._row_ptr = np.ascontiguousarray(matrix.RowPointers, np.int32)
        self._col = np.ascontiguousarray(matrix.ColumnIndices, np.int32)
        self._diag = np.ascontiguousarray(matrix.DiagonalIndices, np.int32)
        vals = np.ascontiguousarray(matrix.Values, np.float64)
        h = C.c_void_p()
        _check(lib.uchol_dmatrix_create(self._n, len(self._col), _native.ptr(self._row_ptr), _native.ptr(self._col),
                                        _vp(vals), C.c_void_p(stream) if stream else None, C.byref(h)))
        self._h = h

    # -- structure and values ---------------------------------------------------
    @property
    def Size(self) -> int:
        return self._n

    RowCount = Size

    @property
    def NonZeroCount(self) -> int:
        return len(self._col)

    @property
    def handle(self):
        return self._h

    @property
    def ValuesPointer(self) -> int:
        """Device address of the values (owned by this object)."""
        p = C.c_void_p()
        _check(_lib().uchol_dmatrix_values(self._h, C.byref(p)))
        return p.value or 0

    @property
    def Values(self) -> np.ndarray:
        """A host copy of the values."""
        out = np.zeros(self.NonZeroCount, np.float64)
        _check(_lib().uchol_dmatrix_get_values(self._h, _vp(out), 0))
        return out

    def SetValues(self, values) -> None:
        v = np.ascontiguousarray(values, np.float64)
        if v.shape != (self.NonZeroCount,):
            raise ArgumentException(f"Expected {self.NonZeroCount} values, got {v.shape}.", "values")
        _check(_lib().uchol_dmatrix_set_values(self._h, _vp(v), 0))

    def SetValuesDevice(self, d_values: int) -> None:
        _check(_lib().uchol_dmatrix_set_values(self._h, C.c_void_p(d_values), 1))

    def SetStream(self, stream: int | None) -> None:
        _check(_lib().uchol_dmatrix_set_stream(self._h, C.c_void_p(stream) if stream else None))

    # -- refresh --------------------------------------------------------------------
    def ClearValues(self) -> None:
        _check(_lib().uchol_dmatrix_clear_values(self._h))

    def AccumulatePlan(self, rows, cols) -> "AccumulatePlan":
        return AccumulatePlan(self, rows, cols)

    def AccumulateAt(self, row: int, col: int, value: float) -> None:
        """One AccumulateAt call (a plan of one item)."""
        self.AccumulatePlan([row], [col]).Apply([value])

    def LineCrossPlan(self, indices) -> "LineCrossPlan":
        return LineCrossPlan(self, indices)

    def LineCross(self, right_hand_side, prescribed_value: float, index: int) -> None:
        """One LineCross call on a host right-hand side (modified in place)."""
        if right_hand_side is None:
            raise ArgumentNullException("rightHandSide")
        if len(right_hand_side) != self._n:
            raise ArgumentException(
                f"The right-hand side length {len(right_hand_side)} does not match the matrix size {self._n}.",
                "rightHandSide")
        if index < 0 or index >= self._n:
            raise ArgumentOutOfRangeException("index")
        self.LineCrossPlan([index]).Apply(right_hand_side, [prescribed_value])

    # -- product ----------------------------------------------------------------------
    def Multiply(self, vector) -> np.ndarray:
        x = np.asarray(vector, np.float64)
        if x.shape[0] != self._n:
            raise ArgumentException(f"Vector length {x.shape[0]} does not match the matrix size {self._n}.")
        xs = np.asfortranarray(x.reshape(self._n, -1))
        y = np.zeros_like(xs, order="F")
        ld = max(1, self._n)
        _check(_lib().uchol_dmatrix_multiply(self._h, xs.shape[1], _vp(xs), ld, _vp(y), ld, 0))
        return y.reshape(x.shape)

    def MultiplyDevice(self, d_x: int, d_y: int, nrhs: int = 1) -> None:
        ld = max(1, self._n)
        _check(_lib().uchol_dmatrix_multiply(self._h, nrhs, C.c_void_p(d_x), ld, C.c_void_p(d_y), ld, 1))

    def close(self) -> None:
        h = getattr(self, "_h", None)
        if h is not None and _native._GPU is not None:
            _native._GPU.uchol_dmatrix_destroy(h)
        self._h = None

    def __del__(self):
        # at interpreter exit the CUDA context goes away with the process: no call into it
        if not sys.is_finalizing():
            self.close()


class _Plan:
    def __init__(self, dm: DeviceSymmetricCSRMatrix):
        self._dm = dm   # keeps the matrix alive while the plan exists
        self._h = None

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _native._GPU is not None and not sys.is_finalizing():
            _native._GPU.uchol_values_plan_destroy(h)
        self._h = None


class AccumulatePlan(_Plan):
    """AccumulateAt(rows[i], cols[i], items[i]) for every item, in list order."""

    def __init__(self, dm: DeviceSymmetricCSRMatrix, rows, cols):
        super().__init__(dm)
        r = np.ascontiguousarray(rows, np.int32)
        c = np.ascontiguousarray(cols, np.int32)
        if r.shape != c.shape or r.ndim != 1:
            raise ArgumentException("rows and cols must be equal-length vectors")
        bad = (r < 0) | (r >= dm.Size) | (c < 0) | (c >= dm.Size)
        if bad.any():
            i = int(np.argmax(bad))
            raise IndexOutOfRangeException(f"Indices are out of range: ({int(r[i])}, {int(c[i])}).")
        self.Count = len(r)
        h = C.c_void_p()
        lib = _lib()
        raise_for_status(lib.uchol_accumulate_plan_create(dm.handle, self.Count, _native.ptr(r), _native.ptr(c),
                                                          C.byref(h)), lib.uchol_last_error())
        self._h = h

    def Apply(self, items) -> None:
        v = np.ascontiguousarray(items, np.float64)
        if v.shape != (self.Count,):
            raise ArgumentException(f"Expected {self.Count} item values, got {v.shape}.", "items")
        _check(_lib().uchol_accumulate(self._dm.handle, self._h, _vp(v), 0))

    def ApplyDevice(self, d_items: int) -> None:
        _check(_lib().uchol_accumulate(self._dm.handle, self._h, C.c_void_p(d_items), 1))


class LineCrossPlan(_Plan):
    """LineCross(rhs, prescribed[t], indices[t]) for every index, in list order."""

    def __init__(self, dm: DeviceSymmetricCSRMatrix, indices):
        super().__init__(dm)
        k = np.ascontiguousarray(indices, np.int32)
        if k.ndim != 1:
            raise ArgumentException("indices must be a vector")
        if len(k) and (k.min() < 0 or k.max() >= dm.Size):
            raise ArgumentOutOfRangeException("index")
        self.Count = len(k)
        h = C.c_void_p()
        lib = _lib()
        raise_for_status(lib.uchol_line_cross_plan_create(dm.handle, self.Count, _native.ptr(k), C.byref(h)),
                         lib.uchol_last_error())
        self._h = h

    def Apply(self, right_hand_side, prescribed) -> None:
        """right_hand_side: host array (n,) or (n, k), modified in place; prescribed: (count,) or (count, k)."""
        n = self._dm.Size
        rhs = right_hand_side
        if not isinstance(rhs, np.ndarray) or rhs.dtype != np.float64:
            raise ArgumentException("the right-hand side must be a float64 numpy array (modified in place)")
        if rhs.shape[0] != n:
            raise ArgumentException(f"The right-hand side length {rhs.shape[0]} does not match the matrix size {n}.",
                                    "rightHandSide")
        k = 1 if rhs.ndim == 1 else rhs.shape[1]
        p = np.asfortranarray(np.asarray(prescribed, np.float64).reshape(self.Count, k))
        work = np.asfortranarray(rhs.reshape(n, k))
        _check(_lib().uchol_line_cross(self._dm.handle, self._h, _vp(work), max(1, n), k, _vp(p),
                                       max(1, self.Count), 0))
        rhs[...] = work.reshape(rhs.shape)

    def ApplyDevice(self, d_rhs: int, d_prescribed: int, nrhs: int = 1, ldr: int | None = None,
                    ldp: int | None = None) -> None:
        _check(_lib().uchol_line_cross(self._dm.handle, self._h, C.c_void_p(d_rhs) if d_rhs else None,
                                       ldr or max(1, self._dm.Size), nrhs,
                                       C.c_void_p(d_prescribed) if d_prescribed else None,
                                       ldp or max(1, self.Count), 1))

    def ApplyValuesOnly(self) -> None:
        """The value changes of the list without a right-hand side."""
        _check(_lib().uchol_line_cross(self._dm.handle, self._h, None, max(1, self._dm.Size), 0, None,
                                       max(1, self.Count), 1))


class JacobiPreconditioner:
    """result = diag(A)^-1 source (CAESolvers/CGGP/JacobiPreconditioner.cs:7-58), built once for
    a matrix.  Given to ConjugateGradientGaussPreSolver.SolveWithInitialGuess it takes priority
    over UsePreconditioner; the device solver forms the inverse diagonal from the matrix's values
    at solve time, the preconditioner's own as long as those values are unchanged."""

    def __init__(self, matrix, pivotTolerance: float = 1e-300):
        if matrix is None:
            raise ArgumentNullException("matrix")
        if not np.isfinite(pivotTolerance) or pivotTolerance <= 0.0:
            raise ArgumentOutOfRangeException("pivotTolerance")
        self.Matrix = matrix
        self.PivotTolerance = pivotTolerance
        self.Size = matrix.Size
        diag = np.array([matrix.GetDiagonal(i) for i in range(self.Size)], np.float64) if self.Size else np.zeros(0)
        bad = ~np.isfinite(diag) | (np.abs(diag) <= pivotTolerance)
        if bad.any():
            raise InvalidOperationException(f"The diagonal element in row {int(np.argmax(bad))} is zero or invalid "
                                            "while building the Jacobi preconditioner.")
        self._inverse = 1.0 / diag

    def Apply(self, source, result) -> None:
        if source is None:
            raise ArgumentNullException("source")
        if result is None:
            raise ArgumentNullException("result")
        if len(source) != self.Size:
            raise ArgumentException("The source vector length does not match the preconditioner size.", "source")
        if len(result) != self.Size:
            raise ArgumentException("The result vector length does not match the preconditioner size.", "result")
        result[:] = self._inverse * np.asarray(source, np.float64)


class IterativeSolverResult:
    """CAESolvers/CGGP/IterativeSolverResult.cs:8-40."""

    def __init__(self, solution, iterations: int, converged: bool, residual_norm: float, relative_residual: float):
        self.Solution = solution
        self.Iterations = iterations
        self.Converged = converged
        self.ResidualNorm = residual_norm
        self.RelativeResidual = relative_residual


class ConjugateGradientGaussPreSolver:
    """Jacobi-preconditioned CG for SPD systems, on the GPU
    (CAESolvers/CGGP/ConjugateGradientGaussPreSolver.cs:40-197)."""

    def __init__(self, UsePreconditioner: bool = True, RelativeTolerance: float = 1e-8, MaxIterations: int = 0,
                 PivotTolerance: float = 1e-300):
        self.UsePreconditioner = UsePreconditioner
        self.RelativeTolerance = RelativeTolerance
        self.MaxIterations = MaxIterations
        self.PivotTolerance = PivotTolerance
        self.LastResult: IterativeSolverResult | None = None
        self.LastResults: list[IterativeSolverResult] = []
        self.LastMilliseconds = 0.0

    def _validate(self):
        if not np.isfinite(self.RelativeTolerance) or self.RelativeTolerance < 0.0:
            raise ArgumentOutOfRangeException("RelativeTolerance")
        if self.MaxIterations < 0:
            raise ArgumentOutOfRangeException("MaxIterations")

    def _options(self, initial_guess: bool) -> _native.CgOptions:
        return _native.CgOptions(float(self.RelativeTolerance), int(self.MaxIterations),
                                 1 if self.UsePreconditioner else 0, 1 if initial_guess else 0,
                                 float(self.PivotTolerance))

    def Solve(self, system: LinearSystem) -> np.ndarray:
        return self.SolveWithInitialGuess(system, None)

    def SolveWithInitialGuess(self, system: LinearSystem, initialGuess, preconditioner=None) -> np.ndarray:
        """x0 = initialGuess (or 0); a given JacobiPreconditioner takes priority over
        UsePreconditioner and must have been built for this system's matrix."""
        self.LastResult = None
        self._validate()
        if system is None:
            raise ArgumentNullException("system")
        matrix = system.Matrix
        n = matrix.Size
        if initialGuess is not None and len(initialGuess) != n:
            raise ArgumentException(f"The initial guess length {len(initialGuess)} does not match the matrix size {n}.")
        if preconditioner is not None and preconditioner.Matrix is not matrix:
            raise ArgumentException("The preconditioner was built for another matrix.", "preconditioner")
        dm = matrix if isinstance(matrix, DeviceSymmetricCSRMatrix) else DeviceSymmetricCSRMatrix(matrix)
        b = np.asfortranarray(np.asarray(system.RightHandSide, np.float64).reshape(n, -1))
        x = np.zeros_like(b, order="F") if initialGuess is None else \
            np.asfortranarray(np.asarray(initialGuess, np.float64).reshape(n, -1))
        res = (_native.CgResult * b.shape[1])()
        opts = self._options(initialGuess is not None)
        if preconditioner is not None:
            opts.use_preconditioner = 1
        ld = max(1, n)
        _check(_lib().uchol_jacobi_pcg(dm.handle, b.shape[1], _vp(b), ld, _vp(x), ld, 0, C.byref(opts), res))
        sol = x.reshape(np.shape(system.RightHandSide))
        self.LastResults = [IterativeSolverResult(sol if b.shape[1] == 1 else x[:, j], r.iterations, bool(r.converged),
                                                  r.residual_norm, r.relative_residual) for j, r in enumerate(res)]
        self.LastResult = self.LastResults[0]
        self.LastMilliseconds = res[0].ms if b.shape[1] else 0.0
        return sol

    def SolveDevice(self, dm: DeviceSymmetricCSRMatrix, d_b: int, d_x: int, nrhs: int = 1,
                    initial_guess: bool = False) -> list:
        """Device buffers (column-major n x nrhs, pointers as integers); returns one result per column."""
        self._validate()
        res = (_native.CgResult * max(1, nrhs))()
        opts = self._options(initial_guess)
        ld = max(1, dm.Size)
        _check(_lib().uchol_jacobi_pcg(dm.handle, nrhs, C.c_void_p(d_b), ld, C.c_void_p(d_x), ld, 1, C.byref(opts),
                                       res))
        self.LastResults = [IterativeSolverResult(None, r.iterations, bool(r.converged), r.residual_norm,
                                                  r.relative_residual) for r in res[:nrhs]]
        self.LastResult = self.LastResults[0] if nrhs else None
        self.LastMilliseconds = res[0].ms if nrhs else 0.0
        return self.LastResults


__all__ = ["DeviceSymmetricCSRMatrix", "AccumulatePlan", "LineCrossPlan", "ConjugateGradientGaussPreSolver",
           "JacobiPreconditioner", "IterativeSolverResult", "InvalidOperationException"]
