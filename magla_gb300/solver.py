"""The UCHOL direct solver with its numeric phase on the GPU.

Python mirror of the reference's public API for this path:

* ``UtduSolverOptions``, ``FillReducingOrdering`` CAESolvers/UCHOL/UtduSymbolicFactorization.cs:8-98
* ``UtduSymbolicFactorization``                   CAESolvers/UCHOL/UtduSymbolicFactorization.cs:109-320
* ``UtduNumericFactorization``                    CAESolvers/UCHOL/UtduNumericFactorization.cs:24-235
* ``SymmetricUtduSolver``                         CAESolvers/UCHOL/SymmetricUtduSolver.cs:45-109
* ``LinearSolver`` / ``DirectLinearSolver``       CAESolvers/LinearSolver.cs:7-31, DirectLinearSolver.cs:6
* ``ResidualCalculator``                          CAESolvers/ResidualCalculator.cs:3-31

The symbolic phase runs on the host (libuchol_host.so, the same integer
arrays the reference computes); ``Factorize`` and ``Solve`` run on the GPU
through libuchol_gpu.so.  There is no CPU numeric path.

GPU extensions of the options: ``Precision`` (FP64 — the plain form — or the
mixed TF32/BF16 forms whose Schur updates run on tensor cores), the outer
block of the tensor-core update, and the refinement tolerance used by
``Solve`` on a mixed-precision factor.
"""
from __future__ import annotations

import copy
import ctypes as C
import enum
import hashlib
import json
import os
import sys

import numpy as np

from . import _native
from .errors import (ArgumentException, ArgumentNullException, InvalidOperationException, raise_for_status)
from .matrix import LinearSystem, SymmetricCSRMatrix


class FillReducingOrdering(enum.IntEnum):
    Natural = 0
    ApproximateMinimumDegree = 1


class Precision(enum.IntEnum):
    FP64 = _native.PRECISION_FP64
    TF32 = _native.PRECISION_TF32
    BF16 = _native.PRECISION_BF16


class UtduSolverOptions:
    def __init__(self, **kw):
        self.Ordering = FillReducingOrdering.ApproximateMinimumDegree
        self.MaxDegreeOfParallelism = 0
        self.SupernodeAmalgamationLimit = 64
        self.PanelWidth = 32
        self.AllowDiagonalRegularization = True
        self.PivotTolerance = 1e-13
        self.DiagonalRegularization = 1e-10
        self.ParallelUpdateThreshold = 1 << 20
        # device extensions
        self.Precision = Precision.FP64
        self.BlockWidth = 0
        self.SmallFrontBuckets = 0   # bit b: fronts of 32b < m <= 32(b+1) rows go whole to one CTA (0 = 0x7)
        self.ChainMergeWidth = 0     # widest device front grouped from a chain of supernodes (0 = 2048, < 0 = off)
        self.InverseBlockWidth = 0   # widest front whose diagonal block is kept inverted for the solves (0 = 2048, < 0 = off)
        self.DeviceMemoryBudget = 0  # bytes; > 0: factorisations needing more fail with OOM before allocating
        # reduced precision breaks down (a pivot regularised or not finite): factorise again in the
        # next higher precision, BF16 -> TF32 -> FP64
        self.PrecisionFallback = True
        self.SplitMinKBlocks = 0     # stream-K threshold of the tensor-core updates (0 = 8, < 0 = never split)
        self.ExtendAddOverlap = 0    # extend-add of contribution columns on a second stream (0 = on, < 0 = off)
        self.ChainMergeFill = 0.0    # largest growth of stored entries a chain grouping may cost (0 = 0.05)
        self.RefinementTolerance = 1e-12
        self.RefinementMaxIterations = 50
        for k, v in kw.items():
            if not hasattr(self, k):
                raise AttributeError(f"unknown option {k}")
            setattr(self, k, v)

    def ResolveWorkerCount(self) -> int:
        requested = self.MaxDegreeOfParallelism if self.MaxDegreeOfParallelism > 0 else (os.cpu_count() or 1)
        return max(1, requested)

    def ResolvePanelWidth(self) -> int:
        return min(128, max(4, self.PanelWidth))

    def _native_options(self) -> _native.Options:
        o = _native.Options()
        o.allow_diagonal_regularization = 1 if self.AllowDiagonalRegularization else 0
        o.pivot_tolerance = float(self.PivotTolerance)
        o.diagonal_regularization = float(self.DiagonalRegularization)
        o.panel_width = int(self.ResolvePanelWidth())
        o.precision = int(self.Precision)
        o.block_width = int(self.BlockWidth)
        o.small_front_buckets = int(self.SmallFrontBuckets)
        o.chain_merge_width = int(self.ChainMergeWidth)
        o.inverse_block_width = int(self.InverseBlockWidth)
        o.device_memory_budget = int(self.DeviceMemoryBudget)
        o.split_min_kblocks = int(self.SplitMinKBlocks)
        o.extend_add_overlap = int(self.ExtendAddOverlap)
        o.chain_merge_fill = float(self.ChainMergeFill)
        return o


# Array selectors of uchol_analysis_copy (include/uchol_host.h)
_A = dict(PERMUTATION=0, INVERSE_PERMUTATION=1, PATTERN_PTR=2, PATTERN_ROWS=3, LOWER_START=4, LOWER_VALUE_PTR=5,
          LOWER_VALUE_INDEX=6, DIAG_VALUE_INDEX=7, ETREE_PARENT=8, COLUMN_COUNTS=9, FIRST_COLUMN=10, SUPERNODE_OF=11,
          SN_PARENT=12, CHILD_PTR=13, CHILDREN=14, FRONT_PTR=15, FRONT_ROWS=16, SLAB_INDEX=17, SLAB_OFFSET=18,
          SLAB_LENGTHS=19)

_FRONT_RETENTION_LIMIT = 1 << 25  # UtduNumericFactorization.cs:264


class UtduSymbolicFactorization:
    """Permutation, factor structure and supernode partition; no matrix values."""

    def __init__(self):
        raise InvalidOperationException("use UtduSymbolicFactorization.Analyze or SymmetricUtduSolver.Analyze")

    @classmethod
    def Analyze(cls, matrix: SymmetricCSRMatrix, options: UtduSolverOptions) -> "UtduSymbolicFactorization":
        if matrix is None:
            raise ArgumentNullException("matrix")
        if options is None:
            raise ArgumentNullException("options")
        lib = _native.host()
        h = C.c_void_p()
        st = lib.uchol_analyze(matrix.Size, matrix.NonZeroCount, _native.ptr(matrix.RowPointers),
                               _native.ptr(matrix.ColumnIndices), int(options.Ordering),
                               max(1, int(options.SupernodeAmalgamationLimit)), C.byref(h))
        raise_for_status(st, lib.uchol_host_last_error())
        return cls._from_analysis(h, matrix)

    @classmethod
    def _from_analysis(cls, h, matrix: SymmetricCSRMatrix) -> "UtduSymbolicFactorization":
        """Takes over an analysis handle of the host library (and destroys it)."""
        lib = _native.host()
        self = cls.__new__(cls)
        try:
            info = _native.AnalysisInfo()
            raise_for_status(lib.uchol_analysis_get_info(h, C.byref(info)), lib.uchol_host_last_error())
            self._info = info
            n, S = info.n, info.supernode_count
            lengths = dict(PERMUTATION=n, INVERSE_PERMUTATION=n, PATTERN_PTR=n + 1, PATTERN_ROWS=info.pattern_entries,
                           LOWER_START=n, LOWER_VALUE_PTR=n + 1, LOWER_VALUE_INDEX=info.lower_entries,
                           DIAG_VALUE_INDEX=n, ETREE_PARENT=n, COLUMN_COUNTS=n, FIRST_COLUMN=S + 1, SUPERNODE_OF=n,
                           SN_PARENT=S, CHILD_PTR=S + 1, CHILDREN=info.child_entries, FRONT_PTR=S + 1,
                           FRONT_ROWS=info.front_row_entries, SLAB_INDEX=S, SLAB_OFFSET=S,
                           SLAB_LENGTHS=info.slab_count)
            self.arrays = {}
            for name, ln in lengths.items():
                a = np.zeros(max(0, ln), np.int32)
                if ln > 0:
                    raise_for_status(lib.uchol_analysis_copy(h, _A[name], _native.ptr(a)), lib.uchol_host_last_error())
                self.arrays[name] = a
        finally:
            lib.uchol_analysis_destroy(h)
        self._matrix_row_ptr = matrix.RowPointers.copy()
        self._matrix_col = matrix.ColumnIndices.copy()
        self._device = None
        return self

    # -- public statistics (UtduSymbolicFactorization.cs:127-234) ----------
    @property
    def Size(self) -> int:
        return self._info.n

    @property
    def Permutation(self) -> np.ndarray:
        return self.arrays["PERMUTATION"]

    @property
    def InversePermutation(self) -> np.ndarray:
        return self.arrays["INVERSE_PERMUTATION"]

    @property
    def MatrixNonZeroCount(self) -> int:
        return self._info.nnz

    @property
    def SupernodeCount(self) -> int:
        return self._info.supernode_count

    @property
    def FactorEntryCount(self) -> int:
        return int(self._info.factor_entry_count)

    @property
    def StrictFactorNonZeroCount(self) -> int:
        return int(self._info.strict_factor_nonzero_count)

    @property
    def FactorOperationCount(self) -> int:
        return int(self._info.factor_operation_count)

    @property
    def MaxFrontSize(self) -> int:
        return self._info.max_front_size

    @property
    def MaxSupernodeWidth(self) -> int:
        return self._info.max_supernode_width

    @property
    def EstimatedFactorBytes(self) -> int:
        return self.FactorEntryCount * 8

    @property
    def MaxFrontBytes(self) -> int:
        m = self.MaxFrontSize
        return m * (m + 1) // 2 * 8

    @property
    def PeakContributionBytes(self) -> int:
        return int(self._info.peak_contribution_entries) * 8

    @property
    def StructureBytes(self) -> int:
        return (self._info.pattern_entries + self._info.lower_entries + self._info.front_row_entries) * 4

    def EstimatePeakBytes(self, worker_count: int) -> int:
        workers = max(1, worker_count)
        retained = min(self.MaxFrontBytes, _FRONT_RETENTION_LIMIT * 8)
        return self.EstimatedFactorBytes + self.StructureBytes + self.PeakContributionBytes + workers * retained + \
            self.MaxFrontBytes

    def EnsureCompatible(self, matrix: SymmetricCSRMatrix) -> None:
        if matrix.Size != self.Size:
            raise ArgumentException(f"Matrix size {matrix.Size} does not match the symbolic factorization "
                                    f"built for {self.Size} equations.")
        if matrix.NonZeroCount != self.MatrixNonZeroCount:
            raise ArgumentException(
                "The matrix sparse structure has changed since symbolic analysis "
                f"(previously {self.MatrixNonZeroCount} nonzero elements, now {matrix.NonZeroCount}). "
                "Symbolic factorization can be reused only when the structure is unchanged. Run Analyze again.")

    # -- device upload (once per pattern) --------------------------------------
    def _desc(self):
        """The C-ABI view of the symbolic arrays (uchol_symbolic_desc) and the arrays it points into."""
        a = self.arrays
        d = _native.SymbolicDesc()
        keep = []

        def p(x):
            x = np.ascontiguousarray(x, np.int32)
            keep.append(x)
            return _native.ptr(x)

        d.n, d.nnz = self.Size, self.MatrixNonZeroCount
        d.row_ptr, d.col = p(self._matrix_row_ptr), p(self._matrix_col)
        d.permutation, d.diag_value_index = p(a["PERMUTATION"]), p(a["DIAG_VALUE_INDEX"])
        d.pattern_ptr, d.pattern_rows = p(a["PATTERN_PTR"]), p(a["PATTERN_ROWS"])
        d.lower_start, d.lower_value_ptr = p(a["LOWER_START"]), p(a["LOWER_VALUE_PTR"])
        d.lower_value_index = p(a["LOWER_VALUE_INDEX"])
        d.supernode_count = self.SupernodeCount
        d.first_column, d.parent = p(a["FIRST_COLUMN"]), p(a["SN_PARENT"])
        d.child_ptr, d.children = p(a["CHILD_PTR"]), p(a["CHILDREN"])
        d.front_ptr, d.front_rows = p(a["FRONT_PTR"]), p(a["FRONT_ROWS"])
        return d, keep

    def EstimateDeviceBytes(self, options: UtduSolverOptions | None = None) -> dict:
        """Device memory of a factorisation with these options (host-side plan, no GPU needed)."""
        lib = _native.gpu()
        d, keep = self._desc()
        o = (options or UtduSolverOptions())._native_options()
        fb, cb, sb = C.c_int64(), C.c_int64(), C.c_int64()
        lv, ln = C.c_int(), C.c_int()
        st = lib.uchol_estimate_device_bytes(C.byref(d), C.byref(o), C.byref(fb), C.byref(cb), C.byref(sb),
                                             C.byref(lv), C.byref(ln))
        raise_for_status(st, lib.uchol_last_error())
        return dict(factor=fb.value, contribution=cb.value, staging=sb.value, levels=lv.value, launches=ln.value)

    def device_handle(self):
        if self._device is None:
            lib = _native.gpu()
            d, keep = self._desc()
            h = C.c_void_p()
            raise_for_status(lib.uchol_symbolic_create(C.byref(d), C.byref(h)), lib.uchol_last_error())
            self._device = h
        return self._device

    def SetStream(self, stream_handle: int | None) -> None:
        """Runs every device call of this pattern and its factors on the given
        CUDA stream (a cudaStream_t as an integer; None = a private stream)."""
        lib = _native.gpu()
        h = self.device_handle()
        raise_for_status(lib.uchol_symbolic_set_stream(h, C.c_void_p(stream_handle) if stream_handle else None),
                         lib.uchol_last_error())

    def __del__(self):
        h = getattr(self, "_device", None)
        # at interpreter exit the CUDA context goes away with the process: no call into it
        if h is not None and _native._GPU is not None and not sys.is_finalizing():
            _native._GPU.uchol_symbolic_destroy(h)
            self._device = None


class UtduNumericFactorization:
    """A = U^T D U on the GPU; Solve handles any number of right-hand sides."""

    def __init__(self, symbolic: UtduSymbolicFactorization, handle, stats: _native.FactorStats,
                 options: UtduSolverOptions, matrix: SymmetricCSRMatrix):
        self._symbolic = symbolic
        self._h = handle
        self._stats = stats
        self._options = options
        self._nnz = matrix.NonZeroCount
        self._diag = None
        self.LastRefinement = None
        self.PrecisionFallbackFrom = []   # precisions given up before this factor's (PrecisionFallback)

    @property
    def Symbolic(self) -> UtduSymbolicFactorization:
        return self._symbolic

    @property
    def Size(self) -> int:
        return self._symbolic.Size

    @property
    def RegularizedPivotCount(self) -> int:
        return self._stats.regularized_pivot_count

    @property
    def NegativePivotCount(self) -> int:
        return self._stats.negative_pivot_count

    @property
    def SmallestPivotMagnitude(self) -> float:
        return self._stats.smallest_pivot_magnitude

    @property
    def LargestPivotMagnitude(self) -> float:
        return self._stats.largest_pivot_magnitude

    @property
    def IsPositiveDefinite(self) -> bool:
        return self.RegularizedPivotCount == 0 and self.NegativePivotCount == 0

    @property
    def Precision(self) -> Precision:
        return Precision(self._options.Precision)

    @property
    def FactorMilliseconds(self) -> float:
        return self._stats.factor_ms

    @property
    def DeviceBytes(self) -> int:
        return int(self._stats.device_bytes)

    @property
    def Diagonal(self) -> np.ndarray:
        if self._diag is None:
            lib = _native.gpu()
            d = np.zeros(self.Size, np.float64)
            raise_for_status(lib.uchol_factor_diagonal(self._h, _native.ptr(d, C.c_double)), lib.uchol_last_error())
            self._diag = d
        return self._diag

    def Solve(self, right_hand_side, out: np.ndarray | None = None) -> np.ndarray:
        """x = A^-1 b (b may be a vector or an n x k block of right-hand sides).

        A FP64 factor is applied once, as in the reference.  A mixed-precision
        factor is refined against the FP64 matrix until the relative residual
        of every column reaches ``RefinementTolerance``.  ``out`` (optional): a
        float64 array of b's shape, column-major for a block (for example in
        page-locked memory), that receives x and is returned.
        """
        if right_hand_side is None:
            raise ArgumentNullException("rightHandSide")
        b = np.asarray(right_hand_side, dtype=np.float64)
        n = self.Size
        if b.shape[0] != n:
            raise ArgumentException(f"The right-hand side length {b.shape[0]} does not match the matrix size {n}.")
        if self.Precision != Precision.FP64:
            return self.SolveRefined(b, self._options.RefinementTolerance, self._options.RefinementMaxIterations,
                                     out=out)
        return self._apply(b, out)

    @staticmethod
    def _out_block(b, out):
        """The column-major n x k block x is written to (a view of ``out`` when given)."""
        if out is None:
            return np.zeros((b.shape[0], 1 if b.ndim == 1 else b.shape[1]), order="F")
        if out.shape != b.shape or out.dtype != np.float64:
            raise ArgumentException(f"out must be a float64 array of shape {b.shape}", "out")
        X = out.reshape(b.shape[0], -1, order="F")
        if not X.flags.f_contiguous or not np.shares_memory(X, out):
            raise ArgumentException("out must be column-major (Fortran order)", "out")
        return X

    def _apply(self, b, out=None):
        lib = _native.gpu()
        vec = b.ndim == 1
        if self.Size == 0:
            return np.zeros(b.shape) if out is None else out
        B = np.asfortranarray(b.reshape(b.shape[0], -1))
        X = self._out_block(b, out)
        k = B.shape[1]
        ld = max(1, B.shape[0])
        st = lib.uchol_solve(self._h, self.Size, k, _native.ptr(B, C.c_double), ld, _native.ptr(X, C.c_double), ld)
        raise_for_status(st, lib.uchol_last_error())
        if out is not None:
            return out
        return X[:, 0].copy() if vec else X

    def SolveRefined(self, right_hand_side, tolerance: float = 1e-10, max_iterations: int = 50, method: int = 0,
                     out: np.ndarray | None = None):
        """Solve with FP64-residual refinement; statistics land in ``LastRefinement``.  ``out`` as in
        ``Solve``."""
        lib = _native.gpu()
        b = np.asarray(right_hand_side, dtype=np.float64)
        if b.shape[0] != self.Size:
            raise ArgumentException(f"The right-hand side length {b.shape[0]} does not match the matrix size {self.Size}.")
        vec = b.ndim == 1
        if self.Size == 0:
            self.LastRefinement = _native.RefineStats()
            return np.zeros(b.shape) if out is None else out
        B = np.asfortranarray(b.reshape(b.shape[0], -1))
        X = self._out_block(b, out)
        ro = _native.RefineOptions(float(tolerance), int(max_iterations), int(method))
        rs = _native.RefineStats()
        ld = max(1, B.shape[0])
        st = lib.uchol_solve_refined(self._h, self.Size, B.shape[1], _native.ptr(B, C.c_double), ld,
                                     _native.ptr(X, C.c_double), ld, C.byref(ro), C.byref(rs))
        self.LastRefinement = rs
        raise_for_status(st, lib.uchol_last_error())
        if out is not None:
            return out
        return X[:, 0].copy() if vec else X

    def DeviceResidualNorms(self, b, x) -> np.ndarray:
        """||b - A x||_2 per column with the device FP64 product."""
        lib = _native.gpu()
        B = np.asfortranarray(np.asarray(b, np.float64).reshape(self.Size, -1))
        X = np.asfortranarray(np.asarray(x, np.float64).reshape(self.Size, -1))
        out = np.zeros(B.shape[1])
        ld = max(1, self.Size)
        st = lib.uchol_residual_norms(self._h, self.Size, B.shape[1], _native.ptr(B, C.c_double), ld,
                                      _native.ptr(X, C.c_double), ld, _native.ptr(out, C.c_double))
        raise_for_status(st, lib.uchol_last_error())
        return out

    def PhaseTimes(self) -> dict:
        """Device milliseconds per factorisation phase (filled when UCHOL_PHASE_TIMES is set)."""
        lib = _native.gpu()
        t = _native.PhaseTimes()
        raise_for_status(lib.uchol_factor_phase_times(self._h, C.byref(t)), lib.uchol_last_error())
        out = {name: getattr(t, name) for name, _ in _native.PhaseTimes._fields_ if name != "solve_kind_ms"}
        out["solve_ms"] = dict(zip(_native.SOLVE_KINDS, list(t.solve_kind_ms)))
        return out

    def Refactorize(self, matrix: SymmetricCSRMatrix) -> None:
        """New values, same pattern, same device storage."""
        self._symbolic.EnsureCompatible(matrix)
        lib = _native.gpu()
        vals = np.ascontiguousarray(matrix.Values, np.float64)
        st = lib.uchol_refactorize(self._h, vals.ctypes.data_as(C.c_void_p), 0, C.byref(self._stats))
        raise_for_status(st, lib.uchol_last_error())
        self._diag = None

    def RefactorizeDevice(self, d_values: int) -> None:
        """Refactorise from matrix values already in device memory (pointer as an integer)."""
        lib = _native.gpu()
        st = lib.uchol_refactorize(self._h, C.c_void_p(d_values), 1, C.byref(self._stats))
        raise_for_status(st, lib.uchol_last_error())
        self._diag = None

    def RefactorizeFrom(self, dmatrix) -> None:
        """Refactorise from the values of a DeviceSymmetricCSRMatrix (same structure): the values
        stay on the device, and the factorisation waits for the refresh work queued on the
        matrix's stream."""
        lib = _native.gpu()
        st = lib.uchol_refactorize_dmatrix(self._h, dmatrix.handle, C.byref(self._stats))
        raise_for_status(st, lib.uchol_last_error())
        self._diag = None

    def SolveRefinedDevice(self, d_b: int, d_x: int, nrhs: int = 1, tolerance: float = 1e-10,
                           max_iterations: int = 100, method: int = 0):
        """Refined solve on device buffers (column-major n x nrhs, pointers as integers)."""
        lib = _native.gpu()
        ro = _native.RefineOptions(float(tolerance), int(max_iterations), int(method))
        rs = _native.RefineStats()
        n = max(1, self.Size)
        st = lib.uchol_solve_refined_device(self._h, self.Size, nrhs, C.c_void_p(d_b), n, C.c_void_p(d_x), n,
                                            C.byref(ro), C.byref(rs))
        self.LastRefinement = rs
        raise_for_status(st, lib.uchol_last_error())
        return rs

    def SolveDevice(self, d_b: int, d_x: int, nrhs: int = 1) -> None:
        lib = _native.gpu()
        n = max(1, self.Size)
        st = lib.uchol_solve_device(self._h, self.Size, nrhs, C.c_void_p(d_b), n, C.c_void_p(d_x), n)
        raise_for_status(st, lib.uchol_last_error())

    @staticmethod
    def ResidualNorm(matrix: SymmetricCSRMatrix, right_hand_side, solution) -> float:
        """||b - A x||_2 in FP64 (UtduNumericFactorization.cs:222-234)."""
        product = matrix.Multiply(solution)
        d = np.asarray(right_hand_side, np.float64) - product
        return float(np.sqrt(np.sum(d * d)))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and _native._GPU is not None and not sys.is_finalizing():
            _native._GPU.uchol_factor_destroy(h)
            self._h = None


class LinearSolver:
    """Type-checked dispatch from a LinearSystem to SolveCore (CAESolvers/LinearSolver.cs:7-31)."""

    MatrixType = SymmetricCSRMatrix

    def Solve(self, system: LinearSystem) -> np.ndarray:
        if system is None:
            raise ArgumentNullException("system")
        matrix = self.GetMatrix(system)
        return self.SolveCore(matrix, system.RightHandSide)

    def GetMatrix(self, system: LinearSystem):
        if system is None:
            raise ArgumentNullException("system")
        if not isinstance(system.Matrix, self.MatrixType):
            raise ArgumentException(f"The solver supports {self.MatrixType.__name__}, but "
                                    f"{type(system.Matrix).__name__} was provided.", "system")
        return system.Matrix

    def SolveCore(self, matrix, right_hand_side):
        raise NotImplementedError


class DirectLinearSolver(LinearSolver):
    pass


class SymmetricUtduSolver(DirectLinearSolver):
    """Direct solver A x = b for SymmetricCSRMatrix with A = U^T D U on the GPU."""

    def __init__(self, options: UtduSolverOptions | None = None):
        if options is None:
            options = UtduSolverOptions()
        self.Options = options

    def Analyze(self, matrix: SymmetricCSRMatrix) -> UtduSymbolicFactorization:
        if matrix is None:
            raise ArgumentNullException("matrix")
        return UtduSymbolicFactorization.Analyze(matrix, self.Options)

    def Factorize(self, matrix: SymmetricCSRMatrix, symbolic: UtduSymbolicFactorization | None = None):
        if matrix is None:
            raise ArgumentNullException("matrix")
        if symbolic is None:
            symbolic = self.Analyze(matrix)
        else:
            symbolic.EnsureCompatible(matrix)
        vals = np.ascontiguousarray(matrix.Values, np.float64)
        return self._factorize_with_fallback(matrix, symbolic, vals.ctypes.data, False)

    @staticmethod
    def _broke_down(stats) -> bool:
        """A reduced-precision factor is unusable when a pivot was regularised (the low-precision
        Schur complement lost definiteness) or a pivot is not finite."""
        return (stats.regularized_pivot_count > 0 or not np.isfinite(stats.smallest_pivot_magnitude)
                or not np.isfinite(stats.largest_pivot_magnitude))

    def _factorize_with_fallback(self, matrix, symbolic, values_ptr, on_device):
        """uchol_factorize[_device] in the options' precision; when PrecisionFallback is set and a
        reduced-precision factor breaks down, again in the next higher precision (the returned
        factor's ``PrecisionFallbackFrom`` lists the precisions given up).  A factor that keeps
        regularised pivots in FP64 is the reference's own result (a singular matrix)."""
        lib = _native.gpu()
        h = symbolic.device_handle()
        order = [Precision.BF16, Precision.TF32, Precision.FP64]
        options = self.Options
        given_up = []
        while True:
            out = C.c_void_p()
            stats = _native.FactorStats()
            opts = options._native_options()
            fn = lib.uchol_factorize_device if on_device else lib.uchol_factorize
            st = fn(h, matrix.Size, matrix.NonZeroCount, C.c_void_p(values_ptr), C.byref(opts), C.byref(out),
                    C.byref(stats))
            p = Precision(options.Precision)
            fall = (options.PrecisionFallback and p != Precision.FP64 and
                    (st == _native.NOT_SPD or (st == _native.OK and self._broke_down(stats))))
            if not fall:
                raise_for_status(st, lib.uchol_last_error())
                f = UtduNumericFactorization(symbolic, out, stats, options, matrix)
                f.PrecisionFallbackFrom = given_up
                return f
            if st == _native.OK:
                lib.uchol_factor_destroy(out)
            given_up.append(p)
            options = copy.copy(options)
            options.Precision = order[order.index(p) + 1]

    def FactorizeDevice(self, matrix: SymmetricCSRMatrix, symbolic: UtduSymbolicFactorization, d_values: int):
        """Factorize with the values already in device memory (pointer as an integer, the
        matrix's value order); ``matrix`` supplies the pattern only."""
        if matrix is None or symbolic is None:
            raise ArgumentNullException("matrix" if matrix is None else "symbolic")
        symbolic.EnsureCompatible(matrix)
        return self._factorize_with_fallback(matrix, symbolic, d_values, True)

    def SolveCore(self, matrix, right_hand_side):
        return self.Factorize(matrix).Solve(right_hand_side)

    # options the autotuner chooses (attribute of UtduSolverOptions -> field of uchol_options)
    _TUNED = (("SmallFrontBuckets", "small_front_buckets"), ("BlockWidth", "block_width"),
              ("ChainMergeWidth", "chain_merge_width"), ("SplitMinKBlocks", "split_min_kblocks"))

    @staticmethod
    def _tuning_key(matrix: SymmetricCSRMatrix, options: UtduSolverOptions) -> str:
        """The pattern and the options that the tuned choices depend on."""
        h = hashlib.sha256()
        h.update(np.asarray([matrix.Size, matrix.NonZeroCount, int(options.Precision), int(options.Ordering),
                             int(options.SupernodeAmalgamationLimit)], np.int64).tobytes())
        h.update(np.ascontiguousarray(matrix.RowPointers, np.int32).tobytes())
        h.update(np.ascontiguousarray(matrix.ColumnIndices, np.int32).tobytes())
        return h.hexdigest()

    def Autotune(self, matrix: SymmetricCSRMatrix, symbolic: UtduSymbolicFactorization | None = None,
                 table: str | os.PathLike | None = None):
        """Picks, per front-size bucket, the kernel that factorises the fronts, and the outer-block
        width, the chain-merge width and the stream-K threshold, by timing refactorisations of this
        matrix (uchol_autotune).

        With ``table`` (a JSON file), a pattern tuned before with the same precision and ordering
        takes its stored choices without timing anything; a new one is timed and added.

        Returns (options, report): a copy of this solver's options with the chosen values, and a
        dict with the number of candidates, the default and best refactorisation times (ms, none
        for a stored entry), the choices and whether they came from the table."""
        if matrix is None:
            raise ArgumentNullException("matrix")
        key = self._tuning_key(matrix, self.Options)
        entries = {}
        if table is not None and os.path.exists(table):
            with open(table) as fh:
                entries = json.load(fh)
        tuned = copy.copy(self.Options)
        if key in entries:
            for attr, field in self._TUNED:
                setattr(tuned, attr, int(entries[key][field]))
            return tuned, dict(entries[key], candidates=0, default_ms=None, best_ms=None, from_table=True)
        if symbolic is None:
            symbolic = self.Analyze(matrix)
        else:
            symbolic.EnsureCompatible(matrix)
        lib = _native.gpu()
        base = self.Options._native_options()
        best = _native.Options()
        rep = _native.AutotuneReport()
        vals = np.ascontiguousarray(matrix.Values, np.float64)
        st = lib.uchol_autotune(symbolic.device_handle(), matrix.Size, matrix.NonZeroCount,
                                _native.ptr(vals, C.c_double), C.byref(base), C.byref(best), C.byref(rep))
        raise_for_status(st, lib.uchol_last_error())
        for attr, field in self._TUNED:
            setattr(tuned, attr, int(getattr(best, field)))
        choices = {field: int(getattr(best, field)) for _, field in self._TUNED}
        report = dict(choices, candidates=rep.candidates, default_ms=rep.default_ms, best_ms=rep.best_ms,
                      from_table=False)
        if table is not None:
            entries[key] = choices
            tmp = f"{table}.tmp"
            with open(tmp, "w") as fh:
                json.dump(entries, fh, indent=1, sort_keys=True)
            os.replace(tmp, table)
        return tuned, report


class BatchedUtduSolver:
    """Many independent systems factorised and solved together.

    The systems form the diagonal blocks of one union matrix.  Each is ordered
    on its own (the options' ordering), and the union is analysed with that
    order, so the elimination forest holds one tree per system with that
    system's own supernodes; every kernel launch of the factorisation and of
    the solves then works on all systems at once.  The reference has no batch
    entry point (its solvers take one ``SymmetricCSRMatrix`` per call); each
    system's factor and solution are those of solving it alone, up to the
    order of floating-point sums.
    """

    def __init__(self, options: UtduSolverOptions | None = None):
        self.Options = options if options is not None else UtduSolverOptions()

    @staticmethod
    def _arrays(matrices):
        if matrices is None:
            raise ArgumentNullException("matrices")
        mats = list(matrices)
        if any(m is None for m in mats):
            raise ArgumentNullException("matrices")
        sizes = np.array([m.Size for m in mats], np.int32)
        rp = [np.ascontiguousarray(m.RowPointers, np.int32) for m in mats]
        cl = [np.ascontiguousarray(m.ColumnIndices, np.int32) for m in mats]
        return mats, sizes, rp, cl

    @staticmethod
    def _ptrs(arrays, ctype):
        P = C.POINTER(ctype)
        return (P * max(1, len(arrays)))(*[a.ctypes.data_as(P) for a in arrays])

    def Union(self, matrices) -> SymmetricCSRMatrix:
        """The block-diagonal union of the systems (values in the systems' order)."""
        mats, sizes, rp, cl = self._arrays(matrices)
        vals = [np.ascontiguousarray(m.Values, np.float64) for m in mats]
        lib = _native.host()
        h = C.c_void_p()
        st = lib.uchol_batch_csr(len(mats), _native.ptr(sizes), self._ptrs(rp, C.c_int), self._ptrs(cl, C.c_int),
                                 self._ptrs(vals, C.c_double), C.byref(h))
        raise_for_status(st, lib.uchol_host_last_error())
        return SymmetricCSRMatrix._from_handle(h)

    def Analyze(self, matrices) -> "BatchedUtduSymbolic":
        mats, sizes, rp, cl = self._arrays(matrices)
        lib = _native.host()
        h = C.c_void_p()
        st = lib.uchol_batch_analyze(len(mats), _native.ptr(sizes), self._ptrs(rp, C.c_int), self._ptrs(cl, C.c_int),
                                     int(self.Options.Ordering), max(1, int(self.Options.SupernodeAmalgamationLimit)),
                                     C.byref(h))
        raise_for_status(st, lib.uchol_host_last_error())
        union = self.Union(mats)
        return BatchedUtduSymbolic(UtduSymbolicFactorization._from_analysis(h, union), sizes)

    def Factorize(self, matrices, symbolic: "BatchedUtduSymbolic | None" = None) -> "BatchedUtduFactorization":
        mats = list(matrices)
        if symbolic is None:
            symbolic = self.Analyze(mats)
        elif len(mats) != len(symbolic.Sizes) or any(m.Size != n for m, n in zip(mats, symbolic.Sizes)):
            raise ArgumentException("The systems do not match the batch analysis.")
        union = self.Union(mats)
        f = SymmetricUtduSolver(self.Options).Factorize(union, symbolic.Union)
        return BatchedUtduFactorization(f, symbolic, self.Options)


class BatchedUtduSymbolic:
    """Analysis of a batch: the union's symbolic factorisation and the system sizes."""

    def __init__(self, union: UtduSymbolicFactorization, sizes):
        self.Union = union
        self.Sizes = np.asarray(sizes, np.int64)
        self.Offsets = np.concatenate([[0], np.cumsum(self.Sizes)]).astype(np.int64)

    @property
    def Count(self) -> int:
        return len(self.Sizes)

    @property
    def FactorOperationCount(self) -> int:
        return self.Union.FactorOperationCount


class BatchedUtduFactorization:
    """Factor of a batch; ``Solve`` takes one right-hand side (vector or n_q x k block) per system."""

    def __init__(self, union_factor: UtduNumericFactorization, symbolic: BatchedUtduSymbolic, options):
        self.Union = union_factor
        self.Symbolic = symbolic
        self._options = options

    def _stack(self, right_hand_sides):
        if right_hand_sides is None:
            raise ArgumentNullException("rightHandSides")
        bs = [np.asarray(b, np.float64) for b in right_hand_sides]
        S = self.Symbolic
        if len(bs) != S.Count:
            raise ArgumentException(f"{len(bs)} right-hand sides for {S.Count} systems.")
        k = bs[0].shape[1] if bs and bs[0].ndim == 2 else 1
        B = np.zeros((int(S.Offsets[-1]), k))
        for q, b in enumerate(bs):
            if b.shape[0] != S.Sizes[q] or (b.ndim == 2 and b.shape[1] != k) or (b.ndim == 1 and k != 1):
                raise ArgumentException(f"The right-hand side of system {q} does not match its size.")
            B[S.Offsets[q]:S.Offsets[q + 1]] = b.reshape(b.shape[0], -1)
        return bs, B

    def _split(self, X, bs):
        S = self.Symbolic
        return [X[S.Offsets[q]:S.Offsets[q + 1]].reshape(bs[q].shape) for q in range(S.Count)]

    def Solve(self, right_hand_sides):
        """Solutions of every system.  A mixed-precision factor is refined until the
        relative residual of every column of every system reaches the tolerance: the
        columns are scaled to unit norm per system and the union is refined to
        tolerance / sqrt(systems)."""
        bs, B = self._stack(right_hand_sides)
        if self.Union.Precision == Precision.FP64:
            return self._split(self.Union._apply(B), bs)
        S = self.Symbolic
        scale = np.ones((S.Count, B.shape[1]))
        for q in range(S.Count):
            blk = B[S.Offsets[q]:S.Offsets[q + 1]]
            nrm = np.linalg.norm(blk, axis=0)
            scale[q] = np.where(nrm > 0, nrm, 1.0)
            B[S.Offsets[q]:S.Offsets[q + 1]] = blk / scale[q]
        tol = self._options.RefinementTolerance / np.sqrt(max(1, S.Count))
        X = self.Union.SolveRefined(B, tol, self._options.RefinementMaxIterations).reshape(B.shape)
        for q in range(S.Count):
            X[S.Offsets[q]:S.Offsets[q + 1]] *= scale[q]
        return self._split(X, bs)

    def Refactorize(self, matrices) -> None:
        mats = list(matrices)
        if len(mats) != self.Symbolic.Count:
            raise ArgumentException("The systems do not match the batch analysis.")
        self.Union.Refactorize(BatchedUtduSolver(self._options).Union(mats))


class ResidualCalculator:
    """FP64 residual and vector norms (CAESolvers/ResidualCalculator.cs:5-30)."""

    def CalculateResidualNorm(self, matrix, right_hand_side, solution) -> float:
        product = matrix.Multiply(solution)
        r = np.asarray(right_hand_side, np.float64) - product
        return float(np.sqrt(np.sum(r * r)))

    def CalculateNorm(self, vector) -> float:
        v = np.asarray(vector, np.float64)
        return float(np.sqrt(np.sum(v * v)))
