"""GB300-native numeric phase of MAGLA's UCHOL direct solver.

Host half (symbolic phase) in libuchol_host.so; device half (numeric
factorisation, solves, FP64 residual, refinement) in libuchol_gpu.so for
sm_103a.  See include/uchol_host.h and include/uchol_gpu.h for the C-ABI.
"""
from .errors import (ArgumentException, ArgumentNullException, ArgumentOutOfRangeException, DeviceOutOfMemoryError,
                     DeviceWaitTimeoutError, IndexOutOfRangeException, InvalidOperationException,
                     RefinementNotConvergedError)
from .device_matrix import (AccumulatePlan, ConjugateGradientGaussPreSolver, DeviceSymmetricCSRMatrix,
                            IterativeSolverResult, JacobiPreconditioner, LineCrossPlan)
from .matrix import LinearSystem, MatrixEntry, SymmetricCSRMatrix, SymmetricCSRMatrixBuilder
from .solver import (BatchedUtduFactorization, BatchedUtduSolver, BatchedUtduSymbolic, DirectLinearSolver,
                     FillReducingOrdering, LinearSolver, Precision, ResidualCalculator, SymmetricUtduSolver,
                     UtduNumericFactorization, UtduSolverOptions, UtduSymbolicFactorization)

__all__ = [
    "ArgumentException", "ArgumentNullException", "ArgumentOutOfRangeException", "DeviceOutOfMemoryError",
    "DeviceWaitTimeoutError", "IndexOutOfRangeException", "InvalidOperationException", "RefinementNotConvergedError",
    "LinearSystem", "MatrixEntry", "SymmetricCSRMatrix", "SymmetricCSRMatrixBuilder", "DirectLinearSolver",
    "BatchedUtduFactorization", "BatchedUtduSolver", "BatchedUtduSymbolic", "FillReducingOrdering", "LinearSolver",
    "Precision", "ResidualCalculator", "SymmetricUtduSolver", "UtduNumericFactorization", "UtduSolverOptions",
    "UtduSymbolicFactorization", "AccumulatePlan", "ConjugateGradientGaussPreSolver", "DeviceSymmetricCSRMatrix",
    "IterativeSolverResult", "JacobiPreconditioner", "LineCrossPlan",
]
