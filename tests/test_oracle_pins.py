"""Pins of the oracle (CPU restatement of the reference numeric phase) to the
known answers held by the reference's own tests:

* diagonal systems, exact solutions (Tests/UCHOL/SymmetricUtduSolverTests.cs:232-245);
* zero right-hand side -> exact zeros (:262-270);
* the 4x4 interface system x = {1, -2, 3, 0.5} (Tests/SymmetricLinearSolverInterfaceTests.cs:26-37);
* the 8x8 workbook system: exact solution and the unpivoted L, D factors
  (Tests/BiCGSTAB/CgComparisonData.cs:8-46);
* singular / indefinite matrices: regularisation and negative-pivot counts,
  strict mode failure (:601-652);
* agreement with dense Gaussian elimination on random sparse systems (:280-301);
* thread-count independence (:389-406) — here bitwise, since the oracle's
  per-supernode arithmetic does not depend on the schedule;
* agreement with an iterative CG solution on the grid 7^3 (:309-328).
"""
import numpy as np
import pytest

import oracle
from magla_gb300 import FillReducingOrdering, SymmetricUtduSolver, UtduSolverOptions
from magla_gb300 import generators as G
from tests import fixtures as F
from tests.conftest import build_vector, max_relative_difference, relative_residual


def factor(matrix, ordering=FillReducingOrdering.ApproximateMinimumDegree, **kw):
    sym = SymmetricUtduSolver(UtduSolverOptions(Ordering=ordering)).Analyze(matrix)
    return sym, oracle.OracleFactor(sym, matrix.Values, **kw)


@pytest.mark.parametrize("diag,expected", [([2.0, 4.0, 5.0], [3.0, 1.0, 2.0]), ([4.0], [2.0]),
                                           ([1e-6, 1e6], [1.0, -1.0])])
def test_diagonal_known_answer(diag, expected):
    m = F.diagonal(diag)
    b = m.Multiply(np.array(expected))
    sym, f = factor(m)
    x = f.Solve(b)
    for e, a in zip(expected, x):
        assert abs(e - a) <= 1e-9 * abs(e) + 1e-12
    # the factor of a diagonal matrix is the identity with D = A's diagonal
    assert np.array_equal(np.sort(f.Diagonal), np.sort(np.array(diag)))


def test_empty_system():
    m = F.diagonal([])
    sym, f = factor(m)
    assert f.Solve(np.zeros(0)).shape == (0,)


def test_zero_rhs_exact_zero():
    m = G.grid_matrix(5, 5, 5, 2)
    sym, f = factor(m)
    assert np.array_equal(f.Solve(np.zeros(m.Size)), np.zeros(m.Size))


def test_interface_system():
    m = F.tridiagonal(4)
    expected = np.array([1.0, -2.0, 3.0, 0.5])
    sym, f = factor(m)
    assert np.max(np.abs(f.Solve(m.Multiply(expected)) - expected)) <= 1e-10


def test_workbook_system_solution_and_factors():
    m = F.cg_matrix()
    sym, f = factor(m, FillReducingOrdering.Natural)
    assert np.max(np.abs(f.Solve(F.CG_RHS) - F.CG_EXACT)) <= 1e-12
    # Natural ordering + elimination-tree postorder; D and L are compared in
    # the permuted order against the workbook's unpivoted factors.
    p = sym.Permutation
    L, d = oracle.dense_ldlt(F.CG_MATRIX[np.ix_(p, p)])
    assert np.allclose(f.Diagonal, d, rtol=1e-13, atol=0)
    if np.array_equal(p, np.arange(8)):
        assert np.allclose(f.Diagonal, F.CG_UPPER_DIAG, rtol=1e-12, atol=0)
        assert np.allclose(L, F.CG_LOWER, rtol=1e-12, atol=1e-15)


def test_workbook_solution_any_ordering():
    m = F.cg_matrix()
    sym, f = factor(m)
    assert np.max(np.abs(f.Solve(F.CG_RHS) - F.CG_EXACT)) <= 1e-12


def test_singular_regularised_and_strict_failure():
    m = F.singular()
    sym, f = factor(m)
    assert f.RegularizedPivotCount > 0
    assert not f.IsPositiveDefinite
    with pytest.raises(oracle.OracleError) as e:
        factor(m, allow_regularization=False)
    assert e.value.status == 3


def test_indefinite_negative_pivot():
    m = F.indefinite()
    sym, f = factor(m)
    assert f.NegativePivotCount > 0
    assert not f.IsPositiveDefinite


@pytest.mark.parametrize("size,density", [(40, 0.02), (55, 0.15), (45, 0.90)])
@pytest.mark.parametrize("ordering", [FillReducingOrdering.ApproximateMinimumDegree, FillReducingOrdering.Natural])
def test_matches_dense_gaussian_elimination(size, density, ordering):
    m = F.random_matrix(size, density, seed=size * 31 + int(density * 1000))
    b = build_vector(size, 7)
    sym, f = factor(m, ordering)
    x = f.Solve(b)
    assert max_relative_difference(x, np.linalg.solve(m.to_dense(), b)) < 1e-9
    assert relative_residual(m, b, x) < 1e-12


@pytest.mark.parametrize("threads", [2, 3, 8, 32])
def test_any_degree_of_parallelism_is_bitwise_identical(threads):
    m = G.grid_matrix(9, 9, 9, 2)
    b = build_vector(m.Size, 17)
    sym, serial = factor(m, workers=1)
    _, par = factor(m, workers=threads, parallel_threshold=1)
    assert np.array_equal(serial.Diagonal, par.Diagonal)
    assert np.array_equal(serial.Solve(b), par.Solve(b))


@pytest.mark.parametrize("scenario", ["tridiagonal", "star", "plate", "block"])
def test_various_structures(scenario):
    m = {"tridiagonal": lambda: F.tridiagonal(400), "star": F.star,
         "plate": lambda: G.grid_matrix(15, 15, 2, 2), "block": lambda: G.grid_matrix(8, 8, 8, 3)}[scenario]()
    b = build_vector(m.Size, 3)
    sym, f = factor(m)
    assert relative_residual(m, b, f.Solve(b)) < 1e-10
    assert f.IsPositiveDefinite


def test_ordering_does_not_change_solution():
    m = G.grid_matrix(6, 6, 6, 2)
    b = build_vector(m.Size, 23)
    _, fn = factor(m, FillReducingOrdering.Natural)
    _, fa = factor(m)
    assert max_relative_difference(fa.Solve(b), fn.Solve(b)) < 1e-9


def test_pivot_range_and_diagonal_against_dense_ldlt():
    m = G.grid_matrix(4, 4, 3, 2)
    sym, f = factor(m)
    p = sym.Permutation
    L, d = oracle.dense_ldlt(m.to_dense()[np.ix_(p, p)])
    assert np.allclose(f.Diagonal, d, rtol=1e-13, atol=0)
    assert f.SmallestPivotMagnitude == np.min(np.abs(d))
    assert f.LargestPivotMagnitude == np.max(np.abs(d))


def test_grid_solution_agrees_with_conjugate_gradients():
    """Tests/UCHOL/SymmetricUtduSolverTests.cs:309-328: the direct solution of the grid 7^3
    (2 unknowns per node) agrees with the Jacobi-PCG solution (RelativeTolerance 1e-12,
    MaxIterations 20000) to 1e-6: the oracle's restatement of MAGLA's
    ConjugateGradientGaussPreSolver (oracle/oracle_values.cpp), and scipy's CG as a second,
    independent iterative solver.  The right-hand side uses the cited test's seed, 11; the
    vector generator is this build's."""
    m = G.grid_matrix(7, 7, 7, 2)
    b = build_vector(m.Size, 11)
    _, f = factor(m)
    x = f.Solve(b)
    xj, _, converged, _, _ = oracle.jacobi_pcg(m, b, tolerance=1e-12, max_iterations=20000)
    assert converged
    assert max_relative_difference(x, xj) < 1e-6
    assert relative_residual(m, b, x) < 1e-12
    spla = pytest.importorskip("scipy.sparse.linalg")
    A = spla.LinearOperator((m.Size, m.Size), matvec=m.Multiply, dtype=np.float64)
    try:
        xc, info = spla.cg(A, b, rtol=1e-12, atol=0.0, maxiter=20 * m.Size)
    except TypeError:   # scipy before 1.12 names the tolerance tol
        xc, info = spla.cg(A, b, tol=1e-12, atol=0.0, maxiter=20 * m.Size)
    assert info == 0
    assert max_relative_difference(x, xc) < 1e-6
