"""Parity of the GPU numeric phase with the oracle (the reference's CPU
algorithm restated) and with the reference's own UCHOL test scenarios
(Tests/UCHOL/SymmetricUtduSolverTests.cs).

Tolerances: FP64 path — D and x agree with the oracle to 1e-12 relative
(summation order differs), relative residuals as in the reference's tests.
Mixed paths — refined to a relative residual <= 1e-10 against the FP64 matrix.
"""
import numpy as np
import pytest

import oracle
from magla_gb300 import (ArgumentException, FillReducingOrdering, InvalidOperationException, LinearSystem, Precision,
                         SymmetricUtduSolver, UtduSolverOptions)
from magla_gb300 import generators as G
from tests import fixtures as F
from tests.conftest import build_vector, max_relative_difference, relative_residual

pytestmark = pytest.mark.gpu

FP64_VS_ORACLE = 1e-12


def solver(**kw):
    return SymmetricUtduSolver(UtduSolverOptions(**kw))


def oracle_for(matrix, **kw):
    opts = UtduSolverOptions(**{k: v for k, v in kw.items() if k in ("Ordering",)})
    sym = SymmetricUtduSolver(opts).Analyze(matrix)
    return sym, oracle.OracleFactor(sym, matrix.Values, **{k: v for k, v in kw.items() if k not in ("Ordering",)})


# ---- known answers -----------------------------------------------------------

@pytest.mark.parametrize("diag,expected", [([2.0, 4.0, 5.0], [3.0, 1.0, 2.0]), ([4.0], [2.0]),
                                           ([1e-6, 1e6], [1.0, -1.0])])
def test_diagonal_system_reproduces_exact_solution(gpu_lib, diag, expected):
    m = F.diagonal(diag)
    b = m.Multiply(np.array(expected))
    x = SymmetricUtduSolver().Solve(LinearSystem(m, b))
    for e, a in zip(expected, x):
        assert abs(e - a) <= 1e-9 * abs(e) + 1e-12


def test_empty_system(gpu_lib):
    m = F.diagonal([])
    x = SymmetricUtduSolver().Solve(LinearSystem(m, np.zeros(0)))
    assert x.shape == (0,)


def test_zero_rhs_gives_exact_zero(gpu_lib):
    m = G.grid_matrix(5, 5, 5, 2)
    x = SymmetricUtduSolver().Solve(LinearSystem(m, np.zeros(m.Size)))
    assert np.array_equal(x, np.zeros(m.Size))


def test_interface_tridiagonal_known_solution(gpu_lib):
    m = F.tridiagonal(4)
    expected = np.array([1.0, -2.0, 3.0, 0.5])
    x = SymmetricUtduSolver().Solve(LinearSystem(m, m.Multiply(expected)))
    assert np.max(np.abs(x - expected)) <= 1e-10


def test_workbook_system_exact_solution_and_factor(gpu_lib):
    m = F.cg_matrix()
    f = solver(Ordering=FillReducingOrdering.Natural).Factorize(m)
    x = f.Solve(F.CG_RHS)
    assert np.max(np.abs(x - F.CG_EXACT)) <= 1e-12
    # With the natural ordering the elimination tree postorder keeps 0..7 in
    # place, so D is the workbook's U diagonal.
    if np.array_equal(f.Symbolic.Permutation, np.arange(8)):
        assert np.allclose(f.Diagonal, F.CG_UPPER_DIAG, rtol=1e-13, atol=0)


# ---- against dense Gaussian elimination and the oracle ----------------------

@pytest.mark.parametrize("size,density", [(40, 0.02), (55, 0.15), (45, 0.90)])
@pytest.mark.parametrize("ordering", [FillReducingOrdering.ApproximateMinimumDegree, FillReducingOrdering.Natural])
def test_random_sparse_matches_dense_and_oracle(gpu_lib, size, density, ordering):
    m = F.random_matrix(size, density, seed=size * 31 + int(density * 1000))
    b = build_vector(size, 7)
    s = solver(Ordering=ordering)
    f = s.Factorize(m)
    x = f.Solve(b)
    expected = np.linalg.solve(m.to_dense(), b)
    assert max_relative_difference(x, expected) < 1e-9
    assert relative_residual(m, b, x) < 1e-12
    sym, of = oracle_for(m, Ordering=ordering)
    assert max_relative_difference(f.Diagonal, of.Diagonal) < FP64_VS_ORACLE
    assert max_relative_difference(x, of.Solve(b)) < FP64_VS_ORACLE


@pytest.mark.parametrize("scenario", ["tridiagonal", "star", "plate", "block"])
def test_various_structures(gpu_lib, scenario):
    m = {"tridiagonal": lambda: F.tridiagonal(400),
         "star": F.star,
         "plate": lambda: G.grid_matrix(15, 15, 2, 2),
         "block": lambda: G.grid_matrix(8, 8, 8, 3)}[scenario]()
    b = build_vector(m.Size, 3)
    f = SymmetricUtduSolver().Factorize(m)
    x = f.Solve(b)
    assert relative_residual(m, b, x) < 1e-10
    assert f.IsPositiveDefinite
    assert f.RegularizedPivotCount == 0
    sym, of = oracle_for(m)
    assert max_relative_difference(f.Diagonal, of.Diagonal) < FP64_VS_ORACLE
    assert max_relative_difference(x, of.Solve(b)) < FP64_VS_ORACLE
    assert abs(f.SmallestPivotMagnitude - of.SmallestPivotMagnitude) <= 1e-12 * of.SmallestPivotMagnitude
    assert abs(f.LargestPivotMagnitude - of.LargestPivotMagnitude) <= 1e-12 * of.LargestPivotMagnitude


@pytest.mark.parametrize("builder", [lambda: G.grid_matrix(9, 9, 9, 2), lambda: G.elasticity(6, 6, 6)[0],
                                     lambda: G.laplacian3d(20, 20, 20), lambda: F.random_matrix(300, 0.9, 5)])
def test_fp64_matches_oracle_d_and_x(gpu_lib, builder):
    m = builder()
    b = build_vector(m.Size, 17)
    f = SymmetricUtduSolver().Factorize(m)
    sym, of = oracle_for(m)
    assert max_relative_difference(f.Diagonal, of.Diagonal) < FP64_VS_ORACLE
    assert max_relative_difference(f.Solve(b), of.Solve(b)) < FP64_VS_ORACLE


def test_large_dense_front_blocked_path(gpu_lib):
    """One supernode of 300 columns: the blocked pivot-panel + trailing update path."""
    m = F.random_matrix(300, 0.9, 11)
    s = solver(Ordering=FillReducingOrdering.Natural)
    f = s.Factorize(m)
    b = build_vector(300, 5)
    x = f.Solve(b)
    sym, of = oracle_for(m, Ordering=FillReducingOrdering.Natural)
    assert sym.MaxFrontSize >= 250
    assert max_relative_difference(f.Diagonal, of.Diagonal) < FP64_VS_ORACLE
    assert max_relative_difference(x, of.Solve(b)) < FP64_VS_ORACLE


def test_ordering_does_not_change_solution(gpu_lib):
    m = G.grid_matrix(6, 6, 6, 2)
    b = build_vector(m.Size, 23)
    nat = solver(Ordering=FillReducingOrdering.Natural).Solve(LinearSystem(m, b))
    amd = solver(Ordering=FillReducingOrdering.ApproximateMinimumDegree).Solve(LinearSystem(m, b))
    assert max_relative_difference(amd, nat) < 1e-9


def test_multiple_rhs_on_one_factorization(gpu_lib):
    m = G.grid_matrix(8, 8, 6, 2)
    f = SymmetricUtduSolver().Factorize(m)
    B = np.stack([build_vector(m.Size, 100 + v) for v in range(5)], axis=1)
    X = f.Solve(B)
    for v in range(5):
        x1 = f.Solve(B[:, v])
        assert relative_residual(m, B[:, v], x1) < 1e-10
        assert relative_residual(m, B[:, v], X[:, v]) < 1e-10
        assert max_relative_difference(X[:, v], x1) < 1e-14


def test_reused_symbolic_after_values_changed(gpu_lib):
    m = G.grid_matrix(8, 8, 5, 2)
    s = SymmetricUtduSolver()
    sym = s.Analyze(m)
    b = build_vector(m.Size, 31)
    first = s.Factorize(m, sym).Solve(b)
    assert relative_residual(m, b, first) < 1e-10
    for i in range(m.Size):
        m.AccumulateAt(i, i, 5.0)
    second = s.Factorize(m, sym).Solve(b)
    assert relative_residual(m, b, second) < 1e-10
    assert max_relative_difference(second, first) > 1e-6


def test_refactorize_in_place(gpu_lib):
    m = G.grid_matrix(8, 8, 5, 2)
    s = SymmetricUtduSolver()
    f = s.Factorize(m)
    b = build_vector(m.Size, 31)
    first = f.Solve(b)
    for i in range(m.Size):
        m.AccumulateAt(i, i, 5.0)
    f.Refactorize(m)
    second = f.Solve(b)
    assert relative_residual(m, b, second) < 1e-10
    assert max_relative_difference(second, first) > 1e-6


def test_symbolic_from_different_structure_throws(gpu_lib):
    s = SymmetricUtduSolver()
    sym = s.Analyze(F.tridiagonal(100))
    with pytest.raises(ArgumentException):
        s.Factorize(G.grid_matrix(5, 5, 4, 1), sym)


@pytest.mark.parametrize("length", [3, 12])
def test_rhs_length_mismatch_throws(gpu_lib, length):
    m = F.tridiagonal(8)
    with pytest.raises(ArgumentException):
        LinearSystem(m, np.zeros(length))
    with pytest.raises(ArgumentException):
        SymmetricUtduSolver().Factorize(m).Solve(np.zeros(length))


def test_singular_matrix_reports_regularization_or_throws(gpu_lib):
    m = F.singular()
    f = solver(AllowDiagonalRegularization=True).Factorize(m)
    assert f.RegularizedPivotCount > 0
    assert not f.IsPositiveDefinite
    sym, of = oracle_for(m)
    assert f.RegularizedPivotCount == of.RegularizedPivotCount
    assert f.NegativePivotCount == of.NegativePivotCount
    with pytest.raises(InvalidOperationException):
        solver(AllowDiagonalRegularization=False).Factorize(m)


def test_indefinite_matrix_reports_negative_pivot(gpu_lib):
    m = F.indefinite()
    f = solver(AllowDiagonalRegularization=True).Factorize(m)
    assert f.NegativePivotCount > 0
    assert not f.IsPositiveDefinite
    sym, of = oracle_for(m)
    assert f.NegativePivotCount == of.NegativePivotCount


@pytest.mark.parametrize("precision", [Precision.TF32, Precision.BF16])
@pytest.mark.parametrize("fixture", [F.singular, F.indefinite])
def test_mixed_pivot_counts_match_the_fp64_path(gpu_lib, precision, fixture):
    """The mixed path's pivot blocks apply the reference's rule in FP64: the same regularised and
    negative counts as the FP64 oracle.  Bucket mask 0x10 sends these small fronts to the blocked
    kernels (k_diag_block) instead of the whole-front FP64 kernel."""
    m = fixture()
    f = solver(Precision=precision, SmallFrontBuckets=0x10, PrecisionFallback=False).Factorize(m)
    assert f.Precision == precision
    sym, of = oracle_for(m)
    assert f.RegularizedPivotCount == of.RegularizedPivotCount
    assert f.NegativePivotCount == of.NegativePivotCount
    with pytest.raises(InvalidOperationException):
        solver(Precision=precision, SmallFrontBuckets=0x10, AllowDiagonalRegularization=False,
               PrecisionFallback=False).Factorize(m)


@pytest.mark.parametrize("fixture", [F.singular, F.indefinite])
def test_precision_fallback_ends_at_fp64_for_a_singular_matrix(gpu_lib, fixture):
    """A reduced-precision factor with a regularised pivot is factorised again in the next
    precision; a matrix that is singular in FP64 too ends with the reference's FP64 result."""
    m = fixture()
    f = solver(Precision=Precision.BF16, SmallFrontBuckets=0x10).Factorize(m)
    assert f.Precision == Precision.FP64
    assert f.PrecisionFallbackFrom == [Precision.BF16, Precision.TF32]
    sym, of = oracle_for(m)
    assert f.RegularizedPivotCount == of.RegularizedPivotCount
    assert f.NegativePivotCount == of.NegativePivotCount
    # an SPD matrix keeps the precision it asked for
    g = solver(Precision=Precision.BF16).Factorize(G.grid_matrix(8, 8, 8, 2))
    assert g.Precision == Precision.BF16 and g.PrecisionFallbackFrom == []


def test_run_twice_is_bitwise_deterministic(gpu_lib):
    m = G.grid_matrix(9, 9, 9, 2)
    b = build_vector(m.Size, 17)
    s = SymmetricUtduSolver()
    x1 = s.Factorize(m).Solve(b)
    x2 = s.Factorize(m).Solve(b)
    assert np.array_equal(x1, x2)


def test_device_residual_matches_reference_product(gpu_lib):
    m = G.elasticity(5, 5, 5)[0]
    b = build_vector(m.Size, 2)
    f = SymmetricUtduSolver().Factorize(m)
    x = f.Solve(b) + build_vector(m.Size, 4) * 1e-3   # a residual well above round-off
    r_dev = f.DeviceResidualNorms(b, x)[0]
    r_ref = oracle.residual_norm(m, b, x)
    assert abs(r_dev - r_ref) <= 1e-12 * r_ref


# ---- mixed precision with refinement ----------------------------------------

@pytest.mark.parametrize("precision", [Precision.TF32, Precision.BF16])
@pytest.mark.parametrize("builder", [lambda: G.grid_matrix(12, 12, 12, 2), lambda: G.elasticity(8, 8, 8)[0],
                                     lambda: F.random_matrix(600, 0.9, 3)])
def test_mixed_precision_refined_reaches_tolerance(gpu_lib, precision, builder):
    m = builder()
    b = build_vector(m.Size, 9)
    f64 = SymmetricUtduSolver().Factorize(m)
    x64 = f64.Solve(b)
    f = solver(Precision=precision).Factorize(m)
    x = f.SolveRefined(b, tolerance=1e-10, max_iterations=60)
    assert relative_residual(m, b, x) <= 1e-10
    assert f.LastRefinement.relative_residual <= 1e-10
    # the low-precision factor is a close preconditioner (its error is set by
    # the FP32 front storage times the conditioning): a wrong tensor-core
    # update would leave a first residual of order one
    assert f.LastRefinement.initial_relative_residual < 3e-2
    assert f.LastRefinement.iterations <= 12
    assert max_relative_difference(x, x64) < 1e-6
    # the pivots (FP64 inside each pivot block, after low-precision Schur updates) stay close
    # to the FP64 factor's
    assert max_relative_difference(f.Diagonal, f64.Diagonal) < 0.05


def test_mixed_precision_multiple_rhs(gpu_lib):
    m = G.grid_matrix(10, 10, 10, 2)
    B = np.stack([build_vector(m.Size, 40 + k) for k in range(4)], axis=1)
    f = solver(Precision=Precision.TF32).Factorize(m)
    X = f.SolveRefined(B, tolerance=1e-10)
    for k in range(4):
        assert relative_residual(m, B[:, k], X[:, k]) <= 1e-10


def test_long_trailing_columns_and_grouped_right_hand_sides(gpu_lib):
    """Natural ordering on a flat mesh gives fronts with up to 2,271 trailing rows: their
    backward column dots are summed in row chunks of 2,048 (then reduced in chunk order),
    and several right-hand sides take the forward tails in groups of four."""
    m, _ = G.elasticity(26, 26, 3)
    opts = dict(Ordering=FillReducingOrdering.Natural)
    sym, of = oracle_for(m, **opts)
    B = np.stack([build_vector(m.Size, 60 + k) for k in range(5)], axis=1)
    f = solver(**opts).Factorize(m, sym)
    X = f.Solve(B)
    for k in range(5):
        assert max_relative_difference(X[:, k], of.Solve(B[:, k])) < FP64_VS_ORACLE
    assert max_relative_difference(f.Solve(B[:, 2]), X[:, 2]) < FP64_VS_ORACLE   # one column alone
    fm = solver(Precision=Precision.TF32, RefinementTolerance=1e-10, **opts).Factorize(m, sym)
    Xm = fm.Solve(B)
    for k in range(5):
        assert relative_residual(m, B[:, k], Xm[:, k]) <= 1e-10


def test_refinement_reports_a_non_finite_residual(gpu_lib):
    """A NaN residual compares false against the tolerance: the refined solve must raise
    instead of returning the NaN solution as converged."""
    from magla_gb300.errors import RefinementNotConvergedError
    m = G.grid_matrix(6, 6, 6, 2)
    b = build_vector(m.Size, 11)
    b[17] = np.nan
    f = solver(Precision=Precision.BF16).Factorize(m)
    with pytest.raises(RefinementNotConvergedError, match="not finite"):
        f.SolveRefined(b, tolerance=1e-10)
    # a finite right-hand side still converges on the same factor
    b[17] = 0.5
    x = f.SolveRefined(b, tolerance=1e-10)
    assert relative_residual(m, b, x) <= 1e-10


def test_symbolic_handle_destroyed_before_its_factor(gpu_lib):
    """A garbage collector may finalise the symbolic object first: the factor stays usable."""
    m = G.grid_matrix(6, 6, 6, 2)
    b = build_vector(m.Size, 5)
    s = SymmetricUtduSolver()
    sym = s.Analyze(m)
    f = s.Factorize(m, sym)
    x0 = f.Solve(b)
    sym.__del__()            # releases the native symbolic handle now
    f.Refactorize(m)
    assert np.array_equal(f.Solve(b), x0)
    f.__del__()


@pytest.mark.gpu
@pytest.mark.parametrize("prec", ["FP64", "TF32"])
def test_solve_into_caller_buffer(gpu_lib, prec):
    """Solve(b, out=x): x receives the solution (column-major block or vector) and is returned."""
    m = G.elasticity(5, 5, 4)[0]
    opts = UtduSolverOptions(Precision=Precision[prec])
    f = SymmetricUtduSolver(opts).Factorize(m)
    B = np.asfortranarray(np.stack([build_vector(m.Size, 7), build_vector(m.Size, 8)], axis=1))
    X = np.zeros_like(B, order="F")
    got = f.Solve(B, out=X)
    assert got is X
    assert np.array_equal(X, f.Solve(B))
    x1 = np.zeros(m.Size)
    assert f.Solve(B[:, 0].copy(), out=x1) is x1
    assert np.array_equal(x1, f.Solve(B[:, 0].copy()))
    with pytest.raises(ArgumentException):
        f.Solve(B, out=np.zeros((m.Size, 2)))   # row-major block


@pytest.mark.gpu
def test_many_rhs_through_inverse_fronts(gpu_lib):
    """33 right-hand sides (three groups of 16 in the trailing-row kernels, five of 8 in the
    inverse-diagonal products) on a natural-order chain of inverse fronts: each column equals
    its own one-column solve to the FP32 accuracy of the factor's application."""
    m = G.elasticity(10, 10, 5)[0]
    opts = UtduSolverOptions(Ordering=FillReducingOrdering.Natural, Precision=Precision.TF32)
    f = SymmetricUtduSolver(opts).Factorize(m)
    B = np.asfortranarray(np.stack([build_vector(m.Size, 200 + k) for k in range(33)], axis=1))
    X = f._apply(B)
    for k in (0, 15, 16, 31, 32):
        xk = f._apply(B[:, k].copy())
        assert max_relative_difference(X[:, k], xk) < 1e-5, k
