"""Oracle of the values refresh and of the Jacobi-preconditioned CG, pinned
against the known answers of the reference's own tests (CPU only).

* LineCross 3x3 system   Tests/SymmetricSparseMatrixCSRTests.cs:16-38
* AccumulateAt           Tests/SymmetricSparseMatrixCSRTests.cs:181-200
* Jacobi-PCG             Tests/CGGP/ConjugateGradientGaussPreSolverTests.cs:55-104
* Jacobi preconditioner  Tests/CGGP/JacobiPreconditionerTests.cs:10-27
* PCG vs direct solve    Tests/UCHOL/SymmetricUtduSolverTests.cs:309-328

and against the host mirror of the container (magla_gb300.matrix), whose
AccumulateAt / LineCross must give the same bits.
"""
import numpy as np
import pytest

import oracle
from magla_gb300 import SymmetricCSRMatrixBuilder
from magla_gb300 import generators as G
from tests.conftest import build_vector


def _build(n, entries):
    b = SymmetricCSRMatrixBuilder(n)
    for r, c, v in entries:
        b.AddToElement(r, c, v)
    return b.Build()


def _diagonal(d):
    return _build(len(d), [(i, i, v) for i, v in enumerate(d)])


def _tridiagonal(n, diagonal, off):
    return _build(n, [(i, i, diagonal) for i in range(n)] + [(i, i + 1, off) for i in range(n - 1)])


def test_line_cross_known_answer():
    m = _build(3, [(0, 0, 4.0), (0, 1, 2.0), (0, 2, -1.0), (1, 1, 5.0), (1, 2, 7.0), (2, 2, 9.0)])
    vals, rhs = oracle.line_cross(m, [11.0, 13.0, 17.0], [2.0], [1])
    assert list(rhs) == [7.0, 2.0, 3.0]
    # structure kept: (0,1) and (1,2) zero, (1,1) one
    pos = {(0, 1): m._find(0, 1), (1, 1): m._find(1, 1), (1, 2): m._find(1, 2), (0, 0): m._find(0, 0)}
    assert vals[pos[(0, 1)]] == 0.0 and vals[pos[(1, 2)]] == 0.0
    assert vals[pos[(1, 1)]] == 1.0 and vals[pos[(0, 0)]] == 4.0
    assert len(vals) == m.NonZeroCount


def test_accumulate_known_answers():
    m = _build(2, [(0, 1, 5.0)])
    vals = oracle.accumulate(m, [1], [0], [1.5])   # reversed order normalises to (0, 1)
    assert vals[m._find(0, 1)] == pytest.approx(6.5, abs=1e-12)
    m = _build(2, [(0, 0, 5.0)])
    with pytest.raises(oracle.OracleError) as e:
        oracle.accumulate(m, [0], [1], [1.0])
    assert e.value.status == 2
    with pytest.raises(oracle.OracleError) as e:
        oracle.accumulate(m, [0], [2], [1.0])
    assert e.value.status == 1


@pytest.mark.parametrize("diag,expected,guess,iters", [
    ([2.0, 4.0, 5.0], [3.0, 1.0, 2.0], None, 1),
    ([2.0, 3.0], [5.0, -2.0], [5.0, -2.0], 0),
    ([4.0, 4.0, 4.0], [0.0, 0.0, 0.0], None, 0),
])
def test_pcg_diagonal_known_answers(diag, expected, guess, iters):
    m = _diagonal(diag)
    b = oracle.multiply(m, np.array(expected))
    x, it, conv, _, _ = oracle.jacobi_pcg(m, b, guess)
    assert conv and it == iters
    assert np.allclose(x, expected, atol=1e-9, rtol=0)


@pytest.mark.parametrize("precondition", [True, False])
def test_pcg_tridiagonal_converges(precondition):
    m = _tridiagonal(5, 4.0, -1.0)
    b = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    x, it, conv, rn, rel = oracle.jacobi_pcg(m, b, tolerance=1e-10, use_preconditioner=precondition)
    assert conv and rel <= 1e-10
    assert np.allclose(oracle.multiply(m, x), b, atol=1e-6, rtol=0)


def test_jacobi_zero_diagonal_fails():
    m = _build(2, [(0, 0, 2.0), (0, 1, 1.0)])   # (1, 1) structurally absent
    with pytest.raises(oracle.OracleError) as e:
        oracle.jacobi_pcg(m, np.array([1.0, 1.0]))
    assert e.value.status == 3 and e.value.column == 1


def test_pcg_not_positive_definite_fails():
    m = _diagonal([-1.0, -2.0])
    with pytest.raises(oracle.OracleError) as e:
        oracle.jacobi_pcg(m, np.array([1.0, 1.0]))
    assert e.value.status == 4


def test_pcg_agrees_with_direct_solve_on_grid():
    m = G.grid_matrix(7, 7, 7, 2)
    b = build_vector(m.Size, 11)
    x, it, conv, _, _ = oracle.jacobi_pcg(m, b, tolerance=1e-12, max_iterations=20000)
    assert conv
    direct = np.linalg.solve(m.to_dense(), b)
    assert np.max(np.abs(x - direct)) / np.max(np.abs(direct)) < 1e-6


def test_oracle_matches_host_container_bit_for_bit():
    """The host mirror's AccumulateAt / LineCross and the oracle: same bits."""
    m = G.elasticity(3, 3, 2)[0]
    rng = np.random.default_rng(5)
    rows = np.repeat(np.arange(m.Size), np.diff(m.RowPointers))
    pick = rng.integers(0, m.NonZeroCount, 400)
    r, c = rows[pick], m.ColumnIndices[pick]
    swap = rng.random(400) < 0.5
    r, c = np.where(swap, c, r), np.where(swap, r, c)
    items = rng.normal(size=400)
    expect = oracle.accumulate(m, r, c, items)
    for i in range(400):
        m.AccumulateAt(int(r[i]), int(c[i]), float(items[i]))
    assert np.array_equal(m.Values, expect)
    idx = rng.choice(m.Size, 30, replace=True)
    pres = rng.normal(size=30)
    rhs0 = build_vector(m.Size, 3)
    vals, rhs = oracle.line_cross(m, rhs0, pres, idx)
    h = rhs0.copy()
    for t in range(30):
        m.LineCross(h, float(pres[t]), int(idx[t]))
    assert np.array_equal(m.Values, vals)
    assert np.array_equal(h, rhs)


def test_device_cg_argument_checks_without_a_gpu():
    """The Jacobi-PCG mirror validates its arguments before any device call
    (ConjugateGradientGaussPreSolver.cs:78-101, IterativeLinearSolver.cs:26-33)."""
    from magla_gb300 import (ArgumentException, ArgumentOutOfRangeException, ConjugateGradientGaussPreSolver,
                             LinearSystem)
    m = _diagonal([2.0, 3.0])
    with pytest.raises(ArgumentOutOfRangeException) as e:
        ConjugateGradientGaussPreSolver(MaxIterations=-1).Solve(LinearSystem(m, [1.0, 1.0]))
    assert e.value.ParamName == "MaxIterations"
    with pytest.raises(ArgumentOutOfRangeException):
        ConjugateGradientGaussPreSolver(RelativeTolerance=-1.0).Solve(LinearSystem(m, [1.0, 1.0]))
    with pytest.raises(ArgumentException):
        ConjugateGradientGaussPreSolver().SolveWithInitialGuess(LinearSystem(m, [1.0, 1.0]), [1.0])


def test_jacobi_preconditioner_known_answers():
    """Tests/CGGP/JacobiPreconditionerTests.cs:10-36, 57-65 (host mirror; no GPU)."""
    from magla_gb300 import (ArgumentException, ConjugateGradientGaussPreSolver, InvalidOperationException,
                             JacobiPreconditioner, LinearSystem)
    p = JacobiPreconditioner(_diagonal([2.0, 4.0, 8.0]))
    result = np.zeros(3)
    p.Apply([4.0, 12.0, -8.0], result)
    assert list(result) == [2.0, 3.0, -1.0]
    with pytest.raises(InvalidOperationException):
        JacobiPreconditioner(_diagonal([2.0, 0.0, 8.0]))
    p2 = JacobiPreconditioner(_diagonal([2.0, 4.0]))
    with pytest.raises(ArgumentException):
        p2.Apply(np.zeros(1), np.zeros(2))
    with pytest.raises(ArgumentException):
        p2.Apply(np.zeros(2), np.zeros(1))
    # a preconditioner built for another matrix (equal values, another object) is refused
    m = _diagonal([2.0, 4.0])
    with pytest.raises(ArgumentException):
        ConjugateGradientGaussPreSolver().SolveWithInitialGuess(LinearSystem(m, [2.0, 4.0]), None,
                                                               JacobiPreconditioner(_diagonal([2.0, 4.0])))
