"""Parity cases at the benchmark configurations: config 1 (3D 7-point Laplacian 20^3,
AMD); config 2 (Q1 elasticity, AMD) against the oracle at 20^3 and refined at its full
40^3; config 3 (elasticity with log-uniform Young's moduli over four decades) at 12^3 and
at its full 40^3 against the FP64 GPU solution; config 5 (natural ordering, repeated
refactorisation with perturbed values, 16 right-hand sides) scaled to 10x10x5 (the full
size is the default bench workload)."""
import numpy as np
import pytest

import oracle
from magla_gb300 import FillReducingOrdering, Precision, SymmetricUtduSolver, UtduSolverOptions
from magla_gb300 import generators as G
from tests.conftest import build_vector, max_relative_difference, relative_residual

pytestmark = pytest.mark.gpu


def test_config1_laplacian20_fp64_matches_the_oracle(gpu_lib):
    m = G.laplacian3d(20, 20, 20)
    assert m.Size == 8000 and m.NonZeroCount == 30800
    b = np.random.default_rng(1).uniform(-1, 1, m.Size)
    s = SymmetricUtduSolver(UtduSolverOptions())
    sym = s.Analyze(m)
    f = s.Factorize(m, sym)
    of = oracle.OracleFactor(sym, m.Values)
    assert max_relative_difference(f.Diagonal, of.Diagonal) < 1e-12
    x = f.Solve(b)
    assert max_relative_difference(x, of.Solve(b)) < 1e-12
    assert relative_residual(m, b, x) < 1e-13


@pytest.mark.parametrize("precision", [Precision.TF32, Precision.BF16])
def test_config3_contrast_reaches_the_tolerance(gpu_lib, precision):
    ex = 12
    E = G.log_uniform_youngs(ex ** 3, 1.0, 1e4, np.random.default_rng(33))
    m, load = G.elasticity(ex, ex, ex, youngs=E)
    b = load + np.random.default_rng(34).uniform(-0.1, 0.1, m.Size)
    s = SymmetricUtduSolver(UtduSolverOptions(Precision=precision, RefinementTolerance=1e-10,
                                              RefinementMaxIterations=200))
    f = s.Factorize(m)
    x = f.Solve(b)
    assert relative_residual(m, b, x) <= 1e-10
    assert f.LastRefinement.iterations <= 60
    # forward error against the FP64 solution
    x64 = SymmetricUtduSolver(UtduSolverOptions()).Factorize(m).Solve(b)
    assert max_relative_difference(x, x64) < 1e-6


def test_config5_natural_refactorisations_with_16_rhs(gpu_lib):
    ex, ey, ez = 10, 10, 5
    rng = np.random.default_rng(55)
    # per-element moduli: no stiffness entry cancels to zero, so every perturbation below keeps
    # the pattern (the reference's 1e-15 drop would otherwise change it with the values)
    E0 = G.log_uniform_youngs(ex * ey * ez, 0.5, 2.0, rng)
    m, load = G.elasticity(ex, ey, ez, youngs=E0)
    opts = UtduSolverOptions(Ordering=FillReducingOrdering.Natural, Precision=Precision.BF16,
                             RefinementTolerance=1e-10)
    s = SymmetricUtduSolver(opts)
    sym = s.Analyze(m)
    f = s.Factorize(m, sym)
    B = rng.uniform(-1, 1, (m.Size, 16))
    for step in range(3):
        E = E0 * (1.0 + rng.uniform(-0.05, 0.05, E0.shape))
        mk, _ = G.elasticity(ex, ey, ez, youngs=E)
        f.Refactorize(mk)                 # same pattern: graph replay
        X = f.Solve(B)
        for j in (0, 7, 15):
            assert relative_residual(mk, B[:, j], X[:, j]) <= 1e-10
    # the last refactorisation equals a fresh factorisation of the same values
    Xf = s.Factorize(mk, sym).Solve(B)
    assert np.array_equal(X, Xf)


def test_config2_elasticity20_fp64_matches_the_oracle(gpu_lib):
    """The config-2 family (Q1 elasticity, E = 1, AMD) at 20^3 elements (27,783 equations):
    FP64 pivots and solution against the oracle."""
    m, load = G.elasticity(20, 20, 20)
    b = load + np.random.default_rng(21).uniform(-0.1, 0.1, m.Size)
    s = SymmetricUtduSolver(UtduSolverOptions())
    sym = s.Analyze(m)
    f = s.Factorize(m, sym)
    of = oracle.OracleFactor(sym, m.Values)
    assert max_relative_difference(f.Diagonal, of.Diagonal) < 1e-11
    x = f.Solve(b)
    assert max_relative_difference(x, of.Solve(b)) < 1e-10
    assert relative_residual(m, b, x) < 1e-12


def test_config2_full_size_bf16_reaches_the_tolerance(gpu_lib):
    """Config 2 at full size (40^3 elements, 206,763 equations, AMD, BF16 Schur updates)."""
    m, load = G.elasticity(40, 40, 40)
    assert m.Size == 206763
    b = load + np.random.default_rng(22).uniform(-0.1, 0.1, m.Size)
    s = SymmetricUtduSolver(UtduSolverOptions(Precision=Precision.BF16, RefinementTolerance=1e-10,
                                              RefinementMaxIterations=100))
    f = s.Factorize(m)
    x = f.Solve(b)
    assert relative_residual(m, b, x) <= 1e-10
    assert f.LastRefinement.iterations <= 15


@pytest.mark.parametrize("precision", [Precision.TF32, Precision.BF16])
def test_config3_full_size_against_fp64(gpu_lib, precision):
    """Config 3 at full size (40^3 elements, Young's modulus log-uniform over four decades):
    refined to 1e-10, and the solution against the FP64 GPU solution."""
    ex = 40
    E = G.log_uniform_youngs(ex ** 3, 1.0, 1e4, np.random.default_rng(20260813))
    m, load = G.elasticity(ex, ex, ex, youngs=E)
    b = load + np.random.default_rng(23).uniform(-0.1, 0.1, m.Size)
    s = SymmetricUtduSolver(UtduSolverOptions(Precision=precision, RefinementTolerance=1e-10,
                                              RefinementMaxIterations=200))
    x = s.Factorize(m).Solve(b)
    assert relative_residual(m, b, x) <= 1e-10
    x64 = SymmetricUtduSolver(UtduSolverOptions()).Factorize(m).Solve(b)
    assert relative_residual(m, b, x64) <= 1e-11   # the direct FP64 solve of this ill-conditioned case
    assert max_relative_difference(x, x64) < 1e-8
