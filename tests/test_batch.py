"""Batches of independent systems (BatchedUtduSolver): the union analysis keeps every
system's own structure, and the union's solutions equal the systems' own solutions."""
import numpy as np
import pytest

import oracle
from magla_gb300 import (ArgumentException, ArgumentNullException, BatchedUtduSolver, FillReducingOrdering, Precision,
                         UtduSolverOptions, UtduSymbolicFactorization)
from magla_gb300 import generators as G
from tests.conftest import build_vector, max_relative_difference


def small_batch(count=7, seed=3):
    return G.laplacian2d_batch(count, seed, (3, 14))


@pytest.mark.parametrize("ordering", [FillReducingOrdering.ApproximateMinimumDegree, FillReducingOrdering.Natural])
def test_union_analysis_keeps_each_systems_structure(ordering):
    mats = small_batch()
    opts = UtduSolverOptions(Ordering=ordering)
    sym = BatchedUtduSolver(opts).Analyze(mats)
    alone = [UtduSymbolicFactorization.Analyze(m, opts) for m in mats]
    assert sym.Union.Size == sum(m.Size for m in mats)
    assert sym.Union.FactorOperationCount == sum(a.FactorOperationCount for a in alone)
    assert sym.Union.FactorEntryCount == sum(a.FactorEntryCount for a in alone)
    assert sym.Union.SupernodeCount == sum(a.SupernodeCount for a in alone)
    # front sizes and widths, system by system
    fc, fp = sym.Union.arrays["FIRST_COLUMN"], sym.Union.arrays["FRONT_PTR"]
    union_fronts = sorted(zip(np.diff(fp).tolist(), np.diff(fc).tolist()))
    single = sorted(f for a in alone for f in zip(np.diff(a.arrays["FRONT_PTR"]).tolist(),
                                                  np.diff(a.arrays["FIRST_COLUMN"]).tolist()))
    assert union_fronts == single
    # each system's equations occupy one contiguous range of the elimination order (one tree each)
    perm = sym.Union.Permutation
    for q in range(sym.Count):
        lo, hi = sym.Offsets[q], sym.Offsets[q + 1]
        pos = np.flatnonzero((perm >= lo) & (perm < hi))
        assert len(pos) == hi - lo and pos[-1] - pos[0] == hi - lo - 1


def test_union_matrix_is_block_diagonal():
    mats = small_batch(4)
    u = BatchedUtduSolver().Union(mats)
    off = 0
    x = [build_vector(m.Size, 10 + q) for q, m in enumerate(mats)]
    y = u.Multiply(np.concatenate(x))
    for q, m in enumerate(mats):
        assert np.allclose(y[off:off + m.Size], m.Multiply(x[q]), rtol=0, atol=1e-13)
        off += m.Size
    assert u.NonZeroCount == sum(m.NonZeroCount for m in mats)


def test_union_factor_on_the_oracle_equals_each_system_alone():
    mats = small_batch(5)
    opts = UtduSolverOptions()
    sym = BatchedUtduSolver(opts).Analyze(mats)
    union = BatchedUtduSolver(opts).Union(mats)
    bs = [build_vector(m.Size, 40 + q) for q, m in enumerate(mats)]
    xu = oracle.OracleFactor(sym.Union, union.Values).Solve(np.concatenate(bs))
    for q, m in enumerate(mats):
        s1 = UtduSymbolicFactorization.Analyze(m, opts)
        x1 = oracle.OracleFactor(s1, m.Values).Solve(bs[q])
        assert max_relative_difference(xu[sym.Offsets[q]:sym.Offsets[q + 1]], x1) < 1e-13


def test_batch_arguments_follow_the_reference_conventions():
    with pytest.raises(ArgumentNullException):
        BatchedUtduSolver().Analyze(None)
    with pytest.raises(ArgumentNullException):
        BatchedUtduSolver().Analyze([G.laplacian2d(3), None])


def test_laplacian2d_shift_is_broadcast_and_checked():
    a = G.laplacian2d(5, 5, 0.5)
    b = G.laplacian2d(5, 5, np.full(25, 0.5))
    assert np.array_equal(a.Values, b.Values)
    with pytest.raises(ValueError):
        G.laplacian2d(5, 5, np.zeros(7))


@pytest.mark.gpu
def test_batch_fp64_matches_each_system_on_the_oracle(gpu_lib):
    mats = G.laplacian2d_batch(12, 11, (8, 40))
    f = BatchedUtduSolver().Factorize(mats)
    bs = [build_vector(m.Size, 70 + q) for q, m in enumerate(mats)]
    xs = f.Solve(bs)
    opts = UtduSolverOptions()
    for q, m in enumerate(mats):
        s1 = UtduSymbolicFactorization.Analyze(m, opts)
        x1 = oracle.OracleFactor(s1, m.Values).Solve(bs[q])
        assert max_relative_difference(xs[q], x1) < 1e-12


@pytest.mark.gpu
@pytest.mark.parametrize("precision", [Precision.BF16, Precision.TF32])
def test_batch_mixed_reaches_the_tolerance_in_every_system(gpu_lib, precision):
    mats = G.laplacian2d_batch(24, 5, (16, 64))
    opts = UtduSolverOptions(Precision=precision, RefinementTolerance=1e-10)
    f = BatchedUtduSolver(opts).Factorize(mats)
    rng = np.random.default_rng(9)
    for k in (1, 8):
        bs = [rng.uniform(-1, 1, (m.Size, k)) for m in mats]
        bs[3] *= 1e-6   # a system with a much smaller right-hand side keeps its own tolerance
        xs = f.Solve(bs)
        for m, b, x in zip(mats, bs, xs):
            for j in range(k):
                r = np.linalg.norm(b[:, j] - m.Multiply(x[:, j])) / np.linalg.norm(b[:, j])
                assert r <= 1e-10


@pytest.mark.gpu
def test_batch_refactorize_equals_fresh_factor(gpu_lib):
    mats = G.laplacian2d_batch(8, 21, (10, 30))
    s = BatchedUtduSolver()
    f = s.Factorize(mats)
    mats2 = G.laplacian2d_batch(8, 21, (10, 30))   # same patterns (same seed), same values
    f.Refactorize(mats2)
    bs = [build_vector(m.Size, q) for q, m in enumerate(mats)]
    xa = f.Solve(bs)
    xb = s.Factorize(mats2).Solve(bs)
    for a, b in zip(xa, xb):
        assert np.array_equal(a, b)
    with pytest.raises(ArgumentException):
        f.Solve(bs[:-1])
