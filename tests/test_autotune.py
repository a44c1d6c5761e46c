"""Per-bucket kernel choice and the autotuner (uchol_autotune): the bucket mask reaches the
execution plan (checked on the host), factors made with any mask match the oracle, and the
tuned options factorise and solve a batch of independent systems (config 4's shape)."""
import numpy as np
import pytest

import oracle
from magla_gb300 import (ArgumentException, BatchedUtduSolver, Precision, SymmetricUtduSolver, UtduSolverOptions)
from magla_gb300 import generators as G
from tests.conftest import build_vector, max_relative_difference, relative_residual


def _launches(sym, **kw):
    return sym.EstimateDeviceBytes(UtduSolverOptions(**kw))["launches"]


@pytest.mark.parametrize("precision", [Precision.FP64, Precision.BF16])
def test_bucket_mask_reaches_the_plan(precision):
    # a 2D Laplacian on a 60 x 60 grid has fronts in every bucket up to 160 rows and beyond
    m = G.laplacian2d(60, 9, np.zeros(3600))
    sym = SymmetricUtduSolver(UtduSolverOptions()).Analyze(m)
    default = _launches(sym, Precision=precision)
    assert _launches(sym, Precision=precision, SmallFrontBuckets=0x7) == default
    # every front up to 160 rows whole in one CTA: fewer blocked-path launches
    assert _launches(sym, Precision=precision, SmallFrontBuckets=0x1F) < default
    # no small-front kernel below 96 rows: more
    assert _launches(sym, Precision=precision, SmallFrontBuckets=0x1) > default


def test_bucket_mask_is_validated():
    m = G.laplacian2d(8, 5, np.zeros(64))
    sym = SymmetricUtduSolver(UtduSolverOptions()).Analyze(m)
    with pytest.raises(ArgumentException, match="small_front_buckets"):
        sym.EstimateDeviceBytes(UtduSolverOptions(SmallFrontBuckets=1 << 5))


@pytest.mark.gpu
@pytest.mark.parametrize("mask", [0x1F, 0x1])
def test_any_bucket_mask_matches_the_oracle(gpu_lib, mask):
    m = G.laplacian2d(60, 9, np.random.default_rng(8).uniform(0.0, 0.1, 3600))
    s = SymmetricUtduSolver(UtduSolverOptions(SmallFrontBuckets=mask))
    sym = s.Analyze(m)
    f = s.Factorize(m, sym)
    of = oracle.OracleFactor(sym, m.Values)
    b = build_vector(m.Size, 21)
    assert max_relative_difference(f.Diagonal, of.Diagonal) < 1e-12
    assert max_relative_difference(f.Solve(b), of.Solve(b)) < 1e-12


@pytest.mark.gpu
def test_autotuned_batch_factorises_and_solves(gpu_lib):
    mats = G.laplacian2d_batch(24, 5, (16, 48))
    bs = BatchedUtduSolver(UtduSolverOptions(Precision=Precision.BF16, RefinementTolerance=1e-10))
    bsym = bs.Analyze(mats)
    tuned, rep = SymmetricUtduSolver(bs.Options).Autotune(bs.Union(mats), bsym.Union)
    # default, 5 buckets toggled, the other block width, 3 chain-merge widths, 3 stream-K thresholds
    assert rep["candidates"] == 13 and not rep["from_table"]
    assert 0.0 < rep["best_ms"] <= rep["default_ms"]
    assert tuned.SmallFrontBuckets == rep["small_front_buckets"] and tuned.BlockWidth == rep["block_width"]
    assert tuned.ChainMergeWidth == rep["chain_merge_width"] and tuned.SplitMinKBlocks == rep["split_min_kblocks"]
    assert tuned.BlockWidth in (64, 128)
    assert tuned.ChainMergeWidth in (0, 512, 2048, -1) and tuned.SplitMinKBlocks in (0, 4, 16, -1)
    f = BatchedUtduSolver(tuned).Factorize(mats, bsym)
    bs_ = [build_vector(mm.Size, 30 + q) for q, mm in enumerate(mats)]
    xs = f.Solve(bs_)
    for mm, b, x in zip(mats, bs_, xs):
        assert relative_residual(mm, b, x) <= 1e-10


@pytest.mark.gpu
def test_autotune_table_is_persisted_and_reloaded(gpu_lib, tmp_path):
    m = G.laplacian2d(48, 5, np.random.default_rng(3).uniform(0.0, 0.1, 48 * 48))
    table = tmp_path / "tuning.json"
    s = SymmetricUtduSolver(UtduSolverOptions(Precision=Precision.TF32))
    tuned, rep = s.Autotune(m, table=table)
    assert not rep["from_table"] and table.exists()
    again, rep2 = s.Autotune(m, table=table)
    assert rep2["from_table"] and rep2["candidates"] == 0
    for attr in ("SmallFrontBuckets", "BlockWidth", "ChainMergeWidth", "SplitMinKBlocks"):
        assert getattr(again, attr) == getattr(tuned, attr)
    # a different precision is a different entry
    _, rep3 = SymmetricUtduSolver(UtduSolverOptions(Precision=Precision.BF16)).Autotune(m, table=table)
    assert not rep3["from_table"]
    b = build_vector(m.Size, 4)
    x = SymmetricUtduSolver(again).Factorize(m).SolveRefined(b, tolerance=1e-10)
    assert relative_residual(m, b, x) <= 1e-10
