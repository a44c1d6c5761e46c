"""Replicas across ranks: the batch is split by system with no data exchange; the
ranks only reduce the step time (max) and a checksum (sum).  Two gloo ranks on
the CPU, the oracle standing in for each rank's GPU factorisation."""
import os
import socket

import numpy as np
import pytest

from magla_gb300.replicas import shard


def test_shards_partition_any_count():
    for count in (0, 1, 5, 256, 257):
        for world in (1, 2, 3, 8):
            parts = [shard(count, r, world) for r in range(world)]
            items = [i for p in parts for i in p]
            assert items == list(range(count))
            sizes = [len(p) for p in parts]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        shard(4, 2, 2)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank_main(rank, world, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        import oracle
        from magla_gb300 import UtduSolverOptions, UtduSymbolicFactorization
        from magla_gb300 import generators as G
        from magla_gb300.replicas import max_over_ranks, shard, sum_over_ranks
        mats = G.laplacian2d_batch(9, 13, (4, 12))
        checksum = 0.0
        for q in shard(len(mats), rank, world):
            m = mats[q]
            b = np.random.default_rng(q).uniform(-1, 1, m.Size)
            sym = UtduSymbolicFactorization.Analyze(m, UtduSolverOptions())
            x = oracle.OracleFactor(sym, m.Values).Solve(b)
            checksum += float(np.sum(x))
        step_time = max_over_ranks(0.25 + rank)
        total = sum_over_ranks(checksum)
        out.put((rank, step_time, total))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_split_the_batch_and_reduce():
    import torch.multiprocessing as mp
    import oracle
    from magla_gb300 import UtduSolverOptions, UtduSymbolicFactorization
    from magla_gb300 import generators as G
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    results = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    mats = G.laplacian2d_batch(9, 13, (4, 12))
    expected = 0.0
    for i, m in enumerate(mats):
        b = np.random.default_rng(i).uniform(-1, 1, m.Size)
        sym = UtduSymbolicFactorization.Analyze(m, UtduSolverOptions())
        expected += float(np.sum(oracle.OracleFactor(sym, m.Values).Solve(b)))
    for rank, step_time, total in results:
        assert step_time == 1.25                      # the slowest rank's time
        assert abs(total - expected) <= 1e-9 * max(1.0, abs(expected))
