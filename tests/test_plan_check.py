"""Host-side invariants of the device execution plan (uchol_check_plan; no GPU needed):
every received contribution column assembled once, side-stream extend-add launches
joined before the contribution update, and the solve's chunked tasks (inverse-diagonal
chunks, forward trailing-row chunks, backward row chunks sized to the SM count and their
reductions) tiling their rows and blocks with distinct partial slots.  Run over AMD trees
and natural-order chains, both precisions, and several SM counts."""
import ctypes as C

import numpy as np
import pytest

import magla_gb300 as mg
from magla_gb300 import _native
from magla_gb300 import generators as G
from magla_gb300.errors import raise_for_status

CASES = [
    ("laplacian 14^3 AMD", lambda: G.laplacian3d(14, 14, 14), "ApproximateMinimumDegree"),
    ("elasticity 20^3 AMD", lambda: G.elasticity(20, 20, 20)[0], "ApproximateMinimumDegree"),
    ("elasticity 24x24x8 natural chain", lambda: G.elasticity(24, 24, 8)[0], "Natural"),
    ("grid 10^3 x2 natural", lambda: G.grid_matrix(10, 10, 10, 2), "Natural"),
]


@pytest.fixture(scope="module")
def lib():
    from magla_gb300 import build
    build.build_all()
    return _native.gpu()


@pytest.mark.parametrize("prec", ["FP64", "TF32"])
def test_plan_invariants(lib, prec):
    total = np.zeros(5, np.int64)
    for _, make, order in CASES:
        m = make()
        base = mg.UtduSolverOptions(Ordering=mg.FillReducingOrdering[order], Precision=mg.Precision[prec])
        sym = mg.SymmetricUtduSolver(base).Analyze(m)
        d, keep = sym._desc()
        for extra in ({}, {"ChainMergeWidth": 512}, {"ChainMergeWidth": -1}, {"InverseBlockWidth": 4096},
                      {"ExtendAddOverlap": -1}):
            o = mg.UtduSolverOptions(Ordering=base.Ordering, Precision=base.Precision, **extra)._native_options()
            for sms in (0, 8, 152):
                counts = (C.c_int * 5)()
                st = lib.uchol_check_plan(C.byref(d), C.byref(o), sms, counts)
                raise_for_status(st, lib.uchol_last_error())
                total += np.array(list(counts))
    # the checks saw the structures they are about
    assert total[0] > 0                          # extend-add items
    assert (total[1] > 0) == (prec != "FP64")    # side-stream launches on the mixed path only
    assert total[2] > 0 and total[3] > 0 and total[4] > 0
