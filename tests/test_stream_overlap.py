"""The side-stream extend-add (ExtendAddOverlap, on by default on the mixed
paths) changes only when the contribution columns are assembled, not what is
added in which order: the factor and the solutions must be bit-identical to
the one-stream factorisation."""
import numpy as np
import pytest

import magla_gb300 as mg
from magla_gb300 import generators as G
from tests.conftest import build_vector

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("case", [
    ("elasticity 10x10x6, natural, TF32", lambda: G.elasticity(10, 10, 6)[0], "Natural", "TF32"),
    ("elasticity 8x8x8, AMD, BF16", lambda: G.elasticity(8, 8, 8)[0], "ApproximateMinimumDegree", "BF16"),
    ("laplacian 24x24x16, AMD, TF32", lambda: G.laplacian3d(24, 24, 16), "ApproximateMinimumDegree", "TF32"),
], ids=lambda c: c[0])
def test_overlap_is_bit_identical(gpu_lib, case):
    _, make, order, prec = case
    m = make()
    b = np.stack([build_vector(m.Size, 3), build_vector(m.Size, 4)], axis=1)
    out = []
    for overlap in (0, -1):
        opts = mg.UtduSolverOptions(Ordering=mg.FillReducingOrdering[order], Precision=mg.Precision[prec],
                                    ExtendAddOverlap=overlap, PrecisionFallback=False)
        f = mg.SymmetricUtduSolver(opts).Factorize(m)
        f.Refactorize(m)   # graph replay
        out.append((f.Diagonal.copy(), f._apply(b).copy()))
    assert np.array_equal(out[0][0], out[1][0])
    assert np.array_equal(out[0][1], out[1][1])
