"""Device-resident values: refresh kernels and the device Jacobi-PCG against the
oracle (oracle/oracle_values.cpp), and the refresh -> refactorisation path
with the values kept on the device.

Refresh results must equal the oracle's sequential calls bit for bit; the
PCG, whose reductions run in another order than the reference's sequential
sums, must match the oracle's iteration count within one step and its
solution to 1e-8 relative (iterates agree to the rounding of the dots
propagated over the run).
"""
import numpy as np
import pytest

import oracle
from magla_gb300 import (ConjugateGradientGaussPreSolver, DeviceSymmetricCSRMatrix, IndexOutOfRangeException,
                         InvalidOperationException, LinearSystem, SymmetricCSRMatrixBuilder, SymmetricUtduSolver,
                         ArgumentOutOfRangeException, ArgumentException, _native)
from magla_gb300 import generators as G
from tests.conftest import build_vector, max_relative_difference, relative_residual

pytestmark = pytest.mark.gpu


def _build(n, entries):
    b = SymmetricCSRMatrixBuilder(n)
    for r, c, v in entries:
        b.AddToElement(r, c, v)
    return b.Build()


def _random_items(m, count, rng):
    rows = np.repeat(np.arange(m.Size), np.diff(m.RowPointers))
    pick = rng.integers(0, m.NonZeroCount, count)
    r, c = rows[pick], m.ColumnIndices[pick]
    swap = rng.random(count) < 0.5
    return np.where(swap, c, r).astype(np.int32), np.where(swap, r, c).astype(np.int32), rng.normal(size=count)


def test_accumulate_matches_oracle_bit_for_bit(gpu_lib):
    m = G.elasticity(6, 6, 6)[0]
    rng = np.random.default_rng(21)
    r, c, items = _random_items(m, 50_000, rng)   # many repeats of each position
    dm = DeviceSymmetricCSRMatrix(m)
    plan = dm.AccumulatePlan(r, c)
    plan.Apply(items)
    expect = oracle.accumulate(m, r, c, items)
    assert np.array_equal(dm.Values, expect)
    # applying twice continues from the refreshed values
    plan.Apply(items * 0.5)
    expect = oracle.accumulate(_with_values(m, expect), r, c, items * 0.5)
    assert np.array_equal(dm.Values, expect)


def _with_values(m, values):
    out = m.__class__.from_triplets(m.Size, np.repeat(np.arange(m.Size), np.diff(m.RowPointers)), m.ColumnIndices,
                                    np.ones(m.NonZeroCount))
    out._val[:] = values
    return out


def test_accumulate_errors(gpu_lib):
    m = _build(2, [(0, 0, 5.0)])
    dm = DeviceSymmetricCSRMatrix(m)
    with pytest.raises(InvalidOperationException):
        dm.AccumulateAt(0, 1, 1.0)
    with pytest.raises(IndexOutOfRangeException):
        dm.AccumulateAt(0, 2, 1.0)
    # the C-ABI's own range check
    import ctypes as C
    rows = np.array([0], np.int32)
    cols = np.array([7], np.int32)
    h = C.c_void_p()
    st = gpu_lib.uchol_accumulate_plan_create(dm.handle, 1, _native.ptr(rows), _native.ptr(cols), C.byref(h))
    assert st == _native.OUT_OF_RANGE
    m = _build(2, [(0, 1, 5.0), (0, 0, 1.0), (1, 1, 1.0)])
    dm = DeviceSymmetricCSRMatrix(m)
    dm.AccumulateAt(1, 0, 1.5)
    assert dm.Values[m._find(0, 1)] == 6.5


def test_line_cross_known_answer(gpu_lib):
    m = _build(3, [(0, 0, 4.0), (0, 1, 2.0), (0, 2, -1.0), (1, 1, 5.0), (1, 2, 7.0), (2, 2, 9.0)])
    dm = DeviceSymmetricCSRMatrix(m)
    rhs = np.array([11.0, 13.0, 17.0])
    dm.LineCross(rhs, 2.0, 1)
    assert list(rhs) == [7.0, 2.0, 3.0]
    v = dm.Values
    assert v[m._find(0, 1)] == 0.0 and v[m._find(1, 2)] == 0.0 and v[m._find(1, 1)] == 1.0
    assert dm.NonZeroCount == m.NonZeroCount


def test_line_cross_list_matches_oracle_bit_for_bit(gpu_lib):
    m = G.elasticity(5, 5, 4)[0]
    rng = np.random.default_rng(8)
    idx = rng.choice(m.Size, 300, replace=True)   # repeated indices and neighbouring constraints
    pres = rng.normal(size=(300, 3))
    rhs0 = np.stack([build_vector(m.Size, 30 + j) for j in range(3)], axis=1)
    vals, expect = oracle.line_cross(m, rhs0, pres, idx)
    dm = DeviceSymmetricCSRMatrix(m)
    rhs = rhs0.copy()
    dm.LineCrossPlan(idx).Apply(rhs, pres)
    assert np.array_equal(rhs, expect)
    assert np.array_equal(dm.Values, vals)


def test_line_cross_errors(gpu_lib):
    m = _build(3, [(0, 0, 1.0), (0, 1, 1.0), (2, 2, 1.0)])   # (1, 1) absent
    dm = DeviceSymmetricCSRMatrix(m)
    with pytest.raises(InvalidOperationException):
        dm.LineCross(np.zeros(3), 1.0, 1)
    with pytest.raises(ArgumentOutOfRangeException):
        dm.LineCross(np.zeros(3), 1.0, 3)
    with pytest.raises(ArgumentException):
        dm.LineCross(np.zeros(2), 1.0, 0)


def test_refresh_on_device_then_refactorize(gpu_lib):
    """Re-assembly on the device (clear, accumulate, Dirichlet rows) feeding the
    factorisation's graph replay: same values as the oracle, same solution as a
    factorisation of the oracle's values."""
    torch = pytest.importorskip("torch")
    m = G.elasticity(8, 8, 6)[0]
    n, nnz = m.Size, m.NonZeroCount
    rows = np.repeat(np.arange(n), np.diff(m.RowPointers)).astype(np.int32)
    cols = np.ascontiguousarray(m.ColumnIndices, np.int32)
    # items: every stored value split in two halves, plus a diagonal shift of 5
    r = np.concatenate([rows, cols, np.arange(n, dtype=np.int32)])
    c = np.concatenate([cols, rows, np.arange(n, dtype=np.int32)])
    items = np.concatenate([m.Values * 0.5, m.Values * 0.5, np.full(n, 5.0)])
    clamped = np.arange(0, n, 7)   # a Dirichlet set
    pres = np.zeros(len(clamped))
    b0 = build_vector(n, 12)

    solver = SymmetricUtduSolver()
    f = solver.Factorize(m)
    dm = DeviceSymmetricCSRMatrix(m)
    acc = dm.AccumulatePlan(r, c)
    lc = dm.LineCrossPlan(clamped)
    d_items = torch.tensor(items, dtype=torch.float64, device="cuda")
    d_rhs = torch.tensor(b0, dtype=torch.float64, device="cuda")
    d_pres = torch.tensor(pres, dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    dm.ClearValues()
    acc.ApplyDevice(d_items.data_ptr())
    lc.ApplyDevice(d_rhs.data_ptr(), d_pres.data_ptr())
    f.RefactorizeFrom(dm)
    torch.cuda.synchronize()

    zero = _with_values(m, np.zeros(nnz))
    v_acc = oracle.accumulate(zero, r, c, items)
    v_ref, rhs_ref = oracle.line_cross(_with_values(m, v_acc), b0, pres, clamped)
    assert np.array_equal(dm.Values, v_ref)
    assert np.array_equal(d_rhs.cpu().numpy(), rhs_ref)
    m_ref = _with_values(m, v_ref)
    x = f.Solve(rhs_ref)
    x_ref = SymmetricUtduSolver().Factorize(m_ref).Solve(rhs_ref)
    assert relative_residual(m_ref, rhs_ref, x) < 1e-10
    assert max_relative_difference(x, x_ref) < 1e-9
    assert np.max(np.abs(x[clamped])) <= 1e-10 * np.max(np.abs(x))   # the prescribed zeros


def test_refactorize_from_rejects_another_structure(gpu_lib):
    m = G.laplacian3d(4, 4, 4)
    f = SymmetricUtduSolver().Factorize(m)
    other = DeviceSymmetricCSRMatrix(G.laplacian3d(4, 4, 3))
    with pytest.raises(ArgumentException):
        f.RefactorizeFrom(other)


@pytest.mark.parametrize("diag,expected,guess,iters", [
    ([2.0, 4.0, 5.0], [3.0, 1.0, 2.0], None, 1),
    ([2.0, 3.0], [5.0, -2.0], [5.0, -2.0], 0),
    ([4.0, 4.0, 4.0], [0.0, 0.0, 0.0], None, 0),
])
def test_pcg_diagonal_known_answers(gpu_lib, diag, expected, guess, iters):
    m = _build(len(diag), [(i, i, v) for i, v in enumerate(diag)])
    b = oracle.multiply(m, np.array(expected))
    s = ConjugateGradientGaussPreSolver()
    x = s.SolveWithInitialGuess(LinearSystem(m, b), guess)
    assert s.LastResult.Converged and s.LastResult.Iterations == iters
    assert np.allclose(x, expected, atol=1e-9, rtol=0)


@pytest.mark.parametrize("precondition", [True, False])
def test_pcg_tridiagonal(gpu_lib, precondition):
    m = _build(5, [(i, i, 4.0) for i in range(5)] + [(i, i + 1, -1.0) for i in range(4)])
    b = np.array([1.0, 2.0, 3.0, 4.0, 5.0])
    s = ConjugateGradientGaussPreSolver(RelativeTolerance=1e-10, UsePreconditioner=precondition)
    x = s.Solve(LinearSystem(m, b))
    assert s.LastResult.Converged and s.LastResult.RelativeResidual <= 1e-10
    assert np.allclose(oracle.multiply(m, x), b, atol=1e-6, rtol=0)


@pytest.mark.parametrize("precondition", [True, False])
def test_pcg_matches_oracle(gpu_lib, precondition):
    m = G.elasticity(6, 6, 5)[0]
    b = build_vector(m.Size, 40)
    x_o, it_o, conv_o, _, _ = oracle.jacobi_pcg(m, b, tolerance=1e-10, use_preconditioner=precondition)
    s = ConjugateGradientGaussPreSolver(RelativeTolerance=1e-10, UsePreconditioner=precondition)
    x = s.Solve(LinearSystem(m, b))
    assert conv_o and s.LastResult.Converged
    assert abs(s.LastResult.Iterations - it_o) <= 1, (s.LastResult.Iterations, it_o)
    assert max_relative_difference(x, x_o) < 1e-8
    assert relative_residual(m, b, x) < 1e-9


def test_pcg_agrees_with_direct_solve(gpu_lib):
    m = G.grid_matrix(7, 7, 7, 2)
    b = build_vector(m.Size, 11)
    s = ConjugateGradientGaussPreSolver(RelativeTolerance=1e-12, MaxIterations=20000)
    x = s.Solve(LinearSystem(m, b))
    assert s.LastResult.Converged
    direct = SymmetricUtduSolver().Factorize(m).Solve(b)
    assert max_relative_difference(x, direct) < 1e-6


def test_pcg_columns_are_independent(gpu_lib):
    """Several right-hand sides at once: each column equals its own single-column run."""
    m = G.laplacian3d(12, 12, 10)
    n = m.Size
    B = np.stack([build_vector(n, 70 + j) * (10.0 ** j) for j in range(3)], axis=1)
    B[:, 2] = 0.0   # a zero column stops before its first step
    s = ConjugateGradientGaussPreSolver(RelativeTolerance=1e-9)
    X = s.Solve(LinearSystem(m, B))
    its = [r.Iterations for r in s.LastResults]
    assert its[2] == 0 and np.all(X[:, 2] == 0.0)
    for j in range(2):
        x1 = ConjugateGradientGaussPreSolver(RelativeTolerance=1e-9).Solve(LinearSystem(m, B[:, j]))
        assert np.array_equal(X[:, j], x1)


def test_pcg_device_buffers(gpu_lib):
    torch = pytest.importorskip("torch")
    m = G.laplacian3d(10, 10, 10)
    n = m.Size
    B = np.stack([build_vector(n, 5), build_vector(n, 6)], axis=1)
    dm = DeviceSymmetricCSRMatrix(m)
    d_b = torch.tensor(B.T.copy(), dtype=torch.float64, device="cuda")
    d_x = torch.zeros_like(d_b)
    torch.cuda.synchronize()
    s = ConjugateGradientGaussPreSolver(RelativeTolerance=1e-10)
    res = s.SolveDevice(dm, d_b.data_ptr(), d_x.data_ptr(), nrhs=2)
    X = d_x.cpu().numpy().T
    assert all(r.Converged for r in res)
    for j in range(2):
        assert relative_residual(m, B[:, j], X[:, j]) < 1e-9
    # the device product
    d_y = torch.zeros_like(d_b)
    dm.MultiplyDevice(d_x.data_ptr(), d_y.data_ptr(), nrhs=2)
    torch.cuda.synchronize()
    Y = d_y.cpu().numpy().T
    assert max_relative_difference(Y[:, 0], oracle.multiply(m, X[:, 0])) < 1e-13


def test_pcg_failures(gpu_lib):
    with pytest.raises(InvalidOperationException):   # zero diagonal (structurally absent)
        ConjugateGradientGaussPreSolver().Solve(LinearSystem(_build(2, [(0, 0, 2.0), (0, 1, 1.0)]), [1.0, 1.0]))
    with pytest.raises(InvalidOperationException):   # p^T A p <= 0
        ConjugateGradientGaussPreSolver().Solve(LinearSystem(_build(2, [(0, 0, -1.0), (1, 1, -2.0)]), [1.0, 1.0]))
    with pytest.raises(ArgumentOutOfRangeException):
        ConjugateGradientGaussPreSolver(MaxIterations=-1).Solve(LinearSystem(_build(1, [(0, 0, 1.0)]), [1.0]))
    m = _build(2, [(0, 0, 1.0), (1, 1, 1.0)])
    with pytest.raises(ArgumentException):
        ConjugateGradientGaussPreSolver().SolveWithInitialGuess(LinearSystem(m, [1.0, 1.0]), [1.0])
    # not converging is a result, not an error
    m = G.laplacian3d(8, 8, 8)
    s = ConjugateGradientGaussPreSolver(RelativeTolerance=1e-14, MaxIterations=3)
    s.Solve(LinearSystem(m, build_vector(m.Size, 1)))
    assert s.LastResult.Iterations == 3 and not s.LastResult.Converged


def test_plan_outlives_its_matrix(gpu_lib):
    """A plan and its matrix are released in either order."""
    m = _build(3, [(0, 0, 4.0), (0, 1, 2.0), (1, 1, 5.0), (2, 2, 9.0)])
    dm = DeviceSymmetricCSRMatrix(m)
    p = dm.AccumulatePlan([0, 1], [1, 1])
    q = dm.LineCrossPlan([2])
    dm.close()
    del p, q
    dm2 = DeviceSymmetricCSRMatrix(m)
    assert np.array_equal(dm2.Values, m.Values)


def test_process_exit_with_live_handles(gpu_lib, tmp_path):
    """A script that keeps matrices, plans and factors in module globals exits cleanly."""
    import subprocess
    import sys
    from pathlib import Path
    root = Path(__file__).resolve().parent.parent
    script = tmp_path / "live.py"
    script.write_text(
        "import sys\n"
        f"sys.path.insert(0, {str(root)!r})\n"
        "import numpy as np\n"
        "import magla_gb300 as mg\n"
        "from magla_gb300 import generators as G\n"
        "m = G.laplacian3d(6, 6, 6)\n"
        "dm = mg.DeviceSymmetricCSRMatrix(m)\n"
        "p = dm.AccumulatePlan([0], [0])\n"
        "q = dm.LineCrossPlan([1])\n"
        "f = mg.SymmetricUtduSolver().Factorize(m)\n"
        "f.RefactorizeFrom(dm)\n"
        "x = mg.ConjugateGradientGaussPreSolver().Solve(mg.LinearSystem(m, np.ones(m.Size)))\n"
        "print('done')\n")
    r = subprocess.run([sys.executable, str(script)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, (r.returncode, r.stderr[-2000:])
    assert "done" in r.stdout


def test_pcg_provided_preconditioner_has_priority(gpu_lib):
    """Tests/CGGP/JacobiPreconditionerTests.cs:38-54: a given preconditioner is reused and wins
    over UsePreconditioner = False (one step each on a diagonal system)."""
    from magla_gb300 import JacobiPreconditioner
    m = _build(3, [(0, 0, 2.0), (1, 1, 4.0), (2, 2, 8.0)])
    pre = JacobiPreconditioner(m)
    s = ConjugateGradientGaussPreSolver(RelativeTolerance=1e-12, UsePreconditioner=False)
    for expected in ([1.0, -2.0, 3.0], [-4.0, 5.0, 0.5]):
        x = s.SolveWithInitialGuess(LinearSystem(m, oracle.multiply(m, np.array(expected))), None, pre)
        assert s.LastResult.Iterations == 1
        assert np.allclose(x, expected, rtol=0, atol=1e-12)
