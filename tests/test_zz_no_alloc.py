"""uchol_residual_norms_static: the residual check for callers that cannot
allocate device memory (an application owning all device memory through its
own pool, a caller recording a CUDA stream capture, a loop that must not
take an allocation's synchronisation).  Its output must match the
allocating entry point uchol_residual_norms on two calls in a row (the
static scratch keeps the previous call's contents), and sizes beyond its
static scratch must be refused with a clear error.

Collected last so that a run stopping at the first failure has already run
every other test.
"""
import ctypes as C

import numpy as np
import pytest

from magla_gb300 import SymmetricUtduSolver, _native
from magla_gb300 import generators as G
from tests.conftest import build_vector

pytestmark = pytest.mark.gpu


def test_static_scratch_residual_matches_allocating_entry_point(gpu_lib):
    torch = pytest.importorskip("torch")
    lib = gpu_lib
    m = G.elasticity(6, 6, 6)[0]
    n, nnz, nrhs = m.Size, m.NonZeroCount, 3
    f = SymmetricUtduSolver().Factorize(m)
    B = np.stack([build_vector(n, 60 + k) for k in range(nrhs)], axis=1)
    # a residual well above round-off, so the two summation orders agree to 1e-12
    X = f.Solve(B) + np.stack([build_vector(n, 80 + k) for k in range(nrhs)], axis=1) * 1e-3
    expected = f.DeviceResidualNorms(B, X)

    dev = torch.device("cuda")
    d_rp = torch.tensor(m.RowPointers, dtype=torch.int32, device=dev)
    d_col = torch.tensor(m.ColumnIndices, dtype=torch.int32, device=dev)
    d_val = torch.tensor(m.Values, dtype=torch.float64, device=dev)
    d_b = torch.tensor(B.T.copy(), dtype=torch.float64, device=dev)   # column j at offset j * n
    d_x = torch.tensor(X.T.copy(), dtype=torch.float64, device=dev)
    d_out = torch.zeros(nrhs, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    for call in range(2):
        d_out.fill_(-1.0)
        st = lib.uchol_residual_norms_static(n, nnz, nrhs, d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                                             d_b.data_ptr(), n, d_x.data_ptr(), n, d_out.data_ptr(), None)
        assert st == _native.OK, lib.uchol_residual_norms_static_error()
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert np.allclose(got, expected, rtol=1e-12, atol=0), (call, got, expected)


def test_static_scratch_with_padded_leading_dimensions(gpu_lib):
    """b and x with leading dimension n + 3 (the padding holds values that must not be read)."""
    torch = pytest.importorskip("torch")
    lib = gpu_lib
    m = G.elasticity(5, 5, 5)[0]
    n, nnz, nrhs, ld = m.Size, m.NonZeroCount, 2, m.Size + 3
    f = SymmetricUtduSolver().Factorize(m)
    B = np.stack([build_vector(n, 90 + k) for k in range(nrhs)], axis=1)
    X = f.Solve(B) + np.stack([build_vector(n, 95 + k) for k in range(nrhs)], axis=1) * 1e-3
    expected = f.DeviceResidualNorms(B, X)
    Bp = np.full((ld, nrhs), 1e30)
    Xp = np.full((ld, nrhs), 1e30)
    Bp[:n], Xp[:n] = B, X
    dev = torch.device("cuda")
    d_rp = torch.tensor(m.RowPointers, dtype=torch.int32, device=dev)
    d_col = torch.tensor(m.ColumnIndices, dtype=torch.int32, device=dev)
    d_val = torch.tensor(m.Values, dtype=torch.float64, device=dev)
    d_b = torch.tensor(Bp.T.copy(), dtype=torch.float64, device=dev)   # column j at offset j * ld
    d_x = torch.tensor(Xp.T.copy(), dtype=torch.float64, device=dev)
    d_out = torch.zeros(nrhs, dtype=torch.float64, device=dev)
    torch.cuda.synchronize()
    for call in range(2):
        st = lib.uchol_residual_norms_static(n, nnz, nrhs, d_rp.data_ptr(), d_col.data_ptr(), d_val.data_ptr(),
                                             d_b.data_ptr(), ld, d_x.data_ptr(), ld, d_out.data_ptr(), None)
        assert st == _native.OK, lib.uchol_residual_norms_static_error()
        torch.cuda.synchronize()
        assert np.allclose(d_out.cpu().numpy(), expected, rtol=1e-12, atol=0), call


def test_static_scratch_rejects_sizes_beyond_its_maximum(gpu_lib):
    torch = pytest.importorskip("torch")
    lib = gpu_lib
    d = torch.zeros(16, dtype=torch.float64, device="cuda")
    too_big = 1 << 20
    st = lib.uchol_residual_norms_static(too_big, 1, 1, d.data_ptr(), d.data_ptr(), d.data_ptr(), d.data_ptr(),
                                         too_big, d.data_ptr(), too_big, d.data_ptr(), None)
    assert st == _native.BAD_ARG
    assert b"exceeds the static scratch" in lib.uchol_residual_norms_static_error()
    st = lib.uchol_residual_norms_static(4, 4, 65, d.data_ptr(), d.data_ptr(), d.data_ptr(), d.data_ptr(), 4,
                                         d.data_ptr(), 4, d.data_ptr(), None)
    assert st == _native.BAD_ARG
