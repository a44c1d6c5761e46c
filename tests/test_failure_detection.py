"""Failure detection without a GPU fault: bounded device waits that run out, and a device
memory budget checked before anything is allocated.

The level solves wait on flags and counters that other CTAs publish; every wait is
bounded (uchol_set_wait_limits).  uchol_check_solve_wait runs a real level-solve launch
with its bulk CTAs withheld, so a chain waits on a counter that nothing publishes: the
wait must expire, the call must report UCHOL_TIMEOUT, and the factor and the device must
stay usable (a normal solve and a new factorisation then match the oracle)."""
import ctypes as C

import numpy as np
import pytest

import oracle
from magla_gb300 import SymmetricUtduSolver, UtduSolverOptions, _native
from magla_gb300 import generators as G
from magla_gb300.errors import DeviceOutOfMemoryError, DeviceWaitTimeoutError, raise_for_status
from tests.conftest import build_vector, max_relative_difference


def _laplacian():
    # AMD on the 16^3 Laplacian: a root separator of 256 columns, four FP64 solve blocks
    return G.laplacian3d(16, 16, 16)


def test_budget_rejects_a_plan_on_the_host():
    m = _laplacian()
    sym = SymmetricUtduSolver().Analyze(m)
    need = sym.EstimateDeviceBytes()
    assert need["factor"] > 0
    with pytest.raises(DeviceOutOfMemoryError, match="budget"):
        sym.EstimateDeviceBytes(UtduSolverOptions(DeviceMemoryBudget=1024))
    sym.EstimateDeviceBytes(UtduSolverOptions(DeviceMemoryBudget=1 << 40))


@pytest.mark.gpu
def test_budget_fails_before_allocation_then_factorisation_works(gpu_lib):
    m = _laplacian()
    with pytest.raises(DeviceOutOfMemoryError, match="budget"):
        SymmetricUtduSolver(UtduSolverOptions(DeviceMemoryBudget=1 << 20)).Factorize(m)
    f = SymmetricUtduSolver(UtduSolverOptions(DeviceMemoryBudget=1 << 40)).Factorize(m)
    b = build_vector(m.Size, 3)
    of = oracle.OracleFactor(f.Symbolic, m.Values)
    assert max_relative_difference(f.Solve(b), of.Solve(b)) < 1e-12


@pytest.mark.gpu
def test_expired_solve_wait_reports_timeout_and_leaves_the_device_usable(gpu_lib):
    lib = _native.gpu()
    m = _laplacian()
    b = build_vector(m.Size, 5)
    s = SymmetricUtduSolver(UtduSolverOptions(InverseBlockWidth=-1))
    f = s.Factorize(m)
    st = lib.uchol_check_solve_wait(f._h, 2.0)
    assert st == _native.TIMEOUT, lib.uchol_last_error()
    with pytest.raises(DeviceWaitTimeoutError):
        raise_for_status(st, lib.uchol_last_error())
    # the same factor, and a new factorisation, still solve correctly
    of = oracle.OracleFactor(f.Symbolic, m.Values)
    xo = of.Solve(b)
    assert max_relative_difference(f.Solve(b), xo) < 1e-12
    assert max_relative_difference(s.Factorize(m).Solve(b), xo) < 1e-12


@pytest.mark.gpu
def test_wait_limits_can_be_set_and_restored(gpu_lib):
    lib = _native.gpu()
    raise_for_status(lib.uchol_set_wait_limits(500.0, 1000.0), lib.uchol_last_error())
    m = _laplacian()
    b = build_vector(m.Size, 6)
    f = SymmetricUtduSolver().Factorize(m)
    x = f.Solve(b)
    raise_for_status(lib.uchol_set_wait_limits(0.0, 0.0), lib.uchol_last_error())   # defaults
    of = oracle.OracleFactor(f.Symbolic, m.Values)
    assert max_relative_difference(x, of.Solve(b)) < 1e-12
