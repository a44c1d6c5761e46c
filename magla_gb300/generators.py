"""Seeded synthetic matrices: the reference's FEM-like grid matrix, 2D/3D
Laplacians, Q1 hexahedral elasticity and random diagonally dominant
matrices.  All go through the reference's construction rules."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native
from .errors import raise_for_status
from .matrix import SymmetricCSRMatrix


def _adopt(st, h):
    lib = _native.host()
    raise_for_status(st, lib.uchol_host_last_error())
    return SymmetricCSRMatrix._from_handle(h)


def grid_matrix(nx: int, ny: int, nz: int, dof: int) -> SymmetricCSRMatrix:
    """BuildGridMatrix of the reference (UtduSolverBenchmark.cs:220-261)."""
    h = C.c_void_p()
    return _adopt(_native.host().uchol_csr_grid(nx, ny, nz, dof, C.byref(h)), h)


def laplacian3d(nx: int, ny: int, nz: int) -> SymmetricCSRMatrix:
    """7-point Laplacian on the interior nodes (Dirichlet eliminated)."""
    h = C.c_void_p()
    return _adopt(_native.host().uchol_csr_laplacian3d(nx, ny, nz, C.byref(h)), h)


def laplacian2d(n: int, stencil: int = 5, shift=None) -> SymmetricCSRMatrix:
    """2D Laplacian on an n x n grid (5- or 9-point stencil, Dirichlet boundary
    eliminated); ``shift`` (a scalar or one value per node) is added to the diagonal."""
    if stencil not in (5, 9):
        raise ValueError("stencil must be 5 or 9")
    h = C.c_void_p()
    s = None
    if shift is not None:
        s = np.ascontiguousarray(np.broadcast_to(np.asarray(shift, np.float64), (n * n,)))
    return _adopt(_native.host().uchol_csr_laplacian2d(n, stencil, _native.ptr(s, C.c_double), C.byref(h)), h)


def laplacian2d_batch(count: int = 256, seed: int = 4, n_range=(16, 128)):
    """Independent 2D Laplacian systems: grid edge n uniform in n_range, 5- or
    9-point stencil chosen at random, diagonal plus uniform[0, 0.1] per node."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        n = int(rng.integers(n_range[0], n_range[1] + 1))
        stencil = 5 if rng.random() < 0.5 else 9
        out.append(laplacian2d(n, stencil, rng.uniform(0.0, 0.1, n * n)))
    return out


def elasticity(ex: int, ey: int, ez: int, youngs=None, nu: float = 0.3, clamp: bool = True):
    """Q1 hexahedral elasticity on unit cubes, face z = 0 clamped with LineCross
    semantics; returns (matrix, body_load) with the consistent load of a unit
    body force in -z."""
    n = 3 * (ex + 1) * (ey + 1) * (ez + 1)
    load = np.zeros(n, np.float64)
    E = None if youngs is None else np.ascontiguousarray(youngs, np.float64)
    if E is not None and E.shape[0] != ex * ey * ez:
        raise ValueError("one Young's modulus per element is required")
    h = C.c_void_p()
    st = _native.host().uchol_csr_elasticity(ex, ey, ez, _native.ptr(E, C.c_double), float(nu), 1 if clamp else 0,
                                             _native.ptr(load, C.c_double), C.byref(h))
    return _adopt(st, h), load


def random_spd(n: int, density: float, rng: np.random.Generator) -> SymmetricCSRMatrix:
    """Random structure, values U[-1,1], strictly dominant diagonal (|offdiag| row sums + 1),
    the construction of the reference test's BuildRandomMatrix with this generator."""
    iu, ju = np.triu_indices(n, 1)
    keep = rng.random(iu.shape[0]) < density
    iu, ju = iu[keep], ju[keep]
    v = rng.random(iu.shape[0]) * 2.0 - 1.0
    off = np.zeros(n)
    np.add.at(off, iu, np.abs(v))
    np.add.at(off, ju, np.abs(v))
    rows = np.concatenate([iu, np.arange(n)]).astype(np.int32)
    cols = np.concatenate([ju, np.arange(n)]).astype(np.int32)
    vals = np.concatenate([v, off + 1.0])
    return SymmetricCSRMatrix.from_triplets(n, rows, cols, vals)


def log_uniform_youngs(elements: int, lo: float, hi: float, rng: np.random.Generator) -> np.ndarray:
    return np.exp(rng.uniform(np.log(lo), np.log(hi), elements))
