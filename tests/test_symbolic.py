"""Host symbolic phase: invariants of the reference's tests plus an
independent brute-force check of the elimination tree, column counts,
supernode partition, row patterns and cost statistics.

The reference's tests pin the symbolic phase only through invariants
(permutation validity, fill reduction, estimate consistency —
Tests/UCHOL/SymmetricUtduSolverTests.cs:438-505, :662-686); the brute-force
restatements below follow the definitions in
CAESolvers/UCHOL/EliminationTree.cs and SupernodalStructure.cs.
"""
import numpy as np
import pytest

from magla_gb300 import (ArgumentException, FillReducingOrdering, SymmetricUtduSolver, UtduSolverOptions,
                         UtduSymbolicFactorization)
from magla_gb300 import generators as G
from tests import fixtures as F


def analyze(m, ordering=FillReducingOrdering.ApproximateMinimumDegree, limit=64):
    return UtduSymbolicFactorization.Analyze(m, UtduSolverOptions(Ordering=ordering, SupernodeAmalgamationLimit=limit))


def permuted_lower_sets(m, perm):
    """Strict lower structure of P^T A P, per column, as Python sets."""
    n = m.Size
    inv = np.empty(n, np.int64)
    inv[perm] = np.arange(n)
    cols = [set() for _ in range(n)]
    for r in range(n):
        for k in range(m.RowPointers[r], m.RowPointers[r + 1]):
            c = m.ColumnIndices[k]
            if c == r:
                continue
            a, b = inv[r], inv[c]
            lo, hi = min(a, b), max(a, b)
            cols[lo].add(hi)
    return cols


def brute_force_factor_structure(m, perm):
    n = m.Size
    low = permuted_lower_sets(m, perm)
    struct = [None] * n
    parent = [-1] * n
    children = [[] for _ in range(n)]
    for j in range(n):
        s = set(low[j])
        for c in children[j]:
            s |= struct[c]
        s.discard(j)
        struct[j] = s
        if s:
            parent[j] = min(s)
            children[parent[j]].append(j)
    counts = [len(s) + 1 for s in struct]
    return struct, parent, counts


def supernodes_restated(parent, counts, limit):
    """Fundamental supernodes + relaxed amalgamation, restated from the definitions."""
    n = len(parent)
    nchild = [0] * n
    for j in range(n):
        if parent[j] >= 0:
            nchild[parent[j]] += 1
    starts = [j for j in range(n) if j == 0 or parent[j - 1] != j or nchild[j] > 1 or counts[j - 1] != counts[j] + 1]
    starts.append(n)
    pref = np.concatenate([[0], np.cumsum(counts)])
    bounds, fronts = [], []
    i = 0
    while i < len(starts) - 1:
        first, last = starts[i], starts[i + 1] - 1
        cols = last - first + 1
        front = counts[first]
        nz = pref[last + 1] - pref[first]
        while i + 1 < len(starts) - 1:
            if parent[last] != last + 1:
                break
            nfirst, nlast = starts[i + 1], starts[i + 2] - 1
            mcols = cols + (nlast - nfirst + 1)
            if mcols > limit:
                break
            mfront = cols + counts[nfirst]
            stored = mfront * mcols - mcols * (mcols - 1) // 2
            mnz = nz + (pref[nlast + 1] - pref[nfirst])
            zeros = stored - mnz
            if zeros > 0:
                frac = zeros / stored
                ok = frac <= 0.8 if mcols <= 4 else frac <= 0.1 if mcols <= 16 else frac <= 0.05 if mcols <= 48 else False
                if not ok:
                    break
            last, cols, front, nz = nlast, mcols, mfront, mnz
            i += 1
        bounds.append(first)
        fronts.append(front)
        i += 1
    bounds.append(n)
    return bounds, fronts


CASES = {
    "grid_4x3x3_dof2": lambda: G.grid_matrix(4, 3, 3, 2),
    "grid_5x5x5_dof1": lambda: G.grid_matrix(5, 5, 5, 1),
    "elasticity_3x3x3": lambda: G.elasticity(3, 3, 3)[0],
    "random_120": lambda: F.random_matrix(120, 0.04, 4),
    "random_60_dense": lambda: F.random_matrix(60, 0.5, 9),
    "star": lambda: F.star(80),
    "two_chains": F.two_chains,
    "tridiagonal": lambda: F.tridiagonal(50),
}


@pytest.mark.parametrize("case", sorted(CASES))
@pytest.mark.parametrize("ordering", [FillReducingOrdering.ApproximateMinimumDegree, FillReducingOrdering.Natural])
def test_structures_match_brute_force(case, ordering):
    m = CASES[case]()
    sym = analyze(m, ordering)
    a = sym.arrays
    perm = a["PERMUTATION"]
    n = m.Size
    assert sorted(perm.tolist()) == list(range(n))
    assert np.array_equal(a["INVERSE_PERMUTATION"][perm], np.arange(n))
    struct, parent, counts = brute_force_factor_structure(m, perm)
    assert a["ETREE_PARENT"].tolist() == parent
    assert a["COLUMN_COUNTS"].tolist() == counts
    # postordered: every parent follows its child
    assert all(p == -1 or p > j for j, p in enumerate(parent))
    assert sym.StrictFactorNonZeroCount == sum(counts)
    bounds, fronts = supernodes_restated(parent, counts, 64)
    assert a["FIRST_COLUMN"].tolist() == bounds
    fp = a["FRONT_PTR"]
    assert np.diff(fp).tolist() == fronts
    # row pattern of each supernode = its columns + union of its columns' structures
    rows = a["FRONT_ROWS"]
    entries = ops = 0
    for s in range(len(bounds) - 1):
        cols = range(bounds[s], bounds[s + 1])
        expect = set(cols)
        for j in cols:
            expect |= struct[j]
        assert rows[fp[s]:fp[s + 1]].tolist() == sorted(expect)
        mm, w = fp[s + 1] - fp[s], bounds[s + 1] - bounds[s]
        entries += mm * w - w * (w - 1) // 2
        ops += sum((mm - k) ** 2 for k in range(w))
    assert sym.FactorEntryCount == entries
    assert sym.FactorOperationCount == ops
    # assembly tree parent = supernode holding the parent of the last column
    snof = a["SUPERNODE_OF"]
    for s in range(len(bounds) - 1):
        pc = parent[bounds[s + 1] - 1]
        assert a["SN_PARENT"][s] == (-1 if pc < 0 else snof[pc])


def test_peak_contribution_restated():
    m = G.grid_matrix(6, 5, 4, 2)
    sym = analyze(m)
    a = sym.arrays
    fp, fc, cp, ch = a["FRONT_PTR"], a["FIRST_COLUMN"], a["CHILD_PTR"], a["CHILDREN"]
    live = peak = 0
    contrib = {}
    for s in range(sym.SupernodeCount):
        mm, w = fp[s + 1] - fp[s], fc[s + 1] - fc[s]
        peak = max(peak, live + mm * (mm + 1) // 2)
        for c in ch[cp[s]:cp[s + 1]]:
            live -= contrib[c]
        t = mm - w
        contrib[s] = t * (t + 1) // 2
        live += contrib[s]
        peak = max(peak, live)
    assert sym.PeakContributionBytes == peak * 8


@pytest.mark.parametrize("scenario", ["grid", "random", "diagonal", "two_chains"])
def test_amd_produces_valid_permutation(scenario):
    m = {"grid": lambda: G.grid_matrix(7, 6, 5, 2), "random": lambda: F.random_matrix(250, 0.02, 99),
         "diagonal": lambda: F.diagonal([float(i) for i in range(1, 61)]), "two_chains": F.two_chains}[scenario]()
    sym = analyze(m)
    assert sorted(sym.Permutation.tolist()) == list(range(m.Size))


def test_amd_isolated_vertices_in_index_order():
    sym = analyze(F.diagonal([float(i) for i in range(1, 61)]))
    assert sym.Permutation.tolist() == list(range(60))


def test_amd_dense_row_ordered_last():
    # the star centre has degree 299 > max(16, 10 sqrt(300)) = 173, so AMD defers it
    from magla_gb300 import _native
    import ctypes as C
    m = F.star(300)
    perm = np.zeros(300, np.int32)
    lib = _native.host()
    st = lib.uchol_amd_order(300, _native.ptr(m.RowPointers), _native.ptr(m.ColumnIndices), _native.ptr(perm))
    assert st == 0
    assert perm[-1] == 0


def test_amd_reduces_fill_compared_to_natural():
    m = G.grid_matrix(12, 12, 12, 1)
    nat = analyze(m, FillReducingOrdering.Natural)
    amd = analyze(m)
    assert amd.StrictFactorNonZeroCount * 2 < nat.StrictFactorNonZeroCount
    assert amd.FactorEntryCount < amd.StrictFactorNonZeroCount * 1.2


def test_amd_is_deterministic():
    m = F.random_matrix(300, 0.03, 12)
    assert np.array_equal(analyze(m).Permutation, analyze(m).Permutation)


def test_consistent_cost_estimates():
    m = G.grid_matrix(10, 10, 10, 2)
    sym = SymmetricUtduSolver().Analyze(m)
    assert sym.Size == m.Size
    assert sym.SupernodeCount > 0
    assert sym.StrictFactorNonZeroCount >= m.NonZeroCount
    assert sym.FactorEntryCount >= sym.StrictFactorNonZeroCount
    assert sym.FactorEntryCount * 8 == sym.EstimatedFactorBytes
    assert sym.EstimatePeakBytes(4) > sym.EstimatedFactorBytes
    assert sym.FactorOperationCount > sym.StrictFactorNonZeroCount
    assert 0 < sym.MaxFrontSize <= m.Size
    assert sorted(sym.Permutation.tolist()) == list(range(m.Size))
    for k in range(sym.Size):
        assert sym.InversePermutation[sym.Permutation[k]] == k


def test_ensure_compatible():
    sym = analyze(F.tridiagonal(100))
    with pytest.raises(ArgumentException):
        sym.EnsureCompatible(G.grid_matrix(5, 5, 4, 1))
    with pytest.raises(ArgumentException):
        sym.EnsureCompatible(F.tridiagonal(101))
    sym.EnsureCompatible(F.tridiagonal(100))


def test_empty_matrix():
    sym = analyze(F.diagonal([]))
    assert sym.Size == 0 and sym.SupernodeCount == 0 and sym.FactorEntryCount == 0
